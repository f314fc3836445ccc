// Host-side declarations shared by the libnbkdt translation units.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/nbkdt.h"
#include "nbk_internal.cuh"

#define NBK_TRY(expr)              \
  do {                             \
    int _s = (expr);               \
    if (_s != NBK_OK) return _s;   \
  } while (0)

namespace nbk {

constexpr int kLocalMax = 1024;  // subtrees up to this size finish in one CTA

// One tree of a forest: particles [pstart, pstart+n) in both input and tree order, nodes
// at [nbase, nbase + heap_slots(n, b)).
struct TreeSpec {
  int64_t pstart, n;
  int nbase;
};

struct BuiltArrays {
  P4* pos = nullptr;
  float4* posf = nullptr;
  V4* vel = nullptr;
  int* perm = nullptr;
  NodeRec* node = nullptr;    // physical / velocity trees
  NodeX* nodex = nullptr;
  NodeS* nodes6 = nullptr;    // phase-space trees
  NodeB6* nodeb6 = nullptr;
  NodeF6* nodef6 = nullptr;
  float4* velf = nullptr;
};

// Stream-ordered device allocations. Scratch allocations made through get() are freed
// together by release_all_scratch(); the device's default memory pool keeps the memory
// cached, so repeated builds do not return to the driver.
// One device allocation carved into several arrays, each starting on a 256-byte boundary
// (one call to the allocator instead of one per array).
struct DevPart {
  void** p;
  size_t bytes;
};
size_t block_bytes(const std::vector<DevPart>& parts);
void carve_block(void* base, const std::vector<DevPart>& parts);
struct DevAlloc;
// A scratch block kept per host thread and slot (0: tree build, 1: FOF labels, 2: FOF
// union-find arrays) for calls that synchronise their stream before they return; blocks
// above 256 MB, or any request when the slot is unusable, come from `fallback` instead.
int thread_scratch_block(int slot, const std::vector<DevPart>& parts, cudaStream_t st,
                         DevAlloc& fallback);
// Waits for the stream when a call leaves early (ok not set): its kernels may still use a
// kept scratch block that the thread's next call would reuse.
struct SyncUnlessOk {
  cudaStream_t st;
  bool ok = false;
  ~SyncUnlessOk() {
    if (!ok) cudaStreamSynchronize(st);
  }
};

struct DevAlloc {
  std::vector<void*> scratch;
  cudaStream_t st = nullptr;
  int get(void** p, size_t bytes);
  int get_block(const std::vector<DevPart>& parts);
  int upload(void* dst, const void* src, size_t bytes, cudaStream_t s);
  void release_all_scratch(cudaStream_t s);
  ~DevAlloc();
};
int dev_malloc(void** p, size_t bytes, cudaStream_t st);
void dev_free(void* p, cudaStream_t st);
// Raise a kernel's dynamic shared-memory limit to `bytes` on the current device (once per
// device and kernel; the attribute is per device).
int ensure_dyn_smem(const void* func, int bytes);
// Test hook behind nbk_debug_set_iteration_cap (fof.cu).
int set_uf_iteration_cap(int cap);

int64_t heap_slots(int64_t n, int b);
int64_t count_nodes(int64_t n, int b);
size_t local_build_smem(int nd = 3);
// Builds every tree of the forest; if root_out is given, the first tree's root node
// (exact bounding box) is copied there before the build's final synchronisation.
int build_forest(const std::vector<TreeSpec>& trees, int b, const double* d_pos_in,
                 const double* d_mass_in, const double* d_vel_in, BuiltArrays& out,
                 DevAlloc& alloc, cudaStream_t st, NodeX* root_out = nullptr);
// The phase-space tree (KDTree with TreeType TPHS): the same rules over the six
// coordinates (x, y, z, vx, vy, vz); d_vel_in is required. Fills pos, posf, vel, velf,
// perm, nodes6, nodeb6 and nodef6; root_out receives the root's exact box.
int build_forest_phase(const std::vector<TreeSpec>& trees, int b, const double* d_pos_in,
                       const double* d_mass_in, const double* d_vel_in, BuiltArrays& out,
                       DevAlloc& alloc, cudaStream_t st, NodeB6* root_out = nullptr);

// ---- kNN family
enum Epi : int {
  kEpiNN = 0,          // neighbour lists
  kEpiDensity = 1,     // CalcDensity scatter
  kEpiDensVel = 2,     // CalcDensity + CalcVelDensity from one search
  kEpiVel = 3,         // CalcVelDensity
  kEpiDensPart = 4,    // CalcDensityParticle (gather only)
  kEpiVelPart = 5,     // CalcVelDensityParticle
  kEpiDensSave = 6,    // CalcDensity scatter + save neighbour lists (adjoint forward)
};

struct KnnArgs {
  TreeView tv;
  int kheap;          // heap size (k, or k+1 for periodic searches)
  int kout;           // entries per output row
  int drop_largest;   // pop the largest entry before writing (periodic FindNearestPos)
  int exclude_self;   // target search: skip the query itself and zero distances
  int periodic;       // search mirror images
  int min_image;      // image gates: 0 = the reference's, 1 = corrected
  int qmode;          // 0: tree particles [q0, q0+nq), 1: coordinates qx, 2: targets qidx
  int q0;
  int nq;
  const double* qx;
  const int* qidx;
  int nsmooth;
  const double* kernel;
  int kernres;
  int* nn;            // nq x kout
  double* d2;
  double* rho;        // tree order (scatter) or query order (particle variants)
  double* vden;
  int* err;
  const double* qv;   // query velocities of coordinate queries (CalcVelDensityPosition)
};
int launch_knn(const KnnArgs& a, int epi, cudaStream_t st);

// ---- phase-space trees (phase.cu)
enum PhaseEpi : int {
  kPhNN = 0,        // FindNearest(tt) / FindNearest(x): neighbour lists
  kPhDensity = 1,   // CalcDensity scatter (tree order)
  kPhDensPart = 2,  // CalcDensityParticle (query order)
};
struct PhaseArgs {
  KnnArgs k;             // queries (qmode 0 / 1 with 6 values per point / 2), heap, outputs;
                         // k.periodic: search the position images (ungated)
  int metric;            // 1: local metric (Aniso 0), 0: plain phase distance (Aniso -1)
  int spacing_periodic;  // the metric spacing searches the images (FindNearest's copy)
  int epi;               // PhaseEpi
};
int launch_phase(const PhaseArgs& a, cudaStream_t st);

// ---- SPH smoothing over the nearest neighbours (smooth.cu)
enum Smooth : int {
  kSmVel = 0,          // CalcSmoothVel (symmetric, every particle)
  kSmVelDisp = 1,      // CalcSmoothVelDisp
  kSmVelSkew = 2,      // CalcSmoothVelSkew
  kSmVelKurt = 3,      // CalcSmoothVelKurtosis
  kSmVelPhys = 4,      // CalcVelDensityWithPhysDensity[Particle]
  kSmVelOne = 5,       // CalcSmoothVel{Particle,Position}
  kSmVelDispOne = 6,   // CalcSmoothVelDisp{Particle,Position}
  kSmMeanOne = 7,      // CalcSmoothLocalMean{Particle,Position}
  kSmDispOne = 8,      // CalcSmoothLocalDisp{Particle,Position}
};
struct SmoothArgs {
  KnnArgs k;              // the search: queries, heap size (Nsmooth, or Nsearch for kSmVelPhys)
  int nsmooth;
  const double* rho;      // densities, input order
  const double* smvel;    // input order [n][3] (every-particle forms) or query order [nq][3]
  const double* disp;     // input order [n][9]
  const double* weight;   // input order [n]
  const double* mean;     // query order [nq]
  double* out;            // input order (every-particle forms, zeroed) or query order
};
int launch_smooth(const SmoothArgs& s, int which, cudaStream_t st);

// ---- batched path: many trees, one persistent launch
struct WorkItem {
  int tree, q0, count, pad;  // queries [q0, q0+count) of tree `tree`
};
struct TreeInfo {
  int pstart, n, nbase, pad;
};
struct BatchArgs {
  const WorkItem* items;
  const TreeInfo* trees;
  int nitems;
  int* counter;         // zeroed before each launch
  int warp_per_query;   // 1: a warp serves one query at a time; 0: a lane per query
};
// Density of every particle of every tree (a.kheap = k, clamped per tree to n-1).
int launch_knn_batch(const KnnArgs& a, const BatchArgs& b, cudaStream_t st);

// ---- FOF / ball / adjoint
struct FofArgs {
  TreeView tv;
  double ll2;          // linking length squared
  int crit;            // 0: plain FOF, 1: FOFCriterion, 2: FOFNN[Dist]Criterion
  int cmp;             // comparator for crit
  double params[8];
  int* parent;         // tree order union-find forest
  int* err;
  const int* nn;       // crit 2: neighbour lists, [n][numnn] tree indices (row = tree index)
  int numnn;
  const double* pval;  // crit 2, FOFNNDistCriterion: per-particle value (tree order) for
  int npc;             //   params[pidx[0..npc)]
  int pidx[8];
  int crit_contained;  // crit 1: every pair the comparator accepts lies inside the search
                       //   region (FOF3d / FOF6d with params[6] <= the position search
                       //   distance^2), so reachability follows from the comparator
};
int run_fof(const FofArgs& a, int nnodes, int minnum, int order, int* d_group_tree,
            int* h_ngroup, DevAlloc& alloc, cudaStream_t st,
            bool defer_count = false);

int run_ball(const TreeView& tv, int qmode, const int* qidx, const double* qx, int nq,
             double fdist2, int exclude_self, int64_t* d_offsets, int* d_out,
             int64_t out_capacity, int64_t* h_total, DevAlloc& alloc, cudaStream_t st);
int run_ball_mark(const TreeView& tv, int target, double fdist2, int imark, int* d_mark,
                  double* d_dist2, const int* d_perm, int target_search, cudaStream_t st);

// d_w_tree is overwritten with w / rho; d_slope holds kernres doubles of scratch.
int run_density_adjoint(const TreeView& tv, int k, const int* d_nn, double* d_w_tree,
                        const double* d_rho_tree, const double* kernel, int kernres,
                        double* d_slope, double* d_gpos_tree, double* d_gmass_tree,
                        cudaStream_t st);

void kernel_table(int kerntype, int kernres, int nd, std::vector<double>& T, double& norm);
void kernel_device_image(const std::vector<double>& T, std::vector<double>& img);

// permutation helpers
int scatter_to_input_order(const double* tree_vals, const int* perm, double* out, int64_t n,
                           int stride, cudaStream_t st);

}  // namespace nbk
