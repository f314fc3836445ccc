// k-nearest-neighbour search and the SPH quantities built on it.
//
// Replaces the recursive depth-first search of SplitNode/LeafNode::FindNearestPos
// (src/KDTree/KDSplitNode.cxx:15-41, 206-231; KDLeafNode.cxx:15-28, 119-130), its periodic
// wrapper (KDSplitNode.cxx:1119-1147) and the per-particle loops of CalcDensity,
// CalcVelDensity, CalcDensityParticle and CalcVelDensityParticle
// (KDCalcSmoothQuantities.cxx:203-389, 768-920).
//
// Work mapping: one warp serves 32 queries that are consecutive in tree order, so they
// sit in one or two neighbouring leaves and want nearly the same nodes. The warp walks
// the tree once for all of them (a node is opened when any lane still needs it), stages
// each opened leaf's particles in shared memory, and every lane tests them against its
// own query. Each lane keeps a bounded max-heap of (d2, index) in shared memory.
//
// Exactness: node pruning and the first candidate test use FP32 lower bounds computed
// with directed rounding from FP32 copies of the coordinates, so they never reject what
// the FP64 test would accept; a candidate that survives is tested in FP64 with the
// reference's arithmetic, d2 = ((dx*dx + dy*dy) + dz*dz), and accepted when d2 < top
// (strict, as the reference's `dist2 < pq->TopPriority()`).
#include <algorithm>

#include "nbk_build.h"

namespace nbk {

namespace {

constexpr int kStack = 64;

template <int KMAX>
struct WarpSmem {
  double hd[KMAX][32];
  int hi[KMAX][32];
  float4 sf[32];  // FP32 copies of the staged leaf particles (the exact ones stay in L1)
  int stk[kStack];
};

template <int KMAX>
__device__ __forceinline__ void heap_sift(WarpSmem<KMAX>& w, int lane, int K, int pos, double d,
                                          int j) {
  while (true) {
    int c = 2 * pos + 1;
    if (c >= K) break;
    double dc = w.hd[c][lane];
    if (c + 1 < K) {
      double dc2 = w.hd[c + 1][lane];
      if (dkey(dc2) > dkey(dc)) {
        c = c + 1;
        dc = dc2;
      }
    }
    if (dkey(d) >= dkey(dc)) break;
    w.hd[pos][lane] = dc;
    w.hi[pos][lane] = w.hi[c][lane];
    pos = c;
  }
  w.hd[pos][lane] = d;
  w.hi[pos][lane] = j;
}

// Remove the root of a heap of size K (returns it).
template <int KMAX>
__device__ __forceinline__ void heap_pop(WarpSmem<KMAX>& w, int lane, int K, double& d, int& j) {
  d = w.hd[0][lane];
  j = w.hi[0][lane];
  double ld = w.hd[K - 1][lane];
  int lj = w.hi[K - 1][lane];
  if (K - 1 > 0) heap_sift<KMAX>(w, lane, K - 1, 0, ld, lj);
}

template <int KMAX>
__device__ void traverse(const TreeView& tv, WarpSmem<KMAX>& w, int lane, bool active,
                         const double xq[3], int self, bool exclude_self, int K, double& top,
                         int* err) {
  const unsigned FULL = 0xffffffffu;
  float qx = __double2float_rn(xq[0]), qy = __double2float_rn(xq[1]),
        qz = __double2float_rn(xq[2]);
  float eps = tv.eps, two_eps = __fmul_ru(2.f, tv.eps);
  long long topk = dkey(top);
  float thr = thresh_hi_bits(topk);
  int sp = 0;
  if (lane == 0) w.stk[0] = 0;
  sp = 1;
  __syncwarp();
  while (sp > 0) {
    int h = w.stk[sp - 1];
    sp--;
    __syncwarp();
    NodeRec r = tv.node[tv.nbase + h];
    bool need = active && box_d2_lo(qx, qy, qz, eps, r) < thr;
    unsigned want = __ballot_sync(FULL, need);
    if (!want) continue;
    if (r.count <= tv.b) {
      for (int c0 = 0; c0 < r.count; c0 += 32) {
        int m = min(32, r.count - c0);
        if (lane < m) w.sf[lane] = tv.posf[r.start + c0 + lane];
        __syncwarp();
        if (need) {
          for (int j = 0; j < m; j++) {
            float4 cf = w.sf[j];
            if (pair_d2_lo(qx, qy, qz, cf.x, cf.y, cf.z, two_eps) < thr) {
              int ti = r.start + c0 + j;
              P4 c = tv.pos[ti];
              double d2 = dist2_exact(xq[0], xq[1], xq[2], c.x, c.y, c.z);
              long long dk = dkey(d2);
              bool ok = dk < topk;  // d2 < top
              if (exclude_self) ok = ok && ti != self && dk != 0;
              if (ok) {
                heap_sift<KMAX>(w, lane, K, 0, d2, ti);
                top = w.hd[0][lane];
                topk = dkey(top);
                thr = thresh_hi_bits(topk);
              }
            }
          }
        }
        __syncwarp();
      }
    } else {
      int hl = 2 * h + 1, hr = 2 * h + 2;
      NodeRec rl = tv.node[tv.nbase + hl], rr = tv.node[tv.nbase + hr];
      float dl = active ? box_d2_lo(qx, qy, qz, eps, rl) : FLT_MAX;
      float dr = active ? box_d2_lo(qx, qy, qz, eps, rr) : FLT_MAX;
      bool nl = active && dl < thr, nr = active && dr < thr;
      unsigned bl = __ballot_sync(FULL, nl), br = __ballot_sync(FULL, nr);
      int leader = __ffs(want) - 1;
      float dl0 = __shfl_sync(FULL, dl, leader), dr0 = __shfl_sync(FULL, dr, leader);
      if (sp + 2 > kStack) {
        if (lane == 0) atomicExch(err, kErrCapacity);
        return;
      }
      // push the farther child first so the nearer one is opened first
      int first = dl0 <= dr0 ? hr : hl, second = dl0 <= dr0 ? hl : hr;
      bool firstneed = dl0 <= dr0 ? (br != 0) : (bl != 0);
      bool secondneed = dl0 <= dr0 ? (bl != 0) : (br != 0);
      if (lane == 0) {
        if (firstneed) w.stk[sp] = first;
      }
      if (firstneed) sp++;
      if (lane == 0) {
        if (secondneed) w.stk[sp] = second;
      }
      if (secondneed) sp++;
      __syncwarp();
    }
  }
}

// One warp's work: up to 32 queries of one tree (lane = query). `qslot` indexes the
// per-query outputs, `self` is the query's tree index (-1 for a coordinate query), K the
// heap size. All lanes of the warp call this together.
template <int KMAX, int EPI>
__device__ void run_warp(const KnnArgs& a, const TreeView& tv, WarpSmem<KMAX>& w, int lane,
                         bool valid, int qi, int self, const double x0[3], int K) {
  for (int s = 0; s < K; s++) {
    w.hd[s][lane] = kMaxValue;
    w.hi[s][lane] = -1;
  }
  double top = kMaxValue;
  __syncwarp();
  int npass = a.periodic ? 8 : 1;
  int near_sq = 7, near_lin = 7;  // walls an image gate could still open across
  for (int pass = 0; pass < npass; pass++) {
    double xq[3];
    bool gate = valid;
    if (pass == 0) {
      xq[0] = x0[0];
      xq[1] = x0[1];
      xq[2] = x0[2];
    } else {
      if (pass == 1 && valid) {
        // top only shrinks from here on, so walls ruled out now stay ruled out: the
        // sqrt(top) > sval gates need a wall closer than sqrt(top), the top > sval gates
        // (2-D and 3-D images of the reference mode) one closer than top
        float4 qf = make_float4(__double2float_rn(x0[0]), __double2float_rn(x0[1]),
                                __double2float_rn(x0[2]), 0.f);
        float top_hi = thresh_hi_bits(dkey(top));
        near_sq = near_walls(qf, tv.period, tv.eps, top_hi);
        near_lin = near_walls_lin(qf, tv.period, tv.eps, top_hi);
      }
      int m = kImageMask[pass];
      bool may = (m & ~((pass <= 3 || a.min_image) ? near_sq : near_lin)) == 0;
      if (!__any_sync(0xffffffffu, valid && may)) continue;
      double sval = reflect(x0, xq, tv.period, kImageMask[pass]);
      // KDSplitNode.cxx:1129 gates 1-D images with sqrt(top) > sval, :1134-1146 the 2-D
      // and 3-D images with top > sval.
      bool g = (pass <= 3 || a.min_image) ? (__dsqrt_rn(top) > sval) : (top > sval);
      gate = gate && may && g;
    }
    if (!__any_sync(0xffffffffu, gate)) continue;
    traverse<KMAX>(tv, w, lane, gate, xq, self, a.exclude_self && pass == 0, K, top, a.err);
  }
  if (!valid) return;

  const int kr = a.kernres;
  const double inv_delta = 0.5 * (double)(kr - 1);  // 1 / table step, exact
  if (EPI == kEpiNN) {
    int Kc = K;
    double d;
    int j;
    if (a.drop_largest) {
      heap_pop<KMAX>(w, lane, Kc, d, j);
      Kc--;
    }
    size_t row = (size_t)qi * a.kout;
    for (int i = a.kout - 1; i >= 0; i--) {
      heap_pop<KMAX>(w, lane, Kc, d, j);
      Kc--;
      a.nn[row + i] = j;
      a.d2[row + i] = d;
    }
    return;
  }
  // density family: the heap holds exactly the k neighbours (target search)
  for (int s = 0; s < K; s++)
    if (w.hi[s][lane] < 0) {
      atomicExch(a.err, kErrTooFew);
      return;
    }
  const double* T = a.kernel;
  P4 me = tv.pos[self];
  if (EPI == kEpiDensity || EPI == kEpiDensVel || EPI == kEpiDensPart || EPI == kEpiDensSave) {
    // KDCalcSmoothQuantities.cxx:260-286
    // One reciprocal per query replaces the per-neighbour divisions (r/h and the table
    // step); the density moves by a few units in the last place, far inside 1e-12.
    double hh = 0.5 * __dsqrt_rn(top);
    double ih = 1.0 / hh;
    double norm = dmul(dmul(ih, ih), ih);  // 1 / h^3 (the reference takes pow(h, 3))
    double wnorm = EPI == kEpiDensPart ? norm : 0.5 * norm;
    double acc = 0.0;
    for (int s = 0; s < K; s++) {
      double d2 = w.hd[s][lane];
      int j = w.hi[s][lane];
      double q = dmul(__dsqrt_rn(d2), ih);
      double wij = dmul(wsm_line(q, kr, inv_delta, T), wnorm);
      double mj = tv.pos[j].m;
      acc = dadd(acc, dmul(wij, mj));
      if (EPI != kEpiDensPart) {
        atomicAdd(&a.rho[j], dmul(wij, me.m));
        if (EPI == kEpiDensSave) a.nn[(size_t)(self - tv.pstart) * K + s] = j;
      }
    }
    if (EPI == kEpiDensPart) a.rho[qi] = acc;
    else atomicAdd(&a.rho[self], acc);
  }
  if (EPI == kEpiDensVel || EPI == kEpiVel || EPI == kEpiVelPart) {
    // KDCalcSmoothQuantities.cxx:354-383: |dv| of the Nsearch neighbours, keep the
    // Nsmooth smallest, h = 0.5 max, sum Wsm(|dv|/h) h^-3 with unit weights.
    V4 vi = tv.vel[self];
    for (int s = 0; s < K; s++) {
      V4 vj = tv.vel[w.hi[s][lane]];
      w.hd[s][lane] = __dsqrt_rn(dist2_exact(vi.x, vi.y, vi.z, vj.x, vj.y, vj.z));
    }
    int ns = a.nsmooth;
    if (ns < K) {
      // max-heap over the first ns values, then keep the ns smallest of the rest
      for (int s = ns / 2 - 1; s >= 0; s--) {
        double d = w.hd[s][lane];
        int j = w.hi[s][lane];
        heap_sift<KMAX>(w, lane, ns, s, d, j);
      }
      for (int s = ns; s < K; s++) {
        double d = w.hd[s][lane];
        if (dkey(d) < dkey(w.hd[0][lane])) heap_sift<KMAX>(w, lane, ns, 0, d, w.hi[s][lane]);
      }
    }
    long long vmaxk = 0;
    for (int s = 0; s < ns; s++) vmaxk = max(vmaxk, dkey(w.hd[s][lane]));
    double hh = 0.5 * __longlong_as_double(vmaxk);
    double ih = 1.0 / hh;
    double norm = dmul(dmul(ih, ih), ih);
    double acc = 0.0;
    for (int s = 0; s < ns; s++) {
      double q = dmul(w.hd[s][lane], ih);
      acc = dadd(acc, dmul(wsm_line(q, kr, inv_delta, T), norm));
    }
    if (EPI == kEpiVelPart) a.vden[qi] = acc;
    else a.vden[self] = acc;
  }
}

template <int KMAX>
constexpr int warps_per_block() {
  return KMAX <= 32 ? 8 : (KMAX <= 64 ? 4 : 2);
}

template <int KMAX, int EPI>
__global__ void __launch_bounds__(32 * warps_per_block<KMAX>()) k_knn(KnnArgs a) {
  constexpr int WPB = warps_per_block<KMAX>();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  WarpSmem<KMAX>* ws = reinterpret_cast<WarpSmem<KMAX>*>(smem_raw);
  int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int gw = blockIdx.x * WPB + warp;
  int qi = gw * 32 + lane;  // query slot
  if (gw * 32 >= a.nq) return;
  const TreeView& tv = a.tv;
  bool valid = qi < a.nq;
  int self = -1;
  double x0[3] = {0, 0, 0};
  if (valid) {
    if (a.qmode == 0) self = a.q0 + qi;
    else if (a.qmode == 2) self = a.qidx[qi];
    if (a.qmode == 1) {
      x0[0] = a.qx[3 * (size_t)qi];
      x0[1] = a.qx[3 * (size_t)qi + 1];
      x0[2] = a.qx[3 * (size_t)qi + 2];
    } else {
      P4 p = tv.pos[self];
      x0[0] = p.x;
      x0[1] = p.y;
      x0[2] = p.z;
    }
  }
  run_warp<KMAX, EPI>(a, tv, ws[warp], lane, valid, qi, self, x0, a.kheap);
}

// Batched density: a persistent grid whose warps pull (tree, query bucket) work items
// from an atomic counter until the list is exhausted; every tree is searched with its
// own k = min(k, n_tree - 1). The loop is bounded by the item count.
template <int KMAX>
__global__ void __launch_bounds__(32 * warps_per_block<KMAX>()) k_knn_batch(KnnArgs a, BatchArgs b) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  WarpSmem<KMAX>* ws = reinterpret_cast<WarpSmem<KMAX>*>(smem_raw);
  int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int guard = 0; guard < b.nitems + 1; guard++) {
    int item = 0;
    if (lane == 0) item = atomicAdd(b.counter, 1);
    item = __shfl_sync(0xffffffffu, item, 0);
    if (item >= b.nitems) break;
    WorkItem it = b.items[item];
    TreeInfo ti = b.trees[it.tree];
    TreeView tv = a.tv;
    tv.n = ti.n;
    tv.pstart = ti.pstart;
    tv.nbase = ti.nbase;
    int K = min(a.kheap, ti.n - 1);
    if (K < 1) continue;
    bool valid = lane < it.count;
    int self = ti.pstart + it.q0 + (valid ? lane : 0);
    P4 p = tv.pos[self];
    double x0[3] = {p.x, p.y, p.z};
    run_warp<KMAX, kEpiDensity>(a, tv, ws[warp], lane, valid, self, self, x0, K);
    __syncwarp();
  }
}

template <int KMAX, int EPI>
int launch_t(const KnnArgs& a, cudaStream_t st) {
  constexpr int WPB = warps_per_block<KMAX>();
  size_t sm = sizeof(WarpSmem<KMAX>) * WPB;
  static bool set = false;
  if (!set) {
    NBK_CUDA_TRY(cudaFuncSetAttribute(k_knn<KMAX, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)sm));
    set = true;
  }
  int warps = (a.nq + 31) / 32;
  int blocks = (warps + WPB - 1) / WPB;
  if (blocks == 0) return NBK_OK;
  static const char* kNames[] = {"knn_nn", "knn_density", "knn_density_veldensity", "knn_veldensity",
                                 "knn_density_particle", "knn_veldensity_particle", "knn_density_save"};
  Phase ph(kNames[EPI], st);
  k_knn<KMAX, EPI><<<blocks, 32 * WPB, sm, st>>>(a); note_launch();
  NBK_CUDA_TRY(cudaGetLastError());
  return NBK_OK;
}

template <int EPI>
int launch_e(const KnnArgs& a, cudaStream_t st) {
  if (a.kheap <= 16) return launch_t<16, EPI>(a, st);
  if (a.kheap <= 33) return launch_t<33, EPI>(a, st);
  if (a.kheap <= 65) return launch_t<65, EPI>(a, st);
  if (a.kheap <= 128) return launch_t<128, EPI>(a, st);
  set_error("k larger than 127 is not supported by the GPU kNN kernels");
  return NBK_ERR_UNSUPPORTED;
}

template <int KMAX>
int launch_batch_t(const KnnArgs& a, const BatchArgs& b, cudaStream_t st) {
  constexpr int WPB = warps_per_block<KMAX>();
  size_t sm = sizeof(WarpSmem<KMAX>) * WPB;
  static int grid = 0;
  if (grid == 0) {
    NBK_CUDA_TRY(cudaFuncSetAttribute(k_knn_batch<KMAX>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    int dev = 0, nsm = 0, per = 0;
    NBK_CUDA_TRY(cudaGetDevice(&dev));
    NBK_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    NBK_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_knn_batch<KMAX>, 32 * WPB, sm));
    grid = nsm * (per > 0 ? per : 1);
  }
  int blocks = std::min(grid, (b.nitems + WPB - 1) / WPB);
  if (blocks <= 0) return NBK_OK;
  Phase ph("knn_density_batch", st);
  k_knn_batch<KMAX><<<blocks, 32 * WPB, sm, st>>>(a, b); note_launch();
  NBK_CUDA_TRY(cudaGetLastError());
  return NBK_OK;
}

}  // namespace

int launch_knn_batch(const KnnArgs& a, const BatchArgs& b, cudaStream_t st) {
  if (a.kheap <= 16) return launch_batch_t<16>(a, b, st);
  if (a.kheap <= 33) return launch_batch_t<33>(a, b, st);
  if (a.kheap <= 65) return launch_batch_t<65>(a, b, st);
  if (a.kheap <= 128) return launch_batch_t<128>(a, b, st);
  set_error("k larger than 127 is not supported by the GPU kNN kernels");
  return NBK_ERR_UNSUPPORTED;
}

int launch_knn(const KnnArgs& a, int epi, cudaStream_t st) {
  switch (epi) {
    case kEpiNN: return launch_e<kEpiNN>(a, st);
    case kEpiDensity: return launch_e<kEpiDensity>(a, st);
    case kEpiDensVel: return launch_e<kEpiDensVel>(a, st);
    case kEpiVel: return launch_e<kEpiVel>(a, st);
    case kEpiDensPart: return launch_e<kEpiDensPart>(a, st);
    case kEpiVelPart: return launch_e<kEpiVelPart>(a, st);
    case kEpiDensSave: return launch_e<kEpiDensSave>(a, st);
  }
  set_error("unknown kNN epilogue");
  return NBK_ERR_INVALID;
}

}  // namespace nbk
