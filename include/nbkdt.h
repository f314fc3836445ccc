/*
 * nbkdt.h -- C ABI of the GB300-native KDTree hot path (tree build, kNN, SPH density,
 * ball search, friends-of-friends), implemented by hand-written sm_103a CUDA kernels in
 * libnbkdt.so.
 *
 * Each entry point replaces one method of the reference C++ class NBody::KDTree
 * (pelahi/NBodylib, src/KDTree/KDTree.h); the comment above each declaration names the
 * reference interface it stands in for. The C++ drop-in class in include/nbkdt/KDTree.hpp
 * and the Python binding in nbodylib_gb300/ are thin layers over these calls.
 *
 * Conventions
 *  - Every call returns an int status (NBK_OK = 0); nbk_last_error() returns a message
 *    for the calling thread's most recent failure. Nothing aborts the process: where the
 *    reference prints and calls exit(1) (e.g. CalcDensity with fewer than k neighbours,
 *    KDCalcSmoothQuantities.cxx:273-276) the call returns NBK_ERR_TOO_FEW.
 *  - Tree order: the tree reorders particles into its own leaf order (the reference
 *    permutes the caller's Particle array, KDTree.h:12-15). "Tree index" means a position
 *    in that order; nbk_get_perm maps tree index -> input index (the reference's ID,
 *    KDTree.cxx:1291). Neighbour lists hold tree indices, as the reference's do
 *    (KDTree.h:295); per-particle quantities (density, FOF groups) are returned in input
 *    order, as the reference's ID-indexed arrays are (KDTree.h:399, :474).
 *  - Memory: by default every pointer argument is host memory and calls are synchronous.
 *    A tree created with NBK_DEVICE_PTRS takes device pointers for all inputs and outputs
 *    on all its calls, runs on its stream (nbk_set_stream) and does not synchronise.
 *  - Arithmetic is FP64 throughout: distances are computed as ((dx*dx + dy*dy) + dz*dz)
 *    with separately rounded operations, as the reference computes them
 *    (DistFunc.h:14-19), so neighbour selection and linking decisions are bit-exact.
 */
#ifndef NBKDT_H
#define NBKDT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define NBK_OK 0
#define NBK_ERR_INVALID 1      /* bad argument (null pointer, k out of range, NaN input) */
#define NBK_ERR_UNSUPPORTED 2  /* a reference option this build does not run on the GPU */
#define NBK_ERR_CUDA 3         /* a CUDA runtime call failed */
#define NBK_ERR_NOMEM 4        /* device or host allocation failed */
#define NBK_ERR_TOO_FEW 5      /* fewer than k neighbours exist (reference: exit(1)) */
#define NBK_ERR_DEVICE 6       /* a device-side bound (iteration cap, capacity) was hit */

/* ---- tree types (KDTree.h:90) and kernel types (KDTree.h:97) ---- */
#define NBK_TPHYS 0
#define NBK_TPROJ 1
#define NBK_TVEL 2
#define NBK_TPHS 3
#define NBK_TMETRIC 4
#define NBK_KSPH 0
#define NBK_KGAUSS 1
#define NBK_KEPAN 2
#define NBK_KTH 3

/* ---- creation flags ---- */
#define NBK_DEVICE_PTRS 1u /* all pointer arguments of this tree's calls are device pointers */

/* ---- kNN variants ---- */
#define NBK_FINDNEAREST 0    /* KDTree::FindNearest(tt, ...)    (KDFindNearest.cxx:247-318) */
#define NBK_FINDNEARESTPOS 1 /* KDTree::FindNearestPos(tt, ...) (KDFindNearest.cxx:320-334) */
#define NBK_FINDNEARESTVEL 2 /* KDTree::FindNearestVel(tt, ...) (KDFindNearest.cxx:335-346),
                                velocity trees */
#define NBK_FINDNEARESTPHASE 3 /* KDTree::FindNearestPhase(tt, ...) (KDFindNearest.cxx:347-361),
                                  phase-space trees: the plain phase distance whatever Aniso */

/* ---- periodic image modes ---- */
/* Reproduce the reference's image gates exactly, including its comparison of a squared
   distance with a distance for the 2-D and 3-D images (KDSplitNode.cxx:1129-1146). */
#define NBK_PERIODIC_REF 0
/* Gate every image by sqrt(top) > wall distance: the exact minimum-image kNN. */
#define NBK_PERIODIC_MIN_IMAGE 1

/* ---- FOF comparators (FOFFunc.h:30-55) ---- */
#define NBK_FOF3D 0
#define NBK_FOFVEL 1
#define NBK_FOF6D 2

typedef struct nbk_tree nbk_tree;
typedef struct nbk_batch nbk_batch;

/* Message for the calling thread's most recent failed call ("" if none). */
const char* nbk_last_error(void);

/* Library version string and the device it runs on. (No reference counterpart.) */
const char* nbk_version(void);

/* Number of CUDA kernels this library has launched since it was loaded; lets a caller
   count the device work of a call sequence. (No reference counterpart.) */
long long nbk_launch_count(void);

/* Phase trace (no reference counterpart; the reference has only ad-hoc std::chrono
   timing macros in src/tests/test_kdtree.cxx:19-22). While enabled, each named phase
   (tree build, kNN search, FOF link, ...) is bracketed by a CUDA event pair on the
   stream it runs on, without synchronising; nbk_trace_json resolves the pending events
   and writes {"phase": {"count": c, "ms": total}, ...} into buf (NUL-terminated) and
   returns the length it needs. */
/* Measured FP64 FMA throughput of the current GPU in GFLOP/s (2 flops per FMA), the
   denominator of the FP64 roofline. (No reference counterpart.) */
int nbk_probe_fp64(double* gflops);

int nbk_trace_enable(int on);
int nbk_trace_reset(void);
int64_t nbk_trace_json(char* buf, int64_t cap);

/* The compute capability (major*10 + minor) of the SASS and PTX that the CUDA runtime
   selected on the current device for one product kernel (the scatter to input order that
   every density call launches): 103 and 103 for an sm_103a build. (No reference
   counterpart.) */
int nbk_kernel_binary_version(int* binary_version, int* ptx_version);

/* ---- test hooks (no reference counterpart: the reference loops without bound and
   exits on failure, KDCalcSmoothQuantities.cxx:273-276, PriorityQueue.h:49-53) ---- */
/* Iteration cap of the union-find loops of FOF, FOFCriterion and FOFNNCriterion on the
   current device (default 2^24; cap <= 0 restores it). A loop that reaches the cap stops,
   sets the call's device error word, and the call returns NBK_ERR_DEVICE. */
int nbk_debug_set_iteration_cap(int cap);
/* Make the device allocation `countdown` allocations from now (0 = the next) fail with
   NBK_ERR_NOMEM, once; a negative countdown disarms. */
int nbk_debug_fail_allocation(long long countdown);
/* Device allocations the library currently holds (trees, batches, per-call scratch not
   yet freed, and the scratch blocks a host thread keeps for its next tree build and FOF
   call, at most 256 MB each, held until the thread exits); a failed call must leave it
   where it was. */
long long nbk_debug_live_allocations(void);

/*
 * Build a tree. Replaces KDTree::KDTree(Particle*, Int_t numparts, Int_t bucket_size,
 * int TreeType, int KernType, int KernRes, int SplittingCriterion, int Aniso,
 * int ScaleSpace, Double_t* Period, ...)  (KDTree.h:229-245, KDTree.cxx:1238-1306).
 *  pos  : n x 3 positions, row-major (x, y, z)
 *  vel  : n x 3 velocities or NULL (needed by nbk_veldensity, nbk_fof_criterion)
 *  mass : n masses or NULL (unit masses)
 *  period: 3 box lengths or NULL (non-periodic)
 * Supported: treetype NBK_TPHYS, NBK_TVEL (velocities required, non-periodic) and
 * NBK_TPHS (velocities required); kernel types all four; splitting 0, scale_space 0;
 * aniso 0 or -1 (for a phase-space tree: 0 the local metric of CalculateMetricSpacing +
 * FindNearestMetric, the reference's default; -1 the plain phase-space distance of
 * FindNearestPhase; other trees ignore it). Anything else returns NBK_ERR_UNSUPPORTED.
 * The tree is built on the GPU with the reference's rules (split dimension of largest
 * spread over the tree's coordinates: x, y, z; vx, vy, vz; or all six; median split with
 * the left child taking ceil(size/2), leaf when size <= bucket_size), so its leaves hold
 * the same particle sets as the reference's.
 * Velocity and phase-space trees run nbk_knn / nbk_knn_targets (FindNearest),
 * nbk_knn_coords, nbk_density / nbk_density_particles (phase space: aniso 0 only) and,
 * for phase-space trees, nbk_fof_criterion; every other call returns NBK_ERR_UNSUPPORTED
 * for them (the reference refuses them or compares positions with velocity cut values).
 */
int nbk_create(const double* pos, const double* vel, const double* mass, int64_t n,
               int bucket_size, int treetype, int kerntype, int kernres,
               int splitting_criterion, int aniso, int scale_space, const double* period,
               unsigned flags, nbk_tree** out);

/* Free the tree. Replaces KDTree::~KDTree (KDTree.cxx:1340-1356); the caller restores
   its own particle order with the permutation (see nbk_get_perm). */
int nbk_destroy(nbk_tree* tree);

/* Set the CUDA stream (a cudaStream_t) the tree's kernels run on; NULL = default. */
int nbk_set_stream(nbk_tree* tree, void* stream);
/* Wait for all work queued on the tree's stream. */
int nbk_sync(nbk_tree* tree);

/* KDTree::GetNumNodes / GetNumLeafNodes / GetBucketSize (KDTree.h:282-284). */
int nbk_get_counts(const nbk_tree* tree, int64_t* numparts, int64_t* numnodes,
                   int64_t* numleafnodes, int32_t* bucket_size);
/* perm[t] = input index of the particle at tree index t (the reference's
   bucket[t].GetID(), KDTree.cxx:1291). */
int nbk_get_perm(const nbk_tree* tree, int32_t* perm);
/* The kernel table (kernres doubles) and its normalisation, as
   KDTree::KernelConstruction builds them (KDTree.cxx:1144-1183). */
int nbk_get_kernel(const nbk_tree* tree, double* table, double* kernnorm);

/*
 * k nearest neighbours of every particle. Replaces KDTree::FindNearest(Int_t** nn,
 * Double_t** dist2, Int_t Nsearch) and FindNearestPos(Int_t**, Double_t**, Int_t)
 * (KDFindNearest.cxx:444-456), i.e. FindNearest(tt)/FindNearestPos(tt) for every tt.
 * variant: NBK_FINDNEAREST, NBK_FINDNEARESTPOS (physical trees), NBK_FINDNEARESTVEL
 * (velocity trees) or NBK_FINDNEARESTPHASE (phase-space trees); periodic_mode as above.
 * nn, d2: n x k, row t = the particle at tree index t; neighbours are tree indices in
 * ascending squared distance. Non-periodic trees exclude the particle itself and any
 * particle at distance 0 (KDLeafNode.cxx:19-21); periodic FindNearest drops the nearest
 * entry (normally the particle itself) and periodic FindNearestPos keeps it
 * (KDFindNearest.cxx:250,315-331).
 */
int nbk_knn(nbk_tree* tree, int k, int variant, int periodic_mode, int32_t* nn, double* d2);

/* FindNearest(tt, ...) / FindNearestPos(tt, ...) (KDFindNearest.cxx:247-334) for a batch
   of target particles (tree indices): row i of nn/d2 belongs to targets[i]; semantics as
   nbk_knn. */
int nbk_knn_targets(nbk_tree* tree, const int32_t* targets, int64_t ntargets, int k,
                    int variant, int periodic_mode, int32_t* nn, double* d2);

/* k nearest neighbours of nq coordinates (nq x 3). Replaces
   KDTree::FindNearestPos(Double_t* x, Int_t* nn, Double_t* dist2, Int_t Nsearch)
   (KDFindNearest.cxx:509-520); nothing is excluded. */
int nbk_knn_points(nbk_tree* tree, const double* x, int64_t nq, int k, int periodic_mode,
                   int32_t* nn, double* d2);

/* k nearest neighbours of nq coordinates in the tree's own space. Replaces
   KDTree::FindNearest(Double_t* x, Int_t* nn, Double_t* dist2, Int_t Nsearch)
   (KDFindNearest.cxx:460-507): x holds 3 positions per row (physical tree, as
   nbk_knn_points with NBK_PERIODIC_REF), 3 velocities (velocity tree) or
   x, y, z, vx, vy, vz (phase-space tree: the plain or local-metric search with the
   ungated position images of a periodic tree, KDSplitNode.cxx:1153-1218). */
int nbk_knn_coords(nbk_tree* tree, const double* x, int64_t nq, int k, int32_t* nn, double* d2);

/* KDTree::FindNearestPhase(Double_t* x, Double_t* v, ...) (KDFindNearest.cxx:542-560) on a
   phase-space tree: the plain phase distance around nq points (x, y, z, vx, vy, vz per
   row), with the ungated position images of a periodic tree, whatever the tree's Aniso. */
int nbk_knn_phase_points(nbk_tree* tree, const double* x, int64_t nq, int k, int32_t* nn,
                         double* d2);

/*
 * SPH density of every particle. Replaces KDTree::CalcDensity(Int_t Nsmooth)
 * (KDCalcSmoothQuantities.cxx:203-305): non-periodic kNN excluding the particle,
 * h = 0.5 sqrt(d2 of the k-th), w = 0.5 Wsm(r/h) h^-3, rho_i += w m_j and rho_j += w m_i.
 * rho: n values in input order (the reference writes Particle::rho). Like the
 * reference, the period is ignored.
 */
int nbk_density(nbk_tree* tree, int k, double* rho);

/* nbk_density without any device allocation (no counterpart in the reference: it exists
   for callers that cannot allocate device memory while they run, e.g. simulation codes
   and in-situ halo finders that reserve the GPU's memory for their own pool at start-up
   and allow no allocation afterwards). The tree must already exist; rho_dev is a
   caller-owned DEVICE buffer of n doubles (input order), whatever the tree's pointer
   mode. The scratch is a static device array of 4,194,304 doubles (32 MiB, held per GPU
   until exit): larger trees return NBK_ERR_INVALID. All calls share it, so calls that
   overlap on the GPU race and must be serialised by the caller. The call runs on the
   tree's device and returns when its GPU work has finished; the first call on each
   device looks the scratch's address up. */
int nbk_density_noalloc(nbk_tree* tree, int k, double* rho_dev);

/* Gather-only density of selected particles. Replaces KDTree::CalcDensityParticle
   (KDCalcSmoothQuantities.cxx:768-843): no 0.5 factor, no scatter.
   targets: tree indices. out: one value per target. */
int nbk_density_particles(nbk_tree* tree, const int32_t* targets, int64_t ntargets, int k,
                          double* out);

/* Velocity-space density. Replaces KDTree::CalcVelDensity(Int_t Nsmooth, Int_t Nsearch)
   (KDCalcSmoothQuantities.cxx:309-389): physical kNN (Nsearch), then the Nsmooth nearest
   in velocity, h = 0.5 max |dv|, sum of Wsm(|dv|/h) h^-3 with unit weights. out: input
   order. Requires velocities. */
int nbk_veldensity(nbk_tree* tree, int nsmooth, int nsearch, double* out);

/* One traversal computing both nbk_density(k) and nbk_veldensity(nsmooth, k): the
   reference's CalcDensity(k) followed by CalcVelDensity(nsmooth, k) use the same
   neighbour search. rho and veldens: input order. */
int nbk_density_veldensity(nbk_tree* tree, int k, int nsmooth, double* rho, double* veldens);

/* Velocity density of selected particles. Replaces KDTree::CalcVelDensityParticle
   (KDCalcSmoothQuantities.cxx:845-920). targets: tree indices. */
int nbk_veldensity_particles(nbk_tree* tree, const int32_t* targets, int64_t ntargets,
                             int nsmooth, int nsearch, double* out);

/* SPH density at arbitrary coordinates. Replaces KDTree::CalcDensityPosition
   (KDCalcSmoothQuantities.cxx:1092-1148) on physical trees: the coordinate search
   (FindNearestPos(x): nothing excluded, never periodic), then the gather of
   CalcDensityParticle. x: nq rows of 3. NBK_ERR_UNSUPPORTED on velocity trees (the
   reference scales by metric factors it never sets there, :1125-1130) and phase-space
   trees; NBK_ERR_TOO_FEW when k exceeds the particle count. */
int nbk_density_points(nbk_tree* tree, const double* x, int64_t nq, int k, double* out);

/* Velocity density at arbitrary coordinates with given velocities. Replaces
   KDTree::CalcVelDensityPosition (KDCalcSmoothQuantities.cxx:1149-1207), physical trees:
   FindNearestPos(x) with nsearch, then as nbk_veldensity_particles with |v - v_j|.
   x, v: nq rows of 3. */
int nbk_veldensity_points(nbk_tree* tree, const double* x, const double* v, int64_t nq,
                          int nsmooth, int nsearch, double* out);

/*
 * SPH smoothing over the Nsmooth nearest neighbours (KDCalcSmoothQuantities.cxx). In all
 * of them rho holds the particles' densities in input order (the reference's
 * densityset = 1: what CalcDensity stored in the particles), or is NULL to run
 * CalcDensity(Nsmooth) first (densityset != 1). Searches ignore the period, as the
 * reference's. Every-particle outputs are in input order; the targets are tree indices and
 * the points (nq, 3) coordinates; their outputs follow the query order. Matrices are 3x3
 * row-major (element (k, l) at 3k + l).
 */
/* KDTree::CalcSmoothVel (KDCalcSmoothQuantities.cxx:480-540). smvel: [n][3]. */
int nbk_smooth_vel(nbk_tree* tree, int nsmooth, const double* rho, double* smvel);
/* KDTree::CalcSmoothVelDisp (:542-615), meanvelset = 1. smvel [n][3] in, disp [n][9] out. */
int nbk_smooth_vel_disp(nbk_tree* tree, int nsmooth, const double* rho, const double* smvel,
                        double* disp);
/* KDTree::CalcSmoothVelSkew (:617-690), meanvelset = veldispset = 1. skew: [n][3]. */
int nbk_smooth_vel_skew(nbk_tree* tree, int nsmooth, const double* rho, const double* smvel,
                        const double* disp, double* skew);
/* KDTree::CalcSmoothVelKurtosis (:692-766), the reference's per-neighbour "- 3" included. */
int nbk_smooth_vel_kurtosis(nbk_tree* tree, int nsmooth, const double* rho, const double* smvel,
                            const double* disp, double* kurt);
/* KDTree::CalcVelDensityWithPhysDensity (:393-478). Its physical smoothing length is half
   the largest squared distance, as the reference computes it (:428); where that sends the
   kernel-table index past the table (neighbour distances below 1), the reference reads
   past its table and this call uses the table's last entry. vden: [n]. */
int nbk_veldensity_physdensity(nbk_tree* tree, int nsmooth, int nsearch, const double* rho,
                               double* vden);
/* KDTree::CalcVelDensityWithPhysDensityParticle (:922-990). */
int nbk_veldensity_physdensity_particles(nbk_tree* tree, const int32_t* targets, int64_t ntargets,
                                         int nsmooth, int nsearch, const double* rho,
                                         double* vden);
/* KDTree::CalcSmoothVelParticle (:992-1036) / CalcSmoothVelPosition (:1209-1253). [nq][3]. */
int nbk_smooth_vel_particles(nbk_tree* tree, const int32_t* targets, int64_t ntargets,
                             int nsmooth, const double* rho, double* smvel);
int nbk_smooth_vel_points(nbk_tree* tree, const double* x, int64_t nq, int nsmooth,
                          const double* rho, double* smvel);
/* KDTree::CalcSmoothVelDispParticle (:1038-1090) / CalcSmoothVelDispPosition (:1255-1305).
   smvel: [nq][3] (the mean velocity of each query), disp: [nq][9]. */
int nbk_smooth_vel_disp_particles(nbk_tree* tree, const int32_t* targets, int64_t ntargets,
                                  int nsmooth, const double* rho, const double* smvel,
                                  double* disp);
int nbk_smooth_vel_disp_points(nbk_tree* tree, const double* x, int64_t nq, int nsmooth,
                               const double* rho, const double* smvel, double* disp);
/* KDTree::CalcSmoothLocalMeanParticle (:1539-1577) / CalcSmoothLocalMeanPosition
   (:1619-1655). weight: [n] in input order; mean: [nq]. */
int nbk_smooth_local_mean_particles(nbk_tree* tree, const int32_t* targets, int64_t ntargets,
                                    int nsmooth, const double* rho, const double* weight,
                                    double* mean);
int nbk_smooth_local_mean_points(nbk_tree* tree, const double* x, int64_t nq, int nsmooth,
                                 const double* rho, const double* weight, double* mean);
/* KDTree::CalcSmoothLocalDispParticle (:1579-1617) / CalcSmoothLocalDispPosition
   (:1657-1693). mean: [nq] (the local mean of each query), disp: [nq]. */
int nbk_smooth_local_disp_particles(nbk_tree* tree, const int32_t* targets, int64_t ntargets,
                                    int nsmooth, const double* rho, const double* weight,
                                    const double* mean, double* disp);
int nbk_smooth_local_disp_points(nbk_tree* tree, const double* x, int64_t nq, int nsmooth,
                                 const double* rho, const double* weight, const double* mean,
                                 double* disp);

/*
 * Fixed-radius search around particles. Replaces KDTree::SearchBallPosTagged(Int_t tt,
 * Double_t fdist2) (KDFindNearest.cxx:618-626, 664-672) for a batch of targets (tree
 * indices): every particle with d2 < fdist2, excluding the target itself; periodic trees
 * search the direct position and every mirror image whose wall distance is below the
 * radius (KDSplitNode.cxx:1389-1414) and then include the target, as the reference does.
 * Results are CSR: offsets[ntargets+1], out = tree indices. If out_capacity is too small
 * the call fills offsets, sets *total and returns NBK_ERR_INVALID without writing out.
 */
int nbk_ball_tagged(nbk_tree* tree, const int32_t* targets, int64_t ntargets, double fdist2,
                    int64_t* offsets, int32_t* out, int64_t out_capacity, int64_t* total);

/* As nbk_ball_tagged for arbitrary coordinates (nq x 3). Replaces
   KDTree::SearchBallPosTagged(Double_t* x, Double_t fdist2) (KDFindNearest.cxx:628-636). */
int nbk_ball_tagged_points(nbk_tree* tree, const double* x, int64_t nq, double fdist2,
                           int64_t* offsets, int32_t* out, int64_t out_capacity,
                           int64_t* total);

/* Replaces KDTree::SearchBallPos(Int_t tt, Double_t fdist2, Int_t imark, Int_t* nn,
   Double_t* dist2) (KDFindNearest.cxx:567-573): nn[ID] = imark and dist2[ID] = d2 for
   every particle found; arrays are input-order and caller-owned, entries not found are
   left untouched. The target is included exactly when the reference includes it (when a
   node on its root-to-leaf path lies wholly inside the radius,
   KDSplitNode.cxx:457-467, KDLeafNode.cxx:250-263). target: tree index. */
int nbk_ball_mark(nbk_tree* tree, int32_t target, double fdist2, int32_t imark, int32_t* nn,
                  double* dist2);

/*
 * Friends-of-friends. Replaces KDTree::FOF(Double_t fdist, Int_t& numgroup, Int_t minnum,
 * int order) (KDFOF.cxx:29-153): particles are linked when d2 < fdist^2 (periodic
 * images as KDSplitNode.cxx:1602-1646). group: input order, 0 = no group; groups are
 * numbered 1..ngroup by their first member in tree order, groups smaller than minnum
 * are dropped; order = 1 renumbers by decreasing size (ties by first member).
 */
int nbk_fof(nbk_tree* tree, double fdist, int32_t minnum, int order, int32_t* group,
            int32_t* ngroup);

/* Replaces KDTree::FOFCriterion(FOFcompfunc cmp, Double_t* params, Int_t& numgroup,
   Int_t minnum, int order) (KDFOF.cxx:157-265) for the comparators FOF3d, FOFVel and
   FOF6d (FOFFunc.h:30-55), selected by `comparator`. params: at least 8 doubles, laid
   out as the reference's (params[0] tree type, [1]/[2] search distance^2, [6]/[7]
   linking lengths^2). An arbitrary host FOFcompfunc cannot run on the GPU: the C++
   drop-in maps the three known functions to this call and reports any other as
   NBK_ERR_UNSUPPORTED. */
int nbk_fof_criterion(nbk_tree* tree, int comparator, const double* params, int32_t minnum,
                      int order, int32_t* group, int32_t* ngroup);

/* Friends-of-friends over given neighbour lists. Replaces KDTree::FOFNNCriterion
   (KDFOF.cxx:380-506): nn holds numnn tree indices per particle, rows by tree index (as
   FindNearest gives them); particle t is linked with each nn[t][j] the comparator accepts.
   The groups are the connected components of those links; groups below minnum are dropped
   and the rest numbered 1..G by decreasing size (equal sizes by their first member in tree
   order; the reference's order among equal sizes follows its priority queue). group: n, in
   input order. */
int nbk_fof_nn_criterion(nbk_tree* tree, int comparator, const double* params, int numnn,
                         const int32_t* nn, int32_t minnum, int32_t* group, int32_t* ngroup);
/* KDTree::FOFNNDistCriterion (KDFOF.cxx:507-640): as nbk_fof_nn_criterion, with
   params[pidx[k]] (k < npc <= 8, pidx[k] <= 7) replaced for each particle t by values[t]
   (tree order) before its comparisons: the value the reference takes from
   distfunc(numNN, dist2[t]), which the caller evaluates (the drop-in class calls the
   caller's function on the host). */
int nbk_fof_nn_dist_criterion(nbk_tree* tree, int comparator, const double* params, int numnn,
                              const int32_t* nn, const double* values, int npc,
                              const int32_t* pidx, int32_t minnum, int32_t* group,
                              int32_t* ngroup);

/*
 * Density adjoint (no reference counterpart; the reference has no gradients).
 * Forward: rho = nbk_density(k). Loss L = sum_i w_i log rho_i. With the neighbour sets
 * and the kernel-table cells frozen at the forward pass, returns dL/dpos (n x 3) and
 * dL/dmass (n), all in input order. Kernel weights are recomputed in the backward
 * kernel, not stored.
 */
int nbk_density_adjoint(nbk_tree* tree, int k, const double* w, double* rho,
                        double* grad_pos, double* grad_mass);

/*
 * Batched path: many independent trees (one per group, e.g. per FOF halo) built and
 * searched together. offsets: ngroups+1 CSR offsets into pos/mass. bucket_size <= 0
 * selects the autotuned leaf size. Replaces a caller loop of
 * KDTree(group particles) + CalcDensity(min(k, n_g - 1)) per group.
 */
int nbk_batch_create(const double* pos, const double* mass, const int64_t* offsets,
                     int64_t ngroups, int bucket_size, int kerntype, int kernres,
                     unsigned flags, nbk_batch** out);
int nbk_batch_destroy(nbk_batch* batch);
int nbk_batch_set_stream(nbk_batch* batch, void* stream);
/* Density of every particle of every group, k clamped per group to n_g - 1. rho: input
   order. use_graph != 0 replays the search as a captured CUDA graph. */
int nbk_batch_density(nbk_batch* batch, int k, double* rho, int use_graph);
/* The plain comparator: the same density computed by one build + one kNN-density
   launch sequence per group, looping over groups on the host. */
int nbk_batch_density_pertree(nbk_batch* batch, int k, double* rho);
/* The search half of the plain comparator: one kNN-density launch per group over the
   forest the batch already built, looping over groups on the host (no builds). */
int nbk_batch_density_pertree_search(nbk_batch* batch, int k, double* rho);
/* The leaf size and query-bucket size in use, and (when autotuned) the tuner's median
   timings of every (leaf size, query bucket, query mapping) candidate as JSON in
   tune_json (NUL-terminated, up to cap bytes). (No reference counterpart.) */
int nbk_batch_get_params(const nbk_batch* batch, int32_t* bucket_size, int32_t* query_bucket,
                         char* tune_json, int64_t cap);
/* How the batched search maps queries to warps: 1 (the default) a warp serves one query
   at a time (its k-list spread over the lanes' registers), 0 a lane serves one query and
   a warp 32 queries of a bucket. The autotuner chooses it with the leaf and bucket sizes.
   (No reference counterpart.) */
int nbk_batch_set_query_mapping(nbk_batch* batch, int warp_per_query);
int nbk_batch_get_query_mapping(const nbk_batch* batch, int32_t* warp_per_query);

#ifdef __cplusplus
}
#endif
#endif /* NBKDT_H */
