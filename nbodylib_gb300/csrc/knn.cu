// k-nearest-neighbour queries and the SPH quantities built on them: the per-particle
// loops of CalcDensity, CalcVelDensity, CalcDensityParticle and CalcVelDensityParticle
// (KDCalcSmoothQuantities.cxx:203-389, 768-920) and the coordinate forms
// CalcDensityPosition / CalcVelDensityPosition (:1092-1207) as epilogues of the warp
// search of knn_core.cuh.
#include <algorithm>
#include <map>
#include <mutex>

#include "knn_core.cuh"
#include "knn_wq.cuh"

namespace nbk {

namespace {

// One warp's work: up to 32 queries of one tree (lane = query). `qslot` indexes the
// per-query outputs, `self` is the query's tree index (-1 for a coordinate query), K the
// heap size. All lanes of the warp call this together.
template <int KMAX, int EPI>
__device__ void run_warp(const KnnArgs& a, const TreeView& tv, WarpSmem<KMAX>& w, int lane,
                         bool valid, int qi, int self, const double x0[3], int K) {
  double top = knn_search<KMAX>(a, tv, w, lane, valid, self, x0, K);
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
  P4 me{};  // the query particle (a coordinate query has none: self = -1)
  if (self >= 0) me = tv.pos[self];
  if (EPI == kEpiDensity || EPI == kEpiDensVel || EPI == kEpiDensPart || EPI == kEpiDensSave) {
    // KDCalcSmoothQuantities.cxx:260-286
    // One reciprocal per query replaces the per-neighbour divisions (r/h and the table
    // step); the density moves by a few units in the last place, far inside 1e-12.
    double hh = 0.5 * __dsqrt_rn(top);
    double ih = 1.0 / hh;
    double norm = dmul(dmul(ih, ih), ih);  // 1 / h^3 (the reference takes pow(h, 3))
    double wnorm = EPI == kEpiDensPart ? norm : 0.5 * norm;
    double acc = 0.0;
    const long long topk = dkey(top);
    for (int s = 0; s < K; s++) {
      double d2 = w.hd[s][lane];
      int j = w.hi[s][lane];
      // the farthest neighbour sits at q = 2 exactly in the reference's arithmetic (the
      // table's last entry, 0 for the compact kernels); the product with 1/h could land
      // an ulp below it, in the previous cell
      double q = dmul(sqrt_newton(d2), ih);
      double wq = dkey(d2) == topk ? T[kr - 1] : wsm_line(q, kr, inv_delta, T);
      double wij = dmul(wq, wnorm);
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
    V4 vi = self >= 0 ? tv.vel[self]
                      : make_v4(a.qv[3 * (size_t)qi], a.qv[3 * (size_t)qi + 1],
                                a.qv[3 * (size_t)qi + 2], 0.0);
    for (int s = 0; s < K; s++) {
      V4 vj = tv.vel[w.hi[s][lane]];
      w.hd[s][lane] = sqrt_newton(dist2_exact(vi.x, vi.y, vi.z, vj.x, vj.y, vj.z));
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
      const double vd = w.hd[s][lane];
      double q = dmul(vd, ih);
      double wq = dkey(vd) == vmaxk ? T[kr - 1] : wsm_line(q, kr, inv_delta, T);  // q = 2
      acc = dadd(acc, dmul(wq, norm));
    }
    if (EPI == kEpiVelPart) a.vden[qi] = acc;
    else a.vden[self] = acc;
  }
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
    if (a.qmode == 2 && (self < 0 || self >= tv.n)) {  // device-resident targets: checked here
      atomicExch(a.err, kErrTarget);
      valid = false;
      self = 0;
    }
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

// ---- warp per query (knn_wq.cuh): target queries

constexpr int kWqWpb = 8;  // warps (queries) per block

// One query's search and epilogue on one warp; `qi` indexes the per-query outputs and
// `self` is the query's tree index. All lanes of the warp call this together.
template <int S, int EPI, bool F32FIRST = false>
__device__ void wq_run(const KnnArgs& a, const TreeView& tv, WqSmem& w, int lane, int qi,
                       int self, const double x0[3], int K) {
  const unsigned FULL = 0xffffffffu;
  WqQuery<S> Q;
  wq_search<S, F32FIRST>(Q, w, a, tv, lane, self, x0, K, a.exclude_self != 0);
  const int kr = a.kernres;
  const double inv_delta = 0.5 * (double)(kr - 1);  // 1 / table step, exact
  if (EPI == kEpiNN) {
    // rows ascending in d2; the popped largest (FindNearestPos on a periodic tree) or the
    // nearest (FindNearest on a periodic tree: k + 1 searched, k written) are left out
    // exactly as the heap version pops them
    int first = K - (a.drop_largest ? 1 : 0) - a.kout;
    size_t row = (size_t)qi * a.kout;
#pragma unroll
    for (int s = 0; s < S; s++) {
      int i = s * 32 + lane - first;
      if (i >= 0 && i < a.kout) {
        a.nn[row + i] = Q.L.idx[s];
        a.d2[row + i] = __longlong_as_double(Q.L.key[s]);
      }
    }
    return;
  }
  // density family: the list holds exactly the k neighbours (target search)
  bool missing = false;
#pragma unroll
  for (int s = 0; s < S; s++) missing |= (s * 32 + lane < K) && Q.L.idx[s] < 0;
  if (__any_sync(FULL, missing)) {
    if (lane == 0) atomicExch(a.err, kErrTooFew);
    return;
  }
  const double* T = a.kernel;
  if (EPI == kEpiDensity || EPI == kEpiDensVel || EPI == kEpiDensPart || EPI == kEpiDensSave) {
    // KDCalcSmoothQuantities.cxx:260-286: one neighbour per lane. 1 / h with
    // h = sqrt(top) / 2 (the reference divides by h) within a few ulps, far inside the
    // 1e-12 density tolerance
    const double me_m = tv.pos[self].m;
    double ih = two_rsqrt(__longlong_as_double(Q.topk));
    double norm = dmul(dmul(ih, ih), ih);  // 1 / h^3 (the reference takes pow(h, 3))
    double wnorm = EPI == kEpiDensPart ? norm : 0.5 * norm;
    double acc = 0.0;
#pragma unroll
    for (int s = 0; s < S; s++) {
      int p = s * 32 + lane;
      if (p >= K) continue;
      double d2 = __longlong_as_double(Q.L.key[s]);
      int j = Q.L.idx[s];
      // the farthest neighbour sits at q = 2 exactly in the reference's arithmetic (the
      // table's last entry); the product with 1/h could land an ulp below it
      double q = dmul(sqrt_newton(d2), ih);
      double wq = Q.L.key[s] == Q.topk ? T[kr - 1] : wsm_line(q, kr, inv_delta, T);
      double wij = dmul(wq, wnorm);
      acc = dadd(acc, dmul(wij, tv.pos[j].m));
      if (EPI != kEpiDensPart) {
        atomicAdd(&a.rho[j], dmul(wij, me_m));
        if (EPI == kEpiDensSave) a.nn[(size_t)(self - tv.pstart) * K + p] = j;
      }
    }
    acc = warp_sum(acc);
    if (lane == 0) {
      if (EPI == kEpiDensPart) a.rho[qi] = acc;
      else atomicAdd(&a.rho[self], acc);
    }
  }
  if (EPI == kEpiDensVel || EPI == kEpiVel || EPI == kEpiVelPart) {
    // KDCalcSmoothQuantities.cxx:354-383: |dv| of the Nsearch neighbours, keep the
    // Nsmooth smallest, h = 0.5 max, sum Wsm(|dv|/h) h^-3 with unit weights
    V4 vi = tv.vel[self];
    long long vk[S];
#pragma unroll
    for (int s = 0; s < S; s++) {
      vk[s] = kWqSent;
      if (s * 32 + lane < K) {
        V4 vj = tv.vel[Q.L.idx[s]];
        vk[s] = dkey(sqrt_newton(dist2_exact(vi.x, vi.y, vi.z, vj.x, vj.y, vj.z)));
      }
    }
    int ns = a.nsmooth;
    bool sel[S];
    if (ns < K) {
      int rk[S];
      wq_ranks<S>(vk, lane, K, rk);
#pragma unroll
      for (int s = 0; s < S; s++) sel[s] = s * 32 + lane < K && rk[s] < ns;
    } else {
#pragma unroll
      for (int s = 0; s < S; s++) sel[s] = s * 32 + lane < K;
    }
    long long vmaxk = 0;
#pragma unroll
    for (int s = 0; s < S; s++)
      if (sel[s]) vmaxk = max(vmaxk, vk[s]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) vmaxk = max(vmaxk, __shfl_xor_sync(FULL, vmaxk, o));
    double ih = recip_newton(0.5 * __longlong_as_double(vmaxk));
    double norm = dmul(dmul(ih, ih), ih);
    double acc = 0.0;
#pragma unroll
    for (int s = 0; s < S; s++) {
      if (!sel[s]) continue;
      double q = dmul(__longlong_as_double(vk[s]), ih);
      double wq = vk[s] == vmaxk ? T[kr - 1] : wsm_line(q, kr, inv_delta, T);  // q = 2
      acc = dadd(acc, dmul(wq, norm));
    }
    acc = warp_sum(acc);
    if (lane == 0) {
      if (EPI == kEpiVelPart) a.vden[qi] = acc;
      else a.vden[self] = acc;
    }
  }
}

// 64 registers per thread (4 blocks of 8 warps per SM): the occupancy outweighs the few
// spills of the two- and four-slot lists (measured at 2^20 and 2^22 clustered particles)
template <int S, int EPI>
__global__ void __launch_bounds__(32 * kWqWpb, 4) k_knn_wq(KnnArgs a) {
  __shared__ WqSmem ws[kWqWpb];
  int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int qi = blockIdx.x * kWqWpb + warp;
  if (qi >= a.nq) return;
  const TreeView& tv = a.tv;
  int self = a.qmode == 0 ? a.q0 + qi : a.qidx[qi];
  if (a.qmode == 2 && (self < 0 || self >= tv.n)) {  // device-resident targets: checked here
    if (lane == 0) atomicExch(a.err, kErrTarget);
    return;
  }
  P4 p = tv.pos[self];
  double x0[3] = {p.x, p.y, p.z};
  wq_run<S, EPI>(a, tv, ws[warp], lane, qi, self, x0, a.kheap);
}

// Batched density, warp per query: the persistent grid's warps pull (tree, query bucket)
// work items and serve the bucket's queries one after another.
// 6 blocks per SM (42 registers): for the many small trees of a batch the occupancy pays
// more than for one large tree (20,000 power-law groups: 17.98 ms against 20.59 ms at 4).
// The batch's one-slot searches run FP32 first (knn_wq.cuh wq_search_f32: 16.2 ms)
template <int S>
__global__ void __launch_bounds__(32 * kWqWpb, 6) k_knn_batch_wq(KnnArgs a, BatchArgs b) {
  __shared__ WqSmem ws[kWqWpb];
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
    for (int q = 0; q < it.count; q++) {
      int self = ti.pstart + it.q0 + q;
      P4 p = tv.pos[self];
      double x0[3] = {p.x, p.y, p.z};
      wq_run<S, kEpiDensity, true>(a, tv, ws[warp], lane, self, self, x0, K);
      __syncwarp();
    }
  }
}

template <int S, int EPI>
int launch_wq(const KnnArgs& a, cudaStream_t st) {
  unsigned blocks = (unsigned)((a.nq + kWqWpb - 1) / kWqWpb);
  if (blocks == 0) return NBK_OK;
  static const char* kNames[] = {"knn_nn", "knn_density", "knn_density_veldensity", "knn_veldensity",
                                 "knn_density_particle", "knn_veldensity_particle", "knn_density_save"};
  Phase ph(kNames[EPI], st);
  k_knn_wq<S, EPI><<<blocks, 32 * kWqWpb, 0, st>>>(a); note_launch();
  NBK_CUDA_TRY(cudaGetLastError());
  return NBK_OK;
}

template <int KMAX, int EPI>
int launch_t(const KnnArgs& a, cudaStream_t st) {
  constexpr int WPB = warps_per_block<KMAX>();
  size_t sm = sizeof(WarpSmem<KMAX>) * WPB;
  NBK_TRY(ensure_dyn_smem((const void*)k_knn<KMAX, EPI>, (int)sm));
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
  if (a.qmode != 1) {  // target queries: a warp per query
    if (a.kheap <= 32) return launch_wq<1, EPI>(a, st);
    if (a.kheap <= 64) return launch_wq<2, EPI>(a, st);
    if (a.kheap <= 128) return launch_wq<4, EPI>(a, st);
  }
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
  // persistent grid: every resident block of this device (cached per device)
  static std::mutex mu;
  static std::map<int, int> grids;
  int dev = 0, grid = 0;
  NBK_CUDA_TRY(cudaGetDevice(&dev));
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = grids.find(dev);
    if (it != grids.end()) grid = it->second;
  }
  if (grid == 0) {
    NBK_TRY(ensure_dyn_smem((const void*)k_knn_batch<KMAX>, (int)sm));
    int nsm = 0, per = 0;
    NBK_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    NBK_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_knn_batch<KMAX>, 32 * WPB, sm));
    grid = nsm * (per > 0 ? per : 1);
    std::lock_guard<std::mutex> lk(mu);
    grids[dev] = grid;
  }
  int blocks = std::min(grid, (b.nitems + WPB - 1) / WPB);
  if (blocks <= 0) return NBK_OK;
  Phase ph("knn_density_batch", st);
  k_knn_batch<KMAX><<<blocks, 32 * WPB, sm, st>>>(a, b); note_launch();
  NBK_CUDA_TRY(cudaGetLastError());
  return NBK_OK;
}

}  // namespace

// Persistent warp-per-query batch kernel: every resident block of this device.
template <int S>
int launch_batch_wq_t(const KnnArgs& a, const BatchArgs& b, cudaStream_t st) {
  static std::mutex mu;
  static std::map<int, int> grids;
  int dev = 0, grid = 0;
  NBK_CUDA_TRY(cudaGetDevice(&dev));
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = grids.find(dev);
    if (it != grids.end()) grid = it->second;
  }
  if (grid == 0) {
    int nsm = 0, per = 0;
    NBK_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    NBK_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_knn_batch_wq<S>,
                                                               32 * kWqWpb, 0));
    grid = nsm * (per > 0 ? per : 1);
    std::lock_guard<std::mutex> lk(mu);
    grids[dev] = grid;
  }
  int blocks = std::min(grid, (b.nitems + kWqWpb - 1) / kWqWpb);
  if (blocks <= 0) return NBK_OK;
  Phase ph("knn_density_batch", st);
  k_knn_batch_wq<S><<<blocks, 32 * kWqWpb, 0, st>>>(a, b); note_launch();
  NBK_CUDA_TRY(cudaGetLastError());
  return NBK_OK;
}

int launch_knn_batch(const KnnArgs& a, const BatchArgs& b, cudaStream_t st) {
  if (b.warp_per_query) {
    if (a.kheap <= 32) return launch_batch_wq_t<1>(a, b, st);
    if (a.kheap <= 64) return launch_batch_wq_t<2>(a, b, st);
    if (a.kheap <= 128) return launch_batch_wq_t<4>(a, b, st);
  }
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
