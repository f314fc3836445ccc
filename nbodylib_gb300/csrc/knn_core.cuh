// Warp-cooperative k-nearest-neighbour search shared by the kNN / SPH density kernels
// (knn.cu) and the SPH smoothing kernels (smooth.cu).
//
// Replaces the recursive depth-first search of SplitNode/LeafNode::FindNearestPos
// (src/KDTree/KDSplitNode.cxx:15-41, 206-231; KDLeafNode.cxx:15-28, 119-130) and its
// periodic wrapper (KDSplitNode.cxx:1119-1147).
//
// Work mapping: one warp serves 32 queries that are consecutive in tree order, so they
// sit in one or two neighbouring leaves and want nearly the same nodes. The warp walks
// the tree once for all of them (a node is opened when any lane still needs it), stages
// each opened leaf's FP32 coordinates in shared memory, and every lane tests them against
// its own query. Each lane keeps a bounded max-heap of (d2, index) in shared memory.
//
// Exactness: node pruning and the first candidate test use FP32 lower bounds computed
// with directed rounding from FP32 copies of the coordinates, so they never reject what
// the FP64 test would accept; a candidate that survives is tested in FP64 with the
// reference's arithmetic, d2 = ((dx*dx + dy*dy) + dz*dz), and accepted when d2 < top
// (strict, as the reference's `dist2 < pq->TopPriority()`).
#pragma once
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
  // the query's own rounding bound (it may lie outside the tree's box); candidates: tv.eps
  float eps = query_eps(tv, xq[0], xq[1], xq[2]), two_eps = __fadd_ru(eps, tv.eps);
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

// The search half of one warp's work: up to 32 queries of one tree (lane = query), the
// direct pass and the periodic image passes with the reference's gates. On return the
// lane's heap holds its K nearest (d2, tree index); returns the largest d2 (the heap top).
// `self` is the query's tree index (-1 for a coordinate query). All lanes call it together.
template <int KMAX>
__device__ double knn_search(const KnnArgs& a, const TreeView& tv, WarpSmem<KMAX>& w, int lane,
                             bool valid, int self, const double x0[3], int K) {
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
        float qeps = query_eps(tv, x0[0], x0[1], x0[2]);
        near_sq = near_walls(qf, tv.period, qeps, top_hi);
        near_lin = near_walls_lin(qf, tv.period, qeps, top_hi);
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
  return top;
}

// Warps per block for a heap bound KMAX (shared memory per warp grows with KMAX).
template <int KMAX>
constexpr int warps_per_block() {
  return KMAX <= 32 ? 8 : (KMAX <= 64 ? 4 : 2);
}

}  // namespace
}  // namespace nbk
