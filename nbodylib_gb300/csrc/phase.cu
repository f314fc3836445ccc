// Searches over a phase-space tree (KDTree with TreeType TPHS): the six coordinates
// (x, y, z, vx, vy, vz) of every particle, a tree split over all six.
//
// Replaces, for such trees:
//   FindNearest(tt) / FindNearest(x)        src/KDTree/KDFindNearest.cxx:247-310, 460-507
//   CalculateMetricSpacing                  KDFindNearest.cxx:34-105 (FindNearest's copy,
//                                           periodic-aware) and KDCalcSmoothQuantities.cxx:
//                                           17-56 (the densities' copy, never periodic)
//   SplitNode/LeafNode::FindNearestPhase    KDSplitNode.cxx:69-95, 260-296; KDLeafNode.cxx:43-56,
//                                           143-161
//   SplitNode/LeafNode::FindNearestMetric   KDSplitNode.cxx:96-121, 303-331; KDLeafNode.cxx:58-71,
//                                           168-179
//   FindNearestPhasePeriodic / ...MetricPeriodic  KDSplitNode.cxx:1085-1097, 1153-1218
//   CalcDensity / CalcDensityParticle       KDCalcSmoothQuantities.cxx:203-305, 768-843
//
// The local-metric search (the reference's default, Aniso = 0) scales the distance at the
// leaves by a per-query metric but prunes with the unscaled incremental offset, so its
// result is not the exact nearest-neighbour set and depends on the order in which the
// tree is walked. Two work mappings give the reference's answer:
//  - warp-cooperative exact search: one warp walks the tree once for 32 consecutive
//    queries (a node is opened when any lane still needs it) and every lane tests the
//    opened leaves against its own query. This is the plain phase distance (Aniso = -1),
//    which is exact, and every local-metric query whose metric weights are all at least
//    1 + 1e-9: for those the reference's unscaled pruning never removes a particle of the
//    final heap, so its result is the exact k nearest in the metric.
//  - per-lane walk for the remaining local-metric queries: the lane walks the tree in
//    exactly the reference's depth-first order (nearer child first; the farther child
//    opened when the FP64 offset sum, rounded as the reference rounds it, is below the
//    heap top at that moment) with the same bounded max-heap, which reproduces the
//    reference's neighbour sets. The walk is stackless over the heap-indexed nodes (the
//    parent of h is (h-1)/2); per depth it keeps the offset sum and the overwritten
//    offset.
//
// The walk skips every subtree whose particles provably cannot enter the heap: when the
// FP32 distance bound of its bounding box (box_lb6f, in the query's own metric, rounded
// down) is at or above an FP32 value above the heap top, walking it would insert nothing
// and so leave the top, and with it every later decision, unchanged. Leaf particles are
// screened the same way (pair_lb6f) before their FP64 distance is computed. The reference's unscaled pruning opens far more of the tree
// than the metric needs (the whole tree, for small velocity offsets), so this bound does
// most of the pruning while the result stays the reference's.
#include "nbk_build.h"

namespace nbk {
namespace {

// Per-thread bounded max-heap in shared memory, one column per thread.
template <int KMAX, int NT>
struct PhHeap {
  double d[KMAX][NT];
  int i[KMAX][NT];
};

// Replace the root (the largest entry) with (d, j) and restore the heap of size K.
template <int KMAX, int NT>
__device__ __forceinline__ void ph_replace_top(PhHeap<KMAX, NT>& H, int t, int K, double d,
                                               int j) {
  int pos = 0;
  while (true) {
    int c = 2 * pos + 1;
    if (c >= K) break;
    double dc = H.d[c][t];
    if (c + 1 < K) {
      double dc2 = H.d[c + 1][t];
      if (dc2 > dc) {
        c = c + 1;
        dc = dc2;
      }
    }
    if (d >= dc) break;
    H.d[pos][t] = dc;
    H.i[pos][t] = H.i[c][t];
    pos = c;
  }
  H.d[pos][t] = d;
  H.i[pos][t] = j;
}

template <int KMAX, int NT>
__device__ __forceinline__ void ph_fill(PhHeap<KMAX, NT>& H, int t, int K) {
  for (int s = 0; s < K; s++) {
    H.d[s][t] = kMaxValue;
    H.i[s][t] = -1;
  }
}

// PhaseDistSqd (DistFunc.h:41-49): ((((dx^2 + dy^2) + dz^2) + dvx^2) + dvy^2) + dvz^2.
__device__ __forceinline__ double phase_d2(const double x[6], const P4& p, const V4& v) {
  double a = dsub(x[0], p.x), b = dsub(x[1], p.y), c = dsub(x[2], p.z);
  double e = dsub(x[3], v.x), f = dsub(x[4], v.y), g = dsub(x[5], v.z);
  double s = dadd(dmul(a, a), dmul(b, b));
  s = dadd(s, dmul(c, c));
  s = dadd(s, dmul(e, e));
  s = dadd(s, dmul(f, f));
  return dadd(s, dmul(g, g));
}
// MetricDistSqd (DistFunc.h:58-65): total += (metric[i] * d) * d from 0, dimension order.
__device__ __forceinline__ double metric_d2(const double x[6], const P4& p, const V4& v,
                                            const double m[6]) {
  const double y[6] = {p.x, p.y, p.z, v.x, v.y, v.z};
  double total = 0.0;
#pragma unroll
  for (int k = 0; k < 6; k++) {
    double d = dsub(x[k], y[k]);
    total = dadd(total, dmul(dmul(m[k], d), d));
  }
  return total;
}

// One depth-first walk of the reference's search from x (a phase-space point). metric:
// the local metric, or nullptr for the plain phase distance. target: a tree index the
// leaves skip (the target forms), or -1. need_pos: leaves accept only distances > 0.
// top: the heap's largest entry, kept current.
template <int KMAX, int NT>
__device__ void ph_walk(const TreeView& tv, PhHeap<KMAX, NT>& H, int t, int K, const double x[6],
                        const double* metric, int target, bool need_pos, double& top, int* err) {
  double m[6] = {1, 1, 1, 1, 1, 1};
  if (metric)
#pragma unroll
    for (int k = 0; k < 6; k++) m[k] = metric[k];
  // FP32 images of the query and of the metric (rounded down) for the bounds
  float q32[6], w32[6], e32[6];
#pragma unroll
  for (int k = 0; k < 6; k++) {
    q32[k] = __double2float_rn(x[k]);
    w32[k] = metric ? __double2float_rd(m[k]) : 1.f;
    // the query may lie outside the tree's box: its own rounding bound, if larger
    e32[k] = fmaxf(tv.eps6[k], __fmul_ru(__double2float_ru(fabs(x[k])), 1.2e-7f));
  }
  float thr = thresh_hi_bits(dkey(top));  // FP32, above top by at least 2^-20 of it
  double off[6] = {0, 0, 0, 0, 0, 0};
  double rd_at[kPhDepth], old_at[kPhDepth];
  const NodeS* N = tv.nodes6 + tv.nbase;
  const NodeF6* F = tv.nodef6 + tv.nbase;
  int h = 0, depth = 0, prev = -1;
  bool down = true;
  rd_at[0] = 0.0;
  while (true) {
    if (down && box_lb6f(q32, w32, e32, F[h]) >= thr) {
      // nothing in this subtree can enter the heap: as if walked, with no insertion
      if (h == 0) break;
      prev = h;
      h = (h - 1) >> 1;
      depth--;
      down = false;
      continue;
    }
    const NodeS nd = N[h];
    if (down && nd.split_dim < 0) {  // a leaf: test its particles in tree order
      for (int i = nd.start; i < nd.start + nd.count; i++) {
        if (i == target) continue;
        const float4 pf = tv.posf[i], vf = tv.velf[i];
        const float c[6] = {pf.x, pf.y, pf.z, vf.x, vf.y, vf.z};
        if (pair_lb6f(q32, c, w32, e32) >= thr) continue;  // its FP64 distance is >= top
        P4 p = tv.pos[i];
        V4 v = tv.vel[i];
        double d2 = metric ? metric_d2(x, p, v, m) : phase_d2(x, p, v);
        if (d2 < top && (!need_pos || d2 > 0)) {
          ph_replace_top<KMAX, NT>(H, t, K, d2, i);
          top = H.d[0][t];
          thr = thresh_hi_bits(dkey(top));
        }
      }
      if (h == 0) break;
      prev = h;
      h = (h - 1) >> 1;
      depth--;
      down = false;
      continue;
    }
    const int cd = nd.split_dim;
    const double xc = get6(x, cd);
    // new_off = x - cut_val < 0 exactly when x < cut_val: an integer compare of order keys
    const bool left_first = okey(xc) < okey(nd.split_val);
    const int nearh = left_first ? 2 * h + 1 : 2 * h + 2;
    const int farh = left_first ? 2 * h + 2 : 2 * h + 1;
    if (down) {  // the nearer child first, with the same offset sum
      if (depth + 1 >= kPhDepth) {
        atomicExch(err, kErrCapacity);
        return;
      }
      rd_at[depth + 1] = rd_at[depth];
      prev = h;
      h = nearh;
      depth++;
      continue;
    }
    if (prev == nearh && box_lb6f(q32, w32, e32, F[farh]) < thr) {
      // back from the nearer child: rd += -old_off*old_off + new_off*new_off, and the
      // farther child is opened when rd < top (a farther child whose bound is above the
      // top inserts nothing whether or not the reference opens it: it is passed over
      // without this FP64 test)
      const double new_off = dsub(xc, nd.split_val);
      const double old = get6(off, cd);
      const double rdf = dadd(rd_at[depth], dadd(dmul(-old, old), dmul(new_off, new_off)));
      if (rdf < top) {
        old_at[depth] = old;
        set6(off, cd, new_off);
        rd_at[depth + 1] = rdf;
        prev = h;
        h = farh;
        depth++;
        down = true;
        continue;
      }
    } else if (prev == farh) {
      set6(off, cd, old_at[depth]);  // back from the farther child: restore the offset
    }
    if (h == 0) break;
    prev = h;
    h = (h - 1) >> 1;
    depth--;
  }
}

// The coordinate search around x with the seven position images of a periodic tree, no
// gate (FindNearestPhasePeriodic / FindNearestMetricPeriodic, KDSplitNode.cxx:1153-1218);
// a tree that is one leaf searches x alone (KDLeafNode.cxx:666-679, 708-711, 725-728).
template <int KMAX, int NT>
__device__ void ph_walk_images(const TreeView& tv, PhHeap<KMAX, NT>& H, int t, int K,
                               const double x[6], const double* metric, bool need_pos,
                               bool periodic, double& top, int* err) {
  ph_walk<KMAX, NT>(tv, H, t, K, x, metric, -1, need_pos, top, err);
  if (!periodic || tv.nodes6[tv.nbase].split_dim < 0) return;
  for (int pass = 1; pass < 8; pass++) {
    double xp[6];
    reflect(x, xp, tv.period, kImageMask[pass]);
    xp[3] = x[3];
    xp[4] = x[4];
    xp[5] = x[5];
    ph_walk<KMAX, NT>(tv, H, t, K, xp, metric, -1, need_pos, top, err);
  }
}

// CalculateMetricSpacing, second half: from the 8 nearest in plain phase space around x
// (held in the first 8 heap rows; a particle at x itself included), the six direct
// offsets to the second nearest (or the next one whose offsets are all non-zero) give
// metric[j] = 1/sr0[j]^2. Returns false when fewer than 8 particles exist.
template <int KMAX, int NT>
__device__ bool ph_spacing_from_heap(const TreeView& tv, const PhHeap<KMAX, NT>& H, int t,
                                     const double x[6], double metric[6]) {
  // the reference pops the heap into ID[7..0]: ID ascending by distance
  double d[8];
  int id[8];
  for (int s = 0; s < 8; s++) {
    d[s] = H.d[s][t];
    id[s] = H.i[s][t];
  }
  for (int a = 1; a < 8; a++)
    for (int b = a; b > 0 && d[b] < d[b - 1]; b--) {
      double td = d[b];
      d[b] = d[b - 1];
      d[b - 1] = td;
      int ti = id[b];
      id[b] = id[b - 1];
      id[b - 1] = ti;
    }
  if (id[7] < 0) return false;
  double sr0[6] = {0, 0, 0, 0, 0, 0};
  double kvol = 0.0;
  for (int ivol = 1; kvol == 0.0 && ivol < 8; ivol++) {
    P4 p = tv.pos[id[ivol]];
    V4 v = tv.vel[id[ivol]];
    const double y[6] = {p.x, p.y, p.z, v.x, v.y, v.z};
    kvol = 1.0;
#pragma unroll
    for (int j = 0; j < 6; j++) {
      sr0[j] = fabs(dsub(y[j], x[j]));
      kvol = dmul(kvol, sr0[j]);
    }
  }
#pragma unroll
  for (int j = 0; j < 6; j++) metric[j] = __ddiv_rn(1.0, dmul(sr0[j], sr0[j]));
  return true;
}

// ---- the warp-cooperative exact search
// One warp serves 32 queries that are consecutive in tree order; it walks the tree once
// for all of them (a node is opened when any lane's FP32 bound in its own weights is
// below its heap top), stages each opened leaf's FP32 coordinates in shared memory, and
// every lane tests them against its own query, exactly (FP64, the reference's arithmetic)
// for the particles its FP32 screen keeps. The result is each lane's exact k nearest.
// That is the reference's answer for the plain phase distance, and for the local metric
// whenever every metric weight is at least 1 + 1e-9: the reference's unscaled offset sum
// is then below the metric distance of every particle of a cell it prunes, so it never
// prunes a particle that belongs in the heap. Lanes with a smaller weight walk the tree
// alone in the reference's order (ph_walk).
constexpr int kPhStack = 64;

template <int KMAX>
struct PhWarp {
  PhHeap<KMAX, 32> H;
  float4 sp[32], sv[32];  // FP32 position / velocity of the staged leaf particles
  int stk[kPhStack];
};

template <int KMAX>
__device__ void ph_coop(const TreeView& tv, PhWarp<KMAX>& w, int lane, bool active,
                        const double x[6], const double* metric, const float w32[6], int skip,
                        bool need_pos, int K, double& top, int* err) {
  const unsigned FULL = 0xffffffffu;
  float q32[6], e32[6];
#pragma unroll
  for (int k = 0; k < 6; k++) {
    q32[k] = __double2float_rn(x[k]);
    e32[k] = fmaxf(tv.eps6[k], __fmul_ru(__double2float_ru(fabs(x[k])), 1.2e-7f));
  }
  float thr = thresh_hi_bits(dkey(top));
  // A first screen of each pair in round to nearest: with dx = fl(q - c) per coordinate
  // and dc = fl(sum w32 dx^2) (relative error below 2^-21), the weighted distance in the
  // exact coordinates is at least (sqrt(dc / (1 + 2^-21)) / (1 + 2^-24) - e0)^2, where
  // e0 = |sqrt(w32) 2 e32| bounds the coordinates' FP32 rounding; so dc >= thr_far =
  // (sqrt(thr) + e0)^2 (1 + 2^-20), every operation rounded up, proves it is >= thr.
  float e0 = 0.f;
#pragma unroll
  for (int k = 0; k < 6; k++) {
    const float t = __fmul_ru(2.f, e32[k]);
    e0 = __fadd_ru(e0, __fmul_ru(__fmul_ru(w32[k], t), t));
  }
  e0 = __fsqrt_ru(e0);
  auto far_of = [&](float t) {
    const float s = __fadd_ru(__fsqrt_ru(t), e0);
    return __fmul_ru(__fmul_ru(s, s), 1.0f + 1.0f / 1048576.0f);
  };
  float thr_far = far_of(thr);
  const NodeS* N = tv.nodes6 + tv.nbase;
  const NodeF6* F = tv.nodef6 + tv.nbase;
  double m[6] = {1, 1, 1, 1, 1, 1};
  if (metric)
#pragma unroll
    for (int k = 0; k < 6; k++) m[k] = metric[k];
  if (lane == 0) w.stk[0] = 0;
  int sp = 1;
  __syncwarp();
  while (sp > 0) {
    const int h = w.stk[sp - 1];
    sp--;
    __syncwarp();
    const bool need = active && box_lb6f(q32, w32, e32, F[h]) < thr;
    const unsigned want = __ballot_sync(FULL, need);
    if (!want) continue;
    const NodeS nd = N[h];
    if (nd.split_dim < 0) {
      for (int c0 = 0; c0 < nd.count; c0 += 32) {
        const int mm = min(32, nd.count - c0);
        if (lane < mm) {
          w.sp[lane] = tv.posf[nd.start + c0 + lane];
          w.sv[lane] = tv.velf[nd.start + c0 + lane];
        }
        __syncwarp();
        if (need) {
          for (int j = 0; j < mm; j++) {
            const int ti = nd.start + c0 + j;
            if (ti == skip) continue;
            const float4 a = w.sp[j], b = w.sv[j];
            const float c[6] = {a.x, a.y, a.z, b.x, b.y, b.z};
            {
              float dc = 0.f;
#pragma unroll
              for (int k = 0; k < 6; k++) {
                const float d = q32[k] - c[k];
                dc = fmaf(w32[k] * d, d, dc);
              }
              if (dc >= thr_far) continue;
            }
            if (pair_lb6f(q32, c, w32, e32) >= thr) continue;
            const P4 p = tv.pos[ti];
            const V4 v = tv.vel[ti];
            const double d2 = metric ? metric_d2(x, p, v, m) : phase_d2(x, p, v);
            if (d2 < top && (!need_pos || d2 > 0)) {
              ph_replace_top<KMAX, 32>(w.H, lane, K, d2, ti);
              top = w.H.d[0][lane];
              thr = thresh_hi_bits(dkey(top));
              thr_far = far_of(thr);
            }
          }
        }
        __syncwarp();
      }
      continue;
    }
    const int hl = 2 * h + 1, hr = 2 * h + 2;
    const float dl = active ? box_lb6f(q32, w32, e32, F[hl]) : FLT_MAX;
    const float dr = active ? box_lb6f(q32, w32, e32, F[hr]) : FLT_MAX;
    const unsigned bl = __ballot_sync(FULL, active && dl < thr);
    const unsigned br = __ballot_sync(FULL, active && dr < thr);
    const int leader = __ffs(want) - 1;
    const float dl0 = __shfl_sync(FULL, dl, leader), dr0 = __shfl_sync(FULL, dr, leader);
    if (sp + 2 > kPhStack) {
      if (lane == 0) atomicExch(err, kErrCapacity);
      return;
    }
    // the farther child (for the first wanting lane) is pushed first, so the nearer opens first
    const bool lfirst = dl0 <= dr0;
    const int first = lfirst ? hr : hl, second = lfirst ? hl : hr;
    const bool fneed = lfirst ? br != 0 : bl != 0, sneed = lfirst ? bl != 0 : br != 0;
    if (fneed) {
      if (lane == 0) w.stk[sp] = first;
      sp++;
    }
    if (sneed) {
      if (lane == 0) w.stk[sp] = second;
      sp++;
    }
    __syncwarp();
  }
}

// The coordinate form with the seven ungated position images of a periodic tree (a tree
// that is one leaf searches x alone), for the warp.
template <int KMAX>
__device__ void ph_coop_images(const TreeView& tv, PhWarp<KMAX>& w, int lane, bool active,
                               const double x[6], const double* metric, const float w32[6],
                               bool need_pos, bool periodic, int K, double& top, int* err) {
  ph_coop<KMAX>(tv, w, lane, active, x, metric, w32, -1, need_pos, K, top, err);
  if (!periodic || tv.nodes6[tv.nbase].split_dim < 0) return;
  for (int pass = 1; pass < 8; pass++) {
    double xp[6];
    reflect(x, xp, tv.period, kImageMask[pass]);
    xp[3] = x[3];
    xp[4] = x[4];
    xp[5] = x[5];
    ph_coop<KMAX>(tv, w, lane, active, xp, metric, w32, -1, need_pos, K, top, err);
  }
}

template <int KMAX>
__host__ __device__ constexpr int ph_warps_per_block() {
  return KMAX <= 16 ? 8 : (KMAX <= 32 ? 4 : (KMAX <= 64 ? 2 : 1));
}

template <int KMAX>
__global__ void __launch_bounds__(32 * ph_warps_per_block<KMAX>()) k_phase(PhaseArgs pa) {
  constexpr int WPB = ph_warps_per_block<KMAX>();
  const KnnArgs& a = pa.k;
  const TreeView& tv = a.tv;
  extern __shared__ __align__(16) unsigned char smem[];
  PhWarp<KMAX>& w = reinterpret_cast<PhWarp<KMAX>*>(smem)[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const int gw = blockIdx.x * WPB + (threadIdx.x >> 5);
  if (gw * 32 >= a.nq) return;  // whole warps only
  const int q = gw * 32 + lane;
  bool valid = q < a.nq;
  // the query: a tree particle (qmode 0: q0 + q; 2: qidx[q]) or a phase-space point
  int self = -1;
  double x[6] = {0, 0, 0, 0, 0, 0};
  if (valid && a.qmode == 1) {
#pragma unroll
    for (int j = 0; j < 6; j++) x[j] = a.qx[6 * (size_t)q + j];
  } else if (valid) {
    const int ti = a.qmode == 0 ? a.q0 + q : a.qidx[q];
    if (ti < 0 || ti >= tv.n) {
      atomicExch(a.err, kErrTarget);
      valid = false;
    } else {
      self = tv.pstart + ti;
      const P4 p = tv.pos[self];
      const V4 v = tv.vel[self];
      x[0] = p.x;
      x[1] = p.y;
      x[2] = p.z;
      x[3] = v.x;
      x[4] = v.y;
      x[5] = v.z;
    }
  }
  const int K = a.kheap;
  const bool periodic = a.periodic != 0;
  const float ones[6] = {1.f, 1.f, 1.f, 1.f, 1.f, 1.f};
  double metric[6] = {1, 1, 1, 1, 1, 1};
  float w32[6] = {1.f, 1.f, 1.f, 1.f, 1.f, 1.f};
  bool coop = valid;
  if (pa.metric) {
    // CalculateMetricSpacing: the exact 8 nearest in plain phase space (a coordinate search)
    if (valid) ph_fill<KMAX, 32>(w.H, lane, 8);
    double top8 = kMaxValue;
    ph_coop_images<KMAX>(tv, w, lane, valid, x, nullptr, ones, false, pa.spacing_periodic != 0,
                         8, top8, a.err);
    if (valid && !ph_spacing_from_heap<KMAX, 32>(tv, w.H, lane, x, metric)) {
      atomicExch(a.err, kErrTooFew);
      valid = false;
    }
    double mmin = metric[0], mmax = metric[0];
#pragma unroll
    for (int j = 0; j < 6; j++) {
      mmin = fmin(mmin, metric[j]);
      mmax = fmax(mmax, metric[j]);
      w32[j] = __double2float_rd(metric[j]);
    }
    coop = valid && mmin >= 1.0 + 1e-9 && mmax < INFINITY;
  }
  const double* mp = pa.metric ? metric : nullptr;
  if (valid) ph_fill<KMAX, 32>(w.H, lane, K);
  double top = kMaxValue;
  if (self >= 0 && !periodic) {
    // the target forms: the target itself and distance 0 are skipped
    ph_coop<KMAX>(tv, w, lane, coop, x, mp, w32, self, true, K, top, a.err);
    if (valid && !coop) ph_walk<KMAX, 32>(tv, w.H, lane, K, x, mp, self, true, top, a.err);
  } else {
    // the coordinate forms (also a periodic target search): the local metric skips
    // distance 0, the plain distance skips nothing
    ph_coop_images<KMAX>(tv, w, lane, coop, x, mp, w32, pa.metric != 0, periodic, K, top,
                         a.err);
    if (valid && !coop)
      ph_walk_images<KMAX, 32>(tv, w.H, lane, K, x, mp, pa.metric != 0, periodic, top, a.err);
  }
  if (!valid) return;
  if (pa.epi == kPhNN) {
    // LoadNN: the heap popped into rows [kout-1 .. 0]; a heap of kout + 1 drops its nearest
    double d[KMAX];
    int id[KMAX];
    for (int s = 0; s < K; s++) {
      d[s] = w.H.d[s][lane];
      id[s] = w.H.i[s][lane];
    }
    for (int s = 1; s < K; s++)
      for (int b = s; b > 0 && d[b] < d[b - 1]; b--) {
        double td = d[b];
        d[b] = d[b - 1];
        d[b - 1] = td;
        int ti = id[b];
        id[b] = id[b - 1];
        id[b - 1] = ti;
      }
    const int skip = K - a.kout;
    for (int s = 0; s < a.kout; s++) {
      int j = id[skip + s];
      a.nn[(size_t)q * a.kout + s] = j >= 0 ? j - tv.pstart : -1;
      a.d2[(size_t)q * a.kout + s] = d[skip + s];
    }
    return;
  }
  // CalcDensity / CalcDensityParticle: h = 0.5 sqrt(top), norm = h^-6 times the product
  // of sqrt(metric[j]) (KDCalcSmoothQuantities.cxx:251-270)
  for (int s = 0; s < K; s++)
    if (w.H.i[s][lane] < 0) {
      atomicExch(a.err, kErrTooFew);
      return;
    }
  const double hh = dmul(0.5, __dsqrt_rn(top));
  const double ih = __ddiv_rn(1.0, hh);
  const double ih2 = dmul(ih, ih);
  double norm = dmul(dmul(ih2, ih2), ih2);
  if (pa.metric) {
    double temp = 1.0;
#pragma unroll
    for (int j = 0; j < 6; j++) temp = dmul(temp, __dsqrt_rn(metric[j]));
    norm = dmul(norm, temp);
  }
  const int kr = a.kernres;
  const double inv_delta = 0.5 * (double)(kr - 1);
  const bool scatter = pa.epi == kPhDensity;
  const double wnorm = scatter ? dmul(0.5, norm) : norm;
  const double mi = tv.pos[self].m;
  double acc = 0.0;
  const long long topk = dkey(top);
  for (int s = 0; s < K; s++) {
    const int j = w.H.i[s][lane];
    const double rij = __dsqrt_rn(w.H.d[s][lane]);
    // the farthest neighbour: q = 2 exactly, the table's last entry
    const double wq = dkey(w.H.d[s][lane]) == topk ? a.kernel[kr - 1]
                                                    : wsm_line(__ddiv_rn(rij, hh), kr, inv_delta, a.kernel);
    const double wv = dmul(wq, wnorm);
    const double mj = tv.pos[j].m;
    acc = dadd(acc, dmul(wv, mj));
    if (scatter) atomicAdd(&a.rho[j - tv.pstart], dmul(wv, mi));
  }
  if (scatter) atomicAdd(&a.rho[self - tv.pstart], acc);
  else a.rho[q] = acc;
}

template <int KMAX>
int launch_phase_t(const PhaseArgs& pa, cudaStream_t st) {
  constexpr int WPB = ph_warps_per_block<KMAX>();
  size_t sm = sizeof(PhWarp<KMAX>) * WPB;
  NBK_TRY(ensure_dyn_smem((const void*)k_phase<KMAX>, (int)sm));
  unsigned warps = (unsigned)((pa.k.nq + 31) / 32);
  k_phase<KMAX><<<(warps + WPB - 1) / WPB, 32 * WPB, sm, st>>>(pa);
  note_launch();
  NBK_CUDA_TRY(cudaGetLastError());
  return NBK_OK;
}

}  // namespace

int launch_phase(const PhaseArgs& pa, cudaStream_t st) {
  if (pa.k.nq <= 0) return NBK_OK;
  Phase ph(pa.epi == kPhNN ? "phase_knn" : "phase_density", st);
  int K = pa.k.kheap;
  if (K < 1 || K > 128 || pa.k.kout > K) {
    set_error("phase-space search: heap size must be in [1, 128]");
    return NBK_ERR_UNSUPPORTED;
  }
  // heaps hold at least the 8 entries of the metric spacing
  if (K <= 16) return launch_phase_t<16>(pa, st);
  if (K <= 32) return launch_phase_t<32>(pa, st);
  if (K <= 64) return launch_phase_t<64>(pa, st);
  return launch_phase_t<128>(pa, st);
}

}  // namespace nbk
