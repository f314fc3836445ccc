// Friends-of-friends on the GPU (replaces KDTree::FOF, src/KDTree/KDFOF.cxx:29-153, and
// the node searches it drives: SplitNode/LeafNode::FOFSearchBall[Periodic],
// KDSplitNode.cxx:921-988, 1602-1646, KDLeafNode.cxx:527-589).
//
// The reference grows one group at a time by breadth-first search; its result is the
// set of connected components of the graph "d2 < ll^2" (with periodic images), numbered
// by the first member met in tree order, groups below minnum dropped. Here:
//  1. prelink: every particle is united with the first particle of its largest
//     "compact" ancestor node (box diagonal certainly below ll, so every pair inside is
//     linked);
//  2. link: one warp per 32 consecutive particles walks the tree with radius ll. A
//     compact node that lies wholly inside a lane's ball is united with that lane's
//     particle in one step; otherwise leaves are tested pair by pair in FP64 with the
//     reference's arithmetic and linked pairs are united. Union-find links the larger
//     root under the smaller (atomicCAS), so every root ends as its component's minimum
//     tree index.
//  3. label: roots of components with at least minnum members get 1..G in increasing
//     root order -- the reference's numbering (discovery order in tree order).
// All FP32 shortcuts are conservative (directed rounding), so the linked pairs are
// exactly those the FP64 test links.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "nbk_build.h"

namespace nbk {

namespace {

// Iteration cap of every union-find loop (root finding, flattening, uniting). The
// default is far above any chain the link phase leaves; a loop that reaches it sets
// kErrIterCap and returns, and the host reports NBK_ERR_DEVICE. Adjustable per device
// through nbk_debug_set_iteration_cap (a test hook that makes the limit run out).
constexpr int kCapDefault = 1 << 24;
__constant__ int c_uf_cap = kCapDefault;

__device__ __forceinline__ int ld_parent(const int* p, int x) {
  return *((volatile const int*)p + x);
}

__device__ __forceinline__ int find_root(int* parent, int x, int* err) {
  for (int it = 0; it < c_uf_cap; it++) {
    int p = ld_parent(parent, x);
    if (p == x) return x;
    int gp = ld_parent(parent, p);
    if (gp != p) atomicCAS(&parent[x], p, gp);
    x = gp;
  }
  atomicExch(err, kErrIterCap);
  return x;
}

__device__ __forceinline__ void unite(int* parent, int a, int b, int* err) {
  const int cap = min(c_uf_cap, 1 << 20);
  for (int it = 0; it < cap; it++) {
    a = find_root(parent, a, err);
    b = find_root(parent, b, err);
    if (a == b) return;
    if (a < b) {
      int t = a;
      a = b;
      b = t;
    }
    int old = atomicCAS(&parent[a], a, b);
    if (old == a) return;
    a = old;
  }
  atomicExch(err, kErrIterCap);
}

__device__ __forceinline__ bool node_compact(const NodeRec& r, float ll2_lo) {
  float ex = __fsub_ru(r.hi[0], r.lo[0]), ey = __fsub_ru(r.hi[1], r.lo[1]),
        ez = __fsub_ru(r.hi[2], r.lo[2]);
  float d = __fadd_ru(__fadd_ru(__fmul_ru(ex, ex), __fmul_ru(ey, ey)), __fmul_ru(ez, ez));
  return d < ll2_lo;
}

__global__ void k_iota(int* p, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = i;
}

// 1. unite each particle with the first particle of its highest compact ancestor
__global__ void k_prelink(FofArgs a) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  const TreeView& tv = a.tv;
  if (t >= tv.n) return;
  int ti = tv.pstart + t;
  float ll2_lo = thresh_lo(a.ll2);
  int h = 0;
  for (int depth = 0; depth < 64; depth++) {
    NodeRec r = tv.node[tv.nbase + h];
    if (node_compact(r, ll2_lo)) {
      if (r.start != ti) unite(a.parent, ti, r.start, a.err);
      return;
    }
    if (r.count <= tv.b) return;
    NodeRec l = tv.node[tv.nbase + 2 * h + 1];
    h = (ti < l.start + l.count) ? 2 * h + 1 : 2 * h + 2;
  }
}

constexpr int kStack = 64;    // depth-first stack of the criterion search (one lane)
constexpr int kWpb = 8;
constexpr int kFStack = 512;  // frontier stack of the link search (one warp)
constexpr int kBatchLimit = kFStack - 128;

struct FofSmem {
  float4 sf[32];
  int par[32];  // parents of the staged leaf particles, read once per leaf
  int stk[kFStack];
};

// Lower bound of the squared distance between two boxes (FP32, directed rounding).
__device__ __forceinline__ float boxbox_d2_lo(const NodeRec& r, const float qlo[3],
                                              const float qhi[3]) {
  float g[3];
#pragma unroll
  for (int d = 0; d < 3; d++)
    g[d] = fmaxf(0.f, fmaxf(__fsub_rd(r.lo[d], qhi[d]), __fsub_rd(qlo[d], r.hi[d])));
  return __fadd_rd(__fadd_rd(__fmul_rd(g[0], g[0]), __fmul_rd(g[1], g[1])), __fmul_rd(g[2], g[2]));
}

// ---- FOFCriterion (KDFOF.cxx:157-265). The comparators of FOFFunc.h:30-55, in the
// reference's operation order: total += (a-b)*(a-b)/params[6] per dimension (FOF6d
// interleaves position and velocity terms), linked when total < 1.
__device__ __forceinline__ bool crit_cmp(int cmp, const double* p, const double xa[3],
                                         const V4& va, const P4& xb, const V4& vb) {
  double total = 0.0;
  double xb3[3] = {xb.x, xb.y, xb.z}, va3[3] = {va.x, va.y, va.z}, vb3[3] = {vb.x, vb.y, vb.z};
#pragma unroll
  for (int j = 0; j < 3; j++) {
    if (cmp == 0 || cmp == 2) {
      double d = dsub(xa[j], xb3[j]);
      total = dadd(total, __ddiv_rn(dmul(d, d), p[6]));
    }
    if (cmp == 1) {
      double d = dsub(va3[j], vb3[j]);
      total = dadd(total, __ddiv_rn(dmul(d, d), p[6]));
    }
    if (cmp == 2) {
      double d = dsub(va3[j], vb3[j]);
      total = dadd(total, __ddiv_rn(dmul(d, d), p[7]));
    }
  }
  return total < 1.0;
}

// 2. One warp links 32 consecutive particles. The traversal is frontier-parallel: each
// step pops up to 32 nodes from the warp's stack, lane i loads node i, drops it when it
// lies farther than ll from the box around all of the warp's query points, and for a
// compact node chases its union-find root, so the dependent loads of up to 32 nodes
// overlap. Surviving inner nodes that are not compact are expanded at once; surviving
// leaves and compact nodes are then tested against every lane's own query.
//
// CRIT3D: FOFCriterion with FOF3d inside its search region, run as FOF with
// ll^2 = params[6]; the FP32 decisions are the same (their 2^-20 margins cover the
// rounding of the comparator's divisions) and the pairs left to FP64 take the comparator.
template <bool CRIT3D>
__global__ void __launch_bounds__(32 * kWpb, 4) k_link(FofArgs a) {
  __shared__ FofSmem sm[kWpb];
  const unsigned FULL = 0xffffffffu;
  int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  FofSmem& w = sm[warp];
  const TreeView& tv = a.tv;
  int q = (blockIdx.x * kWpb + warp) * 32 + lane;
  if ((blockIdx.x * kWpb + warp) * 32 >= tv.n) return;
  bool valid = q < tv.n;
  int self = tv.pstart + (valid ? q : 0);
  P4 me = tv.pos[self];
  double x0[3] = {me.x, me.y, me.z};
  float thr = thresh_hi(a.ll2), ll2_lo = thresh_lo(a.ll2);
  long long ll2k = a.ll2 > 0.0 ? dkey(a.ll2) : 0;  // no link for ll2 <= 0 or NaN
  float eps = tv.eps, two_eps = __fmul_ru(2.f, tv.eps);
  int myroot = find_root(a.parent, self, a.err);  // cached; refreshed when it goes stale
  int npass = tv.periodic ? 8 : 1;
  int near = tv.periodic && valid ? near_walls(tv.posf[self], tv.period, eps, thr) : 0;
  for (int pass = 0; pass < npass; pass++) {
    double xq[3] = {x0[0], x0[1], x0[2]};
    bool active = valid;
    if (pass > 0) {
      // images no lane can open are skipped before any FP64 work
      bool may = (kImageMask[pass] & ~near) == 0;
      if (!__any_sync(FULL, may)) continue;
      double sval = reflect(x0, xq, tv.period, kImageMask[pass]);
      active = active && may && (a.ll2 > dmul(sval, sval));  // KDSplitNode.cxx:1611
    }
    if (!__any_sync(FULL, active)) continue;
    float qx = __double2float_rn(xq[0]), qy = __double2float_rn(xq[1]),
          qz = __double2float_rn(xq[2]);
    // box around the active lanes' query points, widened by eps
    float qlo[3], qhi[3];
    {
      float v[3] = {qx, qy, qz};
#pragma unroll
      for (int d = 0; d < 3; d++) {
        float lo = active ? __fsub_rd(v[d], eps) : FLT_MAX;
        float hi = active ? __fadd_ru(v[d], eps) : -FLT_MAX;
        for (int o = 16; o > 0; o >>= 1) {
          lo = fminf(lo, __shfl_xor_sync(FULL, lo, o));
          hi = fmaxf(hi, __shfl_xor_sync(FULL, hi, o));
        }
        qlo[d] = lo;
        qhi[d] = hi;
      }
    }
    int sp = 1;
    if (lane == 0) w.stk[0] = 0;
    __syncwarp();
    const int first = tv.pstart + (blockIdx.x * kWpb + warp) * 32;  // lane 0's particle
    for (int guard = 0; sp > 0 && guard < (1 << 26); guard++) {
      // above kBatchLimit entries pop one node at a time: a depth-first descent from
      // there adds at most the tree depth, so the stack never exceeds kFStack
      int m = sp <= kBatchLimit ? min(32, sp) : 1;
      int h = 0, root = -1;
      NodeRec r;
      bool keep = false, cpt = false;
      if (lane < m) {
        h = w.stk[sp - 1 - lane];
        r = tv.node[tv.nbase + h];
        // direct pass: a node wholly before the warp's first particle in tree order only
        // holds pairs that particle's own search tests (each pair once, from its lower
        // index), so it is not opened
        keep = boxbox_d2_lo(r, qlo, qhi) < thr && (pass != 0 || r.start + r.count - 1 > first);
        cpt = keep && node_compact(r, ll2_lo);
        if (cpt) root = find_root(a.parent, r.start, a.err);
      }
      __syncwarp();
      sp -= m;
      // a kept node that is neither compact nor a leaf is expanded at once: the lanes'
      // own balls are tested at its leaves
      const bool inner = keep && !cpt && r.count > tv.b;
      unsigned expand = __ballot_sync(FULL, inner);
      unsigned todo = __ballot_sync(FULL, keep && !inner);
      while (todo) {
        int j = __ffs(todo) - 1;
        todo &= todo - 1;
        int rootj = __shfl_sync(FULL, root, j);
        // a compact node already in every active lane's component adds nothing: skipped
        // before its box is broadcast
        if (rootj >= 0 && __all_sync(FULL, rootj == myroot || !active)) continue;
        NodeRec rj;
#pragma unroll
        for (int d = 0; d < 3; d++) {
          rj.lo[d] = __shfl_sync(FULL, r.lo[d], j);
          rj.hi[d] = __shfl_sync(FULL, r.hi[d], j);
        }
        rj.start = __shfl_sync(FULL, r.start, j);
        rj.count = __shfl_sync(FULL, r.count, j);
        bool need = active && box_d2_lo(qx, qy, qz, eps, rj) < thr;
        if (need && rootj >= 0) {
          // a compact node was prelinked: all its particles share one root. If that root
          // is already ours nothing inside can add a link (the parallel form of the
          // reference's BucketFlag, KDLeafNode.cxx:529-588); if the node lies wholly
          // inside the ball, one union links all of it.
          if (rootj != myroot) myroot = find_root(a.parent, myroot, a.err);
          if (rootj == myroot) {
            need = false;
          } else if (box_far_d2_hi(qx, qy, qz, eps, rj) < ll2_lo) {
            unite(a.parent, self, rj.start, a.err);
            myroot = find_root(a.parent, self, a.err);
            need = false;
          }
        }
        if (!__any_sync(FULL, need)) continue;
        if (rj.count > tv.b) {
          expand |= 1u << j;
          continue;
        }
        for (int c0 = 0; c0 < rj.count; c0 += 32) {
          int mm = min(32, rj.count - c0);
          if (lane < mm) {
            w.sf[lane] = tv.posf[rj.start + c0 + lane];
            w.par[lane] = ld_parent(a.parent, rj.start + c0 + lane);
          }
          __syncwarp();
          if (need) {
            for (int jj = 0; jj < mm; jj++) {
              int ti = rj.start + c0 + jj;
              // direct pass: the test is symmetric, so each pair is handled once
              if (pass == 0 && ti <= self) continue;
              // a staged parent equal to our root proves one component for good (links
              // and path halving never separate a component), so no root chase is needed
              int pj = w.par[jj];
              if (pj == myroot || ti == myroot) continue;
              float4 cf = w.sf[jj];
              if (pair_d2_lo(qx, qy, qz, cf.x, cf.y, cf.z, two_eps) < thr) {
                // decided in FP32 when the upper bound is already inside; only pairs
                // within a few FP32 ulps of the linking length take the FP64 test
                bool in = pair_d2_hi(qx, qy, qz, cf.x, cf.y, cf.z, two_eps) < ll2_lo;
                if (!in) {
                  P4 c = tv.pos[ti];
                  if (CRIT3D) in = crit_cmp(0, a.params, xq, make_v4(0, 0, 0, 0), c, make_v4(0, 0, 0, 0));
                  else in = dkey(dist2_exact(xq[0], xq[1], xq[2], c.x, c.y, c.z)) < ll2k;
                }
                if (in) {
                  int rt = find_root(a.parent, pj, a.err);
                  if (rt != myroot) myroot = find_root(a.parent, myroot, a.err);
                  if (rt != myroot) {
                    unite(a.parent, self, ti, a.err);
                    myroot = find_root(a.parent, self, a.err);
                  }
                }
              }
            }
          }
          __syncwarp();
        }
      }
      // children of the expanded nodes: lane i pushes those of its own node
      int ne = __popc(expand);
      if (sp + 2 * ne > kFStack) {
        if (lane == 0) atomicExch(a.err, kErrCapacity);
        return;
      }
      if ((expand >> lane) & 1u) {
        int slot = sp + 2 * __popc(expand & ((1u << lane) - 1u));
        w.stk[slot] = 2 * h + 2;
        w.stk[slot + 1] = 2 * h + 1;
      }
      sp += 2 * ne;
      __syncwarp();
    }
    if (sp > 0 && lane == 0) atomicExch(a.err, kErrIterCap);
  }
}

// Node pruning of SplitNode::FOFSearchCriterion (KDSplitNode.cxx:991-1028): the far child
// is opened when rd + (-old^2 + new^2) * invscaling < 1, with old/new the offsets to the
// cut planes along the path. This reachability is part of the reference's result (pairs
// it never reaches are never compared), so it is reproduced exactly: one thread per
// particle walks the tree with the same split planes, carrying rd and the offsets.
__device__ __forceinline__ double crit_invscaling(const double* p, int cd) {
  int tt = (int)p[0];
  if (tt == 0) return 1.0 / p[1];
  if (tt == 2) return 1.0 / p[2];
  if (tt == 3) return 1.0 / p[(cd < 3) * 1 + (cd >= 3) * 2];
  return 1.0;
}

// ---- FOFNNCriterion / FOFNNDistCriterion (KDFOF.cxx:380-506, 507-640). The reference
// grows groups breadth-first, testing each member t against its listed neighbours
// nn[t][j] with the comparator; every particle ends up tested, and merges join whole
// groups, so its groups are the connected components of the accepted (t, nn[t][j]) edges.
// One thread per particle unites it with each accepted neighbour. For the distance form,
// params[pidx[k]] take the particle's own value before its comparisons, as the reference
// sets them from distfunc(numNN, dist2[t]).
__global__ void __launch_bounds__(256) k_nn_link(FofArgs a) {
  const TreeView& tv = a.tv;
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= tv.n) return;
  int self = tv.pstart + q;
  P4 me = tv.pos[self];
  V4 mv = tv.vel ? tv.vel[self] : make_v4(0, 0, 0, 0);
  double x0[3] = {me.x, me.y, me.z};
  double p[8];
#pragma unroll
  for (int k = 0; k < 8; k++) p[k] = a.params[k];
  if (a.pval)
    for (int k = 0; k < a.npc; k++) {
      double v = a.pval[q];
#pragma unroll
      for (int m = 0; m < 8; m++)
        if (m == a.pidx[k]) p[m] = v;  // static indices keep p in registers
    }
  const int* row = a.nn + (size_t)q * a.numnn;
  for (int j = 0; j < a.numnn; j++) {
    int b = row[j];
    if (b < 0 || b >= tv.n) {
      if (b >= tv.n) atomicExch(a.err, kErrTarget);
      continue;
    }
    if (b == q) continue;
    int bi = tv.pstart + b;
    V4 vb = tv.vel ? tv.vel[bi] : make_v4(0, 0, 0, 0);
    if (crit_cmp(a.cmp, p, x0, mv, tv.pos[bi], vb)) unite(a.parent, self, bi, a.err);
  }
}

__global__ void __launch_bounds__(128) k_crit_link(FofArgs a) {
  const TreeView& tv = a.tv;
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= tv.n) return;
  int self = tv.pstart + q;
  P4 me = tv.pos[self];
  V4 mv = tv.vel ? tv.vel[self] : make_v4(0, 0, 0, 0);
  double x0[3] = {me.x, me.y, me.z};
  int stk_h[kStack];
  double stk_rd[kStack], stk_off[kStack][3];
  // FOF3d and FOF6d accept a pair only if sum dx^2 / params[6] < 1 (FOFFunc.h:30-55): a
  // subtree (or particle) whose FP32 bound of that sum is at or above 1 + 2^-20 holds
  // nothing to link and is passed over (FOFVel is not bounded by positions)
  const float wpos = a.cmp == 1 ? 0.f : __double2float_rd(__ddiv_rd(1.0, a.params[6]));
  const float thr1 = 1.0f + 1.0f / 1048576.0f;
  int npass = tv.periodic ? 8 : 1;
  for (int pass = 0; pass < npass; pass++) {
    double xq[3] = {x0[0], x0[1], x0[2]};
    if (pass > 0) reflect(x0, xq, tv.period, kImageMask[pass]);  // ungated (:1649-1681)
    const float qx = __double2float_rn(xq[0]), qy = __double2float_rn(xq[1]),
                qz = __double2float_rn(xq[2]);
    const float eps = query_eps(tv, xq[0], xq[1], xq[2]), two_eps = __fadd_ru(eps, tv.eps);
    int sp = 0;
    stk_h[0] = 0;
    stk_rd[0] = 0.0;
    stk_off[0][0] = stk_off[0][1] = stk_off[0][2] = 0.0;
    sp = 1;
    while (sp > 0) {
      sp--;
      int h = stk_h[sp];
      double rd = stk_rd[sp];
      double off[3] = {stk_off[sp][0], stk_off[sp][1], stk_off[sp][2]};
      NodeRec r = tv.node[tv.nbase + h];
      if (wpos > 0.f && __fmul_rd(wpos, box_d2_lo(qx, qy, qz, eps, r)) >= thr1) continue;
      if (r.count <= tv.b) {
        for (int i = r.start; i < r.start + r.count; i++) {
          if (i == self) continue;
          if (wpos > 0.f) {
            const float4 cf = tv.posf[i];
            if (__fmul_rd(wpos, pair_d2_lo(qx, qy, qz, cf.x, cf.y, cf.z, two_eps)) >= thr1)
              continue;
          }
          P4 xb = tv.pos[i];
          V4 vb = tv.vel ? tv.vel[i] : make_v4(0, 0, 0, 0);
          if (crit_cmp(a.cmp, a.params, xq, mv, xb, vb)) unite(a.parent, self, i, a.err);
        }
        continue;
      }
      const NodeX& nx = tv.nodex[tv.nbase + h];
      int cd = nx.split_dim;
      double old_off = off[cd];
      double new_off = dsub(xq[cd], nx.split_val);
      int nearh = new_off < 0 ? 2 * h + 1 : 2 * h + 2;
      int farh = new_off < 0 ? 2 * h + 2 : 2 * h + 1;
      double rdf = dadd(rd, dmul(dadd(dmul(-old_off, old_off), dmul(new_off, new_off)),
                                 crit_invscaling(a.params, cd)));
      if (sp + 2 > kStack) {
        atomicExch(a.err, kErrCapacity);
        return;
      }
      if (rdf < 1.0) {
        stk_h[sp] = farh;
        stk_rd[sp] = rdf;
        stk_off[sp][0] = off[0];
        stk_off[sp][1] = off[1];
        stk_off[sp][2] = off[2];
        stk_off[sp][cd] = new_off;
        sp++;
      }
      stk_h[sp] = nearh;
      stk_rd[sp] = rd;
      stk_off[sp][0] = off[0];
      stk_off[sp][1] = off[1];
      stk_off[sp][2] = off[2];
      sp++;
    }
  }
}

constexpr int kCritStack = 512;  // frontier stack of the phase-space link search (one warp)
constexpr int kCritBatchLimit = kCritStack - 128;
struct CritSmem {
  float4 sp[32], sv[32];
  int par[32];
  int stk[kCritStack];
};

// FP32 lower bound of sum_j w[j] * gap_j^2 between the box [qlo, qhi] around a warp's
// query points and a node's FP32 box; every operation rounds down.
__device__ __forceinline__ float boxbox_lb6f(const float qlo[6], const float qhi[6],
                                             const float w[6], const NodeF6& b) {
  float s = 0.f;
#pragma unroll
  for (int j = 0; j < 6; j++) {
    float g = fmaxf(0.f, fmaxf(__fsub_rd(b.lo[j], qhi[j]), __fsub_rd(qlo[j], b.hi[j])));
    s = __fadd_rd(s, __fmul_rd(__fmul_rd(w[j], g), g));
  }
  return s;
}

// FOF6d weights 1/params[6] (positions) and 1/params[7] (velocities) rounded down / up.
__device__ __forceinline__ void fof6d_weights(const double* p, float w_lo[6], float w_hi[6]) {
#pragma unroll
  for (int j = 0; j < 3; j++) {
    w_lo[j] = __double2float_rd(__ddiv_rd(1.0, p[6]));
    w_hi[j] = __double2float_ru(__ddiv_ru(1.0, p[6]));
    w_lo[3 + j] = __double2float_rd(__ddiv_rd(1.0, p[7]));
    w_hi[3 + j] = __double2float_ru(__ddiv_ru(1.0, p[7]));
  }
}

// FOFCriterion with FOF6d inside its search region on a physical tree: the accepted
// pairs are those with sum dx^2 / params[6] + sum dv^2 / params[7] < 1, a unit ball of a
// scaled phase space, whose components do not depend on the tree searched. They are found
// on a phase-space tree built for the call over the same particles (its splits follow the
// velocities where those spread more, so the search prunes in velocity too): one warp per
// 32 particles walks it with FP32 bounds of the comparator's sum and unites the accepted
// pairs (the reference's comparator in FP64 for pairs within a few FP32 ulps of 1); the
// components are then carried over to the physical tree's indices.
__global__ void __launch_bounds__(32 * kWpb) k_crit6_warp(FofArgs a) {
  __shared__ CritSmem sm[kWpb];
  const unsigned FULL = 0xffffffffu;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  CritSmem& w = sm[warp];
  const TreeView& tv = a.tv;
  const int q = (blockIdx.x * kWpb + warp) * 32 + lane;
  if ((blockIdx.x * kWpb + warp) * 32 >= tv.n) return;
  const bool valid = q < tv.n;
  const int self = tv.pstart + (valid ? q : 0);
  const P4 me = tv.pos[self];
  const V4 mv = tv.vel[self];
  const double x0[3] = {me.x, me.y, me.z};
  float w_lo[6], w_hi[6];
  fof6d_weights(a.params, w_lo, w_hi);
  const float thr_hi = 1.0f + 1.0f / 1048576.0f, thr_lo = 1.0f - 1.0f / 1048576.0f;
  const NodeS* N = tv.nodes6 + tv.nbase;
  const NodeF6* F = tv.nodef6 + tv.nbase;
  int myroot = find_root(a.parent, self, a.err);
  const int first = tv.pstart + (blockIdx.x * kWpb + warp) * 32;  // lane 0's particle
  const int npass = (tv.periodic && N[0].split_dim >= 0) ? 8 : 1;
  for (int pass = 0; pass < npass; pass++) {
    double xq[6] = {x0[0], x0[1], x0[2], mv.x, mv.y, mv.z};
    bool active = valid;
    if (pass > 0) {
      // an image links only if its position part can stay below 1: sval^2 < params[6]
      const double sval = reflect(x0, xq, tv.period, kImageMask[pass]);
      active = active && a.params[6] > dmul(sval, sval);
    }
    if (!__any_sync(FULL, active)) continue;
    float q32[6], e32[6];
#pragma unroll
    for (int k = 0; k < 6; k++) {
      q32[k] = __double2float_rn(xq[k]);
      e32[k] = fmaxf(tv.eps6[k], __fmul_ru(__double2float_ru(fabs(xq[k])), 1.2e-7f));
    }
    // box around the active lanes' query intervals
    float qlo[6], qhi[6];
#pragma unroll
    for (int k = 0; k < 6; k++) {
      float lo = active ? __fsub_rd(q32[k], e32[k]) : FLT_MAX;
      float hi = active ? __fadd_ru(q32[k], e32[k]) : -FLT_MAX;
      for (int o = 16; o > 0; o >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(FULL, lo, o));
        hi = fmaxf(hi, __shfl_xor_sync(FULL, hi, o));
      }
      qlo[k] = lo;
      qhi[k] = hi;
    }
    if (lane == 0) w.stk[0] = 0;
    int sp = 1;
    __syncwarp();
    // frontier-parallel: each step pops up to 32 nodes, lane i loads node i and drops it
    // when the warp's query box cannot reach it, so the dependent node loads overlap; the
    // surviving inner nodes are expanded at once, the surviving leaves tested against
    // every lane's own query
    for (int guard = 0; sp > 0 && guard < (1 << 26); guard++) {
      // above kCritBatchLimit entries pop one node at a time: a depth-first descent from
      // there adds at most the tree depth, so the stack never exceeds kCritStack
      const int m = sp <= kCritBatchLimit ? min(32, sp) : 1;
      int h = 0;
      NodeS nd{};
      NodeF6 f{};
      bool keep = false;
      if (lane < m) {
        h = w.stk[sp - 1 - lane];
        nd = N[h];
        f = F[h];
        // direct pass: nodes wholly before the warp's first particle hold only pairs
        // tested from their lower index
        keep = boxbox_lb6f(qlo, qhi, w_lo, f) < thr_hi &&
               (pass != 0 || nd.start + nd.count - 1 > first);
      }
      __syncwarp();
      sp -= m;
      // a kept inner node is expanded at once: the lanes' own queries are tested at its
      // leaves
      const bool inner = keep && nd.split_dim >= 0;
      unsigned expand = __ballot_sync(FULL, inner);
      unsigned todo = __ballot_sync(FULL, keep && !inner);
      while (todo) {
        const int jn = __ffs(todo) - 1;
        todo &= todo - 1;
        NodeF6 fj;
#pragma unroll
        for (int k = 0; k < 6; k++) {
          fj.lo[k] = __shfl_sync(FULL, f.lo[k], jn);
          fj.hi[k] = __shfl_sync(FULL, f.hi[k], jn);
        }
        const bool need = active && box_lb6f(q32, w_lo, e32, fj) < thr_hi;
        if (!__any_sync(FULL, need)) continue;
        if (__shfl_sync(FULL, nd.split_dim, jn) >= 0) {
          expand |= 1u << jn;
          continue;
        }
        const int nstart = __shfl_sync(FULL, nd.start, jn);
        const int ncount = __shfl_sync(FULL, nd.count, jn);
        for (int c0 = 0; c0 < ncount; c0 += 32) {
          const int mm = min(32, ncount - c0);
          if (lane < mm) {
            const int i = nstart + c0 + lane;
            w.sp[lane] = tv.posf[i];
            w.sv[lane] = tv.velf[i];
            w.par[lane] = ld_parent(a.parent, i);
          }
          __syncwarp();
          if (need) {
            for (int jj = 0; jj < mm; jj++) {
              const int ti = nstart + c0 + jj;
              if (ti == self || (pass == 0 && ti < self)) continue;  // direct pass: each pair once
              const int pj = w.par[jj];
              if (pj == myroot || ti == myroot) continue;
              const float4 cp = w.sp[jj], cv = w.sv[jj];
              const float c[6] = {cp.x, cp.y, cp.z, cv.x, cv.y, cv.z};
              if (pair_lb6f(q32, c, w_lo, e32) >= thr_hi) continue;
              bool in = pair_ub6f(q32, c, w_hi, e32) < thr_lo;
              if (!in) in = crit_cmp(2, a.params, xq, mv, tv.pos[ti], tv.vel[ti]);
              if (in) {
                int rt = find_root(a.parent, pj, a.err);
                if (rt != myroot) myroot = find_root(a.parent, myroot, a.err);
                if (rt != myroot) {
                  unite(a.parent, self, ti, a.err);
                  myroot = find_root(a.parent, self, a.err);
                }
              }
            }
          }
          __syncwarp();
        }
      }
      // children of the expanded nodes: lane i pushes those of its own node
      const int ne = __popc(expand);
      if (sp + 2 * ne > kCritStack) {
        if (lane == 0) atomicExch(a.err, kErrCapacity);
        return;
      }
      if ((expand >> lane) & 1u) {
        const int slot = sp + 2 * __popc(expand & ((1u << lane) - 1u));
        w.stk[slot] = 2 * h + 2;
        w.stk[slot + 1] = 2 * h + 1;
      }
      sp += 2 * ne;
      __syncwarp();
    }
    if (sp > 0 && lane == 0) atomicExch(a.err, kErrIterCap);
  }
}

// The phase-space tree's components carried to the physical tree: each particle is united
// with its component's root (perm6: phase-space tree index -> physical tree index).
__global__ void k_carry_roots(const int* parent6, const int* perm6, int* parent, int n,
                              int* err) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  int r = j;
  for (int it = 0; it < c_uf_cap; it++) {
    int p = parent6[r];
    if (p == r) break;
    r = p;
  }
  if (r != j) unite(parent, perm6[j], perm6[r], err);
}

// Positions, velocities and masses of a tree, in its order, as n x 3 arrays (the input
// layout of a build).
__global__ void k_unpack(const P4* pos, const V4* vel, double* p3, double* v3, double* m, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  P4 p = pos[i];
  V4 v = vel[i];
  p3[3 * (size_t)i] = p.x;
  p3[3 * (size_t)i + 1] = p.y;
  p3[3 * (size_t)i + 2] = p.z;
  v3[3 * (size_t)i] = v.x;
  v3[3 * (size_t)i + 1] = v.y;
  v3[3 * (size_t)i + 2] = v.z;
  m[i] = p.m;
}


// FOFCriterion on a phase-space tree (KDFOF.cxx:157-265 with FOFSearchCriterion[Periodic],
// KDSplitNode.cxx:991-1030, 1649-1682, KDLeafNode.cxx:591-619): every particle walks the
// tree with the reference's reachability rule (the farther child when the offset sum,
// scaled per cut dimension by 1/params[1] or 1/params[2], stays below 1) and unites with
// each particle the comparator accepts. The reference's breadth-first grouping equals
// these connected components when each comparator's linking region lies inside the search
// region, so that every link is found from both of its ends.
__global__ void __launch_bounds__(128) k_crit_link6(FofArgs a) {
  const TreeView& tv = a.tv;
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= tv.n) return;
  const int self = tv.pstart + q;
  const P4 me = tv.pos[self];
  const V4 mv = tv.vel[self];
  const double x0[6] = {me.x, me.y, me.z, mv.x, mv.y, mv.z};
  const NodeS* N = tv.nodes6 + tv.nbase;
  const NodeF6* F = tv.nodef6 + tv.nbase;
  // the comparator's weights per coordinate (FOFFunc.h:30-55), rounded down: a subtree (or
  // a particle) whose FP32 bound in them is at or above 1 + 2^-20 holds nothing the
  // comparator accepts (its FP64 sum is >= 1), so it is skipped
  float w[6], e32[6];
#pragma unroll
  for (int j = 0; j < 3; j++) {
    w[j] = a.cmp == 1 ? 0.f : __double2float_rd(__ddiv_rd(1.0, a.params[6]));
    w[3 + j] = a.cmp == 0 ? 0.f : __double2float_rd(__ddiv_rd(1.0, a.params[a.cmp == 1 ? 6 : 7]));
  }
#pragma unroll
  for (int j = 0; j < 6; j++) e32[j] = tv.eps6[j];
  const float thr = 1.0f + 1.0f / 1048576.0f;
  int npass = (tv.periodic && N[0].split_dim >= 0) ? 8 : 1;
  for (int pass = 0; pass < npass; pass++) {
    double x[6];
    reflect(x0, x, tv.period, kImageMask[pass]);  // ungated (KDSplitNode.cxx:1649-1681)
    x[3] = x0[3];
    x[4] = x0[4];
    x[5] = x0[5];
    float q32[6];
#pragma unroll
    for (int j = 0; j < 6; j++) q32[j] = __double2float_rn(x[j]);
    double off[6] = {0, 0, 0, 0, 0, 0};
    double rd_at[kPhDepth], old_at[kPhDepth];
    int h = 0, depth = 0, prev = -1;
    bool down = true;
    rd_at[0] = 0.0;
    while (true) {
      if (down && box_lb6f(q32, w, e32, F[h]) >= thr) {
        if (h == 0) break;
        prev = h;
        h = (h - 1) >> 1;
        depth--;
        down = false;
        continue;
      }
      const NodeS nd = N[h];
      if (down && nd.split_dim < 0) {
        for (int i = nd.start; i < nd.start + nd.count; i++) {
          if (i == self) continue;
          const float4 pf = tv.posf[i], vf = tv.velf[i];
          const float c[6] = {pf.x, pf.y, pf.z, vf.x, vf.y, vf.z};
          if (pair_lb6f(q32, c, w, e32) >= thr) continue;
          if (crit_cmp(a.cmp, a.params, x, mv, tv.pos[i], tv.vel[i])) unite(a.parent, self, i, a.err);
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
      const bool left_first = okey(xc) < okey(nd.split_val);  // new_off < 0
      const int nearh = left_first ? 2 * h + 1 : 2 * h + 2;
      const int farh = left_first ? 2 * h + 2 : 2 * h + 1;
      if (down) {
        if (depth + 1 >= kPhDepth) {
          atomicExch(a.err, kErrCapacity);
          return;
        }
        rd_at[depth + 1] = rd_at[depth];
        prev = h;
        h = nearh;
        depth++;
        continue;
      }
      // a farther child that holds nothing the comparator accepts is passed over without
      // the FP64 reachability test
      if (prev == nearh && box_lb6f(q32, w, e32, F[farh]) < thr) {
        const double new_off = dsub(xc, nd.split_val);
        const double old = get6(off, cd);
        const double rdf = dadd(rd_at[depth], dmul(dadd(dmul(-old, old), dmul(new_off, new_off)),
                                                   crit_invscaling(a.params, cd)));
        if (rdf < 1.0) {
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
        set6(off, cd, old_at[depth]);
      }
      if (h == 0) break;
      prev = h;
      h = (h - 1) >> 1;
      depth--;
    }
  }
}

// Point every particle straight at its root (between phases: no unions in flight).
__global__ void k_compress(int* parent, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int x = i;
  for (int it = 0; it < c_uf_cap; it++) {
    int p = ld_parent(parent, x);
    if (p == x) break;
    x = p;
  }
  parent[i] = x;
}

__global__ void k_flatten_count(int* parent, int n, int* cnt, int* err) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool valid = i < n;
  int x = valid ? i : -1;
  if (valid) {
    int it = 0;
    for (; it < c_uf_cap; it++) {
      int p = parent[x];
      if (p == x) break;
      x = p;
    }
    if (it == c_uf_cap) atomicExch(err, kErrIterCap);
    parent[i] = x;  // no concurrent writers remain; roots are untouched
  }
  // neighbouring particles mostly share a root: one atomic per distinct root in the warp
  unsigned peers = __match_any_sync(0xffffffffu, x);
  if (valid && (threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&cnt[x], __popc(peers));
}

__global__ void k_valid(const int* parent, const int* cnt, int n, int minnum, int* flag) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  flag[i] = (parent[i] == i && cnt[i] >= minnum) ? 1 : 0;
}

// exclusive scan (three-phase, 1024 per block)
__global__ void k_scan_blocks(const int* in, int* out, int* bsum, int n) {
  __shared__ int s[1024];
  int i = blockIdx.x * 1024 + threadIdx.x;
  int v = i < n ? in[i] : 0;
  s[threadIdx.x] = v;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    int t = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
    __syncthreads();
    s[threadIdx.x] += t;
    __syncthreads();
  }
  if (i < n) out[i] = s[threadIdx.x] - v;
  if (threadIdx.x == 1023) bsum[blockIdx.x] = s[1023];
}
__global__ void k_scan_sums(int* bsum, int nb, int* total) {
  __shared__ int run;
  if (threadIdx.x == 0) run = 0;
  __syncthreads();
  for (int c0 = 0; c0 < nb; c0 += 1024) {
    __shared__ int s[1024];
    int i = c0 + threadIdx.x;
    int v = i < nb ? bsum[i] : 0;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
      int t = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
      __syncthreads();
      s[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < nb) bsum[i] = run + s[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == 1023) run += s[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = run;
}
__global__ void k_scan_add(int* out, const int* bsum, int n) {
  int i = blockIdx.x * 1024 + threadIdx.x;
  if (i < n) out[i] += bsum[blockIdx.x];
}

__global__ void k_label(const int* parent, const int* flag, const int* lbl, int n, int* group) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int r = parent[i];
  group[i] = flag[r] ? lbl[r] + 1 : 0;
}

// order = 1: sort keys (size descending, then label) with a bitonic network in global
// memory; then new_label[old] = rank + 1.
__global__ void k_order_keys(const int* parent, const int* flag, const int* lbl, const int* cnt,
                             int n, unsigned long long* keys) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (flag[i]) {
    unsigned size = (unsigned)cnt[i];
    keys[lbl[i]] = ((unsigned long long)(0xffffffffu - size) << 32) | (unsigned)lbl[i];
  }
}
__global__ void k_pad(unsigned long long* keys, int g, int P) {
  int i = g + blockIdx.x * blockDim.x + threadIdx.x;
  if (i < P) keys[i] = ~0ull;
}
__global__ void k_bitonic(unsigned long long* keys, int P, int kk, int jj) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= P) return;
  int u = t ^ jj;
  if (u > t) {
    bool up = (t & kk) == 0;
    unsigned long long a = keys[t], b = keys[u];
    if ((a > b) == up) {
      keys[t] = b;
      keys[u] = a;
    }
  }
}
__global__ void k_rank(const unsigned long long* keys, int g, int* newlbl) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g) return;
  newlbl[(int)(keys[i] & 0xffffffffu)] = i + 1;
}
__global__ void k_relabel(int* group, const int* newlbl, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int g = group[i];
  if (g > 0) group[i] = newlbl[g - 1];
}

}  // namespace

// FOF6d inside its search region on a physical tree (see k_crit6_warp): builds the
// phase-space tree of the same particles, links on it, and unites the physical tree's
// parent forest accordingly.
static int link_fof6d_phase_tree(const FofArgs& a, DevAlloc& alloc, cudaStream_t st) {
  const int n = a.tv.n;
  const int b = a.tv.b;
  double *p3, *v3, *m;
  NBK_TRY(alloc.get((void**)&p3, sizeof(double) * 3 * (size_t)n));
  NBK_TRY(alloc.get((void**)&v3, sizeof(double) * 3 * (size_t)n));
  NBK_TRY(alloc.get((void**)&m, sizeof(double) * (size_t)n));
  k_unpack<<<(n + 255) / 256, 256, 0, st>>>(a.tv.pos + a.tv.pstart, a.tv.vel + a.tv.pstart, p3,
                                             v3, m, n);
  note_launch();
  const int64_t slots = heap_slots(n, b);
  BuiltArrays A6;
  NBK_TRY(alloc.get((void**)&A6.pos, sizeof(P4) * (size_t)n));
  NBK_TRY(alloc.get((void**)&A6.posf, sizeof(float4) * (size_t)n));
  NBK_TRY(alloc.get((void**)&A6.vel, sizeof(V4) * (size_t)n));
  NBK_TRY(alloc.get((void**)&A6.velf, sizeof(float4) * (size_t)n));
  NBK_TRY(alloc.get((void**)&A6.perm, sizeof(int) * (size_t)n));
  NBK_TRY(alloc.get((void**)&A6.nodes6, sizeof(NodeS) * (size_t)slots));
  NBK_TRY(alloc.get((void**)&A6.nodeb6, sizeof(NodeB6) * (size_t)slots));
  NBK_TRY(alloc.get((void**)&A6.nodef6, sizeof(NodeF6) * (size_t)slots));
  NBK_CUDA_TRY(cudaMemsetAsync(A6.nodes6, 0, sizeof(NodeS) * (size_t)slots, st));
  NodeB6 root;
  {
    DevAlloc alloc6;  // the build releases its own scratch when it ends
    alloc6.st = st;
    std::vector<TreeSpec> trees{{0, n, 0}};
    NBK_TRY(build_forest_phase(trees, b, p3, m, v3, A6, alloc6, st, &root));
  }
  FofArgs f = a;
  TreeView& v = f.tv;
  v = TreeView{};
  v.pos = A6.pos;
  v.posf = A6.posf;
  v.vel = A6.vel;
  v.velf = A6.velf;
  v.perm = A6.perm;
  v.nodes6 = A6.nodes6;
  v.nodeb6 = A6.nodeb6;
  v.nodef6 = A6.nodef6;
  v.n = n;
  v.b = b;
  v.periodic = a.tv.periodic;
  for (int d = 0; d < 3; d++) v.period[d] = a.tv.period[d];
  for (int d = 0; d < 6; d++) {
    double mx = std::max(std::fabs(root.lo[d]), std::fabs(root.hi[d])) +
                (d < 3 ? v.period[d] : 0.0);
    v.eps6[d] = (float)std::ldexp(mx, -23) * 1.0001f + 1e-38f;
  }
  v.eps = a.tv.eps;
  int* parent6;
  NBK_TRY(alloc.get((void**)&parent6, sizeof(int) * (size_t)n));
  k_iota<<<(n + 255) / 256, 256, 0, st>>>(parent6, n);
  note_launch();
  f.parent = parent6;
  const int warps = (n + 31) / 32;
  k_crit6_warp<<<(warps + kWpb - 1) / kWpb, 32 * kWpb, 0, st>>>(f);
  note_launch();
  // the phase-space tree's "input" order is the physical tree's order: perm6 maps to it
  k_carry_roots<<<(n + 255) / 256, 256, 0, st>>>(parent6, A6.perm, a.parent + a.tv.pstart, n,
                                                 a.err);
  note_launch();
  NBK_CUDA_TRY(cudaGetLastError());
  return NBK_OK;
}

int run_fof(const FofArgs& a, int nnodes, int minnum, int order, int* d_group_tree,
            int* h_ngroup, DevAlloc& alloc, cudaStream_t st, bool defer_count) {
  (void)nnodes;
  int n = a.tv.n;
  if (n == 0) {
    *h_ngroup = 0;
    return NBK_OK;
  }
  int* cnt;
  int *flag, *lbl, *bsum, *d_total;
  int nb = (n + 1023) / 1024;
  // every caller synchronises its stream before it returns (the group count, or the
  // error word; an early return here waits), so this thread's kept block is free again
  SyncUnlessOk sync_guard{st};
  NBK_TRY(thread_scratch_block(1, {{(void**)&cnt, sizeof(int) * n},
                                   {(void**)&flag, sizeof(int) * n},
                                   {(void**)&lbl, sizeof(int) * n},
                                   {(void**)&bsum, sizeof(int) * (nb + 1)},
                                   {(void**)&d_total, sizeof(int)}},
                               st, alloc));
  k_iota<<<(n + 255) / 256, 256, 0, st>>>(a.parent, n); note_launch();
  // FOFCriterion with FOF3d inside its search region links exactly the pairs with
  // sum dx^2 / params[6] < 1: the FOF kernels with ll^2 = params[6]
  const bool fof3d = a.crit == 1 && a.crit_contained && a.cmp == 0 && !a.tv.nodes6;
  FofArgs f = a;
  if (fof3d) f.ll2 = a.params[6];
  if (!a.crit || fof3d) {
    Phase ph("fof_prelink", st);
    k_prelink<<<(n + 255) / 256, 256, 0, st>>>(f); note_launch();
    k_compress<<<(n + 255) / 256, 256, 0, st>>>(a.parent, n); note_launch();
  }
  int warps = (n + 31) / 32;
  if (a.crit == 2) {
    Phase ph("fof_nn_link", st);
    k_nn_link<<<(n + 255) / 256, 256, 0, st>>>(a); note_launch();
  } else if (a.crit && a.tv.nodes6 && a.crit_contained) {
    // FOF6d inside the search region on a phase-space tree: the warp search directly
    Phase ph("fof_criterion_link", st);
    k_crit6_warp<<<(warps + kWpb - 1) / kWpb, 32 * kWpb, 0, st>>>(a); note_launch();
  } else if (a.crit && a.tv.nodes6) {
    Phase ph("fof_criterion_link", st);
    k_crit_link6<<<(n + 127) / 128, 128, 0, st>>>(a); note_launch();
  } else if (fof3d) {
    Phase ph("fof_criterion_link", st);
    k_link<true><<<(warps + kWpb - 1) / kWpb, 32 * kWpb, 0, st>>>(f); note_launch();
  } else if (a.crit && a.crit_contained && a.cmp == 2) {
    Phase ph("fof_criterion_link", st);
    NBK_TRY(link_fof6d_phase_tree(a, alloc, st));
  } else if (a.crit) {
    Phase ph("fof_criterion_link", st);
    k_crit_link<<<(n + 127) / 128, 128, 0, st>>>(a); note_launch();
  } else {
    Phase ph("fof_link", st);
    k_link<false><<<(warps + kWpb - 1) / kWpb, 32 * kWpb, 0, st>>>(a); note_launch();
  }
  Phase ph_label("fof_label", st);
  NBK_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(int) * n, st));
  k_flatten_count<<<(n + 255) / 256, 256, 0, st>>>(a.parent, n, cnt, a.err); note_launch();
  k_valid<<<(n + 255) / 256, 256, 0, st>>>(a.parent, cnt, n, minnum, flag); note_launch();
  k_scan_blocks<<<nb, 1024, 0, st>>>(flag, lbl, bsum, n); note_launch();
  k_scan_sums<<<1, 1024, 0, st>>>(bsum, nb, d_total); note_launch();
  k_scan_add<<<nb, 1024, 0, st>>>(lbl, bsum, n); note_launch();
  k_label<<<(n + 255) / 256, 256, 0, st>>>(a.parent, flag, lbl, n, d_group_tree); note_launch();
  NBK_CUDA_TRY(cudaGetLastError());
  if (defer_count && !order) {
    // the caller's page-locked h_ngroup is read after the caller's own synchronisation
    NBK_CUDA_TRY(cudaMemcpyAsync(h_ngroup, d_total, sizeof(int), cudaMemcpyDeviceToHost, st));
    sync_guard.ok = true;
    return NBK_OK;
  }
  int total = 0;
  NBK_CUDA_TRY(cudaMemcpyAsync(&total, d_total, sizeof(int), cudaMemcpyDeviceToHost, st));
  NBK_CUDA_TRY(cudaStreamSynchronize(st));
  *h_ngroup = total;
  if (order && total > 1) {
    int P = 1;
    while (P < total) P <<= 1;
    unsigned long long* keys;
    int* newlbl;
    NBK_TRY(alloc.get((void**)&keys, sizeof(unsigned long long) * P));
    NBK_TRY(alloc.get((void**)&newlbl, sizeof(int) * total));
    k_order_keys<<<(n + 255) / 256, 256, 0, st>>>(a.parent, flag, lbl, cnt, n, keys); note_launch();
    if (P > total) k_pad<<<(P - total + 255) / 256, 256, 0, st>>>(keys, total, P); note_launch();
    for (int kk = 2; kk <= P; kk <<= 1)
      for (int jj = kk >> 1; jj > 0; jj >>= 1)
        k_bitonic<<<(P + 255) / 256, 256, 0, st>>>(keys, P, kk, jj); note_launch();
    k_rank<<<(total + 255) / 256, 256, 0, st>>>(keys, total, newlbl); note_launch();
    k_relabel<<<(n + 255) / 256, 256, 0, st>>>(d_group_tree, newlbl, n); note_launch();
    NBK_CUDA_TRY(cudaGetLastError());
  }
  sync_guard.ok = true;  // the count was read above (a synchronisation); callers wait again
  return NBK_OK;
}

// Union-find iteration cap on the current device; cap <= 0 restores the default.
int set_uf_iteration_cap(int cap) {
  int v = cap > 0 ? cap : kCapDefault;
  NBK_CUDA_TRY(cudaMemcpyToSymbol(c_uf_cap, &v, sizeof(int)));
  return NBK_OK;
}

}  // namespace nbk
