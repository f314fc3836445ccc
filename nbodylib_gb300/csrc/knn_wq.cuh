// Warp-per-query k-nearest-neighbour search for target queries (a query that is a
// particle of the tree): the kNN behind CalcDensity, CalcVelDensity, CalcDensityParticle,
// CalcVelDensityParticle and FindNearest / FindNearestPos of tree particles.
//
// Replaces the depth-first search of SplitNode/LeafNode::FindNearestPos(target)
// (src/KDTree/KDSplitNode.cxx:15-41, KDLeafNode.cxx:15-28) with its bounded max-heap
// (src/KDTree/PriorityQueue.h:14-85), and the periodic wrapper of KDSplitNode.cxx:1119-1147.
//
// Work mapping: one warp serves one query. The query's k-list is distributed over the
// warp's registers, sorted: position p = s * 32 + lane holds the p-th smallest (d2, index)
// in slot s of that lane (S slots, k <= 32 S). A batch of candidates enters by a bitonic
// sort over the lanes and a merge with the list (one or two slots), or one candidate at a time
// by a ballot (its position) and a shuffle of the tail one place up; the k-th distance
// (the heap top of the reference) is one shuffle away.
//
// Search order: the query's own subtree first -- the smallest node on its path holding
// more than k particles, found from the tree's split rule by integer arithmetic (left
// child = the first (size - 1) / 2 + 1 particles, leaf when size <= b). An FP32 upper
// bound of the k-th distance over that subtree's particles is found first, then they are
// tested; then the rest of the tree -- the subtrees of the siblings of that node and of
// each of its ancestors -- frontier-parallel: each step pops up to 32 stack nodes, one per
// lane, and prunes them against the k-th distance.
//
// FP64 work: candidates are screened by an FP32 lower bound of their squared distance
// (directed rounding, never below the FP64 value); those that pass are compacted into a
// per-warp queue, and the exact FP64 distance ((dx*dx + dy*dy) + dz*dz), the reference's
// association, is computed 32 queued candidates at a time, so the FP64 instructions run
// with every lane busy. A candidate enters when d2 < the k-th distance (strict, as the
// reference's `dist2 < pq->TopPriority()`); the FP32 screen uses a bound at or above the
// k-th distance, the exact test the current k-th distance, so the result is the exact k
// nearest. The batched kernel's one-slot searches first run the whole search on FP32
// bounds alone (wq_search_f32), then compute FP64 distances only for the particles within
// the final FP32 bound of the k-th distance; for one large tree that extra FP32 work
// costs more than the FP64 it saves, so the direct form above serves it.
#pragma once
#include "nbk_build.h"

namespace nbk {
namespace {

constexpr int kWqStack = 192;      // frontier stack (node indices) per warp
constexpr int kWqBatchLimit = 64;  // above this many entries the stack pops one at a time
constexpr long long kWqSent = 0x7fffffffffffffffll;  // key beyond position k - 1

constexpr int kWqBuf = 256;  // candidates kept per query by the FP32 search

struct WqSmem {
  int stk[kWqStack];
  int queue[64];        // candidates (tree indices) that passed the FP32 screen
  int buf[kWqBuf];      // FP32 search: candidates whose lower bound was within the bound
  unsigned blo[kWqBuf];  // and those lower bounds (FP32 bit patterns)
};

// The sorted k-list of one query: keys are the bit patterns of the non-negative squared
// distances (they order as the values do, on the integer pipe).
template <int S>
struct WqList {
  long long key[S];
  int idx[S];
};

template <int S>
__device__ __forceinline__ void wq_init(WqList<S>& L, int lane, int K) {
  const long long kmax = __double_as_longlong(kMaxValue);
#pragma unroll
  for (int s = 0; s < S; s++) {
    int p = s * 32 + lane;
    L.key[s] = p < K ? kmax : kWqSent;  // the reference pre-fills with (-1, MAXVALUE)
    L.idx[s] = -1;
  }
}

// Key at position p of the list (every lane gets it).
template <int S>
__device__ __forceinline__ long long wq_key_at(const WqList<S>& L, int p) {
  long long v = L.key[0];
#pragma unroll
  for (int s = 1; s < S; s++)
    if ((p >> 5) == s) v = L.key[s];
  return __shfl_sync(0xffffffffu, v, p & 31);
}

// Insert (k, j) (the same on every lane) into a list of K entries; the caller has
// checked k < the key at position K - 1.
template <int S>
__device__ __forceinline__ void wq_insert(WqList<S>& L, int lane, int K, long long k, int j) {
  const unsigned FULL = 0xffffffffu;
  int pos = 0;
#pragma unroll
  for (int s = 0; s < S; s++) pos += __popc(__ballot_sync(FULL, L.key[s] <= k));
#pragma unroll
  for (int s = S - 1; s >= 0; s--) {
    long long up = __shfl_up_sync(FULL, L.key[s], 1);
    int upi = __shfl_up_sync(FULL, L.idx[s], 1);
    if (s > 0) {
      long long c = __shfl_sync(FULL, L.key[s - 1], 31);
      int ci = __shfl_sync(FULL, L.idx[s - 1], 31);
      if (lane == 0) {
        up = c;
        upi = ci;
      }
    }
    int p = s * 32 + lane;
    if (p == pos) {
      L.key[s] = k;
      L.idx[s] = j;
    } else if (p > pos) {
      L.key[s] = up;
      L.idx[s] = upi;
    }
    if (p >= K) {
      L.key[s] = kWqSent;
      L.idx[s] = -1;
    }
  }
}

// Ascending bitonic sort of one (key, index) pair per lane over the warp (equal keys are
// never exchanged).
__device__ __forceinline__ void warp_sort_asc(long long& k, int& j, int lane) {
  const unsigned FULL = 0xffffffffu;
#pragma unroll
  for (int size = 2; size <= 32; size <<= 1) {
#pragma unroll
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      long long ok = __shfl_xor_sync(FULL, k, stride);
      int oj = __shfl_xor_sync(FULL, j, stride);
      bool up = (lane & size) == 0;
      bool lower = (lane & stride) == 0;
      bool take = (lower == up) ? (ok < k) : (ok > k);
      if (take) {
        k = ok;
        j = oj;
      }
    }
  }
}

// Merge a batch sorted ascending over the lanes into a one-slot list of K <= 32 entries:
// the lower half of Batcher's merge (list ascending against the batch reversed; the list
// keeps ties) holds the 32 smallest of both as a bitonic sequence, which five
// half-cleaners sort.
__device__ __forceinline__ void wq_merge1(WqList<1>& L, int lane, int K, long long k, int j) {
  const unsigned FULL = 0xffffffffu;
  long long rk = __shfl_sync(FULL, k, 31 - lane);
  int rj = __shfl_sync(FULL, j, 31 - lane);
  bool tb = rk < L.key[0];
  long long mk = tb ? rk : L.key[0];
  int mj = tb ? rj : L.idx[0];
#pragma unroll
  for (int stride = 16; stride > 0; stride >>= 1) {
    long long ok = __shfl_xor_sync(FULL, mk, stride);
    int oj = __shfl_xor_sync(FULL, mj, stride);
    bool lower = (lane & stride) == 0;
    bool take = lower ? (ok < mk) : (ok > mk);
    if (take) {
      mk = ok;
      mj = oj;
    }
  }
  if (lane >= K) {
    mk = kWqSent;
    mj = -1;
  }
  L.key[0] = mk;
  L.idx[0] = mj;
}

// The same for a two-slot list of K <= 64 entries (positions 0-31 in slot 0, 32-63 in
// slot 1): against the 128-sequence list ascending ++ (batch padded to 64 with +inf)
// reversed, the lower half keeps slot 0 and takes min(slot 1, batch reversed); that
// bitonic 64-sequence is sorted by an in-lane compare-exchange (stride 32) and five
// shuffle half-cleaners per slot.
__device__ __forceinline__ void wq_merge2(WqList<2>& L, int lane, int K, long long k, int j) {
  const unsigned FULL = 0xffffffffu;
  long long rk = __shfl_sync(FULL, k, 31 - lane);
  int rj = __shfl_sync(FULL, j, 31 - lane);
  long long a0 = L.key[0], a1 = L.key[1];
  int i0 = L.idx[0], i1 = L.idx[1];
  if (rk < a1) {
    a1 = rk;
    i1 = rj;
  }
  if (a1 < a0) {
    long long tk = a0;
    a0 = a1;
    a1 = tk;
    int ti = i0;
    i0 = i1;
    i1 = ti;
  }
#pragma unroll
  for (int stride = 16; stride > 0; stride >>= 1) {
    bool lower = (lane & stride) == 0;
    long long o0 = __shfl_xor_sync(FULL, a0, stride);
    int p0 = __shfl_xor_sync(FULL, i0, stride);
    long long o1 = __shfl_xor_sync(FULL, a1, stride);
    int p1 = __shfl_xor_sync(FULL, i1, stride);
    if (lower ? (o0 < a0) : (o0 > a0)) {
      a0 = o0;
      i0 = p0;
    }
    if (lower ? (o1 < a1) : (o1 > a1)) {
      a1 = o1;
      i1 = p1;
    }
  }
  if (lane >= K) {
    a0 = kWqSent;
    i0 = -1;
  }
  if (32 + lane >= K) {
    a1 = kWqSent;
    i1 = -1;
  }
  L.key[0] = a0;
  L.idx[0] = i0;
  L.key[1] = a1;
  L.idx[1] = i1;
}

// Per-warp search state of one query.
template <int S>
struct WqQuery {
  WqList<S> L;
  int K;
  long long topk;  // key at position K - 1
  float thr;       // FP32 value at or above the k-th distance (screens boxes, particles)
  double xq[3];    // the query point of this pass (exact)
  float qx, qy, qz, eps, two_eps;
  int self;        // tree index excluded by the target search (-1: none)
  int qn;          // candidates waiting in the queue
};

template <int S>
__device__ __forceinline__ void wq_set_point(WqQuery<S>& Q, const TreeView& tv, const double x[3]) {
  Q.xq[0] = x[0];
  Q.xq[1] = x[1];
  Q.xq[2] = x[2];
  Q.qx = __double2float_rn(x[0]);
  Q.qy = __double2float_rn(x[1]);
  Q.qz = __double2float_rn(x[2]);
  Q.eps = query_eps(tv, x[0], x[1], x[2]);
  Q.two_eps = __fadd_ru(Q.eps, tv.eps);
}

// Exact FP64 test of the first `cnt` queued candidates (one per lane) and insertion of
// those below the k-th distance.
template <int S>
__device__ void wq_flush(WqQuery<S>& Q, WqSmem& w, const TreeView& tv, int lane, int cnt) {
  const unsigned FULL = 0xffffffffu;
  bool have = lane < cnt;
  int ti = have ? w.queue[lane] : 0;
  long long dk = kWqSent;
  if (have) {
    P4 c = tv.pos[ti];
    double d2 = dist2_exact(Q.xq[0], Q.xq[1], Q.xq[2], c.x, c.y, c.z);
    dk = dkey(d2);
    if (Q.self >= 0 && (ti == Q.self || dk == 0)) dk = kWqSent;  // KDLeafNode.cxx:19-21
  }
  unsigned acc = __ballot_sync(FULL, dk < Q.topk);
  if (S <= 2 && __popc(acc) > 2) {
    // many at once: sort the batch and merge it (the k smallest of list and batch: the
    // same entries the one-by-one strict insertions keep, up to exact ties)
    long long k = dk < Q.topk ? dk : kWqSent;
    int j = ti;
    warp_sort_asc(k, j, lane);
    if (S == 1) wq_merge1(*reinterpret_cast<WqList<1>*>(&Q.L), lane, Q.K, k, j);
    else wq_merge2(*reinterpret_cast<WqList<2>*>(&Q.L), lane, Q.K, k, j);
    Q.topk = wq_key_at<S>(Q.L, Q.K - 1);
    acc = 0;
  }
  while (acc) {
    int src = __ffs(acc) - 1;
    acc &= acc - 1;
    long long k = __shfl_sync(FULL, dk, src);
    int j = __shfl_sync(FULL, ti, src);
    if (k < Q.topk) {  // d2 < top, against the k-th distance of this moment
      wq_insert<S>(Q.L, lane, Q.K, k, j);
      Q.topk = wq_key_at<S>(Q.L, Q.K - 1);
    }
  }
  Q.thr = fminf(Q.thr, thresh_hi_bits(Q.topk));
}

// FP32 screen of one candidate per lane (valid lanes only); survivors join the queue,
// which is flushed 32 at a time.
template <int S>
__device__ __forceinline__ void wq_consider(WqQuery<S>& Q, WqSmem& w, const TreeView& tv,
                                            int lane, bool valid, int ti) {
  const unsigned FULL = 0xffffffffu;
  bool pass = false;
  if (valid) {
    float4 cf = tv.posf[ti];
    pass = pair_d2_lo(Q.qx, Q.qy, Q.qz, cf.x, cf.y, cf.z, Q.two_eps) < Q.thr;
  }
  unsigned pm = __ballot_sync(FULL, pass);
  if (!pm) return;
  if (pass) w.queue[Q.qn + __popc(pm & ((1u << lane) - 1u))] = ti;
  Q.qn += __popc(pm);
  __syncwarp();
  if (Q.qn >= 32) {
    wq_flush<S>(Q, w, tv, lane, 32);
    __syncwarp();
    int rest = Q.qn - 32;
    int moved = lane < rest ? w.queue[32 + lane] : 0;
    __syncwarp();
    if (lane < rest) w.queue[lane] = moved;
    Q.qn = rest;
    __syncwarp();
  }
}

template <int S>
__device__ __forceinline__ void wq_drain(WqQuery<S>& Q, WqSmem& w, const TreeView& tv, int lane) {
  if (Q.qn > 0) {
    wq_flush<S>(Q, w, tv, lane, Q.qn);
    Q.qn = 0;
    __syncwarp();
  }
}

// Every particle of the node range [start, start + count) through the screen.
template <int S>
__device__ __forceinline__ void wq_range(WqQuery<S>& Q, WqSmem& w, const TreeView& tv, int lane,
                                         int start, int count) {
  for (int c0 = 0; c0 < count; c0 += 32)
    wq_consider<S>(Q, w, tv, lane, c0 + lane < count, start + c0 + lane);
}

// ---- FP32 search (target queries, one-slot lists): the whole search runs on FP32
// bounds only. An FP32 k-list keeps the K smallest upper bounds of the squared distance
// (particles other than the query and provably at a non-zero distance), so its last
// entry T bounds the k-th distance from above; every particle whose lower bound is at or
// below the T of the moment is kept in a buffer. Afterwards only the kept particles with
// a lower bound at or below the final T -- the k nearest and the few within the FP32
// rounding of them -- get exact FP64 distances. Bit patterns of non-negative floats order
// as their values; 0xffffffff marks an empty list position (above +inf).
struct WqF32 {
  unsigned fk;   // this lane's position of the FP32 k-list (one slot)
  unsigned tb;   // bits of T, the list's entry K - 1
  int bn;        // particles in the buffer
  bool over;     // the buffer overflowed: the query takes the exact search instead
};

__device__ __forceinline__ void warp_sort_asc_u32(unsigned& k, int lane) {
#pragma unroll
  for (int size = 2; size <= 32; size <<= 1) {
#pragma unroll
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      unsigned ok = __shfl_xor_sync(0xffffffffu, k, stride);
      bool up = (lane & size) == 0;
      bool lower = (lane & stride) == 0;
      bool take = (lower == up) ? (ok < k) : (ok > k);
      if (take) k = ok;
    }
  }
}

// FP32 screen of one candidate per lane (valid lanes only): keep it when its lower
// bound is within T, and let its upper bound into the FP32 k-list.
template <int S>
__device__ __forceinline__ void wq32_consider(const WqQuery<S>& Q, WqF32& F, WqSmem& w,
                                              const TreeView& tv, int lane, bool valid, int ti,
                                              int self, int K) {
  const unsigned FULL = 0xffffffffu;
  unsigned lob = 0xffffffffu, hib = 0xffffffffu;
  if (valid) {
    float4 cf = tv.posf[ti];
    float lo = pair_d2_lo(Q.qx, Q.qy, Q.qz, cf.x, cf.y, cf.z, Q.two_eps);
    lob = __float_as_uint(lo);
    if (lob <= F.tb && ti != self && lo > 0.f)
      hib = __float_as_uint(pair_d2_hi(Q.qx, Q.qy, Q.qz, cf.x, cf.y, cf.z, Q.two_eps));
  }
  bool keep = valid && lob <= F.tb;
  unsigned km = __ballot_sync(FULL, keep);
  if (!km) return;
  int nk = __popc(km);
  if (F.bn + nk > kWqBuf) {
    // drop kept particles that the bound has since excluded
    int nb = 0;
    for (int c0 = 0; c0 < F.bn; c0 += 32) {
      int i = c0 + lane;
      bool stay = i < F.bn && w.blo[i] <= F.tb;
      int bi = stay ? w.buf[i] : 0;
      unsigned bl = stay ? w.blo[i] : 0u;
      unsigned sm = __ballot_sync(FULL, stay);
      __syncwarp();
      if (stay) {
        int d = nb + __popc(sm & ((1u << lane) - 1u));
        w.buf[d] = bi;
        w.blo[d] = bl;
      }
      nb += __popc(sm);
      __syncwarp();
    }
    F.bn = nb;
    if (F.bn + nk > kWqBuf) {
      F.over = true;
      return;
    }
  }
  if (keep) {
    int d = F.bn + __popc(km & ((1u << lane) - 1u));
    w.buf[d] = ti;
    w.blo[d] = lob;
  }
  F.bn += nk;
  __syncwarp();
  // the list takes the batch's upper bounds below T (sorted, then merged)
  if (__ballot_sync(FULL, hib < F.tb)) {
    unsigned k = hib < F.tb ? hib : 0xffffffffu;
    warp_sort_asc_u32(k, lane);
    unsigned rk = __shfl_sync(FULL, k, 31 - lane);
    unsigned m = rk < F.fk ? rk : F.fk;
#pragma unroll
    for (int stride = 16; stride > 0; stride >>= 1) {
      unsigned o = __shfl_xor_sync(FULL, m, stride);
      bool lower = (lane & stride) == 0;
      if (lower ? (o < m) : (o > m)) m = o;
    }
    F.fk = lane < K ? m : 0xffffffffu;
    F.tb = __shfl_sync(FULL, F.fk, K - 1);
  }
}

// Frontier-parallel traversal of every node whose FP32 box bound is below the k-th
// distance: the whole tree when `home` is -1, else the whole tree but the subtree at heap
// index `home` (already searched), which is the union of the subtrees of the siblings of
// home and of each of its ancestors: those are pushed at once, so the first step tests
// them all together instead of descending from the root one level per step. Returns
// false when the stack would overflow (the caller sets the error word).
template <int S, bool F32 = false>
__device__ bool wq_traverse(WqQuery<S>& Q, WqSmem& w, const TreeView& tv, int lane, int home,
                            WqF32* F = nullptr, int self = -1, int K = 0) {
  const unsigned FULL = 0xffffffffu;
  int sp = 0;
  if (home < 0) {
    if (lane == 0) w.stk[0] = 0;
    sp = 1;
  } else {
    // at most 31 levels (n < 2^31), well inside the stack
    for (int h = home; h > 0; h = (h - 1) >> 1) {
      if (lane == 0) w.stk[sp] = (h & 1) ? h + 1 : h - 1;
      sp++;
    }
  }
  __syncwarp();
  for (int guard = 0; sp > 0 && guard < (1 << 24); guard++) {
    int m = sp <= kWqBatchLimit ? min(32, sp) : 1;
    int h = 0;
    NodeRec r{};
    bool need = false;
    if (lane < m) {
      h = w.stk[sp - 1 - lane];
      r = tv.node[tv.nbase + h];
      float blo = box_d2_lo(Q.qx, Q.qy, Q.qz, Q.eps, r);
      need = F32 ? __float_as_uint(blo) <= F->tb : blo < Q.thr;
    }
    __syncwarp();
    sp -= m;
    bool leaf = need && r.count <= tv.b;
    unsigned inner = __ballot_sync(FULL, need && !leaf);
    int ne = __popc(inner);
    if (sp + 2 * ne > kWqStack) return false;
    if ((inner >> lane) & 1u) {
      int slot = sp + 2 * __popc(inner & ((1u << lane) - 1u));
      w.stk[slot] = 2 * h + 2;
      w.stk[slot + 1] = 2 * h + 1;
    }
    sp += 2 * ne;
    // leaves: packed into the 32 lanes (several small leaves per screening step)
    unsigned lm = __ballot_sync(FULL, leaf);
    int fill = 0, my = 0;
    while (lm) {
      int l = __ffs(lm) - 1;
      int st = __shfl_sync(FULL, r.start, l), ct = __shfl_sync(FULL, r.count, l);
      if (fill > 0 && fill + ct > 32) {
        if (F32) wq32_consider<S>(Q, *F, w, tv, lane, lane < fill, my, self, K);
        else wq_consider<S>(Q, w, tv, lane, lane < fill, my);
        fill = 0;
      }
      lm &= lm - 1;
      if (ct > 32) {
        for (int c0 = 0; c0 < ct; c0 += 32) {
          if (F32) wq32_consider<S>(Q, *F, w, tv, lane, c0 + lane < ct, st + c0 + lane, self, K);
          else wq_consider<S>(Q, w, tv, lane, c0 + lane < ct, st + c0 + lane);
        }
        continue;
      }
      if (lane >= fill && lane < fill + ct) my = st + lane - fill;
      fill += ct;
    }
    if (fill > 0) {
      if (F32) wq32_consider<S>(Q, *F, w, tv, lane, lane < fill, my, self, K);
      else wq_consider<S>(Q, w, tv, lane, lane < fill, my);
    }
    __syncwarp();
    if (F32 && F->over) return true;  // the caller redoes the query exactly
  }
  return sp == 0;
}

// Heap index, first particle and size of the smallest node on the path of tree index
// `self` that holds at least `want` particles (the root if none is smaller).
__device__ __forceinline__ void wq_home(const TreeView& tv, int self, int want, int& h,
                                        int& start, int& size) {
  int i = self - tv.pstart;
  int hh = 0, s0 = 0, sz = tv.n;
  h = 0;
  start = tv.pstart;
  size = tv.n;
  while (sz > tv.b) {
    int ls = (sz - 1) / 2 + 1;  // KDTree.cxx:1012, 1025-1030
    if (i < s0 + ls) {
      hh = 2 * hh + 1;
      sz = ls;
    } else {
      hh = 2 * hh + 2;
      s0 += ls;
      sz -= ls;
    }
    if (sz < want) break;
    h = hh;
    start = tv.pstart + s0;
    size = sz;
  }
}

// An FP32 upper bound of the k-th distance from the query's own subtree [hs, hs + hn):
// a value T with at least K particles whose FP32 upper bound of the squared distance is
// at or below T (bisection over the bit patterns, which order as the non-negative values
// do), counting only particles provably at a non-zero distance and other than the query
// (the target search skips those). Returns +inf when fewer than K qualify.
// hn <= 2K + 1 <= 64 S + 1.
template <int S>
__device__ __forceinline__ float wq_home_bound(const WqQuery<S>& Q, const TreeView& tv, int lane,
                                               int self, int hs, int hn, int K) {
  const unsigned FULL = 0xffffffffu;
  constexpr int R = 2 * S + 1;
  unsigned hb[R];
  unsigned mn = 0x7f800000u, mx = 0u;
#pragma unroll
  for (int r = 0; r < R; r++) {
    int c = r * 32 + lane;
    hb[r] = 0x7f800000u;
    if (c < hn) {
      int ti = hs + c;
      float4 cf = tv.posf[ti];
      float lo = pair_d2_lo(Q.qx, Q.qy, Q.qz, cf.x, cf.y, cf.z, Q.two_eps);
      if (ti != self && lo > 0.f) {
        hb[r] = __float_as_uint(pair_d2_hi(Q.qx, Q.qy, Q.qz, cf.x, cf.y, cf.z, Q.two_eps));
        mn = min(mn, hb[r]);
        mx = max(mx, hb[r]);
      }
    }
  }
  mn = __reduce_min_sync(FULL, mn);
  mx = __reduce_max_sync(FULL, mx);
  int cnt = 0;
#pragma unroll
  for (int r = 0; r < R; r++) cnt += hb[r] <= mx ? 1 : 0;
  if (__reduce_add_sync(FULL, cnt) < K) return __uint_as_float(0x7f800000u);
  // invariant: count(<= hi) >= K; 14 halvings bring hi within 2^-14 of the span
  unsigned lo = mn, hi = mx;
  for (int it = 0; it < 14 && lo < hi; it++) {
    unsigned mid = lo + ((hi - lo) >> 1);
    int c = 0;
#pragma unroll
    for (int r = 0; r < R; r++) c += hb[r] <= mid ? 1 : 0;
    if (__reduce_add_sync(FULL, c) >= K) hi = mid;
    else lo = mid + 1;
  }
  return __uint_as_float(hi + 1u);  // strictly above: candidates test lo < thr
}

// Target search of a one-slot list (K <= 32) without periodic images: the FP32 search
// of the whole tree (own subtree, then the siblings of it and of its ancestors), then
// exact FP64 distances for the kept particles within the final bound. Returns false when
// the buffer overflowed (the caller runs wq_search instead) or the stack would.
template <int S>
__device__ bool wq_search_f32(WqQuery<S>& Q, WqSmem& w, const TreeView& tv, int lane, int self,
                              const double x0[3], int K) {
  WqF32 F;
  F.fk = 0xffffffffu;
  F.tb = 0xffffffffu;
  F.bn = 0;
  F.over = false;
  wq_set_point<S>(Q, tv, x0);
  int hh, hs, hn;
  wq_home(tv, self, K + 1, hh, hs, hn);
  for (int c0 = 0; c0 < hn && !F.over; c0 += 32)
    wq32_consider<S>(Q, F, w, tv, lane, c0 + lane < hn, hs + c0 + lane, self, K);
  bool ok = F.over || hh == 0 || wq_traverse<S, true>(Q, w, tv, lane, hh, &F, self, K);
  if (!ok || F.over) return false;
  // exact phase
  wq_init<S>(Q.L, lane, K);
  Q.K = K;
  Q.topk = __double_as_longlong(kMaxValue);
  Q.thr = __uint_as_float(0x7f800000u);
  Q.qn = 0;
  Q.self = self;
  const unsigned FULL = 0xffffffffu;
  for (int c0 = 0; c0 < F.bn; c0 += 32) {
    int i = c0 + lane;
    bool sel = i < F.bn && w.blo[i] <= F.tb;
    int ti = sel ? w.buf[i] : 0;
    unsigned pm = __ballot_sync(FULL, sel);
    if (!pm) continue;
    if (sel) w.queue[Q.qn + __popc(pm & ((1u << lane) - 1u))] = ti;
    Q.qn += __popc(pm);
    __syncwarp();
    if (Q.qn >= 32) {
      wq_flush<S>(Q, w, tv, lane, 32);
      __syncwarp();
      int rest = Q.qn - 32;
      int moved = lane < rest ? w.queue[32 + lane] : 0;
      __syncwarp();
      if (lane < rest) w.queue[lane] = moved;
      Q.qn = rest;
      __syncwarp();
    }
  }
  wq_drain<S>(Q, w, tv, lane);
  return true;
}

// The search of one target query (tree index `self`, position x0): the direct pass
// (seeded with the query's own subtree) and, on a periodic tree, the image passes with
// the reference's gates. exclude_self: the target search of the direct pass skips the
// query and zero distances (KDLeafNode.cxx:19-21). On return Q.L holds the K nearest.
// F32FIRST: one-slot target searches without images take wq_search_f32 first (faster
// for the many small trees of a batch; for one large tree the direct form is faster).
template <int S, bool F32FIRST = false>
__device__ void wq_search(WqQuery<S>& Q, WqSmem& w, const KnnArgs& a, const TreeView& tv,
                          int lane, int self, const double x0[3], int K, bool exclude_self) {
  if (F32FIRST && S == 1 && exclude_self && !a.periodic &&
      wq_search_f32<S>(Q, w, tv, lane, self, x0, K))
    return;
  wq_init<S>(Q.L, lane, K);
  Q.K = K;
  Q.topk = __double_as_longlong(kMaxValue);
  Q.thr = thresh_hi_bits(Q.topk);
  Q.qn = 0;
  Q.self = exclude_self ? self : -1;
  wq_set_point<S>(Q, tv, x0);
  int hh, hs, hn;
  wq_home(tv, self, K + 1, hh, hs, hn);
  if (exclude_self) Q.thr = fminf(Q.thr, wq_home_bound<S>(Q, tv, lane, self, hs, hn, K));
  wq_range<S>(Q, w, tv, lane, hs, hn);
  // with the bound the rest of the tree prunes at once; without it (coordinate search of
  // the direct pass) the queue is flushed first so the k-th distance is known
  if (!exclude_self) wq_drain<S>(Q, w, tv, lane);
  bool ok = hh == 0 || wq_traverse<S>(Q, w, tv, lane, hh);
  wq_drain<S>(Q, w, tv, lane);
  if (ok && a.periodic) {
    Q.self = -1;
    // image passes in the reference's order; the k-th distance only shrinks, so walls
    // ruled out after the direct pass stay ruled out
    float4 qf = make_float4(__double2float_rn(x0[0]), __double2float_rn(x0[1]),
                            __double2float_rn(x0[2]), 0.f);
    float top_hi = thresh_hi_bits(Q.topk);
    float qeps = query_eps(tv, x0[0], x0[1], x0[2]);
    int near_sq = near_walls(qf, tv.period, qeps, top_hi);
    int near_lin = near_walls_lin(qf, tv.period, qeps, top_hi);
    for (int pass = 1; pass < 8 && ok; pass++) {
      int mk = kImageMask[pass];
      bool lin = !(pass <= 3 || a.min_image);
      if ((mk & ~(lin ? near_lin : near_sq)) != 0) continue;
      double xq[3];
      double sval = reflect(x0, xq, tv.period, mk);
      double top = __longlong_as_double(Q.topk);
      // KDSplitNode.cxx:1129 gates 1-D images with sqrt(top) > sval, :1134-1146 the 2-D
      // and 3-D images with top > sval
      bool g = lin ? (top > sval) : (__dsqrt_rn(top) > sval);
      if (!g) continue;
      wq_set_point<S>(Q, tv, xq);
      ok = wq_traverse<S>(Q, w, tv, lane, -1);
      wq_drain<S>(Q, w, tv, lane);
    }
  }
  if (!ok && lane == 0) atomicExch(a.err, kErrCapacity);
}

// Rank of each list entry among the first K by value (ties by position): the nsmooth
// smallest |dv| of CalcVelDensity are those of rank < nsmooth.
template <int S>
__device__ __forceinline__ void wq_ranks(const long long v[S], int lane, int K, int rank[S]) {
#pragma unroll
  for (int s = 0; s < S; s++) rank[s] = 0;
  for (int p = 0; p < K; p++) {
    long long vp = v[0];
#pragma unroll
    for (int s = 1; s < S; s++)
      if ((p >> 5) == s) vp = v[s];
    vp = __shfl_sync(0xffffffffu, vp, p & 31);
#pragma unroll
    for (int s = 0; s < S; s++) {
      int me = s * 32 + lane;
      rank[s] += (vp < v[s] || (vp == v[s] && p < me)) ? 1 : 0;
    }
  }
}

// 2 / sqrt(t) (the 1/h of h = sqrt(t) / 2) to about 2e-16 relative: the FP32 reciprocal
// square root as the start and two Newton steps y (3/2 - t/2 y^2) in FP64. Outside the
// FP32 normal range it takes the FP64 square root and division.
__device__ __forceinline__ double two_rsqrt(double t) {
  const float tf = __double2float_rn(t);
  if (!(tf > 1e-30f && tf < 1e30f)) return 1.0 / (0.5 * __dsqrt_rn(t));
  double y = (double)rsqrtf(tf);
  const double ht = 0.5 * t;
  y = dmul(y, __fma_rn(-ht, dmul(y, y), 1.5));
  y = dmul(y, __fma_rn(-ht, dmul(y, y), 1.5));
  return 2.0 * y;
}
// 1 / x to about 2e-16 relative: the FP32 reciprocal and two Newton steps y (2 - x y).
__device__ __forceinline__ double recip_newton(double x) {
  const float xf = __double2float_rn(x);
  if (!(xf > 1e-30f && xf < 1e30f)) return 1.0 / x;
  double y = (double)__frcp_rn(xf);
  y = dmul(y, __fma_rn(-x, y, 2.0));
  y = dmul(y, __fma_rn(-x, y, 2.0));
  return y;
}

__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x = dadd(x, __shfl_xor_sync(0xffffffffu, x, o));
  return x;
}

}  // namespace
}  // namespace nbk
