// GPU kd-tree build (replaces KDTree::BuildNodes + MedianPos + DetermineSplitDim,
// src/KDTree/KDTree.cxx:970-1055, 328-370, 459-504).
//
// The reference builds recursively: split dimension = largest spread (ties to the lowest
// dimension), split at index start + (size-1)/2 with the left child [start, split+1),
// leaf when size <= b. Because the median partition of a node is unique (up to ties in
// the coordinate), building level by level with the same rules yields nodes holding the
// same particle sets as the reference's, hence the same node counts and bounding boxes.
//
// The same code builds phase-space trees (TreeType TPHS: six coordinates x, y, z, vx, vy,
// vz, SpreadestPhs / MedianPhs, KDTree.cxx:71-100, 414-456); every kernel takes the
// number of coordinates ND as a template parameter.
//
// Phase 1 (levels whose nodes hold more than kLocalMax particles): for all nodes of a
// level at once, over chunks of kChunk particles:
//   bbox      segmented min/max of each coordinate (order-preserving uint64 keys); for
//             the first level only, later levels get it from the partition above them
//   select    6 radix passes (11, 11, 11, 11, 11, 9 bits) find the key of the median
//             particle exactly; pass 0 also picks the split dimension from the box
//   partition stable 3-way (less / equal / greater) scatter into the other buffer
// Phase 2: one CTA per subtree of <= kLocalMax particles finishes it in shared memory:
// one sort per dimension, then level by level stable splits of index lists; it writes
// the final tree-order arrays.
#include <algorithm>
#include <cstring>
#include <vector>

#include "nbk_build.h"

namespace nbk {

namespace {

constexpr int kChunk = 2048;  // 8 particles per thread, loads issued together
constexpr int kThreads = 256;
constexpr int kRounds = kChunk / kThreads;
constexpr int kLevelCap = kLocalMax;  // level lists hold up to 2*size/(b+1) nodes

// The coordinates of the particles being partitioned live in one buffer per ping-pong
// side: coordinate d of particle i at C[d * cs + i] (cs = the buffer's particle count).
// ND = 3 for physical trees (x, y, z), 6 for phase-space trees (x, y, z, vx, vy, vz).
template <int ND>
struct GNodeT {
  int start, size;  // absolute tree-index range
  int node;         // absolute node index
  int dim;
  int k;            // rank still to find inside the current prefix class
  int n_less;       // particles with key below the current prefix class
  int need_eq;      // after selection: equal-key particles that go left
  int total_eq;
  int first_chunk, nchunks;
  int first_diff;   // highest bit where the keys of the split dimension can differ
  unsigned done;    // blocks of this node finished in the current radix pass
  int child[2];     // the children's slots in the next level's list (-1: per-CTA subtree)
  int ncand;        // keys in the current prefix class
  unsigned nfill;   // keys of the class gathered so far (collect mode)
  unsigned long long prefix, mask;
  unsigned long long kmin[ND], kmax[ND];  // node box as order keys (filled by the level above)
};

// Radix passes of the median selection (11-bit digits from each node's highest differing
// key bit: at most six cover a 64-bit key).
constexpr int kPasses = 6;
constexpr int kBins = 2048;
constexpr int kCollect = kThreads;  // a class this small is gathered and ranked by one block
static_assert(kCollect % kThreads == 0, "whole keys per thread");

struct Chunk {
  int g;      // gnode index within the level
  int start;  // absolute start
  int len;
  int off;    // offset of the chunk inside its node
};

struct LRoot {
  int start, size;  // absolute range
  int nbase;        // node index of the tree's root
  int h;            // heap index of this subtree root within its tree
  int buf;          // which ping-pong buffer holds its particles
  int pad;
};

// Node records written by the build: NodeRec + NodeX for ND = 3, NodeS + NodeB6 for 6.
template <int ND>
struct NodeOut;
template <>
struct NodeOut<3> {
  NodeRec* node;
  NodeX* nodex;
  __device__ __forceinline__ void write(int idx, const double* lo, const double* hi, int start,
                                        int count, int dim, double split_val) const {
    NodeRec r;
    NodeX x;
#pragma unroll
    for (int d = 0; d < 3; d++) {
      r.lo[d] = __double2float_rd(lo[d]);
      r.hi[d] = __double2float_ru(hi[d]);
      x.lo[d] = lo[d];
      x.hi[d] = hi[d];
    }
    r.start = start;
    r.count = count;
    x.split_dim = dim;
    x.split_val = split_val;
    x.pad = 0;
    node[idx] = r;
    nodex[idx] = x;
  }
  __device__ __forceinline__ void set_split(int idx, double v) const { nodex[idx].split_val = v; }
};
template <>
struct NodeOut<6> {
  NodeS* nodes;
  NodeB6* nodeb;
  NodeF6* nodef;
  __device__ __forceinline__ void write(int idx, const double* lo, const double* hi, int start,
                                        int count, int dim, double split_val) const {
    NodeS r;
    NodeB6 x;
    NodeF6 f;
#pragma unroll
    for (int d = 0; d < 6; d++) {
      x.lo[d] = lo[d];
      x.hi[d] = hi[d];
      f.lo[d] = __double2float_rd(lo[d]);
      f.hi[d] = __double2float_ru(hi[d]);
    }
    nodef[idx] = f;
    r.split_val = split_val;
    r.split_dim = dim;
    r.start = start;
    r.count = count;
    r.pad = 0;
    nodes[idx] = r;
    nodeb[idx] = x;
  }
  __device__ __forceinline__ void set_split(int idx, double v) const { nodes[idx].split_val = v; }
};

// a[dim] of a small array indexed at run time, kept in registers
template <int ND, typename T>
__device__ __forceinline__ T sel(const T* a, int dim) {
  T r = a[0];
#pragma unroll
  for (int d = 1; d < ND; d++)
    if (dim == d) r = a[d];
  return r;
}

template <int ND>
__global__ void k_init_soa(const double* __restrict__ pos_in, const double* __restrict__ vel_in,
                           double* C, int64_t cs, int* ID, int64_t n, int* err) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  bool bad = false;
#pragma unroll
  for (int d = 0; d < ND; d++) {
    double v = d < 3 ? pos_in[3 * i + d] : vel_in[3 * i + d - 3];
    bad = bad || !(v == v) || isinf(v);
    C[d * cs + i] = v;
  }
  if (bad) atomicExch(err, 1);
  ID[i] = (int)i;
}

__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v) {
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w < v ? w : v;
  }
  return v;
}
__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  return v;
}

template <int ND>
__global__ void __launch_bounds__(kThreads) k_bbox(const Chunk* __restrict__ chunks,
                                                   GNodeT<ND>* g, const double* C, int64_t cs) {
  Chunk c = chunks[blockIdx.x];
  unsigned long long mn[ND], mx[ND];
#pragma unroll
  for (int d = 0; d < ND; d++) {
    mn[d] = ~0ull;
    mx[d] = 0ull;
  }
#pragma unroll
  for (int d = 0; d < ND; d++) {
    double v[kRounds];
#pragma unroll
    for (int r = 0; r < kRounds; r++) {
      int i = r * kThreads + threadIdx.x;
      if (i < c.len) v[r] = C[d * cs + c.start + i];
    }
#pragma unroll
    for (int r = 0; r < kRounds; r++) {
      int i = r * kThreads + threadIdx.x;
      if (i < c.len) {
        unsigned long long k = okey(v[r]);
        mn[d] = min(mn[d], k);
        mx[d] = max(mx[d], k);
      }
    }
  }
  __shared__ unsigned long long s[2 * ND][kThreads / 32];
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int d = 0; d < ND; d++) {
    unsigned long long a = warp_min_u64(mn[d]), b = warp_max_u64(mx[d]);
    if (lane == 0) {
      s[d][w] = a;
      s[ND + d][w] = b;
    }
  }
  __syncthreads();
  if (threadIdx.x < ND) {
    int d = threadIdx.x;
    unsigned long long a = ~0ull, b = 0ull;
    for (int i = 0; i < kThreads / 32; i++) {
      a = min(a, s[d][i]);
      b = max(b, s[ND + d][i]);
    }
    atomicMin(&g[c.g].kmin[d], a);
    atomicMax(&g[c.g].kmax[d], b);
  }
}

// DetermineSplitDim (KDTree.cxx:459-504): spread = max - min per dimension in FP64, the
// first strictly larger spread wins.
template <int ND>
__device__ __forceinline__ int split_dim_of(const GNodeT<ND>& s, double* lo, double* hi) {
#pragma unroll
  for (int d = 0; d < ND; d++) {
    lo[d] = okey_inv(s.kmin[d]);
    hi[d] = okey_inv(s.kmax[d]);
  }
  int dim = 0;
  double cur = dsub(hi[0], lo[0]);
#pragma unroll
  for (int d = 1; d < ND; d++) {
    double sp = dsub(hi[d], lo[d]);
    if (sp > cur) {
      dim = d;
      cur = sp;
    }
  }
  return dim;
}

__device__ __forceinline__ unsigned block_excl_scan(unsigned v, unsigned* tot, unsigned* wsum);

// One radix pass of the median selection for every node of a level. Each block
// histograms one chunk's digits; the last block of a node to finish (arrival counter,
// no waiting) reads the node's histogram, narrows the rank to one digit and clears the
// histogram for the next pass. Pass 0 also fixes the split dimension from the node box
// (each block derives the same one) and writes the node's records.
template <int ND>
__global__ void __launch_bounds__(kThreads) k_radix(const Chunk* __restrict__ chunks,
                                                    GNodeT<ND>* g, const double* Cb, int64_t cs,
                                                    unsigned* hist, unsigned long long* cand,
                                                    int pass, NodeOut<ND> out, int p0, int* err) {
  static_assert(kCollect <= kBins / 2, "the gathered keys share the bins' shared memory");
  __shared__ unsigned long long sk[kBins / 2];  // the bins, or the gathered keys
  unsigned* h = reinterpret_cast<unsigned*>(sk);
  __shared__ unsigned wsum[32], tot;
  __shared__ int s_last;
  Chunk c = chunks[blockIdx.x];
  const GNodeT<ND> s = g[c.g];
  if (s.mask == ~0ull) return;  // the median key of this node is already known
  int dim, first_diff;
  double lo[ND], hi[ND];
  if (pass == 0) {
    dim = split_dim_of<ND>(s, lo, hi);
    unsigned long long x = sel<ND>(s.kmin, dim) ^ sel<ND>(s.kmax, dim);
    first_diff = x ? 63 - __clzll((long long)x) : -1;
  } else {
    dim = s.dim;
    first_diff = s.first_diff;
  }
  const double* C = Cb + (int64_t)dim * cs;
  // digits start at the node's highest differing key bit: pass p resolves the 11 bits
  // below first_diff - 11p (fewer for the last one); the bits above first_diff are common
  // to every key of the node and enter the prefix in pass 0
  const int hi_bit = first_diff - 11 * pass;
  const bool skip = hi_bit < 0;  // no bit left: every key of the node is equal
  const int width = skip ? 1 : min(11, hi_bit + 1), shift = skip ? 0 : hi_bit - width + 1;
  const unsigned long long dmask = skip ? 0ull : ((1ull << width) - 1ull) << shift;
  const unsigned long long common = hi_bit >= 63 ? 0ull : (~0ull << (hi_bit + 1));
  const bool collect = !skip && s.ncand <= kCollect;
  if (collect) {
    // gather the class's keys into this node's slice of the candidate buffer
    double v[kRounds];
#pragma unroll
    for (int r = 0; r < kRounds; r++) {
      int i = r * kThreads + threadIdx.x;
      if (i < c.len) v[r] = C[c.start + i];
    }
    const unsigned lane = threadIdx.x & 31;
#pragma unroll
    for (int r = 0; r < kRounds; r++) {
      int i = r * kThreads + threadIdx.x;
      unsigned long long key = 0;
      bool in = false;
      if (i < c.len) {
        key = okey(v[r]);
        in = (key & s.mask) == s.prefix;
      }
      unsigned b = __ballot_sync(0xffffffffu, in);
      if (b) {
        unsigned base = 0;
        if (lane == (unsigned)(__ffs(b) - 1)) base = atomicAdd(&g[c.g].nfill, (unsigned)__popc(b));
        base = __shfl_sync(0xffffffffu, base, __ffs(b) - 1);
        unsigned slot = base + __popc(b & ((1u << lane) - 1u));
        if (in && slot < (unsigned)kCollect) cand[s.start + slot] = key;
      }
    }
  } else if (!skip) {
    for (int i = threadIdx.x; i < kBins; i += kThreads) h[i] = 0;
    __syncthreads();
    double v[kRounds];
#pragma unroll
    for (int r = 0; r < kRounds; r++) {
      int i = r * kThreads + threadIdx.x;
      if (i < c.len) v[r] = C[c.start + i];
    }
    // the keys of one node share their leading digits, so most lanes of a warp hit the
    // same bin: lanes are grouped by digit and one atomic per distinct digit is issued
#pragma unroll
    for (int r = 0; r < kRounds; r++) {
      int i = r * kThreads + threadIdx.x;
      int digit = -1;
      if (i < c.len) {
        unsigned long long key = okey(v[r]);
        if ((key & s.mask) == s.prefix) digit = (int)((key & dmask) >> shift);
      }
      unsigned peers = __match_any_sync(0xffffffffu, digit);
      if (digit >= 0 && (threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&h[digit], __popc(peers));
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kBins; i += kThreads)
      if (h[i]) atomicAdd(&hist[(size_t)c.g * kBins + i], h[i]);
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(&g[c.g].done, 1u) == (unsigned)s.nchunks - 1u;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  if (threadIdx.x == 0) {
    g[c.g].done = 0u;
    if (pass == 0) {
      g[c.g].dim = dim;
      g[c.g].first_diff = first_diff;
      // the split value is written once the median key is known (k_chunk_scan)
      out.write(s.node, lo, hi, p0 + s.start, s.size, dim, 0.0);
    }
  }
  const unsigned long long kmin_dim = sel<ND>(s.kmin, dim);
  if (skip) {  // all keys equal (first_diff = -1): the median key is the minimum key
    if (threadIdx.x == 0) {
      g[c.g].prefix = kmin_dim;
      g[c.g].mask = ~0ull;
    }
    return;
  }
  // pass 0 adds the bits every key shares
  const unsigned long long base_prefix = pass == 0 ? (kmin_dim & common) : s.prefix;
  const unsigned long long base_mask = pass == 0 ? common : s.mask;
  if (collect) {
    // the k-th smallest of the gathered keys is the median key: thread t holds keys t,
    // t + kThreads, ... and counts the keys below and equal to each
    constexpr int kPerT = kCollect / kThreads;
    int n = min(s.ncand, kCollect);
    if (threadIdx.x == 0 && __ldcg(&g[c.g].nfill) != (unsigned)s.ncand) atomicExch(err, 5);
    unsigned long long mine[kPerT];
#pragma unroll
    for (int q = 0; q < kPerT; q++) {
      const int i = (int)threadIdx.x + q * kThreads;
      mine[q] = i < n ? __ldcg(&cand[s.start + i]) : ~0ull;
      sk[i] = mine[q];
    }
    __syncthreads();
    int below[kPerT], equal[kPerT];
#pragma unroll
    for (int q = 0; q < kPerT; q++) below[q] = equal[q] = 0;
    for (int i = 0; i < n; i++) {
      const unsigned long long o = sk[i];
#pragma unroll
      for (int q = 0; q < kPerT; q++) {
        below[q] += o < mine[q];
        equal[q] += o == mine[q];
      }
    }
    int kr = min(max(s.k, 0), n - 1);
#pragma unroll
    for (int q = 0; q < kPerT; q++) {
      if ((int)threadIdx.x + q * kThreads < n && below[q] <= kr && kr < below[q] + equal[q]) {
        // every holder of the k-th key writes the same value
        g[c.g].prefix = mine[q];
        g[c.g].mask = ~0ull;
      }
    }
    if (threadIdx.x == 0) g[c.g].nfill = 0u;
    return;
  }
  // the digit whose bin holds rank k: each thread owns kBins / kThreads consecutive bins
  constexpr int kPer = kBins / kThreads;
  unsigned* hh = hist + (size_t)c.g * kBins;
  unsigned cnt[kPer], sum = 0;
#pragma unroll
  for (int e = 0; e < kPer; e++) {
    cnt[e] = __ldcg(&hh[threadIdx.x * kPer + e]);
    sum += cnt[e];
  }
  unsigned before = block_excl_scan(sum, &tot, wsum);
  unsigned k = (unsigned)s.k;
  if (before <= k && k < before + sum) {
    int digit = -1;
#pragma unroll
    for (int e = 0; e < kPer; e++) {
      if (digit < 0) {
        if (k < before + cnt[e]) digit = threadIdx.x * kPer + e;
        else before += cnt[e];
      }
    }
    g[c.g].k = (int)(k - before);
    g[c.g].n_less = s.n_less + (int)before;
#pragma unroll
    for (int e = 0; e < kPer; e++)
      if (threadIdx.x * kPer + e == digit) g[c.g].ncand = (int)cnt[e];
    g[c.g].prefix = base_prefix | ((unsigned long long)digit << shift);
    g[c.g].mask = base_mask | dmask;
  }
#pragma unroll
  for (int e = 0; e < kPer; e++) hh[threadIdx.x * kPer + e] = 0u;
}

template <int NT>
__device__ __forceinline__ unsigned block_excl_scan_t(unsigned v, unsigned* tot, unsigned* wsum) {
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  unsigned incl = v;
  for (int o = 1; o < 32; o <<= 1) {
    unsigned t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) wsum[w] = incl;
  __syncthreads();
  if (w == 0) {
    unsigned x = lane < NT / 32 ? wsum[lane] : 0;
    unsigned xi = x;
    for (int o = 1; o < 32; o <<= 1) {
      unsigned t = __shfl_up_sync(0xffffffffu, xi, o);
      if (lane >= o) xi += t;
    }
    if (lane < NT / 32) wsum[lane] = xi - x;
    if (lane == NT / 32 - 1) *tot = xi;
  }
  __syncthreads();
  unsigned r = incl - v + wsum[w];
  __syncthreads();
  return r;
}
__device__ __forceinline__ unsigned block_excl_scan(unsigned v, unsigned* tot, unsigned* wsum) {
  return block_excl_scan_t<kThreads>(v, tot, wsum);
}

// Per chunk: how many keys are below / equal to the median key.
template <int ND>
__device__ __forceinline__ void count_body(int vb, const Chunk* __restrict__ chunks,
                                           const GNodeT<ND>* g, const double* Cb, int64_t cs,
                                           unsigned* cnt_less, unsigned* cnt_eq) {
  Chunk c = chunks[vb];
  const GNodeT<ND>& s = g[c.g];
  unsigned long long piv = s.prefix;
  unsigned a = 0, e = 0;
  const double* C = Cb + (int64_t)s.dim * cs;
  double v[kRounds];
#pragma unroll
  for (int r = 0; r < kRounds; r++) {
    int i = r * kThreads + threadIdx.x;
    if (i < c.len) v[r] = C[c.start + i];
  }
#pragma unroll
  for (int r = 0; r < kRounds; r++) {
    if (r * kThreads + (int)threadIdx.x < c.len) {
      unsigned long long key = okey(v[r]);
      a += key < piv;
      e += key == piv;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    e += __shfl_xor_sync(0xffffffffu, e, o);
  }
  __shared__ unsigned sa[kThreads / 32], se[kThreads / 32];
  if ((threadIdx.x & 31) == 0) {
    sa[threadIdx.x >> 5] = a;
    se[threadIdx.x >> 5] = e;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned ta = 0, te = 0;
    for (int i = 0; i < kThreads / 32; i++) {
      ta += sa[i];
      te += se[i];
    }
    cnt_less[vb] = ta;
    cnt_eq[vb] = te;
  }
}

// For one node (one block): exclusive scan of the chunk counts (chunk order), the split
// value, and the number of equal keys that go left.
template <int ND>
__device__ __forceinline__ void scan_body(int vn, GNodeT<ND>* g, const unsigned* cnt_less,
                                          const unsigned* cnt_eq, unsigned* base_less,
                                          unsigned* base_eq, NodeOut<ND> out) {
  __shared__ unsigned wsum[32];
  __shared__ unsigned tot;
  const GNodeT<ND>& sg = g[vn];
  const int nchunks = sg.nchunks, first_chunk = sg.first_chunk;
  unsigned run_l = 0, run_e = 0;
  for (int c0 = 0; c0 < nchunks; c0 += kThreads) {
    int c = c0 + threadIdx.x;
    // read through L2: in k_count_scan other blocks wrote these counts during the launch
    unsigned vl = c < nchunks ? __ldcg(&cnt_less[first_chunk + c]) : 0;
    unsigned ve = c < nchunks ? __ldcg(&cnt_eq[first_chunk + c]) : 0;
    unsigned el = block_excl_scan(vl, &tot, wsum);
    unsigned tl = tot;
    unsigned ee = block_excl_scan(ve, &tot, wsum);
    unsigned te = tot;
    if (c < nchunks) {
      base_less[first_chunk + c] = run_l + el;
      base_eq[first_chunk + c] = run_e + ee;
    }
    run_l += tl;
    run_e += te;
  }
  if (threadIdx.x == 0) {
    // after selection n_less counts every key below the median key; rank k + 1 particles
    // go left: all of those plus (k_total + 1 - n_less) equal keys.
    int ktot = (sg.size - 1) / 2;
    g[vn].need_eq = ktot + 1 - (int)run_l;
    g[vn].total_eq = (int)run_e;
    g[vn].n_less = (int)run_l;
    out.set_split(sg.node, okey_inv(sg.prefix));
  }
}

// k_count and k_chunk_scan in one launch: each block counts its chunk, and the node's
// last-arriving block (arrival counter, no waiting) scans the node's chunk counts.
template <int ND>
__global__ void __launch_bounds__(kThreads) k_count_scan(const Chunk* __restrict__ chunks,
                                                         GNodeT<ND>* g, const double* Cb,
                                                         int64_t cs, unsigned* cnt_less,
                                                         unsigned* cnt_eq, unsigned* base_less,
                                                         unsigned* base_eq, NodeOut<ND> out) {
  __shared__ int s_last;
  count_body<ND>((int)blockIdx.x, chunks, g, Cb, cs, cnt_less, cnt_eq);
  const int node = chunks[blockIdx.x].g;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0)
    s_last = atomicAdd(&g[node].done, 1u) == (unsigned)g[node].nchunks - 1u;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  scan_body<ND>(node, g, cnt_less, cnt_eq, base_less, base_eq, out);
  if (threadIdx.x == 0) g[node].done = 0u;
}

// Stable 3-way partition of every node of a level around its median key into the other
// buffer. Each warp owns 256 consecutive particles of the chunk, taken 32 at a time, so
// ballots give every particle its rank inside its class and the writes of one class are
// contiguous across the warp; one block scan of the warps' (less, equal, valid) counts
// orders the warps. The children's bounding boxes (order keys of every coordinate) are
// gathered on the way and merged into the next level's nodes.
template <int ND>
__global__ void __launch_bounds__(kThreads) k_scatter(const Chunk* __restrict__ chunks,
                                                      const GNodeT<ND>* __restrict__ g,
                                                      const double* __restrict__ Cb,
                                                      const int* __restrict__ ID,
                                                      double* __restrict__ C2,
                                                      int* __restrict__ ID2, int64_t cs,
                                                      const unsigned* base_less,
                                                      const unsigned* base_eq, int* err,
                                                      GNodeT<ND>* gnext) {
  constexpr int kWarps = kThreads / 32, kPerWarp = kChunk / kWarps;
  __shared__ unsigned wl[kWarps], we[kWarps], wv[kWarps];
  __shared__ unsigned long long bb[kWarps][4 * ND];
  Chunk c = chunks[blockIdx.x];
  const GNodeT<ND>& s = g[c.g];
  const unsigned long long piv = s.prefix;
  const int sdim = s.dim, sstart = s.start, ssize = s.size, sneed = s.need_eq,
            sless = s.n_less, stot = s.total_eq, child0 = s.child[0], child1 = s.child[1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  const double* C = Cb + (int64_t)sdim * cs;
  const int w0 = warp * kPerWarp;
  unsigned cls = 0, nl = 0, ne = 0, nv = 0;
#pragma unroll
  for (int r = 0; r < kPerWarp / 32; r++) {
    int i = w0 + r * 32 + lane;
    unsigned k = 3;
    if (i < c.len) {
      unsigned long long key = okey(C[c.start + i]);
      k = key < piv ? 0u : (key == piv ? 1u : 2u);
    }
    cls |= k << (2 * r);
    nl += __popc(__ballot_sync(0xffffffffu, k == 0));
    ne += __popc(__ballot_sync(0xffffffffu, k == 1));
    nv += __popc(__ballot_sync(0xffffffffu, k != 3));
  }
  if (lane == 0) {
    wl[warp] = nl;
    we[warp] = ne;
    wv[warp] = nv;
  }
  __syncthreads();
  unsigned pl = 0, pe = 0, pv = 0;
  for (int q = 0; q < warp; q++) {
    pl += wl[q];
    pe += we[q];
    pv += wv[q];
  }
  const unsigned bl = base_less[blockIdx.x], be = base_eq[blockIdx.x];
  const int kleft = (ssize - 1) / 2 + 1;
  const int right0 = sstart + kleft;
  const int excess = stot - sneed;
  unsigned rl = bl + pl, re = be + pe;
  unsigned rg = ((unsigned)c.off - bl - be) + (pv - pl - pe);  // greater keys before this warp
  unsigned long long mnl[ND], mxl[ND], mnr[ND], mxr[ND];  // left / right child boxes
#pragma unroll
  for (int d = 0; d < ND; d++) {
    mnl[d] = mnr[d] = ~0ull;
    mxl[d] = mxr[d] = 0ull;
  }
#pragma unroll
  for (int r = 0; r < kPerWarp / 32; r++) {
    unsigned k = (cls >> (2 * r)) & 3u;
    unsigned bL = __ballot_sync(0xffffffffu, k == 0), bE = __ballot_sync(0xffffffffu, k == 1),
             bG = __ballot_sync(0xffffffffu, k == 2);
    if (k != 3) {
      int p = c.start + w0 + r * 32 + lane;
      int dst;
      if (k == 0) {
        dst = sstart + (int)(rl + __popc(bL & lt));
      } else if (k == 1) {
        int e = (int)(re + __popc(bE & lt));
        dst = e < sneed ? sstart + sless + e : right0 + (e - sneed);
      } else {
        dst = right0 + excess + (int)(rg + __popc(bG & lt));
      }
      if (dst < sstart || dst >= sstart + ssize) {  // selection inconsistent: report
        atomicExch(err, 2);
        dst = p;
      }
      const bool to_left = dst < right0;
#pragma unroll
      for (int d = 0; d < ND; d++) {
        double x = Cb[d * cs + p];
        C2[d * cs + dst] = x;
        unsigned long long kk = okey(x);
        if (to_left) {
          mnl[d] = min(mnl[d], kk);
          mxl[d] = max(mxl[d], kk);
        } else {
          mnr[d] = min(mnr[d], kk);
          mxr[d] = max(mxr[d], kk);
        }
      }
      ID2[dst] = ID[p];
    }
    rl += __popc(bL);
    re += __popc(bE);
    rg += __popc(bG);
  }
  if (gnext == nullptr || (child0 < 0 && child1 < 0)) return;
#pragma unroll
  for (int d = 0; d < ND; d++) {
    unsigned long long a = warp_min_u64(mnl[d]), b = warp_max_u64(mxl[d]);
    unsigned long long a2 = warp_min_u64(mnr[d]), b2 = warp_max_u64(mxr[d]);
    if (lane == 0) {
      bb[warp][d] = a;
      bb[warp][ND + d] = b;
      bb[warp][2 * ND + d] = a2;
      bb[warp][3 * ND + d] = b2;
    }
  }
  __syncthreads();
  if (threadIdx.x < 4 * ND) {
    int t = threadIdx.x / (2 * ND), e = threadIdx.x % (2 * ND);
    int child = t == 0 ? child0 : child1;
    if (child >= 0) {
      bool is_min = e < ND;
      unsigned long long v = is_min ? ~0ull : 0ull;
      for (int q = 0; q < kWarps; q++) {
        unsigned long long u = bb[q][threadIdx.x];
        v = is_min ? min(v, u) : max(v, u);
      }
      if (is_min) atomicMin(&gnext[child].kmin[e], v);
      else atomicMax(&gnext[child].kmax[e - ND], v);
    }
  }
}

// ---- phase 1b: one CTA per subtree of at most kMidMax (and more than kLocalMax) particles.
// The CTA splits the subtree's nodes level by level down to the subtrees of at most
// kLocalMax particles that phase 2 finishes; the nodes of one level (at most kMidGroups)
// are split at the same time, each by its own group of warps synchronised by a named
// barrier. Each split makes the same decisions as a global level -- split dimension from
// the node box, the median key by radix passes over the order keys (kept in shared
// memory; the median's class is ranked directly once it holds at most kMidCollect keys),
// the stable 3-way partition into the other buffer, the children's boxes -- with group
// barriers where a global level needs arrival counters and launches.
constexpr int kMidMax = 8192;
constexpr int kMidThreads = 1024;
constexpr int kMidGroups = 4;     // a level of a subtree of <= 8192 holds <= 4 nodes above 1024
constexpr int kMidCollect = 32;   // a class this small is ranked directly by one warp
constexpr int kMidNodes = 2 * kMidGroups;
constexpr int kMidRounds = 8;     // keys per group thread on a level: at most 8192 / 1024
static_assert(kMidMax <= kMidGroups * 2 * kLocalMax, "a subtree level fits in the groups");
static_assert(kMidCollect <= kMidThreads / kMidGroups, "one candidate per group thread");
static_assert(kMidMax <= kMidRounds * kMidThreads, "a level's keys fit the group's rounds");

struct MRoot {
  int start, size;  // absolute range in the ping-pong buffers
  int nbase, h;     // node index of the tree's root, heap index of this subtree root
  int buf;          // which ping-pong buffer holds its particles
  int pad;
};

template <int ND>
struct MNode {
  int start, size, h, pad;
  unsigned long long kmin[ND], kmax[ND];  // box as order keys
};

template <int ND>
struct MidLayout {
  static constexpr size_t key = 0;                                              // u64[kMidMax]
  static constexpr size_t dst = key + sizeof(unsigned long long) * kMidMax;     // int[kMidMax]
  // per group: u32[kBins] bins, or u64[kMidCollect] gathered keys
  static constexpr size_t bins = dst + sizeof(int) * kMidMax;
  static constexpr size_t nodes = bins + sizeof(unsigned) * kBins * kMidGroups;  // MNode[2][kMidNodes]
  static constexpr size_t total = nodes + sizeof(MNode<ND>) * 2 * kMidNodes;
  static_assert(sizeof(unsigned) * kBins >= sizeof(unsigned long long) * kMidCollect,
                "the gathered keys share the bins' shared memory");
  static_assert(nodes % 16 == 0, "MNode alignment");
};

// Barrier of the nt threads of group g (named barrier g + 1; nt a multiple of 32).
__device__ __forceinline__ void group_sync(int g, int nt) {
  asm volatile("bar.sync %0, %1;" ::"r"(g + 1), "r"(nt) : "memory");
}

// Exclusive scan over the nt threads of group g (r: the thread's rank in the group); the
// group's total goes to *tot.
__device__ __forceinline__ unsigned group_excl_scan(unsigned v, int r, int nt, int g,
                                                    unsigned* tot, unsigned* wsum) {
  const int lane = r & 31, w = r >> 5, nw = nt >> 5;
  unsigned incl = v;
  for (int o = 1; o < 32; o <<= 1) {
    unsigned t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) wsum[w] = incl;
  group_sync(g, nt);
  if (w == 0) {
    unsigned x = lane < nw ? wsum[lane] : 0;
    unsigned xi = x;
    for (int o = 1; o < 32; o <<= 1) {
      unsigned t = __shfl_up_sync(0xffffffffu, xi, o);
      if (lane >= o) xi += t;
    }
    if (lane < nw) wsum[lane] = xi - x;
    if (lane == nw - 1) *tot = xi;
  }
  group_sync(g, nt);
  unsigned res = incl - v + wsum[w];
  group_sync(g, nt);
  return res;
}

template <int ND>
__global__ void __launch_bounds__(kMidThreads) k_mid_build(
    const MRoot* __restrict__ roots, double* Ca, int* IDa, double* Cb, int* IDb, int64_t cs,
    NodeOut<ND> out, int* err, int p0) {
  using L = MidLayout<ND>;
  extern __shared__ __align__(16) unsigned char smem[];
  unsigned long long* key_all = (unsigned long long*)(smem + L::key);
  int* dst_all = (int*)(smem + L::dst);
  MNode<ND>* cur = (MNode<ND>*)(smem + L::nodes);
  MNode<ND>* nxt = cur + kMidNodes;
  __shared__ unsigned wsum[kMidGroups][32], tot[kMidGroups];
  __shared__ int n_cur, n_next, s_k[kMidGroups], s_ncand[kMidGroups];
  __shared__ unsigned s_fill[kMidGroups];
  __shared__ unsigned long long s_prefix[kMidGroups];
  // per group: left min, left max, right min, right max
  __shared__ unsigned long long box[kMidGroups][4 * ND];
  const int tid = threadIdx.x, lane = tid & 31;
  const MRoot R = roots[blockIdx.x];
  int buf = R.buf;

  // the subtree root's box (every thread)
  if (tid < 2 * ND) box[0][tid] = tid < ND ? ~0ull : 0ull;
  __syncthreads();
  {
    const double* C = buf ? Cb : Ca;
#pragma unroll
    for (int d = 0; d < ND; d++) {
      unsigned long long mn = ~0ull, mx = 0ull;
      for (int i = tid; i < R.size; i += kMidThreads) {
        unsigned long long k = okey(C[d * cs + R.start + i]);
        mn = min(mn, k);
        mx = max(mx, k);
      }
      mn = warp_min_u64(mn);
      mx = warp_max_u64(mx);
      if (lane == 0) {
        atomicMin(&box[0][d], mn);
        atomicMax(&box[0][ND + d], mx);
      }
    }
  }
  __syncthreads();
  if (tid == 0) {
    MNode<ND> r;
    r.start = R.start;
    r.size = R.size;
    r.h = R.h;
    r.pad = 0;
    for (int d = 0; d < ND; d++) {
      r.kmin[d] = box[0][d];
      r.kmax[d] = box[0][ND + d];
    }
    cur[0] = r;
    n_cur = 1;
    n_next = 0;
  }
  __syncthreads();
  for (int depth = 0; depth < 32; depth++) {
    const int ncur = n_cur;  // read by every thread before thread 0 rewrites it
    if (ncur <= 0) break;
    if (ncur > kMidGroups) {  // cannot happen for subtrees of <= kMidMax particles
      if (tid == 0) atomicExch(err, 3);
      break;
    }
    const int G = ncur <= 1 ? 1 : (ncur <= 2 ? 2 : 4);
    const int nt = kMidThreads / G, g = tid / nt, r = tid - g * nt;
    const double* C = buf ? Cb : Ca;
    const int* I = buf ? IDb : IDa;
    double* C2 = buf ? Ca : Cb;
    int* I2 = buf ? IDa : IDb;
    if (g < ncur) {
      const MNode<ND> nd = cur[g];
      const int S = nd.size, s0 = nd.start;
      unsigned long long* key = key_all + (s0 - R.start);  // the node's slice: disjoint per node
      int* dsti = dst_all + (s0 - R.start);
      unsigned* bin = (unsigned*)(smem + L::bins) + g * kBins;
      unsigned long long* cand = (unsigned long long*)bin;
      // DetermineSplitDim: the first strictly larger FP64 spread wins
      double lo[ND], hi[ND];
#pragma unroll
      for (int d = 0; d < ND; d++) {
        lo[d] = okey_inv(nd.kmin[d]);
        hi[d] = okey_inv(nd.kmax[d]);
      }
      int dim = 0;
      double spread = dsub(hi[0], lo[0]);
#pragma unroll
      for (int d = 1; d < ND; d++) {
        double sp = dsub(hi[d], lo[d]);
        if (sp > spread) {
          dim = d;
          spread = sp;
        }
      }
      const double* Cd = C + (int64_t)dim * cs + s0;
      for (int i = r; i < S; i += nt) key[i] = okey(Cd[i]);
      // the median key: rank kr = (S - 1) / 2 along dim
      const int kr = (S - 1) / 2;
      const unsigned long long kmin_dim = sel<ND>(nd.kmin, dim), kmax_dim = sel<ND>(nd.kmax, dim);
      const unsigned long long x = kmin_dim ^ kmax_dim;
      const int first_diff = x ? 63 - __clzll((long long)x) : -1;
      unsigned long long mask = first_diff < 0 ? ~0ull
                                               : (first_diff >= 63 ? 0ull : (~0ull << (first_diff + 1)));
      unsigned long long prefix = first_diff < 0 ? kmin_dim : (kmin_dim & mask);
      int k = kr, ncand = S;
      group_sync(g, nt);  // keys stored
      for (int pass = 0; mask != ~0ull && pass < kPasses; pass++) {
        if (ncand <= kMidCollect) {
          // the class is small: gather its keys; the k-th smallest of them is the median key
          if (r == 0) s_fill[g] = 0u;
          group_sync(g, nt);
          for (int i = r; i < S; i += nt) {
            const unsigned long long kk = key[i];
            if ((kk & mask) == prefix) {
              unsigned slot = atomicAdd(&s_fill[g], 1u);
              if (slot < (unsigned)kMidCollect) cand[slot] = kk;
            }
          }
          group_sync(g, nt);
          const int n = min(ncand, kMidCollect);
          if (r == 0 && s_fill[g] != (unsigned)ncand) atomicExch(err, 5);
          if (r < n) {
            const unsigned long long mine = cand[r];
            int below = 0, equal = 0;
            for (int i = 0; i < n; i++) {
              const unsigned long long o = cand[i];
              below += o < mine;
              equal += o == mine;
            }
            const int kk = min(max(k, 0), n - 1);
            if (below <= kk && kk < below + equal) s_prefix[g] = mine;  // every holder: same value
          }
          group_sync(g, nt);
          prefix = s_prefix[g];
          mask = ~0ull;
          group_sync(g, nt);  // s_prefix and the gathered keys are read before any reuse
          break;
        }
        const int hi_bit = first_diff - 11 * pass;
        const int width = min(11, hi_bit + 1), shift = hi_bit - width + 1;
        const unsigned long long dmask = ((1ull << width) - 1ull) << shift;
        for (int i = r; i < kBins; i += nt) bin[i] = 0u;
        group_sync(g, nt);
        // whole warps per round (match_any needs every lane): lanes with the same digit
        // add once
        for (int i0 = 0; i0 < S; i0 += nt) {
          const int i = i0 + r;
          int digit = -1;
          if (i < S) {
            const unsigned long long kk = key[i];
            if ((kk & mask) == prefix) digit = (int)((kk & dmask) >> shift);
          }
          const unsigned peers = __match_any_sync(0xffffffffu, digit);
          if (digit >= 0 && lane == __ffs(peers) - 1) atomicAdd(&bin[digit], __popc(peers));
        }
        group_sync(g, nt);
        // the digit whose bin holds rank k: each thread owns kPer consecutive bins
        constexpr int kPerMax = kBins * kMidGroups / kMidThreads;
        const int kPer = kBins / nt;
        unsigned cnt[kPerMax], sum = 0;
#pragma unroll
        for (int q = 0; q < kPerMax; q++) {
          cnt[q] = q < kPer ? bin[r * kPer + q] : 0u;
          sum += cnt[q];
        }
        unsigned before = group_excl_scan(sum, r, nt, g, &tot[g], wsum[g]);
        if (before <= (unsigned)k && (unsigned)k < before + sum) {
          int digit = -1;
#pragma unroll
          for (int q = 0; q < kPerMax; q++) {
            if (digit < 0 && q < kPer) {
              if ((unsigned)k < before + cnt[q]) {
                digit = r * kPer + q;
                s_ncand[g] = (int)cnt[q];
              } else {
                before += cnt[q];
              }
            }
          }
          s_k[g] = k - (int)before;
          s_prefix[g] = prefix | ((unsigned long long)digit << shift);
        }
        group_sync(g, nt);
        k = s_k[g];
        ncand = s_ncand[g];
        prefix = s_prefix[g];
        mask |= dmask;
        group_sync(g, nt);  // the shared values are read before the next pass writes them
      }
      if (mask != ~0ull && r == 0) atomicExch(err, 5);  // selection unfinished: report
      const unsigned long long piv = prefix;
      // the stable 3-way partition: warp w of the group takes WR rounds of 32 consecutive
      // keys; ballots rank each key inside its round and class, one scan over the warps'
      // (less, equal) counts orders the warps (counts packed in one word: both < 2^16)
      const int nw = nt >> 5, w = r >> 5;
      const int WR = (S + nt - 1) / nt;  // rounds per warp: at most kMidRounds
      const int wbase = w * WR * 32;
      unsigned cls = 0, nl = 0, ne = 0;
#pragma unroll
      for (int j = 0; j < kMidRounds; j++) {
        if (j < WR) {
          const int i = wbase + j * 32 + lane;
          unsigned c = 3;
          if (i < S) {
            const unsigned long long kk = key[i];
            c = kk < piv ? 0u : (kk == piv ? 1u : 2u);
          }
          cls |= c << (2 * j);
          nl += __popc(__ballot_sync(0xffffffffu, c == 0));
          ne += __popc(__ballot_sync(0xffffffffu, c == 1));
        }
      }
      if (lane == 0) wsum[g][w] = (nl << 16) | ne;
      group_sync(g, nt);
      if (w == 0) {
        const unsigned v = lane < nw ? wsum[g][lane] : 0u;
        unsigned incl = v;
        for (int o = 1; o < 32; o <<= 1) {
          const unsigned t = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += t;
        }
        if (lane < nw) wsum[g][lane] = incl - v;
        if (lane == nw - 1) tot[g] = incl;
      }
      group_sync(g, nt);
      const unsigned pre = wsum[g][w];
      const int n_less = (int)(tot[g] >> 16), total_eq = (int)(tot[g] & 0xffffu);
      const int kleft = kr + 1, right0 = s0 + kleft;
      const int need_eq = kleft - n_less, excess = total_eq - need_eq;
      if (r == 0) out.write(R.nbase + nd.h, lo, hi, p0 + s0, S, dim, okey_inv(piv));
      // destinations: less, then the first need_eq equal keys on the left; the other equal
      // keys, then greater, on the right; each class in its current order
      unsigned rl = pre >> 16, re = pre & 0xffffu;
      unsigned rg = (unsigned)min(wbase, S) - rl - re;  // greater keys before this warp
      const unsigned lt = (1u << lane) - 1u;
#pragma unroll
      for (int j = 0; j < kMidRounds; j++) {
        if (j < WR) {
          const int i = wbase + j * 32 + lane;
          const unsigned c = (cls >> (2 * j)) & 3u;
          const unsigned bL = __ballot_sync(0xffffffffu, c == 0), bE = __ballot_sync(0xffffffffu, c == 1),
                         bG = __ballot_sync(0xffffffffu, c == 2);
          if (c != 3) {
            int dst;
            if (c == 0) {
              dst = s0 + (int)(rl + __popc(bL & lt));
            } else if (c == 1) {
              const int q = (int)(re + __popc(bE & lt));
              dst = q < need_eq ? s0 + n_less + q : right0 + (q - need_eq);
            } else {
              dst = right0 + excess + (int)(rg + __popc(bG & lt));
            }
            if (dst < s0 || dst >= s0 + S) {  // selection inconsistent: report, keep in bounds
              atomicExch(err, 2);
              dst = s0 + i;
            }
            dsti[i] = dst;
          }
          rl += __popc(bL);
          re += __popc(bE);
          rg += __popc(bG);
        }
      }
      if (r < 4 * ND) box[g][r] = (r % (2 * ND)) < ND ? ~0ull : 0ull;
      group_sync(g, nt);
      // move every coordinate and id; the children's boxes on the way
#pragma unroll
      for (int d = 0; d < ND; d++) {
        unsigned long long mnl = ~0ull, mxl = 0ull, mnr = ~0ull, mxr = 0ull;
        for (int i = r; i < S; i += nt) {
          const double v = C[d * cs + s0 + i];
          const int t = dsti[i];
          C2[d * cs + t] = v;
          const unsigned long long kk = okey(v);
          if (t < right0) {
            mnl = min(mnl, kk);
            mxl = max(mxl, kk);
          } else {
            mnr = min(mnr, kk);
            mxr = max(mxr, kk);
          }
        }
        mnl = warp_min_u64(mnl);
        mxl = warp_max_u64(mxl);
        mnr = warp_min_u64(mnr);
        mxr = warp_max_u64(mxr);
        if (lane == 0) {
          atomicMin(&box[g][d], mnl);
          atomicMax(&box[g][ND + d], mxl);
          atomicMin(&box[g][2 * ND + d], mnr);
          atomicMax(&box[g][3 * ND + d], mxr);
        }
      }
      for (int i = r; i < S; i += nt) I2[dsti[i]] = I[s0 + i];
      group_sync(g, nt);
      if (r == 0) {
        for (int side = 0; side < 2; side++) {
          const int cst = side ? right0 : s0, csz = side ? S - kleft : kleft;
          if (csz <= kLocalMax) continue;  // phase 2 finishes it
          const int slot = atomicAdd(&n_next, 1);
          if (slot >= kMidNodes) {
            atomicExch(err, 3);
            continue;
          }
          MNode<ND> c;
          c.start = cst;
          c.size = csz;
          c.h = 2 * nd.h + 1 + side;
          c.pad = 0;
          for (int d = 0; d < ND; d++) {
            c.kmin[d] = box[g][2 * ND * side + d];
            c.kmax[d] = box[g][2 * ND * side + ND + d];
          }
          nxt[slot] = c;
        }
      }
    }
    __syncthreads();  // every group is done with this level
    if (tid == 0) {
      n_cur = min(n_next, kMidNodes);
      n_next = 0;
    }
    MNode<ND>* t = cur;
    cur = nxt;
    nxt = t;
    buf ^= 1;
    __syncthreads();
  }
}

// ---- phase 2: one CTA per subtree of at most kLocalMax particles.
// The subtree is sorted once along every coordinate (key, then local index). No level
// sorts again: a node's bounding box is the first and last entry of its segment in each
// sorted list, its median along the split dimension is the middle entry of that list,
// and the ND + 1 index lists (the sorted lists and the particle order) are split stably
// into the children's segments with one block scan per level (two lists per scan word).
struct LNode {
  short start, size;  // local range
  int h;              // heap index within the tree
  short kl;           // particles that go left (split nodes)
  short child;        // slot of the left child in the next level's list
  int dim;            // -1 leaf
};

constexpr int kLocalThreads = 512;  // two CTAs of 16 warps per SM for ND = 3 (shared memory)

// Shared-memory layout of k_local_build<ND>.
template <int ND>
struct LocalLayout {
  static constexpr int K = kLocalMax;
  static constexpr int kSortN = ND * K;
  static constexpr int kLists = ND + 1;
  static constexpr int kWords = (kLists + 1) / 2;  // packed scan words per position
  static constexpr size_t coords = 0;                                         // double[ND][K]
  static constexpr size_t skey = coords + sizeof(double) * ND * K;            // u64[kSortN]
  static constexpr size_t id = skey + sizeof(unsigned long long) * kSortN;    // int[K]
  static constexpr size_t sidx = id + sizeof(int) * K;                        // u16[kSortN]
  static constexpr size_t lst = sidx + sizeof(unsigned short) * kSortN;       // u16[2][kLists][K]
  static constexpr size_t lv = lst + sizeof(unsigned short) * 2 * kLists * K;  // LNode[2][cap]
  static constexpr size_t total = lv + sizeof(LNode) * 2 * kLevelCap;
  // reused after the sort, inside skey: scan words, node slots, left flags
  static constexpr size_t sc = skey;                                  // unsigned[kWords][K]
  static constexpr size_t node_at = sc + sizeof(unsigned) * kWords * K;  // short[K]
  static constexpr size_t left = node_at + sizeof(short) * K;           // u8[K]
  static_assert(left + K <= id, "the reused region fits inside the sort keys");
  static_assert(lv % 16 == 0, "LNode alignment");
};

template <int ND>
struct PartOut {
  P4* pos;
  float4* posf;
  V4* vel;
  int* perm;
  float4* velf;  // ND = 6 only
};

template <int ND>
__global__ void __launch_bounds__(kLocalThreads) k_local_build(
    const LRoot* __restrict__ roots, const double* Ca, const int* IDa, const double* Cb,
    const int* IDb, int64_t cs, const double* __restrict__ mass_in,
    const double* __restrict__ vel_in, int b, NodeOut<ND> out, PartOut<ND> po, int* err,
    int p0) {
  using L = LocalLayout<ND>;
  extern __shared__ __align__(16) unsigned char smem[];
  double* cc = (double*)(smem + L::coords);                        // cc[d * K + r]
  unsigned long long* skey = (unsigned long long*)(smem + L::skey);  // sort only
  unsigned* sc = (unsigned*)(smem + L::sc);            // after the sort: packed scans
  short* node_at = (short*)(smem + L::node_at);        // level slot of each position, -1 done
  unsigned char* left = smem + L::left;                // per particle
  int* id = (int*)(smem + L::id);
  unsigned short* sidx = (unsigned short*)(smem + L::sidx);
  unsigned short* lst = (unsigned short*)(smem + L::lst);
  LNode* lv = (LNode*)(smem + L::lv);
  LNode* lv2 = lv + kLevelCap;
  __shared__ int n_cur, n_next;
  __shared__ unsigned wsum[32], tot;
  constexpr int K = L::K;
  constexpr int NL = L::kLists;

  const LRoot R = roots[blockIdx.x];
  const int S = R.size;
  const double* C = R.buf ? Cb : Ca;
  const int* I = R.buf ? IDb : IDa;
  for (int e = threadIdx.x; e < S; e += kLocalThreads) {
#pragma unroll
    for (int d = 0; d < ND; d++) cc[d * K + e] = C[d * cs + R.start + e];
    id[e] = I[R.start + e];
  }
  __syncthreads();
  int P = 1, lgP = 0;
  while (P < S) {
    P <<= 1;
    lgP++;
  }
  const int total = ND * P;
  for (int t = threadIdx.x; t < total; t += kLocalThreads) {
    int d = t >> lgP, r = t & (P - 1);
    if (r < S) {
      skey[t] = okey(cc[d * K + r]);
      sidx[t] = (unsigned short)r;
    } else {
      skey[t] = ~0ull;
      sidx[t] = 0xffff;
    }
  }
  __syncthreads();
  // ND segments of P sorted at once; every segment ascending by (key, local index). A
  // bitonic network: the steps with partner distance jj >= 32 exchange through shared
  // memory (one thread per pair, a barrier per step); the steps with jj <= 16 pair lanes
  // of one warp, so each thread takes its elements e = row * kLocalThreads + tid one row
  // at a time through all of them in registers (shuffles, no barrier).
  const int rows = (total + kLocalThreads - 1) / kLocalThreads;
  for (int kk = 2; kk <= P; kk <<= 1) {
    for (int jj = kk >> 1; jj >= 32; jj >>= 1) {
      for (int q = threadIdx.x; q < total / 2; q += kLocalThreads) {
        const int t = ((q & ~(jj - 1)) << 1) | (q & (jj - 1)), u = t + jj;
        const bool up = ((t & (P - 1)) & kk) == 0;
        const unsigned long long a = skey[t], c = skey[u];
        const unsigned short ia = sidx[t], ic = sidx[u];
        const bool gt = (a > c) || (a == c && ia > ic);
        if (gt == up) {
          skey[t] = c;
          skey[u] = a;
          sidx[t] = ic;
          sidx[u] = ia;
        }
      }
      __syncthreads();
    }
    // the register steps: every kk up to 32 at once, later only jj = 16 .. 1
    const int kk_last = kk < 32 ? min(32, P) : kk;
    for (int row = 0; row < rows; row++) {
      const int e = row * kLocalThreads + threadIdx.x;
      const bool have = e < total;
      unsigned long long a = have ? skey[e] : ~0ull;
      unsigned ia = have ? sidx[e] : 0xffffu;
      for (int k2 = kk; k2 <= kk_last; k2 <<= 1) {
        for (int jj = min(k2 >> 1, 16); jj > 0; jj >>= 1) {
          const unsigned long long c = __shfl_xor_sync(0xffffffffu, a, jj);
          const unsigned ic = __shfl_xor_sync(0xffffffffu, ia, jj);
          const bool lower = (e & jj) == 0;
          const bool up = ((e & (P - 1)) & k2) == 0;
          // the lower element of a pair keeps the smaller (up) or larger (down) one
          const bool other_less = (c < a) || (c == a && ic < ia);
          if (other_less == (lower == up)) {
            a = c;
            ia = ic;
          }
        }
      }
      if (have) {
        skey[e] = a;
        sidx[e] = (unsigned short)ia;
      }
    }
    __syncthreads();
    kk = kk_last;
  }
  unsigned short* cur = lst;
  unsigned short* nxt = lst + NL * K;
#pragma unroll
  for (int d = 0; d < ND; d++) {
    for (int i = threadIdx.x; i < S; i += kLocalThreads) {
      unsigned short q = sidx[d * P + i];
      if (q >= S) {  // a padding slot inside the sorted range: report, keep in bounds
        atomicExch(err, 3);
        q = (unsigned short)i;
      }
      cur[d * K + i] = q;
    }
  }
  __syncthreads();  // the sort keys' region is reused from here on
  for (int i = threadIdx.x; i < S; i += kLocalThreads) {
    cur[ND * K + i] = (unsigned short)i;
    node_at[i] = 0;
  }
  if (threadIdx.x == 0) {
    LNode r0;
    r0.start = 0;
    r0.size = (short)S;
    r0.h = R.h;
    r0.kl = 0;
    r0.child = 0;
    r0.dim = -1;
    lv[0] = r0;
    n_cur = 1;
  }
  __syncthreads();
  for (int depth = 0; depth < 64; depth++) {
    if (threadIdx.x == 0) n_next = 0;
    __syncthreads();
    // A: bounding box, split dimension and median of every node of this level
    for (int j = threadIdx.x; j < n_cur; j += kLocalThreads) {
      LNode nd = lv[j];
      int a0 = nd.start, a1 = nd.start + nd.size - 1;
      double lo[ND], hi[ND];
#pragma unroll
      for (int d = 0; d < ND; d++) {
        lo[d] = cc[d * K + cur[d * K + a0]];
        hi[d] = cc[d * K + cur[d * K + a1]];
      }
      int dim = -1;
      double split = 0.0;
      if (nd.size > b) {
        // DetermineSplitDim: the first strictly larger FP64 spread wins
        dim = 0;
        double spread = dsub(hi[0], lo[0]);
#pragma unroll
        for (int d = 1; d < ND; d++) {
          double sp = dsub(hi[d], lo[d]);
          if (sp > spread) {
            dim = d;
            spread = sp;
          }
        }
        int kl = (nd.size - 1) / 2 + 1;
        int q = cur[dim * K + nd.start + kl - 1];
        split = cc[dim * K + q];
        int slot = atomicAdd(&n_next, 2);
        if (slot + 2 <= kLevelCap) {
          LNode l, r;
          l.start = nd.start;
          l.size = (short)kl;
          l.h = 2 * nd.h + 1;
          r.start = (short)(nd.start + kl);
          r.size = (short)(nd.size - kl);
          r.h = 2 * nd.h + 2;
          l.kl = r.kl = 0;
          l.child = r.child = 0;
          l.dim = r.dim = -1;
          lv2[slot] = l;
          lv2[slot + 1] = r;
        } else {
          atomicExch(err, 4);
        }
        nd.kl = (short)kl;
        nd.child = (short)slot;
      }
      nd.dim = dim;
      lv[j] = nd;
      out.write(R.nbase + nd.h, lo, hi, p0 + R.start + nd.start, nd.size, dim, split);
    }
    __syncthreads();
    if (n_next == 0 || n_next > kLevelCap) break;
    // B: which particles go left, read off the list of their node's split dimension
    for (int i = threadIdx.x; i < S; i += kLocalThreads) {
      const int j = node_at[i];
      if (j >= 0) {
        const LNode nd = lv[j];
        if (nd.dim >= 0) left[cur[nd.dim * K + i]] = (i - nd.start) < nd.kl;
      }
    }
    __syncthreads();
    // C: exclusive scans of the left flags of the NL lists (two packed per word); each
    // thread covers kPerT consecutive positions
    {
      constexpr int kPerT = kLocalMax / kLocalThreads;
      constexpr int NW = L::kWords;
      unsigned f[NW][kPerT], sw[NW];
#pragma unroll
      for (int w = 0; w < NW; w++) sw[w] = 0;
#pragma unroll
      for (int u = 0; u < kPerT; u++) {
        int i = kPerT * threadIdx.x + u;
        bool split_here = false;
        if (i < S) {
          int j = node_at[i];
          split_here = j >= 0 && lv[j].dim >= 0;
        }
#pragma unroll
        for (int w = 0; w < NW; w++) {
          unsigned a = 0;
          if (split_here) {
            a = left[cur[(2 * w) * K + i]];
            if (2 * w + 1 < NL) a |= (unsigned)left[cur[(2 * w + 1) * K + i]] << 16;
          }
          f[w][u] = sw[w];
          sw[w] += a;
        }
      }
#pragma unroll
      for (int w = 0; w < NW; w++) {
        unsigned bw = block_excl_scan_t<kLocalThreads>(sw[w], &tot, wsum);
#pragma unroll
        for (int u = 0; u < kPerT; u++) {
          int i = kPerT * threadIdx.x + u;
          if (i < S) sc[w * K + i] = bw + f[w][u];
        }
      }
    }
    __syncthreads();
    // D: stable split of every list inside its node; positions of leaves stay put
    for (int i = threadIdx.x; i < S; i += kLocalThreads) {
      int j = node_at[i];
      if (j < 0) {
#pragma unroll
        for (int l = 0; l < NL; l++) nxt[l * K + i] = cur[l * K + i];
        continue;
      }
      LNode nd = lv[j];
      if (nd.dim < 0) {
#pragma unroll
        for (int l = 0; l < NL; l++) nxt[l * K + i] = cur[l * K + i];
        node_at[i] = -1;
        continue;
      }
      int rel = i - nd.start;
      unsigned vw[L::kWords];
#pragma unroll
      for (int w = 0; w < L::kWords; w++) vw[w] = sc[w * K + i] - sc[w * K + nd.start];
#pragma unroll
      for (int l = 0; l < NL; l++) {
        unsigned v = vw[l >> 1];
        int before = (int)((l & 1) ? (v >> 16) : (v & 0xffffu));  // left entries before i
        unsigned short q = cur[l * K + i];
        int dst = left[q] ? nd.start + before : nd.start + nd.kl + (rel - before);
        if (dst < nd.start || dst >= nd.start + nd.size) {  // inconsistent split: report
          atomicExch(err, 3);
          dst = i;
        }
        nxt[l * K + dst] = q;
      }
      node_at[i] = (short)(rel < nd.kl ? nd.child : nd.child + 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) n_cur = n_next;
    unsigned short* t = cur;
    cur = nxt;
    nxt = t;
    LNode* tl = lv;
    lv = lv2;
    lv2 = tl;
    __syncthreads();
  }
  // final tree-order arrays: the particle-order list holds every leaf contiguously
  for (int e = threadIdx.x; e < S; e += kLocalThreads) {
    int q = cur[ND * K + e];
    int t = p0 + R.start + e;  // absolute tree index
    int ii = p0 + id[q];       // absolute input index
    double m = mass_in ? mass_in[ii] : 1.0;
    P4 p;
    p.x = cc[q];
    p.y = cc[K + q];
    p.z = cc[2 * K + q];
    p.m = m;
    po.pos[t] = p;
    po.posf[t] = make_float4(__double2float_rn(p.x), __double2float_rn(p.y),
                             __double2float_rn(p.z), 0.f);
    po.perm[t] = ii;
    if (ND == 6) {
      po.vel[t] = make_v4(cc[3 * K + q], cc[4 * K + q], cc[5 * K + q], 0.0);
      po.velf[t] = make_float4(__double2float_rn(cc[3 * K + q]), __double2float_rn(cc[4 * K + q]),
                               __double2float_rn(cc[5 * K + q]), 0.f);
    } else if (po.vel && vel_in) {
      po.vel[t] = make_v4(vel_in[3 * ii], vel_in[3 * ii + 1], vel_in[3 * ii + 2], 0.0);
    }
  }
}

int depth_of(int64_t n, int b) {
  int d = 0;
  while (n > b) {
    n = (n - 1) / 2 + 1;
    d++;
  }
  return d;
}

}  // namespace

size_t local_build_smem(int nd) {
  return nd == 6 ? LocalLayout<6>::total : LocalLayout<3>::total;
}

// One global level of a build plan: its nodes [g0, g0 + ng) and chunks [c0, c0 + nc) in
// the uploaded plan, and the ping-pong buffer holding its particles.
struct PlanLevel {
  int g0, ng, c0, nc, buf;
};
// The last plan built on a host thread (its bytes stay in that thread's page-locked stage;
// one per thread for every dimension count, as the stage is). `stage`/`gen` name the
// staged bytes it describes, so a stage written or replaced since is never mistaken for
// this plan.
struct PlanCache {
  bool valid = false;
  const void* stage = nullptr;
  unsigned long long gen = 0;
  int nd = 0, b = 0;
  std::vector<TreeSpec> trees;
  std::vector<PlanLevel> levels;
  int max_ng = 0;
  size_t nch = 0, nroots = 0, nmroots = 0, bg = 0, bc = 0, br = 0, bm = 0;
};
bool same_trees(const std::vector<TreeSpec>& a, const std::vector<TreeSpec>& b) {
  if (a.size() != b.size()) return false;
  for (size_t i = 0; i < a.size(); i++)
    if (a[i].pstart != b[i].pstart || a[i].n != b[i].n || a[i].nbase != b[i].nbase) return false;
  return true;
}

// One growing page-locked buffer per host thread for the build plans.
struct PinnedStage {
  unsigned char* p = nullptr;
  size_t cap = 0, used = 0;
  unsigned long long gen = 0;  // bumped whenever a plan is written into it
  unsigned char* data() { return p; }
  size_t size() const { return used; }
  ~PinnedStage() {
    if (p) cudaFreeHost(p);
  }
};
PlanCache& plan_cache() {
  static thread_local PlanCache cache;
  return cache;
}

PinnedStage& pinned_stage(size_t bytes) {
  static thread_local PinnedStage st;
  if (bytes > st.cap) {
    if (st.p) cudaFreeHost(st.p);
    st.p = nullptr;
    st.cap = 0;
    st.gen++;  // new memory holds no plan (even at the same address)
    size_t cap = std::max<size_t>(bytes, 1 << 20);
    if (cudaMallocHost((void**)&st.p, cap) == cudaSuccess) st.cap = cap;
    else st.p = nullptr;
  }
  st.used = bytes;
  return st;
}

int64_t heap_slots(int64_t n, int b) {
  int d = depth_of(n, b);
  return (int64_t(1) << (d + 1)) - 1;
}

int64_t count_nodes(int64_t n, int b) {
  // level by level: the split rule gives the nodes of one level at most a few distinct
  // sizes, so counting (size, multiplicity) pairs replaces a walk over every node
  std::vector<std::pair<int64_t, int64_t>> cur{{n, 1}}, nxt;
  int64_t total = 0;
  while (!cur.empty()) {
    nxt.clear();
    for (auto& sm : cur) {
      total += sm.second;
      if (sm.first <= b) continue;
      int64_t l = (sm.first - 1) / 2 + 1;
      for (int64_t c : {l, sm.first - l}) {
        bool found = false;
        for (auto& q : nxt)
          if (q.first == c) {
            q.second += sm.second;
            found = true;
          }
        if (!found) nxt.push_back({c, sm.second});
      }
    }
    cur.swap(nxt);
  }
  return total;
}

// Build every tree of the forest. All arrays live on `st`. Returns NBK status.
template <int ND>
static int build_forest_t(const std::vector<TreeSpec>& trees, int b, const double* d_pos_in,
                          const double* d_mass_in, const double* d_vel_in, NodeOut<ND> nout,
                          PartOut<ND> pout, DevAlloc& alloc, cudaStream_t st, void* root_out,
                          size_t root_bytes, const void* root_src) {
  using GNode = GNodeT<ND>;
  Phase ph("build", st);
  // internal buffers cover only [p0, p0 + ntot), the particles of these trees
  int64_t p0 = trees.empty() ? 0 : trees[0].pstart, pend = 0;
  for (auto& t : trees) {
    p0 = std::min<int64_t>(p0, t.pstart);
    pend = std::max<int64_t>(pend, t.pstart + t.n);
  }
  int64_t ntot = pend - p0;
  if (ntot == 0) return NBK_OK;
  double *Ca, *Cb;
  int *IDa, *IDb, *d_err;
  const int64_t cs = ntot;  // coordinate stride of the ping-pong buffers

  // The whole plan (every global level's nodes and chunks, every subtree handed to the
  // per-CTA phase) depends only on the tree sizes, so it is computed on the host first
  // and uploaded once; the levels then run back to back with no host round trip.
  // The level plan of the last build on this thread stays in the thread's page-locked
  // stage with its key (dimension count, leaf size, trees): a repeated build of the same
  // trees skips the planning and the staging copy and uploads the stage as it is (the
  // previous build's final synchronisation finished its upload).
  PlanCache& cache = plan_cache();
  PinnedStage& stage_now = pinned_stage(0);  // the thread's stage as it is
  const bool hit = cache.valid && cache.stage == stage_now.p && cache.gen == stage_now.gen &&
                   cache.nd == ND && cache.b == b && same_trees(cache.trees, trees);
  if (!hit) {
    cache.valid = false;
    std::vector<LRoot> lroots;
    std::vector<MRoot> mroots;
    struct HN {
      int64_t start, size;
      int h, nbase;
    };
    // a subtree of kLocalMax < size <= kMidMax particles at ping-pong side `side`: one
    // CTA of phase 1b splits it level by level (each level flips the side); its
    // descendants of at most kLocalMax particles go to phase 2 on the side they land on
    auto add_mid = [&](const HN& r, int side) {
      mroots.push_back({(int)r.start, (int)r.size, r.nbase, r.h, side, 0});
      std::vector<HN> lev{r}, down;
      while (!lev.empty()) {
        side ^= 1;
        down.clear();
        for (const HN& x : lev) {
          int64_t l = (x.size - 1) / 2 + 1;
          for (HN c : {HN{x.start, l, 2 * x.h + 1, x.nbase},
                       HN{x.start + l, x.size - l, 2 * x.h + 2, x.nbase}}) {
            if (c.size <= kLocalMax) lroots.push_back({(int)c.start, (int)c.size, c.nbase, c.h, side, 0});
            else down.push_back(c);
          }
        }
        lev.swap(down);
      }
    };
    std::vector<HN> cur, nxt;
    for (auto& t : trees) {
      if (t.n <= 0) continue;
      HN r{t.pstart - p0, t.n, 0, t.nbase};
      if (t.n <= kLocalMax) lroots.push_back({(int)(t.pstart - p0), (int)t.n, t.nbase, 0, 0, 0});
      else if (t.n <= kMidMax) add_mid(r, 0);
      else cur.push_back(r);
    }
    std::vector<GNode> gn;
    std::vector<Chunk> ch;
    std::vector<PlanLevel> levels;
    int buf = 0, max_ng = 0;
    while (!cur.empty()) {
      PlanLevel L{(int)gn.size(), (int)cur.size(), (int)ch.size(), 0, buf};
      for (size_t i = 0; i < cur.size(); i++) {
        GNode g{};
        g.start = (int)cur[i].start;
        g.size = (int)cur[i].size;
        g.node = cur[i].nbase + cur[i].h;
        g.k = (int)((cur[i].size - 1) / 2);  // rank of the median inside the node
        g.ncand = (int)cur[i].size;
        g.child[0] = g.child[1] = -1;
        for (int d = 0; d < ND; d++) {
          g.kmin[d] = ~0ull;  // boxes are merged in with atomics
          g.kmax[d] = 0ull;
        }
        g.first_chunk = (int)ch.size() - L.c0;
        int nc = (int)((cur[i].size + kChunk - 1) / kChunk);
        g.nchunks = nc;
        for (int c = 0; c < nc; c++) {
          int off = c * kChunk;
          int len = (int)std::min<int64_t>(kChunk, cur[i].size - off);
          ch.push_back({(int)i, (int)(cur[i].start + off), len, off});
        }
        gn.push_back(g);
      }
      L.nc = (int)ch.size() - L.c0;
      levels.push_back(L);
      max_ng = std::max(max_ng, L.ng);
      buf ^= 1;
      nxt.clear();
      for (size_t i = 0; i < cur.size(); i++) {
        const HN& c = cur[i];
        int64_t l = (c.size - 1) / 2 + 1;
        HN Lh = {c.start, l, 2 * c.h + 1, c.nbase};
        HN Rh = {c.start + l, c.size - l, 2 * c.h + 2, c.nbase};
        int side = 0;
        for (HN x : {Lh, Rh}) {
          if (x.size <= kLocalMax) {
            lroots.push_back({(int)x.start, (int)x.size, x.nbase, x.h, buf, 0});
          } else if (x.size <= kMidMax) {
            add_mid(x, buf);
          } else {
            gn[L.g0 + i].child[side] = (int)nxt.size();
            nxt.push_back(x);
          }
          side++;
        }
      }
      cur.swap(nxt);
    }
    // one upload: [GNode...][Chunk...][LRoot...][MRoot...]
    size_t bg = sizeof(GNode) * gn.size(), bc = sizeof(Chunk) * ch.size(),
           br = sizeof(LRoot) * lroots.size(), bm = sizeof(MRoot) * mroots.size();
    // staged in page-locked memory so the upload is a plain asynchronous copy (the build's
    // final synchronisation orders it before the buffer is reused by this thread)
    PinnedStage& plan = pinned_stage(bg + bc + br + bm + 16);
    if (!plan.data()) {
      set_error("tree build: page-locked staging allocation failed");
      return NBK_ERR_NOMEM;
    }
    memcpy(plan.data(), gn.data(), bg);
    memcpy(plan.data() + bg, ch.data(), bc);
    memcpy(plan.data() + bg + bc, lroots.data(), br);
    memcpy(plan.data() + bg + bc + br, mroots.data(), bm);
    plan.gen++;
    cache.stage = plan.p;
    cache.gen = plan.gen;
    cache.valid = true;
    cache.nd = ND;
    cache.b = b;
    cache.trees = trees;
    cache.levels = levels;
    cache.max_ng = max_ng;
    cache.nch = ch.size();
    cache.nroots = lroots.size();
    cache.nmroots = mroots.size();
    cache.bg = bg;
    cache.bc = bc;
    cache.br = br;
    cache.bm = bm;
  }
  const std::vector<PlanLevel>& levels = cache.levels;
  const int max_ng = cache.max_ng;
  const size_t nch = cache.nch, nroots = cache.nroots, nmroots = cache.nmroots, bg = cache.bg,
               bc = cache.bc, br = cache.br;
  PinnedStage& plan = pinned_stage(cache.bg + cache.bc + cache.br + cache.bm + 16);
  if (!plan.data()) {
    cache.valid = false;
    set_error("tree build: page-locked staging allocation failed");
    return NBK_ERR_NOMEM;
  }
  // every scratch array of the build in one allocation; the error word and the radix
  // histograms, which start zeroed, come first
  unsigned char* d_plan;
  unsigned long long* d_cand = nullptr;
  unsigned *d_hist = nullptr, *d_cl = nullptr, *d_ce = nullptr, *d_bl = nullptr, *d_be = nullptr;
  const size_t ncall = std::max<size_t>(nch, 1);
  const size_t hist_bytes = levels.empty() ? 0 : sizeof(unsigned) * kBins * max_ng;
  std::vector<DevPart> parts{{(void**)&d_err, sizeof(int)}, {(void**)&d_hist, hist_bytes}};
  const size_t zeroed = block_bytes(parts);
  parts.insert(parts.end(), {{(void**)&Ca, sizeof(double) * ND * ntot},
                             {(void**)&Cb, sizeof(double) * ND * ntot},
                             {(void**)&IDa, sizeof(int) * ntot},
                             {(void**)&IDb, sizeof(int) * ntot},
                             {(void**)&d_plan, plan.size()}});
  if (!levels.empty()) {
    parts.insert(parts.end(), {{(void**)&d_cand, sizeof(unsigned long long) * ntot},
                               {(void**)&d_cl, sizeof(unsigned) * ncall},
                               {(void**)&d_ce, sizeof(unsigned) * ncall},
                               {(void**)&d_bl, sizeof(unsigned) * ncall},
                               {(void**)&d_be, sizeof(unsigned) * ncall}});
  }
  // every way out of this build waits for the stream, so this thread's kept block is free
  NBK_TRY(thread_scratch_block(0, parts, st, alloc));
  NBK_CUDA_TRY(cudaMemsetAsync(d_err, 0, zeroed, st));
  NBK_CUDA_TRY(cudaMemcpyAsync(d_plan, plan.data(), plan.size(), cudaMemcpyHostToDevice, st));
  // every way out of here waits for the stream, so the staging buffer is free again
  struct WaitOnExit {
    cudaStream_t st;
    ~WaitOnExit() { cudaStreamSynchronize(st); }
  } wait_on_exit{st};
  GNode* d_gall = (GNode*)d_plan;
  Chunk* d_call = (Chunk*)(d_plan + bg);
  LRoot* d_r = (LRoot*)(d_plan + bg + bc);
  MRoot* d_m = (MRoot*)(d_plan + bg + bc + br);
  k_init_soa<ND><<<(unsigned)((ntot + 255) / 256), 256, 0, st>>>(
      d_pos_in + 3 * p0, d_vel_in ? d_vel_in + 3 * p0 : nullptr, Ca, cs, IDa, ntot, d_err);
  note_launch();
  NBK_CUDA_TRY(cudaGetLastError());
  for (size_t li = 0; li < levels.size(); li++) {
    const PlanLevel& L = levels[li];
    GNode* d_g = d_gall + L.g0;
    GNode* d_gnext = li + 1 < levels.size() ? d_gall + levels[li + 1].g0 : nullptr;
    Chunk* d_c = d_call + L.c0;
    unsigned *cl = d_cl + L.c0, *ce = d_ce + L.c0, *bl = d_bl + L.c0, *be = d_be + L.c0;
    int nc = L.nc;
    const double* C = L.buf ? Cb : Ca;
    const int* I = L.buf ? IDb : IDa;
    double* C2 = L.buf ? Ca : Cb;
    int* I2 = L.buf ? IDa : IDb;
    // boxes of the first level's nodes; every later level gets them from the scatter above
    if (li == 0) {
      k_bbox<ND><<<nc, kThreads, 0, st>>>(d_c, d_g, C, cs); note_launch();
    }
    for (int pass = 0; pass < kPasses; pass++) {
      k_radix<ND><<<nc, kThreads, 0, st>>>(d_c, d_g, C, cs, d_hist, d_cand, pass, nout, (int)p0,
                                           d_err); note_launch();
    }
    k_count_scan<ND><<<nc, kThreads, 0, st>>>(d_c, d_g, C, cs, cl, ce, bl, be, nout);
    note_launch();
    k_scatter<ND><<<nc, kThreads, 0, st>>>(d_c, d_g, C, I, C2, I2, cs, bl, be, d_err, d_gnext);
    note_launch();
    NBK_CUDA_TRY(cudaGetLastError());
  }
  if (nmroots > 0) {
    size_t sm = MidLayout<ND>::total;
    NBK_TRY(ensure_dyn_smem((const void*)k_mid_build<ND>, (int)sm));
    k_mid_build<ND><<<(unsigned)nmroots, kMidThreads, sm, st>>>(d_m, Ca, IDa, Cb, IDb, cs, nout,
                                                                d_err, (int)p0);
    note_launch();
    NBK_CUDA_TRY(cudaGetLastError());
  }
  if (nroots > 0) {
    size_t sm = LocalLayout<ND>::total;
    NBK_TRY(ensure_dyn_smem((const void*)k_local_build<ND>, (int)sm));
    k_local_build<ND><<<(unsigned)nroots, kLocalThreads, sm, st>>>(
        d_r, Ca, IDa, Cb, IDb, cs, d_mass_in, d_vel_in, b, nout, pout, d_err, (int)p0);
    note_launch();
    NBK_CUDA_TRY(cudaGetLastError());
  }
  if (root_out && root_src)
    NBK_CUDA_TRY(cudaMemcpyAsync(root_out, root_src, root_bytes, cudaMemcpyDeviceToHost, st));
  int h_err = 0;
  NBK_CUDA_TRY(cudaMemcpyAsync(&h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
  NBK_CUDA_TRY(cudaStreamSynchronize(st));
  alloc.release_all_scratch(st);
  if (h_err == 1) {
    set_error("input positions or velocities contain NaN or infinity");
    return NBK_ERR_INVALID;
  }
  if (h_err) {
    set_error("tree build: partition inconsistent (device check, code " + std::to_string(h_err) + ")");
    return NBK_ERR_DEVICE;
  }
  return NBK_OK;
}

int build_forest(const std::vector<TreeSpec>& trees, int b, const double* d_pos_in,
                 const double* d_mass_in, const double* d_vel_in, BuiltArrays& out,
                 DevAlloc& alloc, cudaStream_t st, NodeX* root_out) {
  NodeOut<3> no{out.node, out.nodex};
  PartOut<3> po{out.pos, out.posf, out.vel, out.perm, nullptr};
  const void* src = trees.empty() ? nullptr : (const void*)(out.nodex + trees[0].nbase);
  return build_forest_t<3>(trees, b, d_pos_in, d_mass_in, d_vel_in, no, po, alloc, st, root_out,
                           sizeof(NodeX), src);
}

int build_forest_phase(const std::vector<TreeSpec>& trees, int b, const double* d_pos_in,
                       const double* d_mass_in, const double* d_vel_in, BuiltArrays& out,
                       DevAlloc& alloc, cudaStream_t st, NodeB6* root_out) {
  if (!d_vel_in) {
    set_error("phase-space tree: velocities are required");
    return NBK_ERR_INVALID;
  }
  NodeOut<6> no{out.nodes6, out.nodeb6, out.nodef6};
  PartOut<6> po{out.pos, out.posf, out.vel, out.perm, out.velf};
  const void* src = trees.empty() ? nullptr : (const void*)(out.nodeb6 + trees[0].nbase);
  return build_forest_t<6>(trees, b, d_pos_in, d_mass_in, d_vel_in, no, po, alloc, st, root_out,
                           sizeof(NodeB6), src);
}

}  // namespace nbk
