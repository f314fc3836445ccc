// Fixed-radius searches (replaces KDTree::SearchBallPosTagged / SearchBallPos and their
// node recursions, src/KDTree/KDFindNearest.cxx:567-706, KDSplitNode.cxx:455-686,
// 1341-1456, KDLeafNode.cxx:247-410).
//
// One warp serves 32 queries and walks the tree once for all of them, like the kNN
// kernel. Results are returned as CSR: a counting pass, an exclusive scan, a filling
// pass. Pair decisions are the reference's FP64 test d2 < fdist2 (strict); the whole-node
// shortcut of the reference marks exactly the particles this test accepts (every member
// of a node whose farthest corner is inside the radius passes it, because rounding is
// monotone), so it changes only whether the target itself is reported, which
// nbk_ball_mark reproduces from the exact node boxes.
#include "nbk_build.h"

namespace nbk {

namespace {

constexpr int kStack = 64;
constexpr int kWpb = 8;

struct BallArgs {
  TreeView tv;
  int qmode;  // 0: targets (tree indices), 1: coordinates
  const int* qidx;
  const double* qx;
  int nq;
  double r2;
  int exclude_self;
  int* counts;
  const int64_t* offsets;
  int* out;
  double* outd2;
  int* err;
};

struct BallSmem {
  float4 sf[32];
  P4 sp[32];
  int stk[kStack];
};

template <bool FILL>
__global__ void __launch_bounds__(32 * kWpb) k_ball(BallArgs a) {
  __shared__ BallSmem sm[kWpb];
  const unsigned FULL = 0xffffffffu;
  int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  BallSmem& w = sm[warp];
  const TreeView& tv = a.tv;
  int gw = blockIdx.x * kWpb + warp;
  if (gw * 32 >= a.nq) return;
  int q = gw * 32 + lane;
  bool valid = q < a.nq;
  int self = -1;
  double x0[3] = {0, 0, 0};
  if (valid) {
    if (a.qmode == 0) {
      self = a.qidx[q];
      P4 p = tv.pos[self];
      x0[0] = p.x;
      x0[1] = p.y;
      x0[2] = p.z;
    } else {
      x0[0] = a.qx[3 * (size_t)q];
      x0[1] = a.qx[3 * (size_t)q + 1];
      x0[2] = a.qx[3 * (size_t)q + 2];
    }
  }
  int64_t base = (FILL && valid) ? a.offsets[q] : 0;
  int cnt = 0;
  float thr = thresh_hi(a.r2), r2_lo = thresh_lo(a.r2);
  long long r2k = a.r2 > 0.0 ? dkey(a.r2) : 0;  // nothing is inside r2 <= 0 or NaN
  // the query's own rounding bound, images included (it may lie outside the tree's box)
  float eps = valid ? query_eps(tv, x0[0], x0[1], x0[2]) : tv.eps;
  float two_eps = __fadd_ru(eps, tv.eps);
  int npass = tv.periodic ? 8 : 1;
  int near = 0;
  if (tv.periodic && valid)
    near = near_walls(make_float4(__double2float_rn(x0[0]), __double2float_rn(x0[1]),
                                  __double2float_rn(x0[2]), 0.f),
                      tv.period, eps, thr);
  for (int pass = 0; pass < npass; pass++) {
    double xq[3] = {x0[0], x0[1], x0[2]};
    bool active = valid;
    if (pass > 0) {
      bool may = (kImageMask[pass] & ~near) == 0;
      if (!__any_sync(0xffffffffu, may)) continue;
      double sval = reflect(x0, xq, tv.period, kImageMask[pass]);
      active = active && may && (a.r2 > dmul(sval, sval));  // KDSplitNode.cxx:1356-1373
    }
    if (!__any_sync(FULL, active)) continue;
    float qx = __double2float_rn(xq[0]), qy = __double2float_rn(xq[1]),
          qz = __double2float_rn(xq[2]);
    int sp = 1;
    if (lane == 0) w.stk[0] = 0;
    __syncwarp();
    while (sp > 0) {
      int h = w.stk[sp - 1];
      sp--;
      __syncwarp();
      NodeRec r = tv.node[tv.nbase + h];
      bool need = active && box_d2_lo(qx, qy, qz, eps, r) < thr;
      if (!__any_sync(FULL, need)) continue;
      if (r.count <= tv.b) {
        for (int c0 = 0; c0 < r.count; c0 += 32) {
          int m = min(32, r.count - c0);
          if (lane < m) {
            w.sf[lane] = tv.posf[r.start + c0 + lane];
            w.sp[lane] = tv.pos[r.start + c0 + lane];
          }
          __syncwarp();
          if (need) {
            for (int j = 0; j < m; j++) {
              int ti = r.start + c0 + j;
              if (a.exclude_self && pass == 0 && ti == self) continue;
              float4 cf = w.sf[j];
              if (pair_d2_lo(qx, qy, qz, cf.x, cf.y, cf.z, two_eps) < thr) {
                // FP32 upper bound inside the ball decides without FP64 unless the
                // distance itself is wanted
                double d2 = 0.0;
                bool in = !(FILL && a.outd2) &&
                          pair_d2_hi(qx, qy, qz, cf.x, cf.y, cf.z, two_eps) < r2_lo;
                if (!in) {
                  P4 c = w.sp[j];
                  d2 = dist2_exact(xq[0], xq[1], xq[2], c.x, c.y, c.z);
                  in = dkey(d2) < r2k;  // d2 < r2
                }
                if (in) {
                  if (FILL) {
                    if (base + cnt < a.offsets[q + 1]) {
                      a.out[base + cnt] = ti;
                      if (a.outd2) a.outd2[base + cnt] = d2;
                    } else {
                      atomicExch(a.err, kErrCapacity);  // fill disagrees with count
                    }
                  }
                  cnt++;
                }
              }
            }
          }
          __syncwarp();
        }
      } else {
        int hl = 2 * h + 1, hr = 2 * h + 2;
        NodeRec rl = tv.node[tv.nbase + hl], rr = tv.node[tv.nbase + hr];
        bool nl = need && box_d2_lo(qx, qy, qz, eps, rl) < thr;
        bool nr = need && box_d2_lo(qx, qy, qz, eps, rr) < thr;
        bool anyl = __any_sync(FULL, nl), anyr = __any_sync(FULL, nr);
        if (sp + 2 > kStack) {
          if (lane == 0) atomicExch(a.err, kErrCapacity);
          return;
        }
        if (anyr) {
          if (lane == 0) w.stk[sp] = hr;
          sp++;
        }
        if (anyl) {
          if (lane == 0) w.stk[sp] = hl;
          sp++;
        }
        __syncwarp();
      }
    }
  }
  if (!FILL && valid) a.counts[q] = cnt;
}

__global__ void k_scan64_blocks(const int* in, int64_t* out, int64_t* bsum, int n) {
  __shared__ int64_t s[1024];
  int i = blockIdx.x * 1024 + threadIdx.x;
  int64_t v = i < n ? in[i] : 0;
  s[threadIdx.x] = v;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    int64_t t = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
    __syncthreads();
    s[threadIdx.x] += t;
    __syncthreads();
  }
  if (i < n) out[i] = s[threadIdx.x] - v;
  if (threadIdx.x == 1023) bsum[blockIdx.x] = s[1023];
}
__global__ void k_scan64_sums(int64_t* bsum, int nb, int64_t* total) {
  __shared__ int64_t s[1024];
  __shared__ int64_t run;
  if (threadIdx.x == 0) run = 0;
  __syncthreads();
  for (int c0 = 0; c0 < nb; c0 += 1024) {
    int i = c0 + threadIdx.x;
    int64_t v = i < nb ? bsum[i] : 0;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
      int64_t t = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
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
__global__ void k_scan64_add(int64_t* out, const int64_t* bsum, int n, const int64_t* total) {
  int i = blockIdx.x * 1024 + threadIdx.x;
  if (i < n) out[i] += bsum[blockIdx.x];
  if (i == 0) out[n] = *total;
}

// Whether SearchBallPos(tt) reports the target: a node on the root-to-leaf path is
// flagged by FlagNodeForSearchBallPos (split nodes, KDNode.h:325-332 with
// __checkboundaries :280-291) or the leaf's whole-bucket test holds (KDLeafNode.cxx:
// 250-255), all in FP64 on the exact node boxes.
__global__ void k_mark(TreeView tv, int target, double r2, int imark, const int* found,
                       const double* found_d2, const int64_t* nfound, const int* perm,
                       int* mark, double* dist2, int check_self) {
  int64_t nf = *nfound;
  for (int64_t i = threadIdx.x + blockIdx.x * (int64_t)blockDim.x; i < nf;
       i += (int64_t)blockDim.x * gridDim.x) {
    int id = perm[found[i]];
    mark[id] = imark;
    dist2[id] = found_d2[i];
  }
  if (!check_self || blockIdx.x != 0 || threadIdx.x != 0) return;
  P4 p = tv.pos[target];
  double x[3] = {p.x, p.y, p.z};
  int h = 0;
  bool inc = false;
  for (int depth = 0; depth < 64; depth++) {
    const NodeX& nx = tv.nodex[tv.nbase + h];
    const NodeRec& r = tv.node[tv.nbase + h];
    bool leaf = r.count <= tv.b;
    double me = 0.0;
    for (int d = 0; d < 3; d++) me = fmax(me, dsub(nx.hi[d], nx.lo[d]));
    double maxr2 = 0.0;
    for (int d = 0; d < 3; d++) {
      double da = dsub(x[d], nx.lo[d]), db = dsub(nx.hi[d], x[d]);
      double a2 = dmul(da, da), b2 = dmul(db, db);
      maxr2 = dadd(maxr2, a2 > b2 ? a2 : b2);
    }
    if (leaf) {
      inc = maxr2 < r2;
      break;
    }
    if (!(dmul(me, me) > r2) && maxr2 < r2) {
      inc = true;
      break;
    }
    const NodeRec& l = tv.node[tv.nbase + 2 * h + 1];
    h = (target < l.start + l.count) ? 2 * h + 1 : 2 * h + 2;
  }
  if (inc) {
    int id = perm[target];
    mark[id] = imark;
    dist2[id] = 0.0;
  }
}

}  // namespace

int run_ball(const TreeView& tv, int qmode, const int* qidx, const double* qx, int nq,
             double fdist2, int exclude_self, int64_t* d_offsets, int* d_out,
             int64_t out_capacity, int64_t* h_total, DevAlloc& alloc, cudaStream_t st) {
  if (nq == 0) {
    *h_total = 0;
    NBK_CUDA_TRY(cudaMemsetAsync(d_offsets, 0, sizeof(int64_t), st));
    return NBK_OK;
  }
  int* counts;
  int64_t *bsum, *d_total;
  int* err;
  int nb = (nq + 1023) / 1024;
  NBK_TRY(alloc.get((void**)&counts, sizeof(int) * nq));
  NBK_TRY(alloc.get((void**)&bsum, sizeof(int64_t) * (nb + 1)));
  NBK_TRY(alloc.get((void**)&d_total, sizeof(int64_t)));
  NBK_TRY(alloc.get((void**)&err, sizeof(int)));
  NBK_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), st));
  BallArgs a{};
  a.tv = tv;
  a.qmode = qmode;
  a.qidx = qidx;
  a.qx = qx;
  a.nq = nq;
  a.r2 = fdist2;
  a.exclude_self = exclude_self;
  a.counts = counts;
  a.err = err;
  int warps = (nq + 31) / 32;
  int blocks = (warps + kWpb - 1) / kWpb;
  Phase ph("ball", st);
  k_ball<false><<<blocks, 32 * kWpb, 0, st>>>(a); note_launch();
  k_scan64_blocks<<<nb, 1024, 0, st>>>(counts, d_offsets, bsum, nq); note_launch();
  k_scan64_sums<<<1, 1024, 0, st>>>(bsum, nb, d_total); note_launch();
  k_scan64_add<<<nb, 1024, 0, st>>>(d_offsets, bsum, nq, d_total); note_launch();
  NBK_CUDA_TRY(cudaGetLastError());
  int64_t total = 0;
  int herr = 0;
  NBK_CUDA_TRY(cudaMemcpyAsync(&total, d_total, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  NBK_CUDA_TRY(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  NBK_CUDA_TRY(cudaStreamSynchronize(st));
  *h_total = total;
  if (herr) {
    set_error("ball search: device traversal stack exceeded");
    return NBK_ERR_DEVICE;
  }
  if (total > out_capacity || d_out == nullptr) {
    set_error("ball search: output capacity " + std::to_string(out_capacity) + " < " +
              std::to_string(total) + " results");
    return NBK_ERR_INVALID;
  }
  a.offsets = d_offsets;
  a.out = d_out;
  a.outd2 = nullptr;
  k_ball<true><<<blocks, 32 * kWpb, 0, st>>>(a); note_launch();
  NBK_CUDA_TRY(cudaGetLastError());
  return NBK_OK;
}

int run_ball_mark(const TreeView& tv, int target, double fdist2, int imark, int* d_mark,
                  double* d_dist2, const int* d_perm, int target_search, cudaStream_t st) {
  DevAlloc alloc;
  int* d_t;
  int64_t* d_off;
  int* err;
  NBK_TRY(alloc.get((void**)&d_t, sizeof(int)));
  NBK_TRY(alloc.get((void**)&d_off, sizeof(int64_t) * 2));
  NBK_TRY(alloc.get((void**)&err, sizeof(int)));
  NBK_CUDA_TRY(cudaMemcpyAsync(d_t, &target, sizeof(int), cudaMemcpyHostToDevice, st));
  NBK_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), st));
  // count
  BallArgs a{};
  a.tv = tv;
  a.qmode = 0;
  a.qidx = d_t;
  a.nq = 1;
  a.r2 = fdist2;
  a.exclude_self = target_search;
  int* counts;
  NBK_TRY(alloc.get((void**)&counts, sizeof(int)));
  a.counts = counts;
  a.err = err;
  k_ball<false><<<1, 32 * kWpb, 0, st>>>(a); note_launch();
  int hc = 0;
  NBK_CUDA_TRY(cudaMemcpyAsync(&hc, counts, sizeof(int), cudaMemcpyDeviceToHost, st));
  NBK_CUDA_TRY(cudaStreamSynchronize(st));
  int64_t offs[2] = {0, hc};
  NBK_CUDA_TRY(cudaMemcpyAsync(d_off, offs, sizeof(offs), cudaMemcpyHostToDevice, st));
  int* found;
  double* fd2;
  NBK_TRY(alloc.get((void**)&found, sizeof(int) * (hc + 1)));
  NBK_TRY(alloc.get((void**)&fd2, sizeof(double) * (hc + 1)));
  a.offsets = d_off;
  a.out = found;
  a.outd2 = fd2;
  k_ball<true><<<1, 32 * kWpb, 0, st>>>(a); note_launch();
  k_mark<<<std::max(1, std::min(1024, (hc + 255) / 256)), 256, 0, st>>>(
      tv, target, fdist2, imark, found, fd2, d_off + 1, d_perm, d_mark, d_dist2,
      target_search); note_launch();
  NBK_CUDA_TRY(cudaGetLastError());
  NBK_CUDA_TRY(cudaStreamSynchronize(st));
  alloc.release_all_scratch(st);
  return NBK_OK;
}

}  // namespace nbk
