// SPH smoothing over the Nsmooth nearest neighbours (KDCalcSmoothQuantities.cxx):
//   CalcSmoothVel, CalcSmoothVelDisp, CalcSmoothVelSkew, CalcSmoothVelKurtosis (:480-766),
//   symmetric sums over every particle's neighbours, scattered to both ends of each pair;
//   CalcVelDensityWithPhysDensity[Particle] (:393-478, :922-990);
//   CalcSmoothVel/CalcSmoothVelDisp {Particle,Position} (:992-1091, :1209-1306) and
//   CalcSmoothLocalMean/CalcSmoothLocalDisp {Particle,Position} (:1539-1700), one-sided.
// Each is an epilogue of the warp search of knn_core.cuh: the lane's heap holds its
// neighbours when the search returns, so no neighbour list is stored. Per-particle inputs
// (densities, mean velocities, dispersions, weights) and the every-particle outputs are in
// input order and addressed through the tree's permutation; the scattered sums use FP64
// atomics, so their summation order (not their terms) differs from the reference's.
#include "knn_core.cuh"

namespace nbk {

namespace {

// 1 / x^1.5 as the reference's pow(x, 1.5) in the denominator of the skewness.
__device__ __forceinline__ double inv_pow15(double x) { return 1.0 / dmul(x, __dsqrt_rn(x)); }

template <int KMAX, int SM>
__device__ void smooth_warp(const SmoothArgs& s, const TreeView& tv, WarpSmem<KMAX>& w, int lane,
                            bool valid, int qi, int self, const double x0[3], int K) {
  const KnnArgs& a = s.k;
  double top = knn_search<KMAX>(a, tv, w, lane, valid, self, x0, K);
  if (!valid) return;
  for (int q = 0; q < K; q++)
    if (w.hi[q][lane] < 0) {
      atomicExch(a.err, kErrTooFew);
      return;
    }
  const int kr = a.kernres;
  const double inv_delta = 0.5 * (double)(kr - 1);
  const double* T = a.kernel;

  if (SM == kSmVelPhys) {
    // |dv| of the Nsearch neighbours, the Nsmooth smallest kept (as CalcVelDensity); the
    // physical h is half the largest *squared* distance, as the reference computes it
    // (:428); a table index past the end gives the table's last entry (the reference
    // reads past its table there).
    V4 vi = tv.vel[self];
    P4 pi = tv.pos[self];
    for (int q = 0; q < K; q++) {
      V4 vj = tv.vel[w.hi[q][lane]];
      w.hd[q][lane] = __dsqrt_rn(dist2_exact(vi.x, vi.y, vi.z, vj.x, vj.y, vj.z));
    }
    int ns = min(s.nsmooth, K);
    if (ns < K) {
      for (int q = ns / 2 - 1; q >= 0; q--) {
        double d = w.hd[q][lane];
        int j = w.hi[q][lane];
        heap_sift<KMAX>(w, lane, ns, q, d, j);
      }
      for (int q = ns; q < K; q++) {
        double d = w.hd[q][lane];
        if (dkey(d) < dkey(w.hd[0][lane])) heap_sift<KMAX>(w, lane, ns, 0, d, w.hi[q][lane]);
      }
    }
    long long vmaxk = 0;
    for (int q = 0; q < ns; q++) vmaxk = max(vmaxk, dkey(w.hd[q][lane]));
    double vih = 1.0 / (0.5 * __longlong_as_double(vmaxk));
    double vnorm = dmul(dmul(vih, vih), vih);
    double ih = 1.0 / (0.5 * top);
    double norm = dmul(dmul(ih, ih), ih);
    double ri = s.rho[tv.perm[self]];
    double acc = 0.0;
    for (int q = 0; q < ns; q++) {
      int j = w.hi[q][lane];
      P4 pj = tv.pos[j];
      double rij = __dsqrt_rn(dist2_exact(pi.x, pi.y, pi.z, pj.x, pj.y, pj.z));
      const double vd = w.hd[q][lane];  // the largest |dv| is at q = 2 exactly
      double vw = dmul(dkey(vd) == vmaxk ? T[kr - 1] : wsm_line(dmul(vd, vih), kr, inv_delta, T),
                       vnorm);
      double wij = dmul(wsm_line(dmul(rij, ih), kr, inv_delta, T), norm);
      acc = dadd(acc, dmul(vw, dmul(wij / ri, pi.m)));
    }
    if (a.qmode == 0) s.out[tv.perm[self]] = acc;
    else s.out[qi] = acc;
    return;
  }

  // the SPH weights of the Nsmooth nearest: h = half the largest distance
  double ih = 1.0 / (0.5 * __dsqrt_rn(top));
  const long long topk = dkey(top);
  double norm = dmul(dmul(ih, ih), ih);
  constexpr bool kSym = SM == kSmVel || SM == kSmVelDisp || SM == kSmVelSkew || SM == kSmVelKurt;
  double wnorm = kSym ? 0.5 * norm : norm;  // the symmetric forms carry the 1/2

  if (kSym) {
    const int id = tv.perm[self];
    P4 pi = tv.pos[self];
    V4 vi = tv.vel[self];
    const double vi3[3] = {vi.x, vi.y, vi.z};
    const double tb0 = pi.m / s.rho[id];  // the target's weight factor, times W_ij
    double svi[3] = {0, 0, 0}, ddi[3] = {1, 1, 1};
    if (SM != kSmVel)
      for (int k = 0; k < 3; k++) svi[k] = s.smvel[3 * (size_t)id + k];
    if (SM == kSmVelSkew || SM == kSmVelKurt)
      for (int k = 0; k < 3; k++) ddi[k] = s.disp[9 * (size_t)id + 4 * k];
    double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int q = 0; q < K; q++) {
      int j = w.hi[q][lane];
      int jd = tv.perm[j];
      double wij = dmul(w_at_d2(w.hd[q][lane], topk, ih, kr, inv_delta, T), wnorm);
      P4 pj = tv.pos[j];
      V4 vj = tv.vel[j];
      const double vj3[3] = {vj.x, vj.y, vj.z};
      double ta = dmul(wij / s.rho[jd], pj.m);  // Wij / rho_j * m_j, summed into the target
      double tb = dmul(wij, tb0) ;              // Wij / rho_i * m_i, summed into neighbour j
      if (SM == kSmVel) {
        for (int k = 0; k < 3; k++) {
          acc[k] = dadd(acc[k], dmul(ta, vj3[k]));
          atomicAdd(&s.out[3 * (size_t)jd + k], dmul(tb, vi3[k]));
        }
      } else if (SM == kSmVelDisp) {
        double svj[3];
        for (int k = 0; k < 3; k++) svj[k] = s.smvel[3 * (size_t)jd + k];
        for (int k = 0; k < 3; k++)
          for (int l = 0; l < 3; l++) {
            acc[3 * k + l] = dadd(acc[3 * k + l],
                                  dmul(dmul(ta, dsub(vj3[k], svi[k])), dsub(vj3[l], svi[l])));
            atomicAdd(&s.out[9 * (size_t)jd + 3 * k + l],
                      dmul(dmul(tb, dsub(vi3[k], svj[k])), dsub(vi3[l], svj[l])));
          }
      } else {
        for (int k = 0; k < 3; k++) {
          double dv = dsub(vj3[k], svi[k]);
          double du = dsub(vi3[k], s.smvel[3 * (size_t)jd + k]);
          double djk = s.disp[9 * (size_t)jd + 4 * k];
          if (SM == kSmVelSkew) {
            acc[k] = dadd(acc[k], dmul(dmul(dmul(ta, dv), dv), dv) * inv_pow15(ddi[k]));
            atomicAdd(&s.out[3 * (size_t)jd + k],
                      dmul(dmul(dmul(tb, du), du), du) * inv_pow15(djk));
          } else {
            // the reference subtracts 3 in every neighbour's term
            acc[k] = dadd(acc[k], dsub(dmul(dmul(dmul(dmul(ta, dv), dv), dv), dv) /
                                           dmul(ddi[k], ddi[k]), 3.0));
            atomicAdd(&s.out[3 * (size_t)jd + k],
                      dsub(dmul(dmul(dmul(dmul(tb, du), du), du), du) / dmul(djk, djk), 3.0));
          }
        }
      }
    }
    const int width = SM == kSmVelDisp ? 9 : 3;
    for (int k = 0; k < width; k++) atomicAdd(&s.out[(size_t)width * id + k], acc[k]);
    return;
  }

  // one-sided forms: the query's own sums
  double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  double sv[3] = {0, 0, 0};
  if (SM == kSmVelDispOne)
    for (int k = 0; k < 3; k++) sv[k] = s.smvel[3 * (size_t)qi + k];
  const double mean = SM == kSmDispOne ? s.mean[qi] : 0.0;
  for (int q = 0; q < K; q++) {
    int j = w.hi[q][lane];
    int jd = tv.perm[j];
    double wij = dmul(w_at_d2(w.hd[q][lane], topk, ih, kr, inv_delta, T), wnorm);
    double ta = dmul(wij / s.rho[jd], tv.pos[j].m);
    if (SM == kSmVelOne || SM == kSmVelDispOne) {
      V4 vj = tv.vel[j];
      const double vj3[3] = {vj.x, vj.y, vj.z};
      if (SM == kSmVelOne) {
        for (int k = 0; k < 3; k++) acc[k] = dadd(acc[k], dmul(ta, vj3[k]));
      } else {
        for (int k = 0; k < 3; k++)
          for (int l = 0; l < 3; l++)
            acc[3 * k + l] = dadd(acc[3 * k + l],
                                  dmul(dmul(ta, dsub(vj3[k], sv[k])), dsub(vj3[l], sv[l])));
      }
    } else if (SM == kSmMeanOne) {
      acc[0] = dadd(acc[0], dmul(ta, s.weight[jd]));
    } else {
      double dl = dsub(s.weight[jd], mean);
      acc[0] = dadd(acc[0], dmul(dmul(ta, dl), dl));
    }
  }
  const int width = SM == kSmVelDispOne ? 9 : (SM == kSmVelOne ? 3 : 1);
  for (int k = 0; k < width; k++) s.out[(size_t)width * qi + k] = acc[k];
}

template <int KMAX, int SM>
__global__ void __launch_bounds__(32 * warps_per_block<KMAX>()) k_smooth(SmoothArgs s) {
  constexpr int WPB = warps_per_block<KMAX>();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  WarpSmem<KMAX>* ws = reinterpret_cast<WarpSmem<KMAX>*>(smem_raw);
  const KnnArgs& a = s.k;
  int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int gw = blockIdx.x * WPB + warp;
  int qi = gw * 32 + lane;
  if (gw * 32 >= a.nq) return;
  const TreeView& tv = a.tv;
  bool valid = qi < a.nq;
  int self = -1;
  double x0[3] = {0, 0, 0};
  if (valid) {
    if (a.qmode == 0) self = a.q0 + qi;
    else if (a.qmode == 2) self = a.qidx[qi];
    if (a.qmode == 2 && (self < 0 || self >= tv.n)) {
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
  smooth_warp<KMAX, SM>(s, tv, ws[warp], lane, valid, qi, self, x0, a.kheap);
}

template <int KMAX, int SM>
int launch_st(const SmoothArgs& s, cudaStream_t st) {
  constexpr int WPB = warps_per_block<KMAX>();
  size_t sm = sizeof(WarpSmem<KMAX>) * WPB;
  NBK_TRY(ensure_dyn_smem((const void*)k_smooth<KMAX, SM>, (int)sm));
  int blocks = ((s.k.nq + 31) / 32 + WPB - 1) / WPB;
  if (blocks == 0) return NBK_OK;
  Phase ph("smooth", st);
  k_smooth<KMAX, SM><<<blocks, 32 * WPB, sm, st>>>(s); note_launch();
  NBK_CUDA_TRY(cudaGetLastError());
  return NBK_OK;
}

template <int SM>
int launch_s(const SmoothArgs& s, cudaStream_t st) {
  int k = s.k.kheap;
  if (k <= 16) return launch_st<16, SM>(s, st);
  if (k <= 33) return launch_st<33, SM>(s, st);
  if (k <= 65) return launch_st<65, SM>(s, st);
  if (k <= 128) return launch_st<128, SM>(s, st);
  set_error("smoothing over more than 128 neighbours is not supported");
  return NBK_ERR_UNSUPPORTED;
}

}  // namespace

int launch_smooth(const SmoothArgs& s, int which, cudaStream_t st) {
  switch (which) {
    case kSmVel: return launch_s<kSmVel>(s, st);
    case kSmVelDisp: return launch_s<kSmVelDisp>(s, st);
    case kSmVelSkew: return launch_s<kSmVelSkew>(s, st);
    case kSmVelKurt: return launch_s<kSmVelKurt>(s, st);
    case kSmVelPhys: return launch_s<kSmVelPhys>(s, st);
    case kSmVelOne: return launch_s<kSmVelOne>(s, st);
    case kSmVelDispOne: return launch_s<kSmVelDispOne>(s, st);
    case kSmMeanOne: return launch_s<kSmMeanOne>(s, st);
    case kSmDispOne: return launch_s<kSmDispOne>(s, st);
  }
  set_error("unknown smoothing quantity");
  return NBK_ERR_INVALID;
}

}  // namespace nbk
