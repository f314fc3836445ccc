// Hand-written adjoint of the SPH density (no reference counterpart: the reference has
// no gradients). The forward pass is CalcDensity (KDCalcSmoothQuantities.cxx:203-305):
//   rho_i = sum_{j in N(i)} w_ij m_j + sum_{l : i in N(l)} w_li m_l,
//   w_ij  = 0.5 Wsm(q_ij) h_i^-3,  q_ij = r_ij / h_i,  h_i = 0.5 r_{i,K(i)}
// where K(i) is the farthest of the k neighbours and Wsm interpolates the kernel table.
// With the neighbour sets and each pair's table cell c frozen at the forward pass, Wsm is
// linear in q inside the cell: T(q) = T[c] + (T[c+1]-T[c]) (q - c delta) / delta, so
//   dw/dr = 0.5 h^-4 T'(q),   dw/dh = -0.5 h^-4 (3 T(q) + q T'(q)),   dh_i/dr_iK = 1/2.
// For L = sum_i w_i log rho_i, with g_i = w_i / rho_i and c_ij = g_i m_j + g_j m_i:
//   dL/dm_a = sum_{i: a in N(i)} g_i w_ia + sum_{j in N(a)} g_j w_aj
//   dL/dx_i += c_ij dw/dr (x_i - x_j)/r_ij   (and the opposite on x_j)
//   dL/dx_i += [sum_j c_ij dw/dh] (1/2) (x_i - x_K)/r_iK   (and the opposite on x_K).
// The backward kernel recomputes every weight from the saved neighbour lists (4 B per
// neighbour) instead of storing weights; one thread per particle, FP64 atomics for the
// contributions that land on other particles. The quotients that do not depend on the
// pair (g_i = w_i / rho_i, the table slopes (T[c+1]-T[c])/delta, 1/h, h^-3) are formed
// once; a pair takes 1/r from an FP32 reciprocal square root and two FP64 Newton steps
// (no division, no FP64 square root). Each pair's table cell is the forward pass's
// (int)(r / h * 0.5 * (kernres - 1)): from the fast r / h, and from the correctly rounded
// square root and division whenever the fast value lies within 1e-10 of a cell edge (its
// own error is below 1e-12 there), so the frozen cells are exactly the forward's.
// The forward (the warp-per-query kNN) writes each neighbour row ascending in distance,
// so the row's last entry is the farthest neighbour, the one that set h_i.
#include <algorithm>

#include "nbk_build.h"

namespace nbk {

namespace {

// 1 / sqrt(x) to about 2e-16 relative: the FP32 reciprocal square root and two Newton
// steps y (3/2 - x/2 y^2) in FP64; outside the FP32 normal range the FP64 path.
__device__ __forceinline__ double rsqrt_newton(double x) {
  const float xf = __double2float_rn(x);
  if (!(xf > 1e-30f && xf < 1e30f)) return 1.0 / __dsqrt_rn(x);
  double y = (double)rsqrtf(xf);
  const double hx = 0.5 * x;
  y = y * __fma_rn(-hx, y * y, 1.5);
  y = y * __fma_rn(-hx, y * y, 1.5);
  return y;
}

// g_i = w_i / rho_i in place of w_i (tree order), and the slope of every table cell
// (0 for the last entry, whose cell the forward pass never interpolates).
__global__ void k_adjoint_prep(double* wg, const double* __restrict__ rho, int64_t n,
                               const double* __restrict__ T, int kr, double* slope) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) wg[i] = wg[i] / rho[i];
  if (i < kr) {
    double delta = 2.0 / (double)(kr - 1);
    slope[i] = i < kr - 1 ? (T[i + 1] - T[i]) / delta : 0.0;
  }
}

__global__ void __launch_bounds__(128) k_adjoint(TreeView tv, int K, const int* __restrict__ nn,
                                                 const double* __restrict__ g,
                                                 const double* __restrict__ T,
                                                 const double* __restrict__ slope, int kr,
                                                 double* gpos, double* gmass) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= tv.n) return;
  int ti = tv.pstart + i;
  const int* row = nn + (size_t)i * K;
  P4 xi = tv.pos[ti];
  double gi = g[ti];
  // farthest neighbour: the one that set h_i in the forward pass (the row's last entry)
  const int kf = row[K - 1];
  P4 xk = tv.pos[kf];
  const double best = dist2_exact(xi.x, xi.y, xi.z, xk.x, xk.y, xk.z);
  const double hh = 0.5 * __dsqrt_rn(best);  // the forward's h_i, for the cell edge cases
  const double irk = rsqrt_newton(best);      // 1 / r_iK
  const double ih = 2.0 * irk;                // 1 / h_i
  const double norm = ih * ih * ih;
  const double delta = 2.0 / (double)(kr - 1);
  const double hk = 0.5 * (double)(kr - 1);
  const double nh = -0.5 * norm * ih;  // dw/dh = nh (3 T + q T'), dw/dr = -nh T'
  double A = 0.0, gmi = 0.0, gx = 0.0, gy = 0.0, gz = 0.0;
  for (int s = 0; s < K; s++) {
    int j = row[s];
    P4 xj = tv.pos[j];
    double dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
    double d2 = dist2_exact(xi.x, xi.y, xi.z, xj.x, xj.y, xj.z);
    double ir = rsqrt_newton(d2);  // 1 / r_ij (the target search excluded r = 0)
    double q = d2 * ir * ih;
    double u = q * hk;
    int c = (int)u;
    double fr = u - (double)c;
    if (fr < 1e-10 || fr > 1.0 - 1e-10) c = (int)(__dsqrt_rn(d2) / hh * 0.5 * (double)(kr - 1));
    double Tp = slope[c < kr - 1 ? c : kr - 1];
    double Tq = c < kr - 1 ? __fma_rn(Tp, q - delta * (double)c, T[c]) : T[kr - 1];
    double w = 0.5 * Tq * norm;
    double gj = g[j];
    double cij = gi * xj.m + gj * xi.m;
    atomicAdd(&gmass[j], gi * w);
    gmi += gj * w;
    double dwdr = -nh * Tp;
    double dwdh = nh * (3.0 * Tq + q * Tp);
    A += cij * dwdh;
    double coef = cij * dwdr * ir;
    gx += coef * dx;
    gy += coef * dy;
    gz += coef * dz;
    atomicAdd(&gpos[3 * (size_t)j + 0], -coef * dx);
    atomicAdd(&gpos[3 * (size_t)j + 1], -coef * dy);
    atomicAdd(&gpos[3 * (size_t)j + 2], -coef * dz);
  }
  double ch = A * 0.5 * irk;
  double kx = ch * (xi.x - xk.x), ky = ch * (xi.y - xk.y), kz = ch * (xi.z - xk.z);
  atomicAdd(&gpos[3 * (size_t)kf + 0], -kx);
  atomicAdd(&gpos[3 * (size_t)kf + 1], -ky);
  atomicAdd(&gpos[3 * (size_t)kf + 2], -kz);
  atomicAdd(&gpos[3 * (size_t)ti + 0], gx + kx);
  atomicAdd(&gpos[3 * (size_t)ti + 1], gy + ky);
  atomicAdd(&gpos[3 * (size_t)ti + 2], gz + kz);
  atomicAdd(&gmass[ti], gmi);
}

}  // namespace

int run_density_adjoint(const TreeView& tv, int k, const int* d_nn, double* d_w_tree,
                        const double* d_rho_tree, const double* kernel, int kernres,
                        double* d_slope, double* d_gpos_tree, double* d_gmass_tree,
                        cudaStream_t st) {
  if (tv.n == 0) return NBK_OK;
  NBK_CUDA_TRY(cudaMemsetAsync(d_gpos_tree, 0, sizeof(double) * 3 * tv.n, st));
  NBK_CUDA_TRY(cudaMemsetAsync(d_gmass_tree, 0, sizeof(double) * tv.n, st));
  Phase ph("adjoint_backward", st);
  int64_t m = std::max<int64_t>(tv.n, kernres);
  k_adjoint_prep<<<(unsigned)((m + 255) / 256), 256, 0, st>>>(d_w_tree, d_rho_tree, tv.n, kernel,
                                                               kernres, d_slope);
  note_launch();
  k_adjoint<<<(tv.n + 127) / 128, 128, 0, st>>>(tv, k, d_nn, d_w_tree, kernel, d_slope, kernres,
                                                d_gpos_tree, d_gmass_tree);
  note_launch();
  NBK_CUDA_TRY(cudaGetLastError());
  return NBK_OK;
}

}  // namespace nbk
