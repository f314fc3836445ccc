// Internal types and device helpers shared by the libnbkdt kernels.
//
// HBM layout of a built tree (all arrays in tree order unless noted):
//   P4      pos[n]    x, y, z, mass as FP64 (32 B, two 16-B vector loads)
//   float4  posf[n]   x, y, z rounded to nearest FP32 (candidate filter)
//   V4 vel[n]    vx, vy, vz, 0 (only when velocities were given)
//   int32   perm[n]   tree index -> input index
//   NodeRec node[]    heap-indexed (root 0, children 2h+1 / 2h+2): FP32 bounding box
//                     rounded outward plus the particle range; 32 B per node
//   NodeX   nodex[]   the same nodes with the exact FP64 bounding box and split plane
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cfloat>
#include <string>

namespace nbk {

constexpr double kMaxValue = 1e32;  // MAXVALUE, src/Math/Precision.h
constexpr int kWarp = 32;

struct __align__(32) P4 {
  double x, y, z, m;
};

struct __align__(32) V4 {
  double x, y, z, w;
};
__host__ __device__ __forceinline__ V4 make_v4(double x, double y, double z, double w) {
  V4 v;
  v.x = x;
  v.y = y;
  v.z = z;
  v.w = w;
  return v;
}

struct __align__(16) NodeRec {
  float lo[3];  // bounding box rounded down (lo) and up (hi): contains every particle
  float hi[3];
  int start;    // first particle (tree index, absolute)
  int count;    // particles in the node; 0 marks an unused heap slot
};

struct NodeX {
  double lo[3], hi[3];  // exact FP64 bounding box (min/max of the node's particles)
  double split_val;     // coordinate of the median particle (the reference's cut_val)
  int split_dim;        // -1 for a leaf
  int pad;
};

// Phase-space (six-dimensional) tree nodes, heap-indexed like the physical ones: the
// split record the searches walk and the exact bounding box, in separate arrays.
struct NodeS {
  double split_val;  // coordinate of the median particle along split_dim (cut_val)
  int split_dim;     // 0-2 position, 3-5 velocity; -1 for a leaf
  int start;         // first particle (tree index, absolute)
  int count;         // particles in the node; 0 marks an unused heap slot
  int pad;
};
struct NodeB6 {
  double lo[6], hi[6];
};
struct __align__(16) NodeF6 {  // the same box in FP32, rounded outward
  float lo[6], hi[6];
};

// Device view of one tree (or of one tree of a batch).
struct TreeView {
  const P4* pos;
  const float4* posf;
  const V4* vel;
  const int* perm;
  const NodeRec* node;
  const NodeX* nodex;
  const NodeS* nodes6;   // phase-space trees only (node/nodex are then unused)
  const NodeB6* nodeb6;  // their exact bounding boxes
  const NodeF6* nodef6;  // and the boxes in FP32
  const float4* velf;    // vx, vy, vz rounded to nearest FP32 (phase-space trees)
  float eps6[6];         // per coordinate: bound on |c - float(c)| (images included)
  int n;       // particles in this tree
  int pstart;  // absolute tree index of its first particle
  int nbase;   // index of its root in the node arrays
  int b;       // bucket size
  int periodic;
  double period[3];
  float eps;  // bound on |x - float(x)| for any coordinate or image coordinate
};

// ---- exact FP64 helpers: explicit round-to-nearest ops are never contracted into FMAs
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }

// DistanceSqd (src/KDTree/DistFunc.h:14-19): ((dx*dx + dy*dy) + dz*dz), each op rounded.
__device__ __forceinline__ double dist2_exact(double ax, double ay, double az, double bx,
                                              double by, double bz) {
  double dx = dsub(ax, bx), dy = dsub(ay, by), dz = dsub(az, bz);
  return dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz));
}

// Order-preserving map from FP64 to uint64 (-0.0 is folded onto +0.0 so that equal
// values compare equal, as the reference's FP comparisons treat them).
__host__ __device__ __forceinline__ uint64_t okey(double v) {
#ifdef __CUDA_ARCH__
  uint64_t u = (uint64_t)__double_as_longlong(v);
#else
  uint64_t u;
  memcpy(&u, &v, 8);
#endif
  if (u == 0x8000000000000000ull) u = 0;  // -0.0 -> +0.0 (an integer test: no FP64 op)
  return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
__host__ __device__ __forceinline__ double okey_inv(uint64_t k) {
  uint64_t u = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double v;
  memcpy(&v, &u, 8);
  return v;
#endif
}

// ---- conservative FP32 bounds (never reject what the exact FP64 test would accept)
// Lower bound of the squared distance from a query known to within +-eps of (qx,qy,qz)
// to the box [lo, hi].
__device__ __forceinline__ float box_d2_lo(float qx, float qy, float qz, float eps,
                                           const NodeRec& r) {
  float gx = fmaxf(0.f, fmaxf(__fsub_rd(r.lo[0], __fadd_ru(qx, eps)),
                              __fsub_rd(__fsub_rd(qx, eps), r.hi[0])));
  float gy = fmaxf(0.f, fmaxf(__fsub_rd(r.lo[1], __fadd_ru(qy, eps)),
                              __fsub_rd(__fsub_rd(qy, eps), r.hi[1])));
  float gz = fmaxf(0.f, fmaxf(__fsub_rd(r.lo[2], __fadd_ru(qz, eps)),
                              __fsub_rd(__fsub_rd(qz, eps), r.hi[2])));
  return __fadd_rd(__fadd_rd(__fmul_rd(gx, gx), __fmul_rd(gy, gy)), __fmul_rd(gz, gz));
}
// Upper bound of the squared distance from the query to the farthest box corner.
__device__ __forceinline__ float box_far_d2_hi(float qx, float qy, float qz, float eps,
                                               const NodeRec& r) {
  float ax = fmaxf(__fsub_ru(__fadd_ru(qx, eps), r.lo[0]), __fsub_ru(r.hi[0], __fsub_rd(qx, eps)));
  float ay = fmaxf(__fsub_ru(__fadd_ru(qy, eps), r.lo[1]), __fsub_ru(r.hi[1], __fsub_rd(qy, eps)));
  float az = fmaxf(__fsub_ru(__fadd_ru(qz, eps), r.lo[2]), __fsub_ru(r.hi[2], __fsub_rd(qz, eps)));
  return __fadd_ru(__fadd_ru(__fmul_ru(ax, ax), __fmul_ru(ay, ay)), __fmul_ru(az, az));
}
// Lower bound of the squared distance between a query and a particle whose FP32
// roundings are (qx..) and (cx..), both within eps of the true coordinates.
__device__ __forceinline__ float pair_d2_lo(float qx, float qy, float qz, float cx, float cy,
                                            float cz, float two_eps) {
  float dx = fmaxf(0.f, __fsub_rd(fabsf(__fsub_rz(qx, cx)), two_eps));
  float dy = fmaxf(0.f, __fsub_rd(fabsf(__fsub_rz(qy, cy)), two_eps));
  float dz = fmaxf(0.f, __fsub_rd(fabsf(__fsub_rz(qz, cz)), two_eps));
  return __fadd_rd(__fadd_rd(__fmul_rd(dx, dx), __fmul_rd(dy, dy)), __fmul_rd(dz, dz));
}
// Upper bound of the squared distance between a query and a particle (the counterpart of
// pair_d2_lo): below thresh_lo(t) it proves the FP64 distance is below t without FP64 work.
__device__ __forceinline__ float pair_d2_hi(float qx, float qy, float qz, float cx, float cy,
                                            float cz, float two_eps) {
  float dx = __fadd_ru(qx >= cx ? __fsub_ru(qx, cx) : __fsub_ru(cx, qx), two_eps);
  float dy = __fadd_ru(qy >= cy ? __fsub_ru(qy, cy) : __fsub_ru(cy, qy), two_eps);
  float dz = __fadd_ru(qz >= cz ? __fsub_ru(qz, cz) : __fsub_ru(cz, qz), two_eps);
  return __fadd_ru(__fadd_ru(__fmul_ru(dx, dx), __fmul_ru(dy, dy)), __fmul_ru(dz, dz));
}
// FP32 threshold above any value whose FP64 counterpart could still be below t.
__device__ __forceinline__ float thresh_hi(double t) {
  float f = __double2float_ru(t);
  return __fmul_ru(f, 1.0f + 1.0f / 1048576.0f);
}

// Bound on |c - float(c)| for the coordinates of a query at (x, y, z) and of its periodic
// images: the tree-wide bound covers the tree's particles and their images, but a query
// point may lie anywhere.
__device__ __forceinline__ float query_eps(const TreeView& tv, double x, double y, double z) {
  double m = fmax(fabs(x), fmax(fabs(y), fabs(z)));
  m += fmax(tv.period[0], fmax(tv.period[1], tv.period[2]));
  return fmaxf(tv.eps, __fmul_ru(__double2float_ru(m), 1.2e-7f));
}

// ---- integer forms for non-negative doubles (squared distances, |dv|). Their bit
// patterns read as signed 64-bit integers order exactly as the values do, so compares
// and the FP32 threshold run on the integer pipe; GB300's FP64 pipe retires only about
// two operations per SM clock and is kept for the arithmetic.
__device__ __forceinline__ long long dkey(double v) { return __double_as_longlong(v); }
// An FP32 value >= v (v >= 0 given by its bits), from the bits alone: the mantissa is
// truncated to 23 bits and bumped by one unit when anything was cut; values below the
// smallest normal FP32 map to it, values beyond the FP32 range to +inf.
__device__ __forceinline__ float f32_above(long long bits) {
  unsigned long long u = (unsigned long long)bits;
  int e = (int)(u >> 52);  // sign bit is 0
  if (e < 1023 - 126) return __uint_as_float(0x00800000u);
  if (e > 1023 + 127) return __uint_as_float(0x7f800000u);
  unsigned f = ((unsigned)(e - 1023 + 127) << 23) | (unsigned)((u >> 29) & 0x7fffffu);
  if (u & 0x1fffffffull) f += 1u;  // a carry into the exponent is still an upper bound
  return __uint_as_float(f);
}
// thresh_hi for a non-negative t given by its bits.
__device__ __forceinline__ float thresh_hi_bits(long long tbits) {
  return __fmul_ru(f32_above(tbits), 1.0f + 1.0f / 1048576.0f);
}
// FP32 threshold below which an FP64 value is certainly below t (for "all inside").
__device__ __forceinline__ float thresh_lo(double t) {
  float f = __double2float_rd(t);
  return __fmul_rd(f, 1.0f - 1.0f / 1048576.0f);
}

// PeriodicReflection1D/2D/ND (src/KDTree/DistFunc.h:326-355): image of x0 across the
// walls named by `mask` (bit k = dimension k); returns sval (a distance; for one
// dimension the signed wall distance, otherwise sqrt of the summed squares).
__device__ __forceinline__ double reflect(const double x0[3], double xp[3], const double p[3],
                                          int mask) {
  // every index is a compile-time constant after unrolling, so the arrays stay in registers
  double s = 0.0, s1 = 0.0;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    xp[k] = x0[k];
    if (!((mask >> k) & 1)) continue;
    if (x0[k] < p[k] / 2.0) {
      xp[k] = dadd(x0[k], p[k]);
      s1 = x0[k];
      s = dadd(s, dmul(x0[k], x0[k]));
    } else {
      xp[k] = dsub(x0[k], p[k]);
      s1 = -xp[k];
      s = dadd(s, dmul(xp[k], xp[k]));
    }
  }
  if (__popc(mask) == 1) return s1;
  return __dsqrt_rn(s);
}
// Dimensions in which the query (FP32 copy q, within eps of the exact position) may lie
// closer than sqrt(r2_hi) to a periodic wall (bit k = dimension k). An image across the
// walls of `mask` can only pass a gate "r2 > sval^2" when (mask & ~near) == 0, because
// sval is at least the distance to each crossed wall; r2_hi is an FP32 value at or above r2.
__device__ __forceinline__ int near_walls(float4 q, const double p[3], float eps, float r2_hi) {
  const float v[3] = {q.x, q.y, q.z};
  int near = 0;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    float pk = __double2float_rd(p[k]);
    float d = fminf(__fsub_rd(v[k], eps), __fsub_rd(__fsub_rd(pk, v[k]), eps));
    if (d <= 0.f || __fmul_rd(d, d) < r2_hi) near |= 1 << k;
  }
  return near;
}
// The same for a gate "t > sval" that compares a distance with t itself (t_hi >= t).
__device__ __forceinline__ int near_walls_lin(float4 q, const double p[3], float eps,
                                              float t_hi) {
  const float v[3] = {q.x, q.y, q.z};
  int near = 0;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    float pk = __double2float_rd(p[k]);
    float d = fminf(__fsub_rd(v[k], eps), __fsub_rd(__fsub_rd(pk, v[k]), eps));
    if (d < t_hi) near |= 1 << k;
  }
  return near;
}
// The order in which the reference searches the images: x, y, z, xy, xz, yz, xyz
// (KDSplitNode.cxx:1126-1147).
__device__ __constant__ static const int kImageMask[8] = {0, 1, 2, 4, 3, 5, 6, 7};

// Wsm (KDCalcSmoothQuantities.cxx:12-15) on the host-built table.
__device__ __forceinline__ double wsm(double r, int i, int size, double delta, const double* x) {
  if (i < size - 1) {
    double xi = x[i], xj = x[i + 1];
    return dadd(xi, __ddiv_rn(dmul(dsub(xj, xi), dsub(r, dmul(delta, (double)i))), delta));
  }
  return x[i];
}
// The same interpolation from the table's device image [T | A | B]: on cell i the line
// through T[i] and T[i+1] is A[i] + B[i] q, one FMA. The cell index is the reference's
// (int)(q * 0.5 * (size - 1)); the result differs from wsm() by a few units in the last
// place (the interpolant is continuous across cells, so a neighbouring cell gives the
// same value up to rounding).
__device__ __forceinline__ double wsm_line(double q, int size, double inv_delta,
                                           const double* img) {
  int i = (int)dmul(q, inv_delta);
  if (i < size - 1) return __fma_rn(img[2 * size + i], q, img[size + i]);
  return img[size - 1];
}

// ---- phase-space trees: depth bound of their per-thread walks, six-vector access
constexpr int kPhDepth = 64;
// v[d] of a six-vector indexed at run time (registers, no local memory)
__device__ __forceinline__ double get6(const double v[6], int d) {
  double r = v[0];
#pragma unroll
  for (int k = 1; k < 6; k++)
    if (d == k) r = v[k];
  return r;
}
__device__ __forceinline__ void set6(double v[6], int d, double x) {
#pragma unroll
  for (int k = 0; k < 6; k++)
    if (d == k) v[k] = x;
}


// Lower bound of sum_j w[j] * (x[j] - y[j])^2 over the points y of the box [lo, hi] of a
// phase-space node, rounded down. Any such sum the reference evaluates for a point of the
// box (each difference, product and sum rounded to nearest, all terms non-negative) is at
// least this bound times (1 - 1e-12), so a subtree whose bound times (1 - 1e-12) is at or
// above a threshold holds no point that tests below it.
__device__ __forceinline__ double box_lb6(const double x[6], const double w[6], const NodeB6& b) {
  double s = 0.0;
#pragma unroll
  for (int j = 0; j < 6; j++) {
    double g = 0.0;
    if (x[j] < b.lo[j]) g = __dsub_rd(b.lo[j], x[j]);
    else if (x[j] > b.hi[j]) g = __dsub_rd(x[j], b.hi[j]);
    s = __dadd_rd(s, __dmul_rd(__dmul_rd(w[j], g), g));
  }
  return s;
}
constexpr double kLbShrink = 1.0 - 1e-12;

// FP32 lower bound of sum_j w[j] * gap_j^2 from a query known to within eps[j] of q[j] to
// the FP32 box [lo, hi] (which contains the exact one); every operation rounds down.
__device__ __forceinline__ float box_lb6f(const float q[6], const float w[6], const float eps[6],
                                          const NodeF6& b) {
  float s = 0.f;
#pragma unroll
  for (int j = 0; j < 6; j++) {
    float g = fmaxf(0.f, fmaxf(__fsub_rd(b.lo[j], __fadd_ru(q[j], eps[j])),
                               __fsub_rd(__fsub_rd(q[j], eps[j]), b.hi[j])));
    s = __fadd_rd(s, __fmul_rd(__fmul_rd(w[j], g), g));
  }
  return s;
}
// FP32 lower bound of sum_j w[j] * (x_j - y_j)^2 for two points whose FP32 roundings q, c
// are each within eps[j] of the exact coordinates.
__device__ __forceinline__ float pair_lb6f(const float q[6], const float c[6], const float w[6],
                                           const float eps[6]) {
  float s = 0.f;
#pragma unroll
  for (int j = 0; j < 6; j++) {
    float g = fmaxf(0.f, __fsub_rd(fabsf(__fsub_rz(q[j], c[j])), __fmul_ru(2.f, eps[j])));
    s = __fadd_rd(s, __fmul_rd(__fmul_rd(w[j], g), g));
  }
  return s;
}

// FP32 upper bound of sum_j w[j] * (x_j - y_j)^2 (w rounded up), the counterpart of
// pair_lb6f: below a threshold under 1 it proves the FP64 sum is below 1.
__device__ __forceinline__ float pair_ub6f(const float q[6], const float c[6], const float w[6],
                                           const float eps[6]) {
  float s = 0.f;
#pragma unroll
  for (int j = 0; j < 6; j++) {
    float g = __fadd_ru(q[j] >= c[j] ? __fsub_ru(q[j], c[j]) : __fsub_ru(c[j], q[j]),
                        __fmul_ru(2.f, eps[j]));
    s = __fadd_ru(s, __fmul_ru(__fmul_ru(w[j], g), g));
  }
  return s;
}

// sqrt(x) for the kernel interpolation, to about 2e-14 relative: the FP32 square root as
// the start and one Newton-Raphson (Heron) step in FP64, q0 + (x - q0^2) / (2 q0), whose
// correction uses an FP32 reciprocal (its error only scales the already small correction).
// Outside the FP32 normal range it falls back to the FP64 square root.
__device__ __forceinline__ double sqrt_newton(double x) {
  const float xf = __double2float_rn(x);
  if (!(xf > 1e-30f && xf < 1e30f)) return __dsqrt_rn(x);
  const float q0f = sqrtf(xf);
  const double q0 = (double)q0f;
  const double half_inv = (double)__fdividef(0.5f, q0f);
  return __fma_rn(__fma_rn(-q0, q0, x), half_inv, q0);
}

// W(q) at q = sqrt(d2) / h with h = sqrt(top) / 2 (ih = 1/h): the farthest neighbour
// (d2 == top) is at q = 2 exactly in the reference's arithmetic, the table's last entry
// (0 for the compact kernels); the product with 1/h could land an ulp below, in the
// previous cell.
__device__ __forceinline__ double w_at_d2(double d2, long long topk, double ih, int size,
                                          double inv_delta, const double* img) {
  if (dkey(d2) == topk) return img[size - 1];
  return wsm_line(dmul(__dsqrt_rn(d2), ih), size, inv_delta, img);
}

// ---- device error word: kernels report bounded-wait and capacity failures here
enum DeviceErr : int {
  kErrNone = 0,
  kErrIterCap = 1,   // a union-find or queue loop exceeded its iteration cap
  kErrCapacity = 2,  // an output or stack capacity was exceeded
  kErrTooFew = 3,    // fewer than k neighbours found
  kErrTarget = 4,    // a target index outside the tree (the query is skipped)
};

}  // namespace nbk

// ---- host-side error state (thread local), set by every entry point
namespace nbk {
void set_error(const std::string& msg);
const char* get_error();
void note_launch();  // counts every kernel launch (reported by nbk_launch_count)

// Phase trace: when enabled (nbk_trace_enable), a Phase records a CUDA event pair around
// its scope on the given stream; the elapsed times are resolved when the trace is read.
struct Phase {
  const char* name;
  cudaStream_t st;
  cudaEvent_t a = nullptr, b = nullptr;
  int dev = 0;
  Phase(const char* n, cudaStream_t s);
  ~Phase();
};
}  // namespace nbk

#define NBK_CUDA_TRY(expr)                                                                  \
  do {                                                                                      \
    cudaError_t _e = (expr);                                                                \
    if (_e != cudaSuccess) {                                                                \
      ::nbk::set_error(std::string("CUDA error: ") + cudaGetErrorString(_e) + " at " +      \
                       __FILE__ + ":" + std::to_string(__LINE__) + " (" #expr ")");         \
      return NBK_ERR_CUDA;                                                                  \
    }                                                                                       \
  } while (0)
