// Device capability probe: sustained FP64 FMA throughput of this GPU, the denominator of
// the FP64 roofline the kNN-density kernels are judged against (the driver-measured
// peaks cover HBM bandwidth and bf16 tensor throughput only).
#include "nbk_build.h"

namespace {

// 8 independent FMA chains per thread so the FP64 pipe, not latency, limits the rate.
__global__ void k_fp64_fma(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-9, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4,
         x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; i++) {
    x0 = fma(x0, a, b);
    x1 = fma(x1, a, b);
    x2 = fma(x2, a, b);
    x3 = fma(x3, a, b);
    x4 = fma(x4, a, b);
    x5 = fma(x5, a, b);
    x6 = fma(x6, a, b);
    x7 = fma(x7, a, b);
  }
  double s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == 12345.678) out[threadIdx.x] = s;  // keeps the chains alive
}

}  // namespace

using namespace nbk;

extern "C" int nbk_probe_fp64(double* gflops) {
  if (!gflops) {
    set_error("nbk_probe_fp64: null output");
    return NBK_ERR_INVALID;
  }
  int dev = 0, nsm = 0;
  NBK_CUDA_TRY(cudaGetDevice(&dev));
  NBK_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  double* out = nullptr;
  NBK_TRY(dev_malloc((void**)&out, sizeof(double) * 1024, nullptr));
  const int threads = 512, blocks = nsm * 4, iters = 1 << 14;
  cudaEvent_t a, b;
  NBK_CUDA_TRY(cudaEventCreate(&a));
  NBK_CUDA_TRY(cudaEventCreate(&b));
  k_fp64_fma<<<blocks, threads>>>(out, 256, 1.0000001, 1e-7);  // warm
  note_launch();
  NBK_CUDA_TRY(cudaEventRecord(a));
  k_fp64_fma<<<blocks, threads>>>(out, iters, 1.0000001, 1e-7);
  note_launch();
  NBK_CUDA_TRY(cudaEventRecord(b));
  NBK_CUDA_TRY(cudaEventSynchronize(b));
  float ms = 0;
  NBK_CUDA_TRY(cudaEventElapsedTime(&ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  dev_free(out, nullptr);
  double flops = 2.0 * 8.0 * (double)iters * threads * blocks;
  *gflops = flops / (ms * 1e-3) / 1e9;
  return NBK_OK;
}
