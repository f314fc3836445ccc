// nbk_density_noalloc: the SPH density (CalcDensity) for callers that cannot allocate
// device memory while they run.
//
// Who needs it: simulation codes and in-situ halo finders that reserve the GPU's memory
// for their own pool when they start and allow no other allocation afterwards (a
// cudaMalloc would fail, or take memory their pool counts on), and callers for whom an
// allocation inside a time step is a cost they cannot take (cudaMalloc and cudaFree can
// synchronise the device). nbk_density allocates a tree-order scratch array on every
// call; this variant keeps that scratch in a file-scope static __device__ array instead,
// so a call allocates nothing: the caller passes the tree (built earlier, when
// allocation was allowed) and a device output buffer it owns.
//
// Limits and sharing:
//  - the scratch holds kNoAllocMaxParticles doubles (4,194,304 particles, 32 MiB); every
//    GPU that loads this module keeps it until the process exits. Larger trees are
//    rejected with NBK_ERR_INVALID.
//  - all calls share the one array. Each call zeroes the part it uses before its kernel
//    runs; calls whose work overlaps on the GPU (different streams, or several host
//    threads) race on it and must be serialised by the caller.
//  - the call runs on the device the tree was created on (made current for the call and
//    restored afterwards), and returns once its GPU work has finished: it reads the
//    kernel's error word, as nbk_density does for host-pointer trees.
//  - set-up: the first call on each device looks up the array's device address with
//    cudaGetSymbolAddress (with that device current) and caches it.
#include <mutex>

#include "nbk_build.h"

namespace nbk {
int density_into_scratch(nbk_tree* t, int k, double* scratch, double* rho_dev);
int64_t tree_size(const nbk_tree* t);
int tree_device(const nbk_tree* t);
}  // namespace nbk

using namespace nbk;

namespace {

constexpr int64_t kNoAllocMaxParticles = int64_t(1) << 22;
static __device__ __align__(256) double g_density_scratch[kNoAllocMaxParticles];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
double* g_scratch_of_device[kMaxDevices] = {};

// Device address of the scratch array on device `dev`, which must be current (looked up
// once per device).
int scratch_for_device(int dev, double** out) {
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("nbk_density_noalloc: device ordinal beyond the supported 64");
    return NBK_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_scratch_of_device[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_density_scratch);
    if (e != cudaSuccess || p == nullptr) {
      set_error(std::string("nbk_density_noalloc: cudaGetSymbolAddress failed: ") +
                cudaGetErrorString(e));
      return NBK_ERR_CUDA;
    }
    g_scratch_of_device[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_of_device[dev];
  return NBK_OK;
}

// Makes `dev` current for the guard's lifetime and restores the caller's device.
struct DeviceGuard {
  int prev = -1;
  int enter(int dev) {
    NBK_CUDA_TRY(cudaGetDevice(&prev));
    if (prev != dev) NBK_CUDA_TRY(cudaSetDevice(dev));
    return NBK_OK;
  }
  ~DeviceGuard() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
};

}  // namespace

extern "C" int nbk_density_noalloc(nbk_tree* tree, int k, double* rho_dev) {
  try {
    if (!tree || !rho_dev) {
      set_error("nbk_density_noalloc: null argument");
      return NBK_ERR_INVALID;
    }
    int64_t n = tree_size(tree);
    if (n > kNoAllocMaxParticles) {
      set_error("nbk_density_noalloc: the tree has " + std::to_string(n) +
                " particles; the static scratch holds at most " +
                std::to_string(kNoAllocMaxParticles));
      return NBK_ERR_INVALID;
    }
    int dev = tree_device(tree);
    DeviceGuard g;
    NBK_TRY(g.enter(dev));
    double* scratch = nullptr;
    NBK_TRY(scratch_for_device(dev, &scratch));
    return density_into_scratch(tree, k, scratch, rho_dev);
  } catch (const std::exception& e) {
    set_error(std::string("nbk_density_noalloc: exception: ") + e.what());
    return NBK_ERR_INVALID;
  }
}
