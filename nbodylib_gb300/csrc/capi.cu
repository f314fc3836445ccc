// extern "C" entry points of libnbkdt (declared in include/nbkdt.h).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <tuple>

#include "nbk_build.h"

namespace nbk {

namespace {
thread_local std::string g_err;

bool g_pool_ready = false;
void ensure_pool() {
  if (g_pool_ready) return;
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess) {
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t thr = ~0ull;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
  }
  g_pool_ready = true;
}

// The smoothing kernels of src/KDTree/SmoothingKernels.h:32-56 (evaluated on the host
// once, to build the table the GPU interpolates).
double w_sph(double r, double h) {
  double rh = r / h;
  if (rh <= 1.0) return (1.0 - 0.75 * (2.0 - rh) * (rh * rh));
  else if (rh > 1.0 && rh <= 2.0) return 0.25 * (2.0 - rh) * (2.0 - rh) * (2.0 - rh);
  return 0;
}
double w_th(double r, double h) { return (r / h * 0.5 <= 1.0); }
double w_gauss(double r, double h) {
  double rh = r / h * 2.0;
  return std::exp(-0.5 * std::pow(rh, 2.0));
}
double w_epan(double r, double h) {
  double rh = r / h * 0.5;
  return rh <= 1.0 ? (1.0 - rh * rh) : 0.;
}

}  // namespace

// KDTree::KernelConstruction (KDTree.cxx:1144-1183) for ND dimensions; Gamma(ND/2+1)
// from std::tgamma.
void kernel_table(int kerntype, int kernres, int nd, std::vector<double>& T, double& norm) {
  double kn = 1.0 / nd * std::pow(M_1_PI, nd / 2.) * std::tgamma(nd / 2. + 1.);
  double (*f)(double, double) = w_sph;
  if (kerntype == NBK_KGAUSS) {
    f = w_gauss;
    kn *= std::pow(0.5 * M_1_PI, nd / 2.);
  } else if (kerntype == NBK_KEPAN) {
    f = w_epan;
    kn *= nd * (nd + 2.) * std::pow(0.5, nd + 1.);
  } else if (kerntype == NBK_KTH) {
    f = w_th;
  } else {
    f = w_sph;
    kn *= nd * (nd + 1.) * (nd + 2.) * (nd + 3.) / (6 * (std::pow(2., nd + 1) - 1.));
  }
  norm = kn;
  double delta = 2.0 / (double)(kernres - 1);
  T.resize(kernres);
  for (int i = 0; i < kernres; i++) T[i] = kn * f(i * delta, 1.0);
}

// Device kernel tables are shared by every tree of one (device, kernel, resolution,
// dimension count): built
// and uploaded once per process, never freed (a few tens of KB each).
struct KernelEntry {
  std::vector<double> table;
  double norm = 0;
  double* d_img = nullptr;
};
static int cached_kernel(int kerntype, int kernres, int nd, const KernelEntry** out) {
  static std::mutex mu;
  static std::map<std::tuple<int, int, int, int>, KernelEntry> cache;
  int dev = 0;
  NBK_CUDA_TRY(cudaGetDevice(&dev));
  auto key = std::make_tuple(dev, kerntype, kernres, nd);
  // the entries never move or go away, so a thread can keep its last one
  static thread_local std::tuple<int, int, int, int> last_key{-1, -1, -1, -1};
  static thread_local const KernelEntry* last = nullptr;
  if (last && last_key == key) {
    *out = last;
    return NBK_OK;
  }
  std::lock_guard<std::mutex> lock(mu);
  auto it = cache.find(key);
  if (it == cache.end()) {
    KernelEntry e;
    kernel_table(kerntype, kernres, nd, e.table, e.norm);
    std::vector<double> img;
    kernel_device_image(e.table, img);
    NBK_CUDA_TRY(cudaMalloc((void**)&e.d_img, sizeof(double) * img.size()));
    NBK_CUDA_TRY(cudaMemcpy(e.d_img, img.data(), sizeof(double) * img.size(),
                            cudaMemcpyHostToDevice));
    it = cache.emplace(key, std::move(e)).first;
  }
  *out = &it->second;
  last_key = key;
  last = &it->second;
  return NBK_OK;
}

// Device image of a kernel table: [T | A | B] with W(q) = A[i] + B[i] q on cell i, the
// same line through T[i] and T[i+1] as the reference's interpolation (one FMA per
// neighbour instead of a division and five more operations).
void kernel_device_image(const std::vector<double>& T, std::vector<double>& img) {
  int kr = (int)T.size();
  double delta = 2.0 / (double)(kr - 1), inv_delta = 0.5 * (double)(kr - 1);
  img.assign(3 * (size_t)kr, 0.0);
  for (int i = 0; i < kr; i++) {
    img[i] = T[i];
    double slope = i + 1 < kr ? (T[i + 1] - T[i]) * inv_delta : 0.0;
    img[kr + i] = T[i] - slope * (delta * i);
    img[2 * kr + i] = slope;
  }
}

namespace {

__global__ void k_scatter_d(const double* tv, const int* perm, double* out, int64_t n,
                            int stride) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int64_t o = perm[i];
  for (int s = 0; s < stride; s++) out[o * stride + s] = tv[i * stride + s];
}
__global__ void k_gather_d(const double* in, const int* perm, double* out, int64_t n) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = in[perm[i]];
}
__global__ void k_scatter_i(const int* tv, const int* perm, int* out, int64_t n) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[perm[i]] = tv[i];
}
}  // namespace

void set_error(const std::string& msg) { g_err = msg; }
const char* get_error() { return g_err.c_str(); }

static std::atomic<long long> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

namespace {
struct PendingPhase {
  std::string name;
  cudaEvent_t a, b;
  int dev;
};
struct TraceAcc {
  long long count = 0;
  double ms = 0;
};
std::mutex g_trace_mu;
std::atomic<bool> g_trace_on{false};
std::vector<PendingPhase> g_pending;
std::map<std::string, TraceAcc> g_trace;
// resolved events are kept for reuse (creating events costs host time inside the very
// call sequence being traced); keyed by device, as events belong to one
std::map<int, std::vector<cudaEvent_t>> g_event_pool;

cudaEvent_t pooled_event(int dev) {
  {
    std::lock_guard<std::mutex> lk(g_trace_mu);
    auto& v = g_event_pool[dev];
    if (!v.empty()) {
      cudaEvent_t e = v.back();
      v.pop_back();
      return e;
    }
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

void resolve_pending() {
  std::lock_guard<std::mutex> lk(g_trace_mu);
  for (auto& p : g_pending) {
    cudaEventSynchronize(p.b);
    float ms = 0;
    cudaEventElapsedTime(&ms, p.a, p.b);
    auto& acc = g_trace[p.name];
    acc.count++;
    acc.ms += ms;
    g_event_pool[p.dev].push_back(p.a);
    g_event_pool[p.dev].push_back(p.b);
  }
  g_pending.clear();
}
}  // namespace

Phase::Phase(const char* n, cudaStream_t s) : name(n), st(s) {
  if (!g_trace_on.load(std::memory_order_relaxed)) return;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return;
  cudaGetDevice(&dev);
  a = pooled_event(dev);
  b = pooled_event(dev);
  cudaEventRecord(a, st);
}
Phase::~Phase() {
  if (!a) return;
  cudaEventRecord(b, st);
  std::lock_guard<std::mutex> lk(g_trace_mu);
  g_pending.push_back({name, a, b, dev});
}

// Live device allocations made through dev_malloc (freed through dev_free), and the
// test hook that makes one chosen future allocation fail (-1: disarmed).
static std::atomic<long long> g_live_allocs{0};
static std::atomic<long long> g_fail_countdown{-1};

int dev_malloc(void** p, size_t bytes, cudaStream_t st) {
  ensure_pool();
  long long c = g_fail_countdown.load(std::memory_order_relaxed);
  while (c >= 0 && !g_fail_countdown.compare_exchange_weak(c, c - 1)) {
  }
  if (c == 0) {
    set_error(std::string("device allocation of ") + std::to_string(bytes) +
              " bytes failed: injected failure (nbk_debug_fail_allocation)");
    *p = nullptr;
    return NBK_ERR_NOMEM;
  }
  cudaError_t e = cudaMallocAsync(p, std::max<size_t>(bytes, 16), st);
  if (e != cudaSuccess) {
    set_error(std::string("device allocation of ") + std::to_string(bytes) +
              " bytes failed: " + cudaGetErrorString(e));
    *p = nullptr;
    return NBK_ERR_NOMEM;
  }
  g_live_allocs.fetch_add(1, std::memory_order_relaxed);
  return NBK_OK;
}
void dev_free(void* p, cudaStream_t st) {
  if (!p) return;
  cudaFreeAsync(p, st);
  g_live_allocs.fetch_sub(1, std::memory_order_relaxed);
}

int ensure_dyn_smem(const void* func, int bytes) {
  static std::mutex mu;
  static std::map<std::pair<int, const void*>, int> done;
  int dev = 0;
  NBK_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  auto key = std::make_pair(dev, func);
  auto it = done.find(key);
  if (it != done.end() && it->second >= bytes) return NBK_OK;
  NBK_CUDA_TRY(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  done[key] = bytes;
  return NBK_OK;
}
size_t block_bytes(const std::vector<DevPart>& parts) {
  size_t total = 0;
  for (auto& q : parts) total += (std::max<size_t>(q.bytes, 16) + 255) & ~size_t(255);
  return total;
}
void carve_block(void* base, const std::vector<DevPart>& parts) {
  size_t off = 0;
  for (auto& q : parts) {
    *q.p = static_cast<char*>(base) + off;
    off += (std::max<size_t>(q.bytes, 16) + 255) & ~size_t(255);
  }
}
// Per-thread scratch blocks for calls that end with a synchronisation of their stream
// (the tree build; FOF), so the block is idle again when the call returns and the next
// call on this thread can reuse it instead of going to the allocator. Blocks above
// kThreadScratchMax are not kept. A kept block stays allocated until the thread exits.
constexpr size_t kThreadScratchMax = size_t(256) << 20;
struct ThreadScratch {
  void* p = nullptr;
  size_t cap = 0;
  int dev = -1;
  ~ThreadScratch() {
    if (p) {
      cudaFree(p);
      g_live_allocs.fetch_sub(1, std::memory_order_relaxed);
    }
  }
};
int thread_scratch_block(int slot, const std::vector<DevPart>& parts, cudaStream_t st,
                         DevAlloc& fallback) {
  static thread_local ThreadScratch keep[3];
  size_t bytes = block_bytes(parts);
  int dev = 0;
  NBK_CUDA_TRY(cudaGetDevice(&dev));
  if (slot < 0 || slot > 2 || bytes > kThreadScratchMax) return fallback.get_block(parts);
  ThreadScratch& k = keep[slot];
  if (!k.p || k.cap < bytes || k.dev != dev) {
    if (k.p && k.dev == dev) {
      dev_free(k.p, st);
    } else if (k.p) {  // another device's block: cudaFree finds its device itself
      cudaFree(k.p);
      g_live_allocs.fetch_sub(1, std::memory_order_relaxed);
    }
    k.p = nullptr;
    k.cap = 0;
    NBK_TRY(dev_malloc(&k.p, bytes, st));
    k.cap = bytes;
    k.dev = dev;
  }
  carve_block(k.p, parts);
  return NBK_OK;
}

int DevAlloc::get_block(const std::vector<DevPart>& parts) {
  void* base = nullptr;
  NBK_TRY(get(&base, block_bytes(parts)));
  carve_block(base, parts);
  return NBK_OK;
}
int DevAlloc::get(void** p, size_t bytes) {
  NBK_TRY(dev_malloc(p, bytes, st));
  scratch.push_back(*p);
  return NBK_OK;
}
int DevAlloc::upload(void* dst, const void* src, size_t bytes, cudaStream_t s) {
  NBK_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s));
  return NBK_OK;
}
void DevAlloc::release_all_scratch(cudaStream_t s) {
  for (void* p : scratch) dev_free(p, s);
  scratch.clear();
}
DevAlloc::~DevAlloc() { release_all_scratch(st); }

int scatter_to_input_order(const double* tree_vals, const int* perm, double* out, int64_t n,
                           int stride, cudaStream_t st) {
  if (n == 0) return NBK_OK;
  k_scatter_d<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(tree_vals, perm, out, n, stride); note_launch();
  NBK_CUDA_TRY(cudaGetLastError());
  return NBK_OK;
}

}  // namespace nbk

using namespace nbk;

struct nbk_tree {
  int64_t n = 0;
  int device = 0;  // the CUDA device the tree's arrays live on (current at nbk_create)
  int b = 16, treetype = 0, kerntype = 0, kernres = 1000;
  int aniso = 0;  // phase-space trees: -1 plain phase distance, 0 local metric
  bool periodic = false;
  double period[3] = {0, 0, 0};
  unsigned flags = 0;
  cudaStream_t st = nullptr;
  bool has_vel = false;
  BuiltArrays arr;
  int64_t nslots = 0, numnodes = 0, numleaves = 0;
  std::vector<double> h_kernel;
  double kernnorm = 0;
  double* d_kernel = nullptr;
  float eps = 0;
  float eps6[6] = {0, 0, 0, 0, 0, 0};
  int* d_err = nullptr;
  void* block = nullptr;  // the one device allocation holding every array above
  bool dev() const { return flags & NBK_DEVICE_PTRS; }
  TreeView view() const {
    TreeView v{};
    v.pos = arr.pos;
    v.posf = arr.posf;
    v.vel = arr.vel;
    v.perm = arr.perm;
    v.node = arr.node;
    v.nodex = arr.nodex;
    v.nodes6 = arr.nodes6;
    v.nodeb6 = arr.nodeb6;
    v.nodef6 = arr.nodef6;
    v.velf = arr.velf;
    for (int d = 0; d < 6; d++) v.eps6[d] = eps6[d];
    v.n = (int)n;
    v.pstart = 0;
    v.nbase = 0;
    v.b = b;
    // a tree that is a single leaf searches without images (KDLeafNode.cxx:658-661)
    v.periodic = (periodic && n > b) ? 1 : 0;
    for (int d = 0; d < 3; d++) v.period[d] = period[d];
    v.eps = eps;
    return v;
  }
};

// Frees every device array a tree owns (null entries are skipped; the frees are ordered on
// the tree's stream); a failed nbk_create also waits for the stream.
static void free_tree_arrays(nbk_tree* t, bool wait) {
  cudaStream_t st = t->st;
  dev_free(t->block, st);  // every array of the tree lives in this one allocation
  t->block = nullptr;
  t->arr = BuiltArrays();
  t->d_err = nullptr;  // t->d_kernel belongs to the process-wide kernel cache
  if (wait) cudaStreamSynchronize(st);
}

#define API_BEGIN try {
#define API_END                                          \
  }                                                      \
  catch (const std::exception& e) {                      \
    set_error(std::string("exception: ") + e.what());    \
    return NBK_ERR_INVALID;                              \
  }

namespace {

// Device staging for one call: host pointers are copied in/out, device pointers used as
// they are.
struct Stage {
  nbk_tree* t;
  DevAlloc alloc;
  std::vector<std::pair<void*, std::pair<void*, size_t>>> outs;  // (host, (dev, bytes))
  explicit Stage(nbk_tree* tt) : t(tt) { alloc.st = tt->st; }
  template <class T>
  int in(const T* host_or_dev, size_t count, const T** dev) {
    if (t->dev() || host_or_dev == nullptr) {
      *dev = host_or_dev;
      return NBK_OK;
    }
    T* d;
    NBK_TRY(alloc.get((void**)&d, sizeof(T) * count));
    NBK_CUDA_TRY(cudaMemcpyAsync(d, host_or_dev, sizeof(T) * count, cudaMemcpyHostToDevice, t->st));
    *dev = d;
    return NBK_OK;
  }
  template <class T>
  int out(T* host_or_dev, size_t count, T** dev, bool copy_existing = false) {
    if (t->dev()) {
      *dev = host_or_dev;
      return NBK_OK;
    }
    T* d;
    NBK_TRY(alloc.get((void**)&d, sizeof(T) * count));
    if (copy_existing)
      NBK_CUDA_TRY(cudaMemcpyAsync(d, host_or_dev, sizeof(T) * count, cudaMemcpyHostToDevice, t->st));
    outs.push_back({(void*)host_or_dev, {(void*)d, sizeof(T) * count}});
    *dev = d;
    return NBK_OK;
  }
  int finish() {
    for (auto& o : outs)
      NBK_CUDA_TRY(cudaMemcpyAsync(o.first, o.second.first, o.second.second,
                                   cudaMemcpyDeviceToHost, t->st));
    if (!t->dev()) NBK_CUDA_TRY(cudaStreamSynchronize(t->st));
    return NBK_OK;
  }
};

// Status for a device error word already read back.
int err_status(int h, const char* what) {
  if (h == kErrTooFew) {
    set_error(std::string(what) + ": fewer than k neighbours were found for some particle");
    return NBK_ERR_TOO_FEW;
  }
  if (h == kErrTarget) {
    set_error(std::string(what) + ": a target index is outside the tree");
    return NBK_ERR_INVALID;
  }
  if (h) {
    set_error(std::string(what) + ": device bound exceeded (code " + std::to_string(h) + ")");
    return NBK_ERR_DEVICE;
  }
  return NBK_OK;
}

int check_err(nbk_tree* t, const char* what) {
  int h = 0;
  NBK_CUDA_TRY(cudaMemcpyAsync(&h, t->d_err, sizeof(int), cudaMemcpyDeviceToHost, t->st));
  NBK_CUDA_TRY(cudaStreamSynchronize(t->st));
  return err_status(h, what);
}

// A few page-locked scalars per host thread, so that small device-to-host reads can be
// queued without blocking and collected by one later synchronisation (null if the
// page-locked allocation failed: callers then read synchronously).
struct PinnedScalars {
  int i[8];
  double d[8];
};
PinnedScalars* pinned_scalars() {
  static thread_local PinnedScalars* p = nullptr;
  static thread_local bool tried = false;
  if (!p && !tried) {
    tried = true;
    void* q = nullptr;
    if (cudaMallocHost(&q, sizeof(PinnedScalars)) == cudaSuccess) p = (PinnedScalars*)q;
  }
  return p;
}

int clear_err(nbk_tree* t) {
  NBK_CUDA_TRY(cudaMemsetAsync(t->d_err, 0, sizeof(int), t->st));
  return NBK_OK;
}

KnnArgs base_args(nbk_tree* t) {
  KnnArgs a{};
  a.tv = t->view();
  a.kernel = t->d_kernel;
  a.kernres = t->kernres;
  a.err = t->d_err;
  return a;
}

int check_tree(const nbk_tree* t) {
  if (!t) {
    set_error("null tree handle");
    return NBK_ERR_INVALID;
  }
  return NBK_OK;
}

// The entry points that only a physical tree supports: on velocity and phase-space trees
// the reference either refuses them (CalcVelDensity, the smoothing family) or compares
// positions with velocity or phase-space cut values (ball searches, FOF), which
// KDTree::GetPosition(j) answers past the end of its three-element array for j > 2.
int check_phys(const nbk_tree* t, const char* what) {
  NBK_TRY(check_tree(t));
  if (t->treetype != NBK_TPHYS) {
    set_error(std::string(what) + ": runs on physical trees only (TreeType TPHYS)");
    return NBK_ERR_UNSUPPORTED;
  }
  return NBK_OK;
}

}  // namespace

namespace nbk {
// CalcDensity with caller-supplied memory only: `scratch` (t->n doubles, tree order) and
// the device output `rho_dev` (t->n doubles, input order). Used by nbk_density_noalloc
// (noalloc.cu), which owns the scratch; nothing here allocates.
int density_into_scratch(nbk_tree* t, int k, double* scratch, double* rho_dev) {
  if (!t || !scratch || !rho_dev || k < 1) {
    set_error("nbk_density_noalloc: invalid argument");
    return NBK_ERR_INVALID;
  }
  if (t->treetype == NBK_TPHS) {
    set_error("nbk_density_noalloc: physical and velocity trees only");
    return NBK_ERR_UNSUPPORTED;
  }
  if (k > t->n - 1) {
    set_error("nbk_density_noalloc: k = " + std::to_string(k) + " exceeds the " +
              std::to_string(t->n - 1) + " other particles");
    return NBK_ERR_TOO_FEW;
  }
  NBK_CUDA_TRY(cudaMemsetAsync(scratch, 0, sizeof(double) * t->n, t->st));
  NBK_TRY(clear_err(t));
  KnnArgs a = base_args(t);
  a.tv.periodic = 0;  // CalcDensity ignores the period (KDCalcSmoothQuantities.cxx:227)
  a.kheap = k;
  a.kout = k;
  a.exclude_self = 1;
  a.qmode = 0;
  a.nq = (int)t->n;
  a.rho = scratch;
  NBK_TRY(launch_knn(a, kEpiDensity, t->st));
  NBK_TRY(scatter_to_input_order(scratch, t->arr.perm, rho_dev, t->n, 1, t->st));
  return check_err(t, "nbk_density_noalloc");
}
int64_t tree_size(const nbk_tree* t) { return t ? t->n : 0; }
int tree_device(const nbk_tree* t) { return t ? t->device : 0; }
}  // namespace nbk

extern "C" {

const char* nbk_last_error(void) { return get_error(); }

long long nbk_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

int nbk_kernel_binary_version(int* binary_version, int* ptx_version) {
  cudaFuncAttributes fa{};
  // k_scatter_d: the scatter back to input order that every density call launches
  NBK_CUDA_TRY(cudaFuncGetAttributes(&fa, (const void*)k_scatter_d));
  if (binary_version) *binary_version = fa.binaryVersion;
  if (ptx_version) *ptx_version = fa.ptxVersion;
  return NBK_OK;
}

int nbk_debug_set_iteration_cap(int cap) { return set_uf_iteration_cap(cap); }

int nbk_debug_fail_allocation(long long countdown) {
  g_fail_countdown.store(countdown < 0 ? -1 : countdown);
  return NBK_OK;
}

long long nbk_debug_live_allocations(void) {
  return g_live_allocs.load(std::memory_order_relaxed);
}

int nbk_trace_enable(int on) {
  g_trace_on.store(on != 0);
  return NBK_OK;
}

int nbk_trace_reset(void) {
  resolve_pending();
  std::lock_guard<std::mutex> lk(g_trace_mu);
  g_trace.clear();
  return NBK_OK;
}

int64_t nbk_trace_json(char* buf, int64_t cap) {
  resolve_pending();
  std::string s = "{";
  {
    std::lock_guard<std::mutex> lk(g_trace_mu);
    bool first = true;
    for (auto& kv : g_trace) {
      char tmp[256];
      snprintf(tmp, sizeof(tmp), "%s\"%s\": {\"count\": %lld, \"ms\": %.6f}", first ? "" : ", ",
               kv.first.c_str(), kv.second.count, kv.second.ms);
      s += tmp;
      first = false;
    }
  }
  s += "}";
  if (buf && cap > 0) {
    int64_t m = std::min<int64_t>(cap - 1, (int64_t)s.size());
    memcpy(buf, s.data(), m);
    buf[m] = 0;
  }
  return (int64_t)s.size() + 1;
}

const char* nbk_version(void) {
  static std::string v;
  int dev = 0;
  cudaDeviceProp p{};
  if (cudaGetDevice(&dev) == cudaSuccess && cudaGetDeviceProperties(&p, dev) == cudaSuccess)
    v = std::string("nbkdt 0.1 sm_103a; device ") + p.name;
  else
    v = "nbkdt 0.1 sm_103a; no device";
  return v.c_str();
}

int nbk_create(const double* pos, const double* vel, const double* mass, int64_t n,
               int bucket_size, int treetype, int kerntype, int kernres,
               int splitting_criterion, int aniso, int scale_space, const double* period,
               unsigned flags, nbk_tree** out) {
  API_BEGIN
  if (!out || !pos) {
    set_error("nbk_create: null pointer argument");
    return NBK_ERR_INVALID;
  }
  *out = nullptr;
  if (n < 1 || n > (int64_t)0x7fffff00) {
    set_error("nbk_create: particle count must be in [1, 2^31)");
    return NBK_ERR_INVALID;
  }
  if (bucket_size < 1) {
    set_error("nbk_create: bucket size must be >= 1");
    return NBK_ERR_INVALID;
  }
  if (bucket_size >= kLocalMax) {
    set_error("nbk_create: bucket sizes >= 1024 are not supported on the GPU");
    return NBK_ERR_UNSUPPORTED;
  }
  if (treetype != NBK_TPHYS && treetype != NBK_TVEL && treetype != NBK_TPHS) {
    set_error("nbk_create: tree types TPHYS, TVEL and TPHS run on the GPU (TPROJ and TMETRIC do not)");
    return NBK_ERR_UNSUPPORTED;
  }
  if ((treetype == NBK_TVEL || treetype == NBK_TPHS) && !vel) {
    set_error("nbk_create: velocity and phase-space trees need velocities");
    return NBK_ERR_INVALID;
  }
  if (treetype == NBK_TVEL && period) {
    set_error("nbk_create: periodic velocity trees are not supported");
    return NBK_ERR_UNSUPPORTED;
  }
  if (splitting_criterion != 0 || scale_space != 0 || (aniso != 0 && aniso != -1)) {
    set_error("nbk_create: splitting criterion and space scaling other than 0, and the anisotropic metric tensor (Aniso 1), are not supported");
    return NBK_ERR_UNSUPPORTED;
  }
  std::unique_ptr<nbk_tree> t(new nbk_tree);
  // a failed creation frees whatever device arrays it had already allocated
  struct FreeOnFailure {
    nbk_tree* t;
    ~FreeOnFailure() {
      if (t) free_tree_arrays(t, true);
    }
  } guard{t.get()};
  NBK_CUDA_TRY(cudaGetDevice(&t->device));
  t->n = n;
  t->b = bucket_size;
  t->treetype = treetype;
  t->aniso = aniso;
  t->kerntype = (kerntype >= NBK_KSPH && kerntype <= NBK_KTH) ? kerntype : NBK_KSPH;
  t->kernres = kernres < 100 ? 100 : kernres;  // KDTree.cxx:1145-1148
  t->flags = flags;
  // a device-resident period is read back with the build's own final synchronisation
  // (queued into page-locked memory) and checked after it; a host one is checked now
  PinnedScalars* ps = (period && (flags & NBK_DEVICE_PTRS)) ? pinned_scalars() : nullptr;
  auto take_period = [&](const double* per) -> int {
    for (int d = 0; d < 3; d++) {
      if (!(per[d] > 0)) {
        set_error("nbk_create: period entries must be positive");
        return NBK_ERR_INVALID;
      }
      t->period[d] = per[d];
    }
    t->periodic = true;
    return NBK_OK;
  };
  if (period) {
    if (flags & NBK_DEVICE_PTRS) {
      if (ps) {
        NBK_CUDA_TRY(cudaMemcpyAsync(ps->d, period, sizeof(double) * 3, cudaMemcpyDeviceToHost,
                                     t->st));
      } else {
        double per[3];
        NBK_CUDA_TRY(cudaMemcpy(per, period, sizeof(per), cudaMemcpyDeviceToHost));
        NBK_TRY(take_period(per));
      }
    } else {
      NBK_TRY(take_period(period));
    }
  }
  t->has_vel = vel != nullptr;
  cudaStream_t st = t->st;
  {
    const KernelEntry* ke;
    NBK_TRY(cached_kernel(t->kerntype, t->kernres, treetype == NBK_TPHS ? 6 : 3, &ke));
    t->h_kernel = ke->table;
    t->kernnorm = ke->norm;
    t->d_kernel = ke->d_img;  // shared, not owned by the tree
  }
  t->nslots = heap_slots(n, bucket_size);
  t->numnodes = count_nodes(n, bucket_size);
  {
    int64_t nl = 0;
    // leaves = nodes - internal nodes; a binary tree has internal = leaves - 1
    nl = (t->numnodes + 1) / 2;
    t->numleaves = nl;
  }
  BuiltArrays& A = t->arr;
  {
    // every array of the tree in one allocation; the error word and the node arrays that
    // start zeroed come first, so one memset clears them
    const bool phs = treetype == NBK_TPHS;
    std::vector<DevPart> parts{{(void**)&t->d_err, sizeof(int)}};
    if (phs) {
      parts.push_back({(void**)&A.nodes6, sizeof(NodeS) * t->nslots});
      parts.push_back({(void**)&A.nodeb6, sizeof(NodeB6) * t->nslots});
    } else {
      parts.push_back({(void**)&A.node, sizeof(NodeRec) * t->nslots});
      parts.push_back({(void**)&A.nodex, sizeof(NodeX) * t->nslots});
    }
    size_t zeroed = block_bytes(parts);
    parts.push_back({(void**)&A.pos, sizeof(P4) * n});
    parts.push_back({(void**)&A.posf, sizeof(float4) * n});
    parts.push_back({(void**)&A.perm, sizeof(int) * n});
    if (vel) parts.push_back({(void**)&A.vel, sizeof(V4) * n});
    if (phs) {
      parts.push_back({(void**)&A.nodef6, sizeof(NodeF6) * t->nslots});
      parts.push_back({(void**)&A.velf, sizeof(float4) * n});
    }
    NBK_TRY(dev_malloc(&t->block, block_bytes(parts), st));
    carve_block(t->block, parts);
    NBK_CUDA_TRY(cudaMemsetAsync(t->block, 0, zeroed, st));
  }
  DevAlloc alloc;
  alloc.st = st;
  const double *d_pos = pos, *d_vel = vel, *d_mass = mass;
  if (!(flags & NBK_DEVICE_PTRS)) {
    double *a, *v = nullptr, *m = nullptr;
    std::vector<DevPart> parts{{(void**)&a, sizeof(double) * 3 * n}};
    if (vel) parts.push_back({(void**)&v, sizeof(double) * 3 * n});
    if (mass) parts.push_back({(void**)&m, sizeof(double) * n});
    NBK_TRY(alloc.get_block(parts));
    NBK_CUDA_TRY(cudaMemcpyAsync(a, pos, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
    if (vel)
      NBK_CUDA_TRY(cudaMemcpyAsync(v, vel, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
    if (mass)
      NBK_CUDA_TRY(cudaMemcpyAsync(m, mass, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    d_pos = a;
    d_vel = v;
    d_mass = m;
  }
  std::vector<TreeSpec> trees{{0, n, 0}};
  // the root's exact box comes back with the build's own final synchronisation
  double rlo[3], rhi[3];
  if (treetype == NBK_TPHS) {
    NodeB6 root;
    NBK_TRY(build_forest_phase(trees, bucket_size, d_pos, d_mass, d_vel, A, alloc, st, &root));
    for (int d = 0; d < 3; d++) {
      rlo[d] = root.lo[d];
      rhi[d] = root.hi[d];
    }
    // FP32 rounding bound per phase-space coordinate (position images included)
    for (int d = 0; d < 6; d++) {
      double m = std::max(std::fabs(root.lo[d]), std::fabs(root.hi[d])) +
                 (d < 3 ? t->period[d] : 0.0);
      t->eps6[d] = (float)std::ldexp(m, -23) * 1.0001f + 1e-38f;
    }
  } else {
    // a velocity tree is the same tree over the velocities (FindNearestVel,
    // BoundaryandMeanVel, MedianVel): positions and velocities trade places on the device
    if (treetype == NBK_TVEL) std::swap(d_pos, d_vel);
    NodeX root;
    NBK_TRY(build_forest(trees, bucket_size, d_pos, d_mass, d_vel, A, alloc, st, &root));
    for (int d = 0; d < 3; d++) {
      rlo[d] = root.lo[d];
      rhi[d] = root.hi[d];
    }
  }
  if (ps) NBK_TRY(take_period(ps->d));  // the build has synchronised the stream
  // FP32 rounding bound for coordinates and image coordinates
  double maxabs = 0;
  for (int d = 0; d < 3; d++)
    maxabs = std::max(maxabs, std::max(std::fabs(rlo[d]), std::fabs(rhi[d])));
  double maxper = std::max(t->period[0], std::max(t->period[1], t->period[2]));
  t->eps = (float)std::ldexp(maxabs + maxper, -23) * 1.0001f + 1e-38f;
  alloc.release_all_scratch(st);
  guard.t = nullptr;
  *out = t.release();
  return NBK_OK;
  API_END
}

int nbk_destroy(nbk_tree* t) {
  if (!t) return NBK_OK;
  free_tree_arrays(t, false);
  delete t;
  return NBK_OK;
}

int nbk_set_stream(nbk_tree* t, void* stream) {
  NBK_TRY(check_tree(t));
  t->st = (cudaStream_t)stream;
  return NBK_OK;
}

int nbk_sync(nbk_tree* t) {
  NBK_TRY(check_tree(t));
  NBK_CUDA_TRY(cudaStreamSynchronize(t->st));
  return NBK_OK;
}

int nbk_get_counts(const nbk_tree* t, int64_t* numparts, int64_t* numnodes,
                   int64_t* numleafnodes, int32_t* bucket_size) {
  NBK_TRY(check_tree(t));
  if (numparts) *numparts = t->n;
  if (numnodes) *numnodes = t->numnodes;
  if (numleafnodes) *numleafnodes = t->numleaves;
  if (bucket_size) *bucket_size = t->b;
  return NBK_OK;
}

int nbk_get_perm(const nbk_tree* t, int32_t* perm) {
  NBK_TRY(check_tree(t));
  if (!perm) {
    set_error("nbk_get_perm: null output");
    return NBK_ERR_INVALID;
  }
  NBK_CUDA_TRY(cudaMemcpyAsync(perm, t->arr.perm, sizeof(int) * t->n,
                               t->dev() ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, t->st));
  if (!t->dev()) NBK_CUDA_TRY(cudaStreamSynchronize(t->st));
  return NBK_OK;
}

int nbk_get_kernel(const nbk_tree* t, double* table, double* kernnorm) {
  NBK_TRY(check_tree(t));
  if (table) memcpy(table, t->h_kernel.data(), sizeof(double) * t->kernres);
  if (kernnorm) *kernnorm = t->kernnorm;
  return NBK_OK;
}

// Phase-space trees: FindNearest(tt) for qmode 0 (every particle) / 2 (targets) and
// FindNearest(x) for qmode 1 (six values per point), through the reference's own walk
// (phase.cu). A periodic target search grows the heap by one and drops its nearest entry
// (KDFindNearest.cxx:250, 310).
static int phase_nn(nbk_tree* t, int qmode, const int* dq, const double* dx, int64_t nq, int k,
                    int* dnn, double* dd2, bool metric) {
  PhaseArgs pa{};
  pa.k = base_args(t);
  pa.k.periodic = t->periodic ? 1 : 0;
  pa.k.kheap = (t->periodic && qmode != 1) ? k + 1 : k;
  pa.k.kout = k;
  pa.k.qmode = qmode;
  pa.k.qidx = dq;
  pa.k.qx = dx;
  pa.k.nq = (int)nq;
  pa.k.nn = dnn;
  pa.k.d2 = dd2;
  pa.metric = metric ? 1 : 0;
  pa.spacing_periodic = t->periodic ? 1 : 0;
  pa.epi = kPhNN;
  return launch_phase(pa, t->st);
}

static int knn_variant_ok(const nbk_tree* t, int variant, const char* what) {
  if (variant < NBK_FINDNEAREST || variant > NBK_FINDNEARESTPHASE) {
    set_error(std::string(what) + ": unknown variant");
    return NBK_ERR_INVALID;
  }
  static const int tree_of[4] = {-1, NBK_TPHYS, NBK_TVEL, NBK_TPHS};
  static const char* name_of[4] = {"", "FindNearestPos", "FindNearestVel", "FindNearestPhase"};
  if (variant != NBK_FINDNEAREST && t->treetype != tree_of[variant]) {
    set_error(std::string(what) + ": " + name_of[variant] + " runs on " +
              (variant == NBK_FINDNEARESTPOS ? "physical" :
               variant == NBK_FINDNEARESTVEL ? "velocity" : "phase-space") + " trees only");
    return NBK_ERR_UNSUPPORTED;
  }
  if (t->treetype == NBK_TPHS && t->n < 8 && t->aniso == 0 && variant == NBK_FINDNEAREST) {
    set_error(std::string(what) + ": the local metric needs at least 8 particles (the reference exits)");
    return NBK_ERR_TOO_FEW;
  }
  return NBK_OK;
}

int nbk_knn(nbk_tree* t, int k, int variant, int periodic_mode, int32_t* nn, double* d2) {
  API_BEGIN
  NBK_TRY(check_tree(t));
  if (k < 1 || !nn || !d2) {
    set_error("nbk_knn: k must be >= 1 and outputs non-null");
    return NBK_ERR_INVALID;
  }
  NBK_TRY(knn_variant_ok(t, variant, "nbk_knn"));
  Stage S(t);
  int *dnn;
  double* dd2;
  NBK_TRY(S.out(nn, (size_t)t->n * k, &dnn));
  NBK_TRY(S.out(d2, (size_t)t->n * k, &dd2));
  NBK_TRY(clear_err(t));
  if (t->treetype == NBK_TPHS) {
    NBK_TRY(phase_nn(t, 0, nullptr, nullptr, t->n, k, dnn, dd2,
                     t->aniso == 0 && variant != NBK_FINDNEARESTPHASE));
    NBK_TRY(S.finish());
    if (!t->dev()) NBK_TRY(check_err(t, "nbk_knn"));
    return NBK_OK;
  }
  KnnArgs a = base_args(t);
  bool per = t->periodic;  // the heap grows by one whenever a period is set
  a.kheap = per ? k + 1 : k;
  a.kout = k;
  a.drop_largest = (per && variant == NBK_FINDNEARESTPOS) ? 1 : 0;
  a.periodic = a.tv.periodic;
  a.exclude_self = a.tv.periodic ? 0 : 1;
  a.min_image = periodic_mode == NBK_PERIODIC_MIN_IMAGE;
  a.qmode = 0;
  a.q0 = 0;
  a.nq = (int)t->n;
  a.nn = dnn;
  a.d2 = dd2;
  NBK_TRY(launch_knn(a, kEpiNN, t->st));
  NBK_TRY(S.finish());
  if (!t->dev()) NBK_TRY(check_err(t, "nbk_knn"));
  return NBK_OK;
  API_END
}

int nbk_knn_targets(nbk_tree* t, const int32_t* targets, int64_t nt, int k, int variant,
                    int periodic_mode, int32_t* nn, double* d2) {
  API_BEGIN
  NBK_TRY(check_tree(t));
  if (k < 1 || !targets || !nn || !d2 || nt < 0) {
    set_error("nbk_knn_targets: invalid argument");
    return NBK_ERR_INVALID;
  }
  NBK_TRY(knn_variant_ok(t, variant, "nbk_knn_targets"));
  if (nt == 0) return NBK_OK;
  if (!t->dev())
    for (int64_t i = 0; i < nt; i++)
      if (targets[i] < 0 || targets[i] >= t->n) {
        set_error("nbk_knn_targets: target index out of range");
        return NBK_ERR_INVALID;
      }
  Stage S(t);
  const int* dt;
  int* dnn;
  double* dd2;
  NBK_TRY(S.in(targets, nt, &dt));
  NBK_TRY(S.out(nn, (size_t)nt * k, &dnn));
  NBK_TRY(S.out(d2, (size_t)nt * k, &dd2));
  NBK_TRY(clear_err(t));
  if (t->treetype == NBK_TPHS) {
    NBK_TRY(phase_nn(t, 2, dt, nullptr, nt, k, dnn, dd2,
                     t->aniso == 0 && variant != NBK_FINDNEARESTPHASE));
    NBK_TRY(S.finish());
    if (!t->dev()) NBK_TRY(check_err(t, "nbk_knn_targets"));
    return NBK_OK;
  }
  KnnArgs a = base_args(t);
  bool per = t->periodic;
  a.kheap = per ? k + 1 : k;
  a.kout = k;
  a.drop_largest = (per && variant == NBK_FINDNEARESTPOS) ? 1 : 0;
  a.periodic = a.tv.periodic;
  a.exclude_self = a.tv.periodic ? 0 : 1;
  a.min_image = periodic_mode == NBK_PERIODIC_MIN_IMAGE;
  a.qmode = 2;
  a.qidx = dt;
  a.nq = (int)nt;
  a.nn = dnn;
  a.d2 = dd2;
  NBK_TRY(launch_knn(a, kEpiNN, t->st));
  NBK_TRY(S.finish());
  if (!t->dev()) NBK_TRY(check_err(t, "nbk_knn_targets"));
  return NBK_OK;
  API_END
}

int nbk_knn_points(nbk_tree* t, const double* x, int64_t nq, int k, int periodic_mode,
                   int32_t* nn, double* d2) {
  API_BEGIN
  NBK_TRY(check_phys(t, "nbk_knn_points"));
  if (k < 1 || !x || !nn || !d2 || nq < 0) {
    set_error("nbk_knn_points: invalid argument");
    return NBK_ERR_INVALID;
  }
  if (nq == 0) return NBK_OK;
  Stage S(t);
  const double* dx;
  int* dnn;
  double* dd2;
  NBK_TRY(S.in(x, (size_t)nq * 3, &dx));
  NBK_TRY(S.out(nn, (size_t)nq * k, &dnn));
  NBK_TRY(S.out(d2, (size_t)nq * k, &dd2));
  NBK_TRY(clear_err(t));
  KnnArgs a = base_args(t);
  a.kheap = k;
  a.kout = k;
  a.periodic = a.tv.periodic;
  a.exclude_self = 0;
  a.min_image = periodic_mode == NBK_PERIODIC_MIN_IMAGE;
  a.qmode = 1;
  a.qx = dx;
  a.nq = (int)nq;
  a.nn = dnn;
  a.d2 = dd2;
  NBK_TRY(launch_knn(a, kEpiNN, t->st));
  NBK_TRY(S.finish());
  if (!t->dev()) NBK_TRY(check_err(t, "nbk_knn_points"));
  return NBK_OK;
  API_END
}


int nbk_knn_coords(nbk_tree* t, const double* x, int64_t nq, int k, int32_t* nn, double* d2) {
  API_BEGIN
  NBK_TRY(check_tree(t));
  if (k < 1 || !x || !nn || !d2 || nq < 0) {
    set_error("nbk_knn_coords: invalid argument");
    return NBK_ERR_INVALID;
  }
  if (t->treetype == NBK_TPHYS) return nbk_knn_points(t, x, nq, k, NBK_PERIODIC_REF, nn, d2);
  NBK_TRY(knn_variant_ok(t, NBK_FINDNEAREST, "nbk_knn_coords"));
  if (nq == 0) return NBK_OK;
  const int nd = t->treetype == NBK_TPHS ? 6 : 3;
  Stage S(t);
  const double* dx;
  int* dnn;
  double* dd2;
  NBK_TRY(S.in(x, (size_t)nq * nd, &dx));
  NBK_TRY(S.out(nn, (size_t)nq * k, &dnn));
  NBK_TRY(S.out(d2, (size_t)nq * k, &dd2));
  NBK_TRY(clear_err(t));
  if (t->treetype == NBK_TPHS) {
    NBK_TRY(phase_nn(t, 1, nullptr, dx, nq, k, dnn, dd2, t->aniso == 0));
  } else {  // velocity tree (never periodic): FindNearestVel(x) over the swapped arrays
    KnnArgs a = base_args(t);
    a.kheap = k;
    a.kout = k;
    a.periodic = 0;
    a.exclude_self = 0;
    a.qmode = 1;
    a.qx = dx;
    a.nq = (int)nq;
    a.nn = dnn;
    a.d2 = dd2;
    NBK_TRY(launch_knn(a, kEpiNN, t->st));
  }
  NBK_TRY(S.finish());
  if (!t->dev()) NBK_TRY(check_err(t, "nbk_knn_coords"));
  return NBK_OK;
  API_END
}

int nbk_knn_phase_points(nbk_tree* t, const double* x, int64_t nq, int k, int32_t* nn,
                         double* d2) {
  API_BEGIN
  NBK_TRY(check_tree(t));
  if (k < 1 || !x || !nn || !d2 || nq < 0) {
    set_error("nbk_knn_phase_points: invalid argument");
    return NBK_ERR_INVALID;
  }
  NBK_TRY(knn_variant_ok(t, NBK_FINDNEARESTPHASE, "nbk_knn_phase_points"));
  if (nq == 0) return NBK_OK;
  Stage S(t);
  const double* dx;
  int* dnn;
  double* dd2;
  NBK_TRY(S.in(x, (size_t)nq * 6, &dx));
  NBK_TRY(S.out(nn, (size_t)nq * k, &dnn));
  NBK_TRY(S.out(d2, (size_t)nq * k, &dd2));
  NBK_TRY(clear_err(t));
  NBK_TRY(phase_nn(t, 1, nullptr, dx, nq, k, dnn, dd2, false));
  NBK_TRY(S.finish());
  if (!t->dev()) NBK_TRY(check_err(t, "nbk_knn_phase_points"));
  return NBK_OK;
  API_END
}

// CalcDensity / CalcDensityParticle on a phase-space tree with the local metric: qmode 0
// scatters into `trho` (tree order), qmode 2 gathers into `out` (query order).
static int phase_density(nbk_tree* t, int qmode, const int* dq, int64_t nq, int k, double* rho) {
  if (t->aniso != 0) {
    set_error("phase-space density needs the local metric (Aniso 0); with Aniso -1 the "
              "reference multiplies uninitialised metric arrays");
    return NBK_ERR_UNSUPPORTED;
  }
  if (t->n < 8) {
    set_error("phase-space density: the local metric needs at least 8 particles");
    return NBK_ERR_TOO_FEW;
  }
  PhaseArgs pa{};
  pa.k = base_args(t);
  pa.k.periodic = 0;  // CalcDensity ignores the period, and its metric spacing too
  pa.k.kheap = k;
  pa.k.kout = k;
  pa.k.qmode = qmode;
  pa.k.qidx = dq;
  pa.k.nq = (int)nq;
  pa.k.rho = rho;
  pa.metric = 1;
  pa.spacing_periodic = 0;
  pa.epi = qmode == 0 ? kPhDensity : kPhDensPart;
  return launch_phase(pa, t->st);
}

static int density_common(nbk_tree* t, int k, int nsmooth, double* rho, double* vden, int epi) {
  if (k < 1) {
    set_error("density: k must be >= 1");
    return NBK_ERR_INVALID;
  }
  if (k > t->n - 1) {
    set_error("density: k = " + std::to_string(k) + " exceeds the " +
              std::to_string(t->n - 1) + " other particles (the reference exits here)");
    return NBK_ERR_TOO_FEW;
  }
  if ((epi == kEpiVel || epi == kEpiDensVel) && !t->has_vel) {
    set_error("velocity density needs velocities at nbk_create");
    return NBK_ERR_INVALID;
  }
  if (epi != kEpiDensity && t->treetype != NBK_TPHYS) {
    set_error("velocity density runs on physical trees only");
    return NBK_ERR_UNSUPPORTED;
  }
  Stage S(t);
  double *drho = nullptr, *dv = nullptr, *trho = nullptr, *tv = nullptr;
  if (rho) NBK_TRY(S.out(rho, t->n, &drho));
  if (vden) NBK_TRY(S.out(vden, t->n, &dv));
  if (rho) {
    NBK_TRY(S.alloc.get((void**)&trho, sizeof(double) * t->n));
    NBK_CUDA_TRY(cudaMemsetAsync(trho, 0, sizeof(double) * t->n, t->st));
  }
  if (vden) NBK_TRY(S.alloc.get((void**)&tv, sizeof(double) * t->n));
  NBK_TRY(clear_err(t));
  if (t->treetype == NBK_TPHS) {
    NBK_TRY(phase_density(t, 0, nullptr, t->n, k, trho));
    NBK_TRY(scatter_to_input_order(trho, t->arr.perm, drho, t->n, 1, t->st));
    NBK_TRY(S.finish());
    if (!t->dev()) NBK_TRY(check_err(t, "density"));
    return NBK_OK;
  }
  KnnArgs a = base_args(t);
  a.tv.periodic = 0;  // CalcDensity ignores the period (KDCalcSmoothQuantities.cxx:227)
  a.kheap = k;
  a.kout = k;
  a.exclude_self = 1;
  a.qmode = 0;
  a.nq = (int)t->n;
  a.nsmooth = nsmooth;
  a.rho = trho;
  a.vden = tv;
  NBK_TRY(launch_knn(a, epi, t->st));
  if (rho) NBK_TRY(scatter_to_input_order(trho, t->arr.perm, drho, t->n, 1, t->st));
  if (vden) NBK_TRY(scatter_to_input_order(tv, t->arr.perm, dv, t->n, 1, t->st));
  NBK_TRY(S.finish());
  if (!t->dev()) NBK_TRY(check_err(t, "density"));
  return NBK_OK;
}

int nbk_density(nbk_tree* t, int k, double* rho) {
  API_BEGIN
  NBK_TRY(check_tree(t));
  if (!rho) {
    set_error("nbk_density: null output");
    return NBK_ERR_INVALID;
  }
  return density_common(t, k, k, rho, nullptr, kEpiDensity);
  API_END
}

int nbk_veldensity(nbk_tree* t, int nsmooth, int nsearch, double* out) {
  API_BEGIN
  NBK_TRY(check_tree(t));
  if (!out || nsmooth < 1) {
    set_error("nbk_veldensity: invalid argument");
    return NBK_ERR_INVALID;
  }
  if (nsmooth > nsearch) nsmooth = nsearch;  // KDCalcSmoothQuantities.cxx:319-322
  return density_common(t, nsearch, nsmooth, nullptr, out, kEpiVel);
  API_END
}

int nbk_density_veldensity(nbk_tree* t, int k, int nsmooth, double* rho, double* veldens) {
  API_BEGIN
  NBK_TRY(check_tree(t));
  if (!rho || !veldens || nsmooth < 1) {
    set_error("nbk_density_veldensity: invalid argument");
    return NBK_ERR_INVALID;
  }
  if (nsmooth > k) nsmooth = k;
  return density_common(t, k, nsmooth, rho, veldens, kEpiDensVel);
  API_END
}

static int particles_common(nbk_tree* t, const int32_t* targets, int64_t nt, int k, int nsmooth,
                            double* out, int epi) {
  if (!targets || !out || nt < 0 || k < 1) {
    set_error("invalid argument");
    return NBK_ERR_INVALID;
  }
  if (k > t->n - 1) {
    set_error("k exceeds the number of other particles");
    return NBK_ERR_TOO_FEW;
  }
  if (epi == kEpiVelPart && !t->has_vel) {
    set_error("velocity density needs velocities at nbk_create");
    return NBK_ERR_INVALID;
  }
  if (epi != kEpiDensPart && t->treetype != NBK_TPHYS) {
    set_error("velocity density runs on physical trees only");
    return NBK_ERR_UNSUPPORTED;
  }
  if (nt == 0) return NBK_OK;
  if (!t->dev()) {
    for (int64_t i = 0; i < nt; i++)
      if (targets[i] < 0 || targets[i] >= t->n) {
        set_error("target index out of range");
        return NBK_ERR_INVALID;
      }
  }
  Stage S(t);
  const int* dt;
  double* dout;
  NBK_TRY(S.in(targets, nt, &dt));
  NBK_TRY(S.out(out, nt, &dout));
  NBK_TRY(clear_err(t));
  if (t->treetype == NBK_TPHS) {
    NBK_TRY(phase_density(t, 2, dt, nt, k, dout));
    NBK_TRY(S.finish());
    if (!t->dev()) NBK_TRY(check_err(t, "particle density"));
    return NBK_OK;
  }
  KnnArgs a = base_args(t);
  a.tv.periodic = 0;
  a.kheap = k;
  a.kout = k;
  a.exclude_self = 1;
  a.qmode = 2;
  a.qidx = dt;
  a.nq = (int)nt;
  a.nsmooth = nsmooth;
  a.rho = dout;
  a.vden = dout;
  NBK_TRY(launch_knn(a, epi, t->st));
  NBK_TRY(S.finish());
  if (!t->dev()) NBK_TRY(check_err(t, "particle density"));
  return NBK_OK;
}

// The SPH smoothing family (KDCalcSmoothQuantities.cxx). qmode 0: every particle,
// 2: targets (tree indices, as the reference's bucket index), 1: coordinates. rho: the
// particles' densities in input order (the reference's densityset = 1), or null to run
// CalcDensity(nsmooth) first (densityset != 1).
static int smooth_common(nbk_tree* t, int which, int qmode, const int32_t* targets,
                         const double* points, int64_t nq, int nsmooth, int nsearch,
                         const double* rho, const double* smvel, const double* disp,
                         const double* weight, const double* mean, double* out) {
  if (!out || nsmooth < 1 || (qmode == 2 && !targets) || (qmode == 1 && !points) || nq < 0) {
    set_error("smoothing: invalid argument");
    return NBK_ERR_INVALID;
  }
  if (which == kSmVelPhys) {
    if (nsearch < 1) {
      set_error("smoothing: nsearch must be >= 1");
      return NBK_ERR_INVALID;
    }
    if (nsmooth > nsearch) nsmooth = nsearch;  // KDCalcSmoothQuantities.cxx:404-407
  }
  bool needs_vel = which != kSmMeanOne && which != kSmDispOne;
  if (needs_vel && !t->has_vel) {
    set_error("smoothing: this quantity needs velocities at nbk_create");
    return NBK_ERR_INVALID;
  }
  if (((which == kSmVelDisp || which == kSmVelSkew || which == kSmVelKurt ||
        which == kSmVelDispOne) && !smvel) ||
      ((which == kSmVelSkew || which == kSmVelKurt) && !disp) ||
      ((which == kSmMeanOne || which == kSmDispOne) && !weight) ||
      (which == kSmDispOne && !mean)) {
    set_error("smoothing: a required input array is null");
    return NBK_ERR_INVALID;
  }
  int K = which == kSmVelPhys ? nsearch : nsmooth;
  if (K > t->n - (qmode == 1 ? 0 : 1)) {
    set_error("smoothing: " + std::to_string(K) + " neighbours requested from a tree of " +
              std::to_string(t->n) + " particles");
    return NBK_ERR_TOO_FEW;
  }
  if (qmode == 0) nq = t->n;
  if (qmode == 2 && !t->dev()) {
    for (int64_t i = 0; i < nq; i++)
      if (targets[i] < 0 || targets[i] >= t->n) {
        set_error("smoothing: target index out of range");
        return NBK_ERR_INVALID;
      }
  }
  if (nq == 0) return NBK_OK;
  const int width = (which == kSmVelDisp || which == kSmVelDispOne) ? 9
                    : (which == kSmVelPhys || which == kSmMeanOne || which == kSmDispOne) ? 1 : 3;
  Stage S(t);
  const int32_t* dt = nullptr;
  const double *dx = nullptr, *drho = nullptr, *dsv = nullptr, *ddisp = nullptr, *dw = nullptr,
               *dmean = nullptr;
  double* dout = nullptr;
  if (qmode == 2) NBK_TRY(S.in(targets, nq, &dt));
  if (qmode == 1) NBK_TRY(S.in(points, 3 * nq, &dx));
  if (rho) {
    NBK_TRY(S.in(rho, t->n, &drho));
  } else {
    double *scratch, *r;
    NBK_TRY(S.alloc.get((void**)&scratch, sizeof(double) * t->n));
    NBK_TRY(S.alloc.get((void**)&r, sizeof(double) * t->n));
    NBK_TRY(density_into_scratch(t, nsmooth, scratch, r));
    drho = r;
  }
  if (smvel) NBK_TRY(S.in(smvel, 3 * (qmode == 0 ? t->n : nq), &dsv));
  if (disp) NBK_TRY(S.in(disp, 9 * t->n, &ddisp));
  if (weight) NBK_TRY(S.in(weight, t->n, &dw));
  if (mean) NBK_TRY(S.in(mean, nq, &dmean));
  NBK_TRY(S.out(out, (size_t)width * nq, &dout));
  if (qmode == 0 && which != kSmVelPhys)
    NBK_CUDA_TRY(cudaMemsetAsync(dout, 0, sizeof(double) * width * nq, t->st));
  NBK_TRY(clear_err(t));
  KnnArgs a = base_args(t);
  a.tv.periodic = 0;  // the smoothing functions search without images, as CalcDensity
  a.kheap = K;
  a.kout = K;
  a.exclude_self = qmode != 1;
  a.qmode = qmode;
  a.qidx = dt;
  a.qx = dx;
  a.nq = (int)nq;
  a.nsmooth = nsmooth;
  SmoothArgs sa{a, nsmooth, drho, dsv, ddisp, dw, dmean, dout};
  NBK_TRY(launch_smooth(sa, which, t->st));
  NBK_TRY(S.finish());
  if (!t->dev()) NBK_TRY(check_err(t, "smoothing"));
  return NBK_OK;
}

int nbk_smooth_vel(nbk_tree* t, int nsmooth, const double* rho, double* smvel) {
  API_BEGIN
  NBK_TRY(check_phys(t, "nbk_smooth_vel"));
  return smooth_common(t, kSmVel, 0, nullptr, nullptr, 0, nsmooth, 0, rho, nullptr, nullptr,
                       nullptr, nullptr, smvel);
  API_END
}

int nbk_smooth_vel_disp(nbk_tree* t, int nsmooth, const double* rho, const double* smvel,
                        double* disp) {
  API_BEGIN
  NBK_TRY(check_phys(t, "nbk_smooth_vel_disp"));
  return smooth_common(t, kSmVelDisp, 0, nullptr, nullptr, 0, nsmooth, 0, rho, smvel, nullptr,
                       nullptr, nullptr, disp);
  API_END
}

int nbk_smooth_vel_skew(nbk_tree* t, int nsmooth, const double* rho, const double* smvel,
                        const double* disp, double* skew) {
  API_BEGIN
  NBK_TRY(check_phys(t, "nbk_smooth_vel_skew"));
  return smooth_common(t, kSmVelSkew, 0, nullptr, nullptr, 0, nsmooth, 0, rho, smvel, disp,
                       nullptr, nullptr, skew);
  API_END
}

int nbk_smooth_vel_kurtosis(nbk_tree* t, int nsmooth, const double* rho, const double* smvel,
                            const double* disp, double* kurt) {
  API_BEGIN
  NBK_TRY(check_phys(t, "nbk_smooth_vel_kurtosis"));
  return smooth_common(t, kSmVelKurt, 0, nullptr, nullptr, 0, nsmooth, 0, rho, smvel, disp,
                       nullptr, nullptr, kurt);
  API_END
}

int nbk_veldensity_physdensity(nbk_tree* t, int nsmooth, int nsearch, const double* rho,
                               double* vden) {
  API_BEGIN
  NBK_TRY(check_phys(t, "nbk_veldensity_physdensity"));
  return smooth_common(t, kSmVelPhys, 0, nullptr, nullptr, 0, nsmooth, nsearch, rho, nullptr,
                       nullptr, nullptr, nullptr, vden);
  API_END
}

int nbk_veldensity_physdensity_particles(nbk_tree* t, const int32_t* targets, int64_t nt,
                                         int nsmooth, int nsearch, const double* rho,
                                         double* vden) {
  API_BEGIN
  NBK_TRY(check_phys(t, "nbk_veldensity_physdensity_particles"));
  return smooth_common(t, kSmVelPhys, 2, targets, nullptr, nt, nsmooth, nsearch, rho, nullptr,
                       nullptr, nullptr, nullptr, vden);
  API_END
}

int nbk_smooth_vel_particles(nbk_tree* t, const int32_t* targets, int64_t nt, int nsmooth,
                             const double* rho, double* smvel) {
  API_BEGIN
  NBK_TRY(check_phys(t, "nbk_smooth_vel_particles"));
  return smooth_common(t, kSmVelOne, 2, targets, nullptr, nt, nsmooth, 0, rho, nullptr, nullptr,
                       nullptr, nullptr, smvel);
  API_END
}

int nbk_smooth_vel_points(nbk_tree* t, const double* x, int64_t nq, int nsmooth,
                          const double* rho, double* smvel) {
  API_BEGIN
  NBK_TRY(check_phys(t, "nbk_smooth_vel_points"));
  return smooth_common(t, kSmVelOne, 1, nullptr, x, nq, nsmooth, 0, rho, nullptr, nullptr,
                       nullptr, nullptr, smvel);
  API_END
}

int nbk_smooth_vel_disp_particles(nbk_tree* t, const int32_t* targets, int64_t nt, int nsmooth,
                                  const double* rho, const double* smvel, double* disp) {
  API_BEGIN
  NBK_TRY(check_phys(t, "nbk_smooth_vel_disp_particles"));
  return smooth_common(t, kSmVelDispOne, 2, targets, nullptr, nt, nsmooth, 0, rho, smvel,
                       nullptr, nullptr, nullptr, disp);
  API_END
}

int nbk_smooth_vel_disp_points(nbk_tree* t, const double* x, int64_t nq, int nsmooth,
                               const double* rho, const double* smvel, double* disp) {
  API_BEGIN
  NBK_TRY(check_phys(t, "nbk_smooth_vel_disp_points"));
  return smooth_common(t, kSmVelDispOne, 1, nullptr, x, nq, nsmooth, 0, rho, smvel, nullptr,
                       nullptr, nullptr, disp);
  API_END
}

int nbk_smooth_local_mean_particles(nbk_tree* t, const int32_t* targets, int64_t nt,
                                    int nsmooth, const double* rho, const double* weight,
                                    double* mean) {
  API_BEGIN
  NBK_TRY(check_phys(t, "nbk_smooth_local_mean_particles"));
  return smooth_common(t, kSmMeanOne, 2, targets, nullptr, nt, nsmooth, 0, rho, nullptr,
                       nullptr, weight, nullptr, mean);
  API_END
}

int nbk_smooth_local_mean_points(nbk_tree* t, const double* x, int64_t nq, int nsmooth,
                                 const double* rho, const double* weight, double* mean) {
  API_BEGIN
  NBK_TRY(check_phys(t, "nbk_smooth_local_mean_points"));
  return smooth_common(t, kSmMeanOne, 1, nullptr, x, nq, nsmooth, 0, rho, nullptr, nullptr,
                       weight, nullptr, mean);
  API_END
}

int nbk_smooth_local_disp_particles(nbk_tree* t, const int32_t* targets, int64_t nt,
                                    int nsmooth, const double* rho, const double* weight,
                                    const double* mean, double* disp) {
  API_BEGIN
  NBK_TRY(check_phys(t, "nbk_smooth_local_disp_particles"));
  return smooth_common(t, kSmDispOne, 2, targets, nullptr, nt, nsmooth, 0, rho, nullptr,
                       nullptr, weight, mean, disp);
  API_END
}

int nbk_smooth_local_disp_points(nbk_tree* t, const double* x, int64_t nq, int nsmooth,
                                 const double* rho, const double* weight, const double* mean,
                                 double* disp) {
  API_BEGIN
  NBK_TRY(check_phys(t, "nbk_smooth_local_disp_points"));
  return smooth_common(t, kSmDispOne, 1, nullptr, x, nq, nsmooth, 0, rho, nullptr, nullptr,
                       weight, mean, disp);
  API_END
}

int nbk_density_particles(nbk_tree* t, const int32_t* targets, int64_t nt, int k, double* out) {
  API_BEGIN
  NBK_TRY(check_tree(t));
  return particles_common(t, targets, nt, k, k, out, kEpiDensPart);
  API_END
}

int nbk_veldensity_particles(nbk_tree* t, const int32_t* targets, int64_t nt, int nsmooth,
                             int nsearch, double* out) {
  API_BEGIN
  NBK_TRY(check_tree(t));
  if (nsmooth > nsearch) nsmooth = nsearch;
  return particles_common(t, targets, nt, nsearch, nsmooth, out, kEpiVelPart);
  API_END
}

// CalcDensityPosition / CalcVelDensityPosition (KDCalcSmoothQuantities.cxx:1092-1207):
// coordinate queries on a physical tree, nothing excluded, never periodic; the density is
// the gather of CalcDensityParticle, the velocity density uses the given velocities.
static int positions_common(nbk_tree* t, const double* x, const double* v, int64_t nq, int k,
                            int nsmooth, double* out, int epi) {
  if (!x || !out || nq < 0 || k < 1 || (epi == kEpiVelPart && !v)) {
    set_error("position density: invalid argument");
    return NBK_ERR_INVALID;
  }
  if (t->treetype != NBK_TPHYS) {
    // velocity trees: the reference scales the normalisation by metric factors it never
    // sets (KDCalcSmoothQuantities.cxx:1125-1130); phase-space trees: not supported here
    set_error("position density runs on physical trees only");
    return NBK_ERR_UNSUPPORTED;
  }
  if (epi == kEpiVelPart && !t->has_vel) {
    set_error("velocity density needs velocities at nbk_create");
    return NBK_ERR_INVALID;
  }
  if (k > t->n) {
    set_error("position density: k exceeds the number of particles");
    return NBK_ERR_TOO_FEW;
  }
  if (nq == 0) return NBK_OK;
  Stage S(t);
  const double *dx, *dv = nullptr;
  double* dout;
  NBK_TRY(S.in(x, (size_t)nq * 3, &dx));
  if (epi == kEpiVelPart) NBK_TRY(S.in(v, (size_t)nq * 3, &dv));
  NBK_TRY(S.out(out, nq, &dout));
  NBK_TRY(clear_err(t));
  KnnArgs a = base_args(t);
  a.tv.periodic = 0;
  a.kheap = k;
  a.kout = k;
  a.exclude_self = 0;
  a.qmode = 1;
  a.qx = dx;
  a.qv = dv;
  a.nq = (int)nq;
  a.nsmooth = nsmooth;
  a.rho = dout;
  a.vden = dout;
  NBK_TRY(launch_knn(a, epi, t->st));
  NBK_TRY(S.finish());
  if (!t->dev()) NBK_TRY(check_err(t, "position density"));
  return NBK_OK;
}

int nbk_density_points(nbk_tree* t, const double* x, int64_t nq, int k, double* out) {
  API_BEGIN
  NBK_TRY(check_tree(t));
  return positions_common(t, x, nullptr, nq, k, k, out, kEpiDensPart);
  API_END
}

int nbk_veldensity_points(nbk_tree* t, const double* x, const double* v, int64_t nq,
                          int nsmooth, int nsearch, double* out) {
  API_BEGIN
  NBK_TRY(check_tree(t));
  if (nsmooth > nsearch) nsmooth = nsearch;
  return positions_common(t, x, v, nq, nsearch, nsmooth, out, kEpiVelPart);
  API_END
}

static int ball_common(nbk_tree* t, int qmode, const int32_t* targets, const double* x,
                       int64_t nq, double fdist2, int64_t* offsets, int32_t* out,
                       int64_t out_capacity, int64_t* total) {
  if (nq < 0 || !offsets || !total) {
    set_error("ball search: invalid argument");
    return NBK_ERR_INVALID;
  }
  Stage S(t);
  const int* dt = nullptr;
  const double* dx = nullptr;
  if (qmode == 0) NBK_TRY(S.in(targets, nq, &dt));
  else NBK_TRY(S.in(x, nq * 3, &dx));
  int64_t* doff;
  NBK_TRY(S.out(offsets, nq + 1, &doff));
  int* dout = nullptr;
  if (t->dev()) dout = out;
  TreeView tv = t->view();
  // the target version excludes the target (KDLeafNode.cxx:369-382); periodic trees use
  // the coordinate version, which keeps it (KDSplitNode.cxx:1382-1387)
  int excl = (qmode == 0 && !tv.periodic && !t->periodic) ? 1 : 0;
  int64_t tot = 0;
  if (!t->dev()) {
    // count first, then size the device output
    int s = run_ball(tv, qmode, dt, dx, (int)nq, fdist2, excl, doff, nullptr, 0, &tot, S.alloc, t->st);
    *total = tot;
    if (s != NBK_OK && s != NBK_ERR_INVALID) return s;
    if (tot > out_capacity || !out) {
      NBK_TRY(S.finish());
      set_error("ball search: output capacity " + std::to_string(out_capacity) + " < " +
                std::to_string(tot) + " results");
      return NBK_ERR_INVALID;
    }
    NBK_TRY(S.out(out, std::max<int64_t>(tot, 1), &dout));
    NBK_TRY(run_ball(tv, qmode, dt, dx, (int)nq, fdist2, excl, doff, dout, tot, &tot, S.alloc, t->st));
    NBK_TRY(S.finish());
    return NBK_OK;
  }
  int s = run_ball(tv, qmode, dt, dx, (int)nq, fdist2, excl, doff, dout, out_capacity, &tot, S.alloc, t->st);
  *total = tot;
  return s;
}

int nbk_ball_tagged(nbk_tree* t, const int32_t* targets, int64_t ntargets, double fdist2,
                    int64_t* offsets, int32_t* out, int64_t out_capacity, int64_t* total) {
  API_BEGIN
  NBK_TRY(check_phys(t, "nbk_ball_tagged"));
  return ball_common(t, 0, targets, nullptr, ntargets, fdist2, offsets, out, out_capacity, total);
  API_END
}

int nbk_ball_tagged_points(nbk_tree* t, const double* x, int64_t nq, double fdist2,
                           int64_t* offsets, int32_t* out, int64_t out_capacity,
                           int64_t* total) {
  API_BEGIN
  NBK_TRY(check_phys(t, "nbk_ball_tagged_points"));
  return ball_common(t, 1, nullptr, x, nq, fdist2, offsets, out, out_capacity, total);
  API_END
}

int nbk_ball_mark(nbk_tree* t, int32_t target, double fdist2, int32_t imark, int32_t* nn,
                  double* dist2) {
  API_BEGIN
  NBK_TRY(check_phys(t, "nbk_ball_mark"));
  if (!nn || !dist2 || target < 0 || target >= t->n) {
    set_error("nbk_ball_mark: invalid argument");
    return NBK_ERR_INVALID;
  }
  Stage S(t);
  int* dnn;
  double* dd2;
  NBK_TRY(S.out(nn, t->n, &dnn, true));
  NBK_TRY(S.out(dist2, t->n, &dd2, true));
  TreeView tv = t->view();
  int target_search = (!t->periodic) ? 1 : 0;
  NBK_TRY(run_ball_mark(tv, target, fdist2, imark, dnn, dd2, t->arr.perm, target_search, t->st));
  NBK_TRY(S.finish());
  return NBK_OK;
  API_END
}

int nbk_fof(nbk_tree* t, double fdist, int32_t minnum, int order, int32_t* group,
            int32_t* ngroup) {
  API_BEGIN
  NBK_TRY(check_phys(t, "nbk_fof"));
  if (!group || !ngroup || !(fdist >= 0)) {
    set_error("nbk_fof: invalid argument");
    return NBK_ERR_INVALID;
  }
  Stage S(t);
  int* dg;
  NBK_TRY(S.out(group, t->n, &dg));
  int *parent, *gtree;
  // the call ends with a synchronisation (an early return waits too), so this thread's
  // kept block is free again then
  SyncUnlessOk sync_guard{t->st};
  NBK_TRY(thread_scratch_block(2, {{(void**)&parent, sizeof(int) * t->n},
                                   {(void**)&gtree, sizeof(int) * t->n}},
                               t->st, S.alloc));
  NBK_TRY(clear_err(t));
  FofArgs a{};
  a.tv = t->view();
  a.ll2 = fdist * fdist;
  a.parent = parent;
  a.err = t->d_err;
  int ng = 0;
  // the group count and the error word come back together, in one synchronisation
  PinnedScalars* ps = order == 0 ? pinned_scalars() : nullptr;
  NBK_TRY(run_fof(a, (int)t->nslots, minnum, order, gtree, ps ? &ps->i[0] : &ng, S.alloc, t->st,
                  ps != nullptr));
  if (t->n > 0) {
    k_scatter_i<<<(unsigned)((t->n + 255) / 256), 256, 0, t->st>>>(gtree, t->arr.perm, dg, t->n); note_launch();
    NBK_CUDA_TRY(cudaGetLastError());
  }
  NBK_TRY(S.finish());
  if (ps) {
    NBK_CUDA_TRY(cudaMemcpyAsync(&ps->i[1], t->d_err, sizeof(int), cudaMemcpyDeviceToHost, t->st));
    NBK_CUDA_TRY(cudaStreamSynchronize(t->st));
    sync_guard.ok = true;  // synchronised above
    NBK_TRY(err_status(ps->i[1], "nbk_fof"));
    ng = ps->i[0];
  } else {
    sync_guard.ok = true;  // check_err synchronises
    NBK_TRY(check_err(t, "nbk_fof"));
  }
  *ngroup = ng;
  return NBK_OK;
  API_END
}

int nbk_fof_criterion(nbk_tree* t, int comparator, const double* params, int32_t minnum,
                      int order, int32_t* group, int32_t* ngroup) {
  API_BEGIN
  NBK_TRY(check_tree(t));
  if (!group || !ngroup || !params) {
    set_error("nbk_fof_criterion: invalid argument");
    return NBK_ERR_INVALID;
  }
  if (comparator < NBK_FOF3D || comparator > NBK_FOF6D) {
    set_error("nbk_fof_criterion: only the FOF3d, FOFVel and FOF6d comparators run on the GPU");
    return NBK_ERR_UNSUPPORTED;
  }
  if (comparator != NBK_FOF3D && !t->has_vel) {
    set_error("nbk_fof_criterion: FOFVel and FOF6d need velocities at nbk_create");
    return NBK_ERR_INVALID;
  }
  if (t->treetype == NBK_TVEL) {
    // FOFSearchCriterion compares GetPhase(cut_dim), a position, with a velocity cut value
    set_error("nbk_fof_criterion: runs on physical and phase-space trees");
    return NBK_ERR_UNSUPPORTED;
  }
  double p[8];
  if (t->dev()) NBK_CUDA_TRY(cudaMemcpy(p, params, sizeof(p), cudaMemcpyDeviceToHost));
  else memcpy(p, params, sizeof(p));
  Stage S(t);
  int* dg;
  NBK_TRY(S.out(group, t->n, &dg));
  int *parent, *gtree;
  NBK_TRY(S.alloc.get((void**)&parent, sizeof(int) * t->n));
  NBK_TRY(S.alloc.get((void**)&gtree, sizeof(int) * t->n));
  NBK_TRY(clear_err(t));
  FofArgs a{};
  a.tv = t->view();
  a.crit = 1;
  a.cmp = comparator;
  for (int i = 0; i < 8; i++) a.params[i] = p[i];
  {
    // the position search distance^2 of FOFSearchCriterion (its invscaling, from
    // params[0]); when FOF3d / FOF6d accept only pairs inside it, reachability follows
    // from the comparator and the warp-cooperative search applies
    int tt = (int)p[0];
    double s1 = (tt == NBK_TPHYS || tt == NBK_TPHS) ? p[1] : (tt == NBK_TVEL ? p[2] : 1.0);
    if (t->treetype == NBK_TPHYS) {
      a.crit_contained = (comparator == NBK_FOF3D || comparator == NBK_FOF6D) && p[6] > 0 &&
                         s1 > 0 && p[6] <= s1 && (comparator != NBK_FOF6D || p[7] > 0);
    } else {
      // a phase-space tree also cuts velocities, scaled by 1/params[2] for TPHS params
      double s2 = tt == NBK_TPHS ? p[2] : s1;
      a.crit_contained = comparator == NBK_FOF6D && p[6] > 0 && p[7] > 0 && s1 > 0 && s2 > 0 &&
                         p[6] <= s1 && p[7] <= s2;
    }
  }
  a.parent = parent;
  a.err = t->d_err;
  int ng = 0;
  NBK_TRY(run_fof(a, (int)t->nslots, minnum, order, gtree, &ng, S.alloc, t->st));
  k_scatter_i<<<(unsigned)((t->n + 255) / 256), 256, 0, t->st>>>(gtree, t->arr.perm, dg, t->n);
  note_launch();
  NBK_CUDA_TRY(cudaGetLastError());
  NBK_TRY(S.finish());
  NBK_TRY(check_err(t, "nbk_fof_criterion"));
  *ngroup = ng;
  return NBK_OK;
  API_END
}

// FOF over given neighbour lists: nn rows by tree index, numnn tree indices per row;
// values (tree order) replace params[pidx[k]] per target for the distance form.
static int fof_nn_common(nbk_tree* t, int comparator, const double* params, int numnn,
                         const int32_t* nn, const double* values, int npc, const int32_t* pidx,
                         int32_t minnum, int32_t* group, int32_t* ngroup) {
  if (!group || !ngroup || !params || !nn || numnn < 0 || npc < 0 || npc > 8 ||
      (npc > 0 && (!values || !pidx))) {
    set_error("nbk_fof_nn_criterion: invalid argument");
    return NBK_ERR_INVALID;
  }
  if (comparator < NBK_FOF3D || comparator > NBK_FOF6D) {
    set_error("nbk_fof_nn_criterion: only the FOF3d, FOFVel and FOF6d comparators run on the GPU");
    return NBK_ERR_UNSUPPORTED;
  }
  if (comparator != NBK_FOF3D && !t->has_vel) {
    set_error("nbk_fof_nn_criterion: FOFVel and FOF6d need velocities at nbk_create");
    return NBK_ERR_INVALID;
  }
  double p[8];
  int32_t pi[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (t->dev()) {
    NBK_CUDA_TRY(cudaMemcpy(p, params, sizeof(p), cudaMemcpyDeviceToHost));
    if (npc) NBK_CUDA_TRY(cudaMemcpy(pi, pidx, sizeof(int32_t) * npc, cudaMemcpyDeviceToHost));
  } else {
    memcpy(p, params, sizeof(p));
    if (npc) memcpy(pi, pidx, sizeof(int32_t) * npc);
  }
  for (int k = 0; k < npc; k++)
    if (pi[k] < 0 || pi[k] > 7) {
      set_error("nbk_fof_nn_dist_criterion: parameter index outside params[0..7]");
      return NBK_ERR_INVALID;
    }
  Stage S(t);
  const int32_t* dnn;
  const double* dval = nullptr;
  int* dg;
  NBK_TRY(S.in(nn, (size_t)t->n * numnn, &dnn));
  if (npc) NBK_TRY(S.in(values, t->n, &dval));
  NBK_TRY(S.out(group, t->n, &dg));
  int *parent, *gtree;
  NBK_TRY(S.alloc.get((void**)&parent, sizeof(int) * t->n));
  NBK_TRY(S.alloc.get((void**)&gtree, sizeof(int) * t->n));
  NBK_TRY(clear_err(t));
  FofArgs a{};
  a.tv = t->view();
  a.crit = 2;
  a.cmp = comparator;
  for (int i = 0; i < 8; i++) a.params[i] = p[i];
  a.parent = parent;
  a.err = t->d_err;
  a.nn = dnn;
  a.numnn = numnn;
  a.pval = dval;
  a.npc = npc;
  for (int k = 0; k < npc; k++) a.pidx[k] = pi[k];
  int ng = 0;
  // groups are numbered by decreasing size, as the reference's (KDFOF.cxx:493-503)
  NBK_TRY(run_fof(a, (int)t->nslots, minnum, 1, gtree, &ng, S.alloc, t->st));
  k_scatter_i<<<(unsigned)((t->n + 255) / 256), 256, 0, t->st>>>(gtree, t->arr.perm, dg, t->n);
  note_launch();
  NBK_CUDA_TRY(cudaGetLastError());
  NBK_TRY(S.finish());
  NBK_TRY(check_err(t, "nbk_fof_nn_criterion"));
  *ngroup = ng;
  return NBK_OK;
}

int nbk_fof_nn_criterion(nbk_tree* t, int comparator, const double* params, int numnn,
                         const int32_t* nn, int32_t minnum, int32_t* group, int32_t* ngroup) {
  API_BEGIN
  NBK_TRY(check_phys(t, "nbk_fof_nn_criterion"));
  return fof_nn_common(t, comparator, params, numnn, nn, nullptr, 0, nullptr, minnum, group,
                       ngroup);
  API_END
}

int nbk_fof_nn_dist_criterion(nbk_tree* t, int comparator, const double* params, int numnn,
                              const int32_t* nn, const double* values, int npc,
                              const int32_t* pidx, int32_t minnum, int32_t* group,
                              int32_t* ngroup) {
  API_BEGIN
  NBK_TRY(check_phys(t, "nbk_fof_nn_dist_criterion"));
  return fof_nn_common(t, comparator, params, numnn, nn, values, npc, pidx, minnum, group,
                       ngroup);
  API_END
}

int nbk_density_adjoint(nbk_tree* t, int k, const double* w, double* rho, double* grad_pos,
                        double* grad_mass) {
  API_BEGIN
  NBK_TRY(check_phys(t, "nbk_density_adjoint"));
  if (!w || !rho || !grad_pos || !grad_mass || k < 1) {
    set_error("nbk_density_adjoint: invalid argument");
    return NBK_ERR_INVALID;
  }
  if (k > t->n - 1) {
    set_error("nbk_density_adjoint: k exceeds the number of other particles");
    return NBK_ERR_TOO_FEW;
  }
  Stage S(t);
  const double* dw;
  double *drho, *dgp, *dgm;
  NBK_TRY(S.in(w, t->n, &dw));
  NBK_TRY(S.out(rho, t->n, &drho));
  NBK_TRY(S.out(grad_pos, 3 * t->n, &dgp));
  NBK_TRY(S.out(grad_mass, t->n, &dgm));
  int* nn;
  double *trho, *tw, *tgp, *tgm, *tslope;
  NBK_TRY(S.alloc.get((void**)&nn, sizeof(int) * t->n * k));
  NBK_TRY(S.alloc.get((void**)&tslope, sizeof(double) * t->kernres));
  NBK_TRY(S.alloc.get((void**)&trho, sizeof(double) * t->n));
  NBK_TRY(S.alloc.get((void**)&tw, sizeof(double) * t->n));
  NBK_TRY(S.alloc.get((void**)&tgp, sizeof(double) * 3 * t->n));
  NBK_TRY(S.alloc.get((void**)&tgm, sizeof(double) * t->n));
  NBK_CUDA_TRY(cudaMemsetAsync(trho, 0, sizeof(double) * t->n, t->st));
  NBK_TRY(clear_err(t));
  // forward: CalcDensity, keeping each particle's neighbour list
  KnnArgs a = base_args(t);
  a.tv.periodic = 0;
  a.kheap = k;
  a.kout = k;
  a.exclude_self = 1;
  a.qmode = 0;
  a.nq = (int)t->n;
  a.rho = trho;
  a.nn = nn;
  NBK_TRY(launch_knn(a, kEpiDensSave, t->st));
  k_gather_d<<<(unsigned)((t->n + 255) / 256), 256, 0, t->st>>>(dw, t->arr.perm, tw, t->n);
  note_launch();
  NBK_TRY(run_density_adjoint(a.tv, k, nn, tw, trho, t->d_kernel, t->kernres, tslope, tgp, tgm,
                              t->st));
  NBK_TRY(scatter_to_input_order(trho, t->arr.perm, drho, t->n, 1, t->st));
  NBK_TRY(scatter_to_input_order(tgp, t->arr.perm, dgp, t->n, 3, t->st));
  NBK_TRY(scatter_to_input_order(tgm, t->arr.perm, dgm, t->n, 1, t->st));
  NBK_TRY(S.finish());
  if (!t->dev()) NBK_TRY(check_err(t, "nbk_density_adjoint"));
  return NBK_OK;
  API_END
}



}  // extern "C"
