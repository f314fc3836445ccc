// Batched path: many independent trees (one per group, as a halo finder builds per FOF
// group) built and searched together. Replaces a caller loop of
//   KDTree(group particles, b) ; CalcDensity(min(k, n_g - 1))
// (src/KDTree/KDTree.cxx:1238-1306, KDCalcSmoothQuantities.cxx:203-305) per group.
//
//  - build: every group is one tree of a forest; one build_forest call builds them all
//    (groups of <= 1024 particles are finished by one CTA each, larger groups go through
//    the level-synchronous phase together).
//  - search: one persistent launch; its warps pull (group, query bucket) work items, the
//    largest groups first, from an atomic counter.
//  - the zeroing, the search and the scatter back to input order are captured once into
//    a CUDA graph per (k, output) and replayed.
//  - leaf size and query-bucket size are chosen by a small autotuner (bucket_size <= 0 at
//    creation): it times build + search for each candidate on the caller's data.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <numeric>
#include <string>

#include "nbk_build.h"

using namespace nbk;

struct nbk_batch {
  int64_t ntot = 0, ngroups = 0;
  int b = 16, qb = 32;
  int wpq = 1;  // query mapping: 1 a warp per query, 0 a lane per query (32 per warp)
  int kerntype = 0, kernres = 1000;
  unsigned flags = 0;
  cudaStream_t st = nullptr;
  bool own_stream = false;
  std::vector<int64_t> off;
  std::vector<TreeSpec> trees;
  BuiltArrays arr;
  double* d_pos_in = nullptr;
  double* d_mass_in = nullptr;
  bool own_inputs = false;
  TreeInfo* d_trees = nullptr;
  WorkItem* d_items = nullptr;
  int nitems = 0;
  int* d_counter = nullptr;
  int* d_err = nullptr;
  double* d_kernel = nullptr;
  std::vector<double> h_kernel;
  std::vector<double> h_kernel_img;
  double kernnorm = 0;
  double* d_rho_tree = nullptr;
  double* d_rho_out = nullptr;
  float eps = 0;
  std::map<std::pair<int, double*>, cudaGraphExec_t> graphs;
  std::string tune;
  bool dev() const { return flags & NBK_DEVICE_PTRS; }
  TreeView base_view() const {
    TreeView v{};
    v.pos = arr.pos;
    v.posf = arr.posf;
    v.vel = arr.vel;
    v.perm = arr.perm;
    v.node = arr.node;
    v.nodex = arr.nodex;
    v.b = b;
    v.periodic = 0;
    v.eps = eps;
    return v;
  }
};

namespace {

__global__ void k_maxabs(const double* p, int64_t n3, unsigned long long* out) {
  unsigned long long m = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n3;
       i += (int64_t)gridDim.x * blockDim.x) {
    double a = fabs(p[i]);
    unsigned long long u = (unsigned long long)__double_as_longlong(a);
    m = u > m ? u : m;
  }
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long w = __shfl_xor_sync(0xffffffffu, m, o);
    m = w > m ? w : m;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

void free_arrays(nbk_batch* B) {
  dev_free(B->arr.pos, B->st);
  dev_free(B->arr.posf, B->st);
  dev_free(B->arr.perm, B->st);
  dev_free(B->arr.node, B->st);
  dev_free(B->arr.nodex, B->st);
  dev_free(B->d_trees, B->st);
  dev_free(B->d_items, B->st);
  B->arr = BuiltArrays();
  B->d_trees = nullptr;
  B->d_items = nullptr;
}

void drop_graphs(nbk_batch* B) {
  for (auto& g : B->graphs) cudaGraphExecDestroy(g.second);
  B->graphs.clear();
}

// Everything a batch owns on the device (null entries skipped), its graphs and its
// stream; used by nbk_batch_destroy and by a failed nbk_batch_create.
void batch_release(nbk_batch* B) {
  drop_graphs(B);
  free_arrays(B);
  if (B->own_inputs) {
    dev_free(B->d_pos_in, B->st);
    dev_free(B->d_mass_in, B->st);
  }
  void* owned[] = {B->d_kernel, B->d_counter, B->d_err, B->d_rho_tree, B->d_rho_out};
  for (void* p : owned) dev_free(p, B->st);
  B->d_pos_in = B->d_mass_in = B->d_kernel = B->d_rho_tree = B->d_rho_out = nullptr;
  B->d_counter = B->d_err = nullptr;
  if (B->st) cudaStreamSynchronize(B->st);
  if (B->own_stream && B->st) cudaStreamDestroy(B->st);
  B->st = nullptr;
  B->own_stream = false;
}

// Work items: (tree, q0, count) buckets of qb queries, largest trees first.
int make_items(nbk_batch* B, int qb) {
  std::vector<int> order(B->ngroups);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int c) { return B->trees[a].n > B->trees[c].n; });
  std::vector<WorkItem> items;
  items.reserve(B->ntot / qb + B->ngroups);
  for (int g : order)
    for (int64_t q = 0; q < B->trees[g].n; q += qb)
      items.push_back({g, (int)q, (int)std::min<int64_t>(qb, B->trees[g].n - q), 0});
  dev_free(B->d_items, B->st);
  NBK_TRY(dev_malloc((void**)&B->d_items, sizeof(WorkItem) * std::max<size_t>(1, items.size()), B->st));
  NBK_CUDA_TRY(cudaMemcpyAsync(B->d_items, items.data(), sizeof(WorkItem) * items.size(),
                               cudaMemcpyHostToDevice, B->st));
  NBK_CUDA_TRY(cudaStreamSynchronize(B->st));
  B->nitems = (int)items.size();
  B->qb = qb;
  drop_graphs(B);
  return NBK_OK;
}

// (Re)build every tree with leaf size b.
int batch_build(nbk_batch* B, int b) {
  free_arrays(B);
  drop_graphs(B);
  B->b = b;
  int64_t nb = 0;
  B->trees.resize(B->ngroups);
  std::vector<TreeInfo> info(B->ngroups);
  for (int64_t g = 0; g < B->ngroups; g++) {
    int64_t n = B->off[g + 1] - B->off[g];
    B->trees[g] = {B->off[g], n, (int)nb};
    info[g] = {(int)B->off[g], (int)n, (int)nb, 0};
    nb += n > 0 ? heap_slots(n, b) : 0;
  }
  int64_t n = B->ntot;
  cudaStream_t st = B->st;
  NBK_TRY(dev_malloc((void**)&B->arr.pos, sizeof(P4) * std::max<int64_t>(n, 1), st));
  NBK_TRY(dev_malloc((void**)&B->arr.posf, sizeof(float4) * std::max<int64_t>(n, 1), st));
  NBK_TRY(dev_malloc((void**)&B->arr.perm, sizeof(int) * std::max<int64_t>(n, 1), st));
  NBK_TRY(dev_malloc((void**)&B->arr.node, sizeof(NodeRec) * std::max<int64_t>(nb, 1), st));
  NBK_TRY(dev_malloc((void**)&B->arr.nodex, sizeof(NodeX) * std::max<int64_t>(nb, 1), st));
  NBK_CUDA_TRY(cudaMemsetAsync(B->arr.node, 0, sizeof(NodeRec) * std::max<int64_t>(nb, 1), st));
  NBK_TRY(dev_malloc((void**)&B->d_trees, sizeof(TreeInfo) * std::max<int64_t>(B->ngroups, 1), st));
  NBK_CUDA_TRY(cudaMemcpyAsync(B->d_trees, info.data(), sizeof(TreeInfo) * info.size(),
                               cudaMemcpyHostToDevice, st));
  DevAlloc alloc;
  alloc.st = st;
  std::vector<TreeSpec> nonempty;
  for (auto& t : B->trees)
    if (t.n > 0) nonempty.push_back(t);
  NBK_TRY(build_forest(nonempty, b, B->d_pos_in, B->d_mass_in, nullptr, B->arr, alloc, st));
  return make_items(B, B->qb);
}

KnnArgs batch_args(nbk_batch* B, int k) {
  KnnArgs a{};
  a.tv = B->base_view();
  a.kheap = k;
  a.kout = k;
  a.exclude_self = 1;
  a.kernel = B->d_kernel;
  a.kernres = B->kernres;
  a.rho = B->d_rho_tree;
  a.err = B->d_err;
  return a;
}

// The batched density sequence on the batch stream (capturable).
int density_sequence(nbk_batch* B, int k, double* out) {
  NBK_CUDA_TRY(cudaMemsetAsync(B->d_rho_tree, 0, sizeof(double) * B->ntot, B->st));
  NBK_CUDA_TRY(cudaMemsetAsync(B->d_counter, 0, sizeof(int), B->st));
  KnnArgs a = batch_args(B, k);
  BatchArgs ba{B->d_items, B->d_trees, B->nitems, B->d_counter, B->wpq};
  NBK_TRY(launch_knn_batch(a, ba, B->st));
  NBK_TRY(scatter_to_input_order(B->d_rho_tree, B->arr.perm, out, B->ntot, 1, B->st));
  return NBK_OK;
}

int run_density(nbk_batch* B, int k, double* out, int use_graph) {
  if (!use_graph) return density_sequence(B, k, out);
  auto key = std::make_pair(k * 2 + B->wpq, out);
  auto it = B->graphs.find(key);
  if (it == B->graphs.end()) {
    // first use outside capture sets kernel attributes and sizes the persistent grid
    NBK_TRY(density_sequence(B, k, out));
    NBK_CUDA_TRY(cudaStreamSynchronize(B->st));
    cudaGraph_t g;
    NBK_CUDA_TRY(cudaStreamBeginCapture(B->st, cudaStreamCaptureModeThreadLocal));
    int s = density_sequence(B, k, out);
    cudaError_t e = cudaStreamEndCapture(B->st, &g);
    if (s != NBK_OK) return s;
    NBK_CUDA_TRY(e);
    cudaGraphExec_t ex;
    NBK_CUDA_TRY(cudaGraphInstantiate(&ex, g, 0));
    cudaGraphDestroy(g);
    it = B->graphs.emplace(key, ex).first;
  }
  NBK_CUDA_TRY(cudaGraphLaunch(it->second, B->st));
  note_launch();
  return NBK_OK;
}

int check_batch_err(nbk_batch* B) {
  int h = 0;
  NBK_CUDA_TRY(cudaMemcpyAsync(&h, B->d_err, sizeof(int), cudaMemcpyDeviceToHost, B->st));
  NBK_CUDA_TRY(cudaStreamSynchronize(B->st));
  if (h) {
    set_error("batched density: device check failed (code " + std::to_string(h) + ")");
    return h == kErrTooFew ? NBK_ERR_TOO_FEW : NBK_ERR_DEVICE;
  }
  return NBK_OK;
}

float elapsed_ms(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0;
  cudaEventSynchronize(b);
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

struct EventPair {
  cudaEvent_t a = nullptr, b = nullptr;
  EventPair() {
    cudaEventCreate(&a);
    cudaEventCreate(&b);
  }
  ~EventPair() {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
  }
};

float median3(float x, float y, float z) {
  return std::max(std::min(x, y), std::min(std::max(x, y), z));
}

// Autotuner: leaf size b, query-bucket size qb and the query mapping (a warp per query,
// or a lane per query with 32 queries per warp) minimising build + batched search for the
// caller's groups with k = 32 (the density workload's k). Every candidate is timed three
// times after a warm-up run and scored by the medians.
int autotune(nbk_batch* B) {
  const int bs[] = {8, 12, 16, 24, 32};
  const int qbs[] = {16, 32};
  const int wpqs[] = {1, 0};
  EventPair ev;
  double best = 1e30;
  int bb = 16, bq = 32, bw = 1;
  std::string rep = "{";
  for (int b : bs) {
    B->qb = 32;
    float tb[3];
    for (int r = 0; r < 3; r++) {
      cudaEventRecord(ev.a, B->st);
      NBK_TRY(batch_build(B, b));
      cudaEventRecord(ev.b, B->st);
      tb[r] = elapsed_ms(ev.a, ev.b);
    }
    float build_ms = median3(tb[0], tb[1], tb[2]);
    for (int qb : qbs) {
      NBK_TRY(make_items(B, qb));
      for (int wpq : wpqs) {
        B->wpq = wpq;
        NBK_TRY(density_sequence(B, 32, B->d_rho_out));  // warm
        float td[3];
        for (int r = 0; r < 3; r++) {
          cudaEventRecord(ev.a, B->st);
          NBK_TRY(density_sequence(B, 32, B->d_rho_out));
          cudaEventRecord(ev.b, B->st);
          td[r] = elapsed_ms(ev.a, ev.b);
        }
        float dens_ms = median3(td[0], td[1], td[2]);
        double score = build_ms + dens_ms;
        char tmp[160];
        snprintf(tmp, sizeof(tmp), "%s\"b%d_qb%d_wpq%d\": [%.4f, %.4f]",
                 rep.size() > 1 ? ", " : "", b, qb, wpq, build_ms, dens_ms);
        rep += tmp;
        if (score < best) {
          best = score;
          bb = b;
          bq = qb;
          bw = wpq;
        }
      }
    }
  }
  rep += "}";
  NBK_TRY(check_batch_err(B));
  B->tune = "{\"chosen\": {\"b\": " + std::to_string(bb) + ", \"qb\": " + std::to_string(bq) +
            ", \"warp_per_query\": " + std::to_string(bw) +
            "}, \"runs_per_candidate\": 3, \"median_ms_build_search\": " + rep + "}";
  B->qb = bq;
  B->wpq = bw;
  return batch_build(B, bb);
}

}  // namespace

#define BAPI_BEGIN try {
#define BAPI_END                                         \
  }                                                      \
  catch (const std::exception& e) {                      \
    set_error(std::string("exception: ") + e.what());    \
    return NBK_ERR_INVALID;                              \
  }

extern "C" {

int nbk_batch_create(const double* pos, const double* mass, const int64_t* offsets,
                     int64_t ngroups, int bucket_size, int kerntype, int kernres,
                     unsigned flags, nbk_batch** out) {
  BAPI_BEGIN
  if (!out || !pos || !offsets || ngroups < 1) {
    set_error("nbk_batch_create: invalid argument");
    return NBK_ERR_INVALID;
  }
  *out = nullptr;
  if (bucket_size >= kLocalMax) {
    set_error("nbk_batch_create: bucket sizes >= 1024 are not supported");
    return NBK_ERR_UNSUPPORTED;
  }
  std::unique_ptr<nbk_batch> B(new nbk_batch);
  // a failed creation frees whatever it had already allocated
  struct ReleaseOnFailure {
    nbk_batch* B;
    ~ReleaseOnFailure() {
      if (B) batch_release(B);
    }
  } guard{B.get()};
  B->ngroups = ngroups;
  B->flags = flags;
  B->kerntype = (kerntype >= NBK_KSPH && kerntype <= NBK_KTH) ? kerntype : NBK_KSPH;
  B->kernres = kernres < 100 ? 100 : kernres;
  NBK_CUDA_TRY(cudaStreamCreateWithFlags(&B->st, cudaStreamNonBlocking));
  B->own_stream = true;
  B->off.resize(ngroups + 1);
  if (flags & NBK_DEVICE_PTRS)
    NBK_CUDA_TRY(cudaMemcpy(B->off.data(), offsets, sizeof(int64_t) * (ngroups + 1),
                            cudaMemcpyDeviceToHost));
  else
    memcpy(B->off.data(), offsets, sizeof(int64_t) * (ngroups + 1));
  if (B->off[0] != 0) {
    set_error("nbk_batch_create: offsets[0] must be 0");
    return NBK_ERR_INVALID;
  }
  for (int64_t g = 0; g < ngroups; g++)
    if (B->off[g + 1] < B->off[g]) {
      set_error("nbk_batch_create: offsets must be non-decreasing");
      return NBK_ERR_INVALID;
    }
  B->ntot = B->off[ngroups];
  if (B->ntot > (int64_t)0x7fffff00) {
    set_error("nbk_batch_create: more than 2^31 particles");
    return NBK_ERR_INVALID;
  }
  int64_t n = std::max<int64_t>(B->ntot, 1);
  cudaStream_t st = B->st;
  if (flags & NBK_DEVICE_PTRS) {
    B->d_pos_in = const_cast<double*>(pos);
    B->d_mass_in = const_cast<double*>(mass);
  } else {
    B->own_inputs = true;  // before the allocations: a failed one frees the other
    NBK_TRY(dev_malloc((void**)&B->d_pos_in, sizeof(double) * 3 * n, st));
    NBK_CUDA_TRY(cudaMemcpyAsync(B->d_pos_in, pos, sizeof(double) * 3 * B->ntot,
                                 cudaMemcpyHostToDevice, st));
    if (mass) {
      NBK_TRY(dev_malloc((void**)&B->d_mass_in, sizeof(double) * n, st));
      NBK_CUDA_TRY(cudaMemcpyAsync(B->d_mass_in, mass, sizeof(double) * B->ntot,
                                   cudaMemcpyHostToDevice, st));
    }
  }
  kernel_table(B->kerntype, B->kernres, 3, B->h_kernel, B->kernnorm);
  kernel_device_image(B->h_kernel, B->h_kernel_img);
  NBK_TRY(dev_malloc((void**)&B->d_kernel, sizeof(double) * B->h_kernel_img.size(), st));
  NBK_CUDA_TRY(cudaMemcpyAsync(B->d_kernel, B->h_kernel_img.data(),
                               sizeof(double) * B->h_kernel_img.size(), cudaMemcpyHostToDevice, st));
  NBK_TRY(dev_malloc((void**)&B->d_counter, sizeof(int), st));
  NBK_TRY(dev_malloc((void**)&B->d_err, sizeof(int), st));
  NBK_CUDA_TRY(cudaMemsetAsync(B->d_err, 0, sizeof(int), st));
  NBK_TRY(dev_malloc((void**)&B->d_rho_tree, sizeof(double) * n, st));
  NBK_TRY(dev_malloc((void**)&B->d_rho_out, sizeof(double) * n, st));
  // FP32 rounding bound of every coordinate
  unsigned long long* d_m;
  DevAlloc tmp;  // frees d_m on every path out
  tmp.st = st;
  NBK_TRY(tmp.get((void**)&d_m, sizeof(unsigned long long)));
  NBK_CUDA_TRY(cudaMemsetAsync(d_m, 0, sizeof(unsigned long long), st));
  if (B->ntot > 0) {
    k_maxabs<<<256, 256, 0, st>>>(B->d_pos_in, 3 * B->ntot, d_m);
    note_launch();
  }
  unsigned long long hm = 0;
  NBK_CUDA_TRY(cudaMemcpyAsync(&hm, d_m, sizeof(hm), cudaMemcpyDeviceToHost, st));
  NBK_CUDA_TRY(cudaStreamSynchronize(st));
  double maxabs;
  memcpy(&maxabs, &hm, sizeof(double));
  if (!std::isfinite(maxabs)) {
    set_error("nbk_batch_create: positions contain NaN or infinity");
    return NBK_ERR_INVALID;
  }
  B->eps = (float)std::ldexp(maxabs, -23) * 1.0001f + 1e-38f;
  if (bucket_size <= 0) NBK_TRY(autotune(B.get()));
  else NBK_TRY(batch_build(B.get(), bucket_size));
  guard.B = nullptr;
  *out = B.release();
  return NBK_OK;
  BAPI_END
}

int nbk_batch_destroy(nbk_batch* B) {
  if (!B) return NBK_OK;
  batch_release(B);
  delete B;
  return NBK_OK;
}

int nbk_batch_set_stream(nbk_batch* B, void* stream) {
  if (!B) {
    set_error("null batch");
    return NBK_ERR_INVALID;
  }
  cudaStreamSynchronize(B->st);
  if (B->own_stream) cudaStreamDestroy(B->st);
  B->own_stream = false;
  B->st = (cudaStream_t)stream;
  return NBK_OK;
}

int nbk_batch_get_params(const nbk_batch* B, int32_t* bucket_size, int32_t* query_bucket,
                         char* tune_json, int64_t cap) {
  if (!B) {
    set_error("null batch");
    return NBK_ERR_INVALID;
  }
  if (bucket_size) *bucket_size = B->b;
  if (query_bucket) *query_bucket = B->qb;
  if (tune_json && cap > 0) {
    int64_t m = std::min<int64_t>(cap - 1, (int64_t)B->tune.size());
    memcpy(tune_json, B->tune.data(), m);
    tune_json[m] = 0;
  }
  return NBK_OK;
}

int nbk_batch_set_query_mapping(nbk_batch* B, int warp_per_query) {
  if (!B || (warp_per_query != 0 && warp_per_query != 1)) {
    set_error("nbk_batch_set_query_mapping: null batch or mapping other than 0 / 1");
    return NBK_ERR_INVALID;
  }
  B->wpq = warp_per_query;
  return NBK_OK;
}

int nbk_batch_get_query_mapping(const nbk_batch* B, int32_t* warp_per_query) {
  if (!B || !warp_per_query) {
    set_error("nbk_batch_get_query_mapping: null argument");
    return NBK_ERR_INVALID;
  }
  *warp_per_query = B->wpq;
  return NBK_OK;
}

int nbk_batch_density(nbk_batch* B, int k, double* rho, int use_graph) {
  BAPI_BEGIN
  if (!B || !rho || k < 1) {
    set_error("nbk_batch_density: invalid argument");
    return NBK_ERR_INVALID;
  }
  double* out = B->dev() ? rho : B->d_rho_out;
  NBK_CUDA_TRY(cudaMemsetAsync(B->d_err, 0, sizeof(int), B->st));
  NBK_TRY(run_density(B, k, out, use_graph));
  if (!B->dev()) {
    NBK_CUDA_TRY(cudaMemcpyAsync(rho, out, sizeof(double) * B->ntot, cudaMemcpyDeviceToHost, B->st));
    NBK_TRY(check_batch_err(B));
  }
  return NBK_OK;
  BAPI_END
}

// The plain method: per group, (optionally) a tree build and one kNN-density launch, in a
// host loop over groups.
static int pertree(nbk_batch* B, int k, double* rho, bool build) {
  if (!B || !rho || k < 1) {
    set_error("nbk_batch_density_pertree: invalid argument");
    return NBK_ERR_INVALID;
  }
  double* out = B->dev() ? rho : B->d_rho_out;
  cudaStream_t st = B->st;
  NBK_CUDA_TRY(cudaMemsetAsync(B->d_err, 0, sizeof(int), st));
  NBK_CUDA_TRY(cudaMemsetAsync(B->d_rho_tree, 0, sizeof(double) * B->ntot, st));
  for (int64_t g = 0; g < B->ngroups; g++) {
    const TreeSpec& ts = B->trees[g];
    if (ts.n < 2) continue;
    if (build) {
      DevAlloc alloc;
      alloc.st = st;
      std::vector<TreeSpec> one{ts};
      NBK_TRY(build_forest(one, B->b, B->d_pos_in, B->d_mass_in, nullptr, B->arr, alloc, st));
    }
    KnnArgs a = batch_args(B, std::min<int64_t>(k, ts.n - 1));
    a.tv.n = (int)ts.n;
    a.tv.pstart = (int)ts.pstart;
    a.tv.nbase = ts.nbase;
    a.qmode = 0;
    a.q0 = (int)ts.pstart;
    a.nq = (int)ts.n;
    NBK_TRY(launch_knn(a, kEpiDensity, st));
  }
  NBK_TRY(scatter_to_input_order(B->d_rho_tree, B->arr.perm, out, B->ntot, 1, st));
  if (!B->dev())
    NBK_CUDA_TRY(cudaMemcpyAsync(rho, out, sizeof(double) * B->ntot, cudaMemcpyDeviceToHost, st));
  NBK_TRY(check_batch_err(B));
  return NBK_OK;
}

int nbk_batch_density_pertree(nbk_batch* B, int k, double* rho) {
  BAPI_BEGIN
  return pertree(B, k, rho, true);
  BAPI_END
}

int nbk_batch_density_pertree_search(nbk_batch* B, int k, double* rho) {
  BAPI_BEGIN
  return pertree(B, k, rho, false);
  BAPI_END
}

}  // extern "C"
