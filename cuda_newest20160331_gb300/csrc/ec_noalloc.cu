// Eigenvector centrality for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc at the point where they need
// centrality: a process whose device memory is fully reserved by its own
// pool (another framework's caching allocator holding the rest of HBM), or
// an embedder that forbids the library any allocation after load so that
// its memory use stays fixed and known in advance.  bna_ec_noalloc serves
// them: it runs the same power-iteration kernels as bna_ec, but its working
// vectors, block partials and iteration state live in one file-scope
// __device__ array of fixed size, so the call itself allocates nothing (no
// cudaMalloc / cudaFree, no context, no pinned buffer, no graph).  The
// caller passes the CSR and the output vector.
//
// It is called from ordinary host code: it issues CUDA calls (memset, kernel
// launches, copies, a stream synchronisation), which CUDA does not allow
// inside a stream callback or a cudaLaunchHostFunc function.
//
// Limits and sharing rules:
//   - N <= kNoAllocMaxN (262,144 vertices); larger graphs get
//     BNA_SCRATCH_LIMIT.  The array holds 4 * kNoAllocMaxN doubles plus block
//     partials and state (about 8 MB); every GPU that loads the library keeps
//     it until the process exits.
//   - Every call shares the array.  Calls that overlap on a GPU (two host
//     threads, or two streams running at once) race on it; serialise them.
//   - The first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (a one-time set-up per device, done with that
//     device current).  Make that first call before any stream capture.  The
//     address is kept per CUDA context (its unique id): after a
//     cudaDeviceReset the next call looks it up again in the new context.
#include <algorithm>
#include <mutex>

#include <cuda.h>

#include "common.cuh"

namespace bna {
size_t ec_state_bytes();
cudaError_t launch_ec_init(int n, double* u, float2* uf, double* parts, void* st, int grid,
                           int max_iter, cudaStream_t stream);
cudaError_t launch_ec_iter(int n, const int32_t* rp, const int32_t* ci, const float* val,
                           const double* vald, long long nnz_used, const double* u,
                           const float2* uf, double* un, float2* unf, double* parts, void* st,
                           int grid, int max_iter, double eps, cudaStream_t stream);
void ec_state_read(const void* host_copy, double* lam2, double* lambda_used, double* e1,
                   double* e2, int* iter, int* done);
int ec_state_err(const void* host_copy);
int ec_coop_grid(int n, int sms);
cudaError_t launch_ec_coop(int n, const int32_t* rp, const int32_t* ci, const float* val,
                           const double* vald, long long nnz_used, double* u, float2* uf,
                           double* parts, void* st, int grid, int it_end, int max_iter,
                           double eps, cudaStream_t stream);
}  // namespace bna

namespace {

constexpr int kNoAllocMaxN = 1 << 18;
constexpr int kNoAllocMaxGrid = 1024;
constexpr size_t kStateDoubles = 16;  // >= sizeof(EcState) / 8
// two double iterates, their two (hi, lo) float copies, block partials, state
constexpr size_t kScratchDoubles =
    4 * (size_t)kNoAllocMaxN + 3 * (size_t)kNoAllocMaxGrid + kStateDoubles;

// The scratch.  Host code must not take its address directly (that is a host
// stand-in); the device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) double g_ec_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
double* g_scratch_ptr[kMaxDevices] = {};
int g_sms[kMaxDevices] = {};
unsigned long long g_ctx_id[kMaxDevices] = {};

// Unique id of the current CUDA context (cuCtxGetId through the runtime's
// driver entry point), or 0 when it cannot be read.
unsigned long long current_ctx_id() {
  using Fn = CUresult (*)(CUcontext, unsigned long long*);
  static Fn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      return (Fn) nullptr;
    }
    return reinterpret_cast<Fn>(p);
  }();
  unsigned long long id = 0;
  if (!fn || fn(nullptr, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// One-time set-up per device and context (the device must be current).
int32_t setup_device(int dev, double** ptr, int* sms) {
  if (dev < 0 || dev >= kMaxDevices) return BNA_BAD_ARG;
  std::lock_guard<std::mutex> lk(g_setup_mu);
  const unsigned long long ctx = current_ctx_id();
  if (!g_scratch_ptr[dev] || ctx == 0 || ctx != g_ctx_id[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_ec_scratch) != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      return BNA_CUDA_ERROR;
    }
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
      cudaGetLastError();
      return BNA_CUDA_ERROR;
    }
    g_sms[dev] = n;
    g_scratch_ptr[dev] = static_cast<double*>(p);
    g_ctx_id[dev] = ctx;
  }
  *ptr = g_scratch_ptr[dev];
  *sms = g_sms[dev];
  return BNA_OK;
}

}  // namespace

extern "C" int32_t bna_ec_noalloc(const bna_csr* csr_dev, int32_t max_iter, double eps,
                                  double* ec_dev, double* lambda, int32_t* iters, void* stream) {
  using namespace bna;
  if (!csr_dev || !ec_dev || csr_dev->n < 1 || !csr_dev->row_ptr ||
      (csr_dev->nnz > 0 && !csr_dev->col_idx) || csr_dev->nnz < 0)
    return BNA_BAD_ARG;
  if (csr_dev->n > kNoAllocMaxN) return BNA_SCRATCH_LIMIT;
  if (ec_state_bytes() > kStateDoubles * sizeof(double)) return BNA_INTERNAL;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return BNA_CUDA_ERROR;
  }
  double* scratch = nullptr;
  int sms = 0;
  int32_t s = setup_device(dev, &scratch, &sms);
  if (s != BNA_OK) return s;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const int n = csr_dev->n;
  const int grid = std::max(1, std::min(sms * 4, kNoAllocMaxGrid));
  double* u = scratch;                                                   // 2 * kNoAllocMaxN
  float2* uf = reinterpret_cast<float2*>(scratch + 2 * (size_t)kNoAllocMaxN);  // 2 * kNoAllocMaxN
  double* parts = scratch + 4 * (size_t)kNoAllocMaxN;                   // 3 * kNoAllocMaxGrid
  void* state = parts + 3 * (size_t)kNoAllocMaxGrid;    // kStateDoubles
  const long long nnz_used = 2 * (csr_dev->nnz / 2);
  // The array keeps the previous call's contents: the state block (with the
  // last-block counter) must start at zero; u and the partials are fully
  // written by the init kernel before they are read.
  cudaError_t e = cudaMemsetAsync(state, 0, ec_state_bytes(), st);
  if (e == cudaSuccess) e = launch_ec_init(n, u, uf, parts, state, grid, max_iter, st);
  if (e != cudaSuccess) return BNA_CUDA_ERROR;
  alignas(16) unsigned char host_state[kStateDoubles * sizeof(double)];
  double lam2 = 0, lam = 0, e1 = 0, e2 = 0;
  int it = 0, done = 0;
  // the same choice as bna_ec: small graphs run as one persistent launch
  // (its 2 x grid x 3 partials fit the partials region: grid <= SM count)
  const int cgrid = std::min(ec_coop_grid(n, sms), kNoAllocMaxGrid / 2);
  if (cgrid > 0) {
    e = launch_ec_coop(n, csr_dev->row_ptr, csr_dev->col_idx, csr_dev->val, nullptr, nnz_used, u,
                       uf, parts, state, cgrid, max_iter, max_iter, eps, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(host_state, state, ec_state_bytes(), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return BNA_CUDA_ERROR;
    if (ec_state_err(host_state)) return BNA_TIMEOUT;
    ec_state_read(host_state, &lam2, &lam, &e1, &e2, &it, &done);
    done = 1;
  }
  const int chunk = 32;
  for (int launched = 0; launched < max_iter && !done; launched += chunk) {
    for (int k = 0; k < chunk; ++k) {
      const int gi = launched + k;
      const size_t cur = (size_t)(gi & 1) * n, nxt = (size_t)((gi + 1) & 1) * n;
      e = launch_ec_iter(n, csr_dev->row_ptr, csr_dev->col_idx, csr_dev->val, nullptr, nnz_used,
                         u + cur, uf + cur, u + nxt, uf + nxt, parts, state, grid, max_iter, eps,
                         st);
      if (e != cudaSuccess) return BNA_CUDA_ERROR;
    }
    // pageable stack buffer: the copy is synchronous with respect to the host
    e = cudaMemcpyAsync(host_state, state, ec_state_bytes(), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return BNA_CUDA_ERROR;
    ec_state_read(host_state, &lam2, &lam, &e1, &e2, &it, &done);
  }
  if (max_iter <= 0) {
    e = cudaMemcpyAsync(host_state, state, ec_state_bytes(), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return BNA_CUDA_ERROR;
    ec_state_read(host_state, &lam2, &lam, &e1, &e2, &it, &done);
  }
  e = cudaMemcpyAsync(ec_dev, u + (size_t)(it & 1) * n, (size_t)n * sizeof(double),
                      cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return BNA_CUDA_ERROR;
  if (lambda) *lambda = lam;
  if (iters) *iters = it;
  return (e1 <= eps || e2 <= eps) ? BNA_OK : BNA_NOT_CONVERGED;
}
