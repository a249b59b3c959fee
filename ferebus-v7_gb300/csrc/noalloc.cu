// fgpu_loglik_noalloc: one log-likelihood evaluation that allocates nothing.
//
// Who needs it: hosts that may not call cudaMalloc at the moment they want a
// likelihood -- a Fortran/OpenACC host whose device memory is owned by the
// OpenACC runtime's data regions, or a host whose caching pool forbids side
// allocations.  They pass device pointers for the inputs and outputs; every
// intermediate (feature planes, the kernel matrix K, log-det partials,
// status words, descriptors) lives in one file-scope device array of fixed
// size, so N is limited to NOALLOC_MAX_N and the feature planes to
// NOALLOC_MAX_PLANES.  The descriptors travel as kernel arguments, so the
// call enqueues its work and returns without waiting for the stream.
//
// The array is shared by every call in the process on that device and keeps
// the previous call's contents; the status words are cleared at the start of
// each call.  Two calls whose work overlaps on the GPU (different streams,
// or different host threads) race on the array: serialise them.
//
// Set-up: the first call on a device resolves the array's device address
// with cudaGetSymbolAddress (with that device current) and caches it; make
// that first call before any stream capture begins.
#include "../../include/fgpu.h"
#include "fgpu_internal.h"

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

namespace fgpu {
namespace {

constexpr int NOALLOC_MAX_N = FGPU_NOALLOC_MAX_N;
constexpr int NOALLOC_MAX_PLANES = FGPU_NOALLOC_MAX_PLANES;
constexpr int NA_NC = NOALLOC_MAX_N;               // Nc = N rounded up to TB
constexpr int NA_LD = NA_NC + TB;
constexpr int NA_STEPS = NA_NC / TB;

constexpr size_t align256(size_t v) { return (v + 255) / 256 * 256; }
constexpr size_t OFF_PROB = 0;
constexpr size_t OFF_SPEC = align256(OFF_PROB + sizeof(Prob));
constexpr size_t OFF_PLANES = align256(OFF_SPEC + sizeof(Spec));
constexpr size_t OFF_K = align256(OFF_PLANES + sizeof(double) * NOALLOC_MAX_PLANES * NA_NC);
constexpr size_t OFF_LOGDET = align256(OFF_K + sizeof(double) * (size_t)NA_LD * NA_NC);
constexpr size_t OFF_STATUS = align256(OFF_LOGDET + sizeof(double) * (NA_STEPS + 1));
constexpr size_t OFF_OUT = align256(OFF_STATUS + sizeof(int) * 4);
constexpr size_t OFF_Z = align256(OFF_OUT + sizeof(double) * 8);
constexpr size_t SCRATCH_BYTES = align256(OFF_Z + sizeof(double) * NA_NC);  // about 9.5 MB
static_assert(SCRATCH_BYTES < (size_t)16 << 20, "no-alloc scratch must stay modest");

// The scratch.  In host code this name is only a stand-in: kernels get the
// address resolved by cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[SCRATCH_BYTES];

std::mutex g_addr_mu;
unsigned char* g_addr[128];

struct PlaneMap {
  int n;
  int dim[NOALLOC_MAX_PLANES];
  int kind[NOALLOC_MAX_PLANES];  // 0: x, 1: sin(x/2), 2: cos(x/2), 3: x (cyclic-wrapped dim)
};

// planes[p][i] from the caller's column-major X(N, d) on the device.
__global__ void k_noalloc_planes(const double* __restrict__ X, int N, int Nc, PlaneMap pm,
                                 double* __restrict__ planes) {
  const int p = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= pm.n || i >= Nc) return;
  double v = 0.0;
  if (i < N) {
    const double x = X[(size_t)pm.dim[p] * N + i];
    v = pm.kind[p] == 1 ? sin(x / 2.0) : (pm.kind[p] == 2 ? cos(x / 2.0) : x);
  }
  planes[(size_t)p * Nc + i] = v;
}

// The call's descriptors reach the scratch as kernel arguments (no host
// staging buffer, so the call never waits for earlier work on the stream),
// and the status words start at zero.
__global__ void k_noalloc_desc(Prob P, Spec sp, Prob* __restrict__ pd, Spec* __restrict__ sd,
                               int* __restrict__ status) {
  if (threadIdx.x == 0) {
    *pd = P;
    *sd = sp;
    for (int k = 0; k < 4; ++k) status[k] = 0;
  }
}

int scratch_address(int dev, unsigned char** out) {
  if (dev < 0 || dev >= 128) return internal_fail(FGPU_ENODEV, "device index out of range");
  std::lock_guard<std::mutex> lk(g_addr_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      std::string m = std::string("cudaGetSymbolAddress(no-alloc scratch): ") + cudaGetErrorString(e);
      return internal_fail(FGPU_ECUDA, m.c_str());
    }
    g_addr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_addr[dev];
  return 0;
}

#define NA_CK(call)                                                                  \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess) {                                                         \
      std::string m_ = std::string(#call) + ": " + cudaGetErrorString(e_);           \
      return internal_fail(FGPU_ECUDA, m_.c_str());                                  \
    }                                                                                \
  } while (0)

}  // namespace
}  // namespace fgpu

using namespace fgpu;

extern "C" int fgpu_loglik_noalloc(int N, int d, const double* X_dev, const double* y_dev, const double* mu_dev,
                                   const int* kspec, int nkspec, int likelihood, double noise, int optimise_noise,
                                   const double* theta_dev, double* ll_dev, int* info_dev, void* stream) {
  internal_clear_error();
  if (N < 1 || d < 1) return internal_fail(FGPU_EINVAL, "N and d must be positive");
  if (N > NOALLOC_MAX_N) {
    std::string m = "fgpu_loglik_noalloc: N=" + std::to_string(N) + " exceeds the fixed scratch limit of " +
                    std::to_string(NOALLOC_MAX_N) + " training points (use fgpu_create/fgpu_loglik)";
    return internal_fail(FGPU_EINVAL, m.c_str());
  }
  if (!X_dev || !y_dev || !kspec || !theta_dev || !ll_dev || !info_dev)
    return internal_fail(FGPU_EINVAL, "NULL input or output pointer");
  if (likelihood != FGPU_MARGINAL && likelihood != FGPU_CONCENTRATED)
    return internal_fail(FGPU_EINVAL, "likelihood must be 0 (marginal) or 1 (concentrated)");
  if (likelihood == FGPU_MARGINAL && !mu_dev) return internal_fail(FGPU_EINVAL, "marginal likelihood needs mu");
  Spec sp;
  std::vector<int> plane_dim, plane_kind;
  int rc = internal_compile_spec(kspec, nkspec, d, sp, plane_dim, plane_kind);
  if (rc) return rc;
  if (sp.nplanes > NOALLOC_MAX_PLANES) {
    std::string m = "fgpu_loglik_noalloc: " + std::to_string(sp.nplanes) +
                    " feature planes exceed the fixed scratch limit of " + std::to_string(NOALLOC_MAX_PLANES);
    return internal_fail(FGPU_EINVAL, m.c_str());
  }
  int dev = 0;
  NA_CK(cudaGetDevice(&dev));
  unsigned char* base = nullptr;
  if ((rc = scratch_address(dev, &base)) != 0) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  const int Nc = (N + TB - 1) / TB * TB, ld = Nc + TB, nsteps = Nc / TB;
  Prob P;
  memset(&P, 0, sizeof(P));
  P.N = N;
  P.Nc = Nc;
  P.ld = ld;
  P.nsteps = nsteps;
  P.nrhs = likelihood == FGPU_CONCENTRATED ? 2 : 1;
  P.likelihood = likelihood;
  P.optimise_noise = optimise_noise ? 1 : 0;
  P.nkparams = sp.nkparams;
  P.noise = noise;
  P.planes = reinterpret_cast<const double*>(base + OFF_PLANES);
  P.y = y_dev;
  P.mu = mu_dev ? mu_dev : y_dev;  // never read for the concentrated likelihood
  P.spec = reinterpret_cast<const Spec*>(base + OFF_SPEC);
  P.theta = theta_dev;
  P.K = reinterpret_cast<double*>(base + OFF_K);
  P.logdet_part = reinterpret_cast<double*>(base + OFF_LOGDET);
  P.status = reinterpret_cast<int*>(base + OFF_STATUS);
  P.out = reinterpret_cast<double*>(base + OFF_OUT);
  P.z = reinterpret_cast<double*>(base + OFF_Z);
  P.ll_dst = ll_dev;
  P.info_dst = info_dev;
  PlaneMap pm;
  memset(&pm, 0, sizeof(pm));
  pm.n = sp.nplanes;
  for (int p = 0; p < sp.nplanes; ++p) {
    pm.dim[p] = plane_dim[p];
    pm.kind[p] = plane_kind[p];
  }
  static_assert(sizeof(Prob) + sizeof(Spec) + 3 * sizeof(void*) <= 4000, "descriptors fit the kernel arguments");
  k_noalloc_desc<<<1, 32, 0, s>>>(P, sp, reinterpret_cast<Prob*>(base + OFF_PROB),
                                  reinterpret_cast<Spec*>(base + OFF_SPEC), reinterpret_cast<int*>(base + OFF_STATUS));
  NA_CK(cudaGetLastError());
  long long n = 1;
  if (sp.nplanes > 0) {
    k_noalloc_planes<<<dim3((Nc + 255) / 256, sp.nplanes), 256, 0, s>>>(
        X_dev, N, Nc, pm, reinterpret_cast<double*>(base + OFF_PLANES));
    NA_CK(cudaGetLastError());
    ++n;
  }
  const Prob* Pd = reinterpret_cast<const Prob*>(base + OFF_PROB);
  NA_CK(launch_build(Pd, 1, nsteps, sp.nplanes, s));
  ++n;
  for (int step = 0; step < nsteps; ++step) {
    NA_CK(launch_potf2(Pd, 1, step, s));
    NA_CK(launch_trsm(Pd, 1, step, nsteps, s));
    n += 2;
    if (nsteps - step - 1 > 0) {
      NA_CK(launch_update(Pd, 1, step, nsteps, s));
      ++n;
    }
  }
  NA_CK(launch_finalize(Pd, 1, s));
  ++n;
  internal_add_launches(n);
  return 0;
}
