// thorin_noalloc.cu -- conservation integrals of caller-owned device fields
// without any device allocation.
//
// Who needs this: a host program that has already given all free GPU memory
// to its own pool allocator (so a cudaMalloc here would fail), or a
// monitoring hook called inside a latency-critical loop, where a cudaMalloc
// is not acceptable because it can synchronise the device.  Such callers
// hand in their own device arrays and get the gas mass, angular momentum and
// total energy back in a device array of their own.
//
// The per-ring partial sums live in a fixed file-scope device array sized
// for the largest ring count the reference supports (MAX1D = 16384 rings,
// src_main/types.h:65).  Its device address is looked up once per GPU, on
// the first call made while that GPU is current, and again whenever the
// GPU's current context is not the one of the last look-up (a
// cudaDeviceReset destroys the context and with it the array's old
// address); make the first call, and the first after a reset, before any
// stream capture.  Every call on a GPU reuses the same array and
// overwrites each ring's slot before reading it, so nothing has to start at
// zero; two calls whose kernels overlap on the same GPU (e.g. issued on
// different streams without ordering) race on the array and must not be
// made.
#include <cuda.h>
#include <mutex>
#include <string>
#include "thorin_kernels.cuh"

#define NOALLOC_MAX_RINGS 16384
#define NOALLOC_SLOTS 3          // mass, momentum, energy per ring

static __device__ __align__(256) double g_noalloc_partials[NOALLOC_MAX_RINGS * NOALLOC_SLOTS];

// GasTotalMass, GasMomentum, GasTotalEnergy (SideEuler.c:26-80, 523-565) of
// one ring per block.
__global__ void k_integrals_ring(const double *__restrict__ rho, const double *__restrict__ vr,
                                 const double *__restrict__ vt, const double *__restrict__ e,
                                 const double *__restrict__ surf, const double *__restrict__ rinf,
                                 const double *__restrict__ rsup, const double *__restrict__ rmed, int ns,
                                 double omega_frame, double *__restrict__ part)
{
  const int i = blockIdx.x;
  const double S = surf[i], rm = rmed[i], ri = rinf[i], rs = rsup[i];
  double m = 0.0, am = 0.0, en = 0.0;
  for (int j = threadIdx.x; j < ns; j += blockDim.x) {
    const int l = j + i * ns;
    const int ljm = (j == 0) ? i * ns + ns - 1 : l - 1;
    const int ljp = (j == ns - 1) ? i * ns : l + 1;
    m += S * rho[l];
    am += S * (rho[l] + rho[ljm]) * rm * (vt[l] + omega_frame * rm);
    double vrc = (rm - ri) * vr[l + ns] + (rs - rm) * vr[l];
    vrc /= (rs - ri);
    const double vtc = 0.5 * (vt[l] + vt[ljp]) + rm * omega_frame;
    en += 0.5 * S * rho[l] * (vrc * vrc + vtc * vtc) + S * e[l];
  }
  m = block_reduce(m, OpAdd(), 0.0);
  am = block_reduce(am, OpAdd(), 0.0);
  en = block_reduce(en, OpAdd(), 0.0);
  if (threadIdx.x == 0) {
    part[NOALLOC_SLOTS * i + 0] = m;
    part[NOALLOC_SLOTS * i + 1] = am;
    part[NOALLOC_SLOTS * i + 2] = en;
  }
}

__global__ void __launch_bounds__(1024) k_integrals_rings_sum(const double *__restrict__ part, int nr, double *__restrict__ out)
{
  for (int q = 0; q < NOALLOC_SLOTS; q++) {
    double s = 0.0;
    for (int i = threadIdx.x; i < nr; i += blockDim.x) s += part[NOALLOC_SLOTS * i + q];
    s = block_reduce(s, OpAdd(), 0.0);
    if (threadIdx.x == 0) out[q] = (q == 1) ? 0.5 * s : s;
    __syncthreads();
  }
}

static std::mutex g_noalloc_mutex;
static double *g_noalloc_ptr[64];
static unsigned long long g_noalloc_ctx[64];    // context ID of each look-up (IDs are never reused)
// Message of the last failure, read back through thorin_gpu_last_error().
extern thread_local std::string g_last_error;
#define g_noalloc_error g_last_error

// ID of the calling thread's current CUDA context (0 if there is none).
// The two driver calls are reached through the runtime's entry-point query,
// so the library needs no link against the driver library (and still loads
// on a machine without one).
static unsigned long long current_context_id()
{
  typedef CUresult (*GetCurrentFn)(CUcontext *);
  typedef CUresult (*GetIdFn)(CUcontext, unsigned long long *);
  static GetCurrentFn get_current = nullptr;
  static GetIdFn get_id = nullptr;
  if (!get_current || !get_id) {
    void *f1 = nullptr, *f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
        q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
      return 0;
    get_current = (GetCurrentFn)f1;
    get_id = (GetIdFn)f2;
  }
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
  if (get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// Device address of the partials array on the current GPU, looked up the
// first time this GPU is seen and again when its context has changed.
static int noalloc_scratch(double **ptr)
{
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) { g_noalloc_error = std::string("cudaGetDevice: ") + cudaGetErrorString(e); return THORIN_ERR_CUDA; }
  if (dev < 0 || dev >= 64) { g_noalloc_error = "device index out of range"; return THORIN_ERR_ARG; }
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  unsigned long long ctx = current_context_id();
  if (!g_noalloc_ptr[dev] || ctx == 0 || ctx != g_noalloc_ctx[dev]) {
    // the look-up also makes the runtime set up the device's primary context
    // when none is current yet
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_partials);
    if (e != cudaSuccess || !p) {
      g_noalloc_error = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
      return THORIN_ERR_CUDA;
    }
    g_noalloc_ptr[dev] = (double *)p;
    g_noalloc_ctx[dev] = current_context_id();
  }
  *ptr = g_noalloc_ptr[dev];
  return THORIN_OK;
}

extern "C" int thorin_integrals_static(const double *rho, const double *vrad, const double *vtheta,
                                       const double *energy, const double *surf, const double *rinf,
                                       const double *rsup, const double *rmed, int nrad, int nsec, double omega_frame,
                                       double *out, void *stream)
{
  if (nrad < 1 || nrad > NOALLOC_MAX_RINGS) {
    g_noalloc_error = "nrad must be in 1.." + std::to_string(NOALLOC_MAX_RINGS) + " (size of the fixed partials array)";
    return THORIN_ERR_ARG;
  }
  if (nsec < 1 || !rho || !vrad || !vtheta || !energy || !surf || !rinf || !rsup || !rmed || !out) {
    g_noalloc_error = "nsec must be positive and every array pointer non-null";
    return THORIN_ERR_ARG;
  }
  double *part = nullptr;
  int rc = noalloc_scratch(&part);
  if (rc != THORIN_OK) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  k_integrals_ring<<<nrad, 256, 0, s>>>(rho, vrad, vtheta, energy, surf, rinf, rsup, rmed, nsec, omega_frame, part);
  k_integrals_rings_sum<<<1, 1024, 0, s>>>(part, nrad, out);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) { g_noalloc_error = std::string("launch: ") + cudaGetErrorString(e); return THORIN_ERR_CUDA; }
  return THORIN_OK;
}
