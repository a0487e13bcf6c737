// thorin_selftest.cu -- on-device checks of the kernels' division routines
// (div_fast, div_slope) against IEEE division, conditional graph nodes, and
// the FP64 FMA peak.
#include <string>
#include "thorin_kernels.cuh"

extern thread_local std::string g_last_error;

// splitmix64 finaliser as a counter-based random source
__device__ __forceinline__ unsigned long long st_mix(unsigned long long z)
{
  z += 0x9e3779b97f4a7c15ULL;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}

// random double with uniform mantissa, exponent uniform in [-emax, emax], random sign
__device__ __forceinline__ double st_value(unsigned long long key, double emax)
{
  const unsigned long long a = st_mix(key), b = st_mix(key ^ 0x5bd1e995ULL);
  const double u = (double)(a >> 11) * (1.0 / 9007199254740992.0);
  const double m = 1.0 + (double)(b >> 11) * (1.0 / 9007199254740992.0);
  const double v = m * exp2(-emax + 2.0 * emax * u);
  return (b & 1ULL) ? -v : v;
}

__global__ void k_selftest_division(long long n, unsigned long long seed, double emax,
                                    unsigned long long *__restrict__ out)
{
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const double x = st_value(seed + 2ULL * (unsigned long long)t, emax);
  const double d = st_value(seed + 2ULL * (unsigned long long)t + 1ULL, emax);
  const long long a = __double_as_longlong(x / d), b = __double_as_longlong(div_fast(x, d));
  const unsigned long long u = (unsigned long long)(a > b ? a - b : b - a);
  if (u) {
    atomicAdd(out, 1ULL);
    atomicMax(out + 1, u);
  }
}

extern "C" int thorin_selftest_division(long long n, unsigned long long seed, double max_exponent,
                                        unsigned long long *mismatches, unsigned long long *max_ulp)
{
  if (n < 1 || !mismatches || !max_ulp || !(max_exponent >= 0.0 && max_exponent <= 1000.0)) {
    g_last_error = "selftest_division: n >= 1, 0 <= max_exponent <= 1000 and output pointers required";
    return THORIN_ERR_ARG;
  }
  unsigned long long *dev = nullptr, host[2] = {0ULL, 0ULL};
  cudaError_t e = cudaMalloc((void **)&dev, sizeof(host));
  if (e == cudaSuccess) e = cudaMemset(dev, 0, sizeof(host));
  if (e == cudaSuccess) {
    k_selftest_division<<<(unsigned)((n + 255) / 256), 256>>>(n, seed, max_exponent, dev);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(host, dev, sizeof(host), cudaMemcpyDeviceToHost);
  if (dev) cudaFree(dev);
  if (e != cudaSuccess) {
    g_last_error = std::string("selftest_division: ") + cudaGetErrorString(e);
    return THORIN_ERR_CUDA;
  }
  *mismatches = host[0];
  *max_ulp = host[1];
  return THORIN_OK;
}

// Conditional graph nodes as the SOR sweep loop uses them.  Every part is
// bounded: an IF node runs its body at most once, and the WHILE check runs
// only after the IF checks have shown that a kernel's condition value of 0
// skips the body and 1 runs it.
__global__ void k_st_setcond(cudaGraphConditionalHandle h, unsigned v)
{
  if (threadIdx.x == 0) cudaGraphSetConditional(h, v);
}

__global__ void k_st_count(int *c, cudaGraphConditionalHandle h, int limit, int loop)
{
  if (threadIdx.x == 0) {
    const int n = ++c[0];
    if (loop) cudaGraphSetConditional(h, n < limit ? 1u : 0u);
  }
}

// One graph: k_st_setcond(v), then IF (body k_st_count) when loop == 0, or
// WHILE with default 1 (body k_st_count, which clears the condition at
// `limit`) when loop == 1.  Returns the count.
static cudaError_t st_cond_graph(int loop, unsigned v, int limit, int *dev, int *count)
{
  cudaGraph_t g;
  cudaError_t e = cudaGraphCreate(&g, 0);
  if (e != cudaSuccess) return e;
  cudaGraphConditionalHandle h;
  cudaGraphNode_t n1, n2, n3;
  cudaGraphNodeParams np = {};
  cudaKernelNodeParams kp = {};
  void *a1[] = {&h, &v};
  void *a2[] = {&dev, &h, &limit, &loop};
  cudaGraphExec_t ge = nullptr;
  e = cudaGraphConditionalHandleCreate(&h, g, loop ? 1u : 0u, cudaGraphCondAssignDefault);
  if (e == cudaSuccess && !loop) {
    kp.func = (void *)k_st_setcond;
    kp.gridDim = dim3(1);
    kp.blockDim = dim3(32);
    kp.kernelParams = a1;
    e = cudaGraphAddKernelNode(&n1, g, nullptr, 0, &kp);
  }
  if (e == cudaSuccess) {
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = loop ? cudaGraphCondTypeWhile : cudaGraphCondTypeIf;
    np.conditional.size = 1;
    e = cudaGraphAddNode(&n2, g, loop ? nullptr : &n1, nullptr, loop ? 0 : 1, &np);
  }
  if (e == cudaSuccess) {
    kp.func = (void *)k_st_count;
    kp.gridDim = dim3(1);
    kp.blockDim = dim3(32);
    kp.kernelParams = a2;
    e = cudaGraphAddKernelNode(&n3, np.conditional.phGraph_out[0], nullptr, 0, &kp);
  }
  if (e == cudaSuccess) e = cudaMemset(dev, 0, sizeof(int));
  if (e == cudaSuccess) e = cudaGraphInstantiate(&ge, g, 0);
  if (e == cudaSuccess) e = cudaGraphLaunch(ge, 0);
  if (e == cudaSuccess) e = cudaMemcpy(count, dev, sizeof(int), cudaMemcpyDeviceToHost);
  if (ge) cudaGraphExecDestroy(ge);
  cudaGraphDestroy(g);
  return e;
}

extern "C" int thorin_selftest_graph_conditional(int *if_zero, int *if_one, int *while_count)
{
  if (!if_zero || !if_one || !while_count) {
    g_last_error = "selftest_graph_conditional: output pointers required";
    return THORIN_ERR_ARG;
  }
  *if_zero = *if_one = *while_count = -1;
  int *dev = nullptr;
  cudaError_t e = cudaMalloc((void **)&dev, sizeof(int));
  if (e == cudaSuccess) e = st_cond_graph(0, 0u, 0, dev, if_zero);
  if (e == cudaSuccess) e = st_cond_graph(0, 1u, 0, dev, if_one);
  if (e == cudaSuccess && *if_zero == 0 && *if_one == 1) e = st_cond_graph(1, 1u, 5, dev, while_count);
  if (dev) cudaFree(dev);
  if (e != cudaSuccess) {
    g_last_error = std::string("selftest_graph_conditional: ") + cudaGetErrorString(e);
    return THORIN_ERR_CUDA;
  }
  return THORIN_OK;
}

// Nested conditional nodes, as a whole-DT graph would use them: an outer
// WHILE node (the substep loop) whose body holds an inner WHILE node (the
// SOR sweep loop).  Both loops are bounded: the outer body resets the inner
// counter, sets the inner condition to 1 and counts itself, clearing its own
// condition at outer_limit; the inner body counts, clearing its condition at
// inner_limit.  (A handle's default value is assigned once per launch of the
// whole graph, not at each run of the body that holds it, so a nested loop
// must be re-armed by a kernel before it.)  c[0] = outer runs, c[1] = inner
// runs in this outer run, c[2] = inner runs in all.
__global__ void k_st_outer(int *c, cudaGraphConditionalHandle h, int limit, cudaGraphConditionalHandle hin)
{
  if (threadIdx.x == 0) {
    const int n = ++c[0];
    c[1] = 0;
    cudaGraphSetConditional(hin, 1u);
    cudaGraphSetConditional(h, n < limit ? 1u : 0u);
  }
}

__global__ void k_st_inner(int *c, cudaGraphConditionalHandle h, int limit)
{
  if (threadIdx.x == 0) {
    const int n = ++c[1];
    c[2]++;
    cudaGraphSetConditional(h, n < limit ? 1u : 0u);
  }
}

extern "C" int thorin_selftest_graph_nested(int *outer, int *inner_total)
{
  if (!outer || !inner_total) {
    g_last_error = "selftest_graph_nested: output pointers required";
    return THORIN_ERR_ARG;
  }
  *outer = *inner_total = -1;
  int *dev = nullptr, host[3] = {0, 0, 0};
  int olim = 3, ilim = 4;
  cudaGraph_t g = nullptr;
  cudaGraphExec_t ge = nullptr;
  cudaGraphConditionalHandle ho, hi;
  cudaGraphNodeParams po = {}, pi = {};
  cudaKernelNodeParams kp = {};
  cudaGraphNode_t no, nk, ni, nik;
  void *ao[] = {&dev, &ho, &olim, &hi};
  void *ai[] = {&dev, &hi, &ilim};
  cudaError_t e = cudaMalloc((void **)&dev, 3 * sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(dev, 0, 3 * sizeof(int));
  if (e == cudaSuccess) e = cudaGraphCreate(&g, 0);
  if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&ho, g, 1u, cudaGraphCondAssignDefault);
  if (e == cudaSuccess) {
    po.type = cudaGraphNodeTypeConditional;
    po.conditional.handle = ho;
    po.conditional.type = cudaGraphCondTypeWhile;
    po.conditional.size = 1;
    e = cudaGraphAddNode(&no, g, nullptr, nullptr, 0, &po);
  }
  cudaGraph_t body = (e == cudaSuccess) ? po.conditional.phGraph_out[0] : nullptr;
  if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&hi, body, 1u, cudaGraphCondAssignDefault);
  if (e == cudaSuccess) {
    kp.func = (void *)k_st_outer;
    kp.gridDim = dim3(1);
    kp.blockDim = dim3(32);
    kp.kernelParams = ao;
    e = cudaGraphAddKernelNode(&nk, body, nullptr, 0, &kp);
  }
  if (e == cudaSuccess) {
    pi.type = cudaGraphNodeTypeConditional;
    pi.conditional.handle = hi;
    pi.conditional.type = cudaGraphCondTypeWhile;
    pi.conditional.size = 1;
    e = cudaGraphAddNode(&ni, body, &nk, nullptr, 1, &pi);
  }
  if (e == cudaSuccess) {
    kp.func = (void *)k_st_inner;
    kp.kernelParams = ai;
    e = cudaGraphAddKernelNode(&nik, pi.conditional.phGraph_out[0], nullptr, 0, &kp);
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&ge, g, 0);
  if (e == cudaSuccess) e = cudaGraphLaunch(ge, 0);
  if (e == cudaSuccess) e = cudaMemcpy(host, dev, sizeof(host), cudaMemcpyDeviceToHost);
  if (ge) cudaGraphExecDestroy(ge);
  if (g) cudaGraphDestroy(g);
  if (dev) cudaFree(dev);
  if (e != cudaSuccess) {
    g_last_error = std::string("selftest_graph_nested: ") + cudaGetErrorString(e);
    return THORIN_ERR_CUDA;
  }
  *outer = host[0];
  *inner_total = host[2];
  return THORIN_OK;
}

// FP64 fused multiply-add throughput of the current GPU: eight independent
// FMA chains per thread, one wave of blocks per multiprocessor times eight.
__global__ void __launch_bounds__(256) k_selftest_dfma(double *__restrict__ out, int iters, double a, double b)
{
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1.0, x2 = x0 + 2.0, x3 = x0 + 3.0;
  double x4 = x0 + 4.0, x5 = x0 + 5.0, x6 = x0 + 6.0, x7 = x0 + 7.0;
  for (int k = 0; k < iters; k++) {
    x0 = __fma_rn(x0, a, b); x1 = __fma_rn(x1, a, b); x2 = __fma_rn(x2, a, b); x3 = __fma_rn(x3, a, b);
    x4 = __fma_rn(x4, a, b); x5 = __fma_rn(x5, a, b); x6 = __fma_rn(x6, a, b); x7 = __fma_rn(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

__global__ void k_selftest_slope_division(long long n, unsigned long long seed, double emax,
                                          unsigned long long *__restrict__ out)
{
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const double x = st_value(seed + 2ULL * (unsigned long long)t, emax);
  const double d = st_value(seed + 2ULL * (unsigned long long)t + 1ULL, emax);
  const long long a = __double_as_longlong(x / d), b = __double_as_longlong(div_slope(x, d));
  const unsigned long long u = (unsigned long long)(a > b ? a - b : b - a);
  if (u) atomicMax(out, u);
}

extern "C" int thorin_selftest_slope_division(long long n, unsigned long long seed, double max_exponent,
                                              unsigned long long *max_ulp)
{
  if (n < 1 || !max_ulp || !(max_exponent >= 0.0 && max_exponent <= 1000.0)) {
    g_last_error = "selftest_slope_division: n >= 1, 0 <= max_exponent <= 1000 and an output pointer required";
    return THORIN_ERR_ARG;
  }
  unsigned long long *dev = nullptr, host = 0ULL;
  cudaError_t e = cudaMalloc((void **)&dev, sizeof(host));
  if (e == cudaSuccess) e = cudaMemset(dev, 0, sizeof(host));
  if (e == cudaSuccess) {
    k_selftest_slope_division<<<(unsigned)((n + 255) / 256), 256>>>(n, seed, max_exponent, dev);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(&host, dev, sizeof(host), cudaMemcpyDeviceToHost);
  if (dev) cudaFree(dev);
  if (e != cudaSuccess) {
    g_last_error = std::string("selftest_slope_division: ") + cudaGetErrorString(e);
    return THORIN_ERR_CUDA;
  }
  *max_ulp = host;
  return THORIN_OK;
}

extern "C" int thorin_selftest_fp64_peak(double *gflops)
{
  if (!gflops) {
    g_last_error = "selftest_fp64_peak: output pointer required";
    return THORIN_ERR_ARG;
  }
  int dev = 0, nsm = 1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int nb = nsm * 8, nt = 256, iters = 4096;
  double *out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaMalloc((void **)&out, sizeof(double) * nb * nt);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e == cudaSuccess) {
    k_selftest_dfma<<<nb, nt>>>(out, 64, 1.0000001, 1e-9);          // warm-up
    cudaEventRecord(e0);
    k_selftest_dfma<<<nb, nt>>>(out, iters, 1.0000001, 1e-9);
    cudaEventRecord(e1);
    e = cudaEventSynchronize(e1);
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (out) cudaFree(out);
  if (e != cudaSuccess || ms <= 0.f) {
    g_last_error = std::string("selftest_fp64_peak: ") + cudaGetErrorString(e);
    return THORIN_ERR_CUDA;
  }
  *gflops = 2.0 * 8.0 * iters * (double)nb * nt / (ms * 1e6);
  return THORIN_OK;
}

// ---------------------------------------------------------------------------
// Tensor-core layout check: one CTA computes D[128][32] = A[128][64] *
// B[32][64]^T with bf16 operands in the K-major, no-swizzle shared-memory
// layout the network kernels use ([k/8][row][16 bytes]) and FP32
// accumulation in TMEM.  The operands sit at the start of a 200 KB shared
// buffer, so any reading of the descriptors stays inside the allocation.
#include "tc_umma.cuh"

__global__ void __launch_bounds__(128) k_selftest_umma(const uint16_t *__restrict__ A, const uint16_t *__restrict__ B,
                                                        float *__restrict__ D, int *__restrict__ status)
{
  extern __shared__ unsigned char smem_raw[];
  unsigned char *s = (unsigned char *)(((uintptr_t)smem_raw + 127) & ~(uintptr_t)127);
  unsigned char *sA = s, *sB = s + 8 * 128 * 16;
  uint64_t *bar = (uint64_t *)(sB + 8 * 32 * 16);
  uint32_t *tslot = (uint32_t *)(bar + 1);
  const int tid = threadIdx.x, warp = tid >> 5;
  for (int c = tid; c < 128 * 8; c += 128) {       // row m, k-group kg
    const int m = c >> 3, kg = c & 7;
    *(uint4 *)(sA + kg * 2048 + m * 16) = *(const uint4 *)(A + m * 64 + kg * 8);
  }
  for (int c = tid; c < 32 * 8; c += 128) {
    const int n = c >> 3, kg = c & 7;
    *(uint4 *)(sB + kg * 512 + n * 16) = *(const uint4 *)(B + n * 64 + kg * 8);
  }
  if (tid == 0) umma::mbar_init(bar, 1);
  if (warp == 0) umma::tmem_alloc(tslot, 32);
  umma::fence_smem_async();
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *tslot;
  if (tid == 0) {
    const uint32_t a0 = umma::smem_addr(sA), b0 = umma::smem_addr(sB);
    for (int ks = 0; ks < 4; ks++)
      umma::mma_bf16(tmem, umma::desc(a0 + ks * 4096, 2048, 128), umma::desc(b0 + ks * 1024, 512, 128),
                     umma::idesc_bf16(128, 32), ks > 0);
    umma::mma_commit(bar);
  }
  __syncwarp();
  bool ok = umma::mbar_wait(bar, 0, 1LL << 26);
  ok = __syncthreads_and(ok);
  if (ok) {
    umma::fence_after_sync();
    float v[32];
    umma::tmem_ld<32>(tmem + ((uint32_t)(warp * 32) << 16), v);
    for (int n = 0; n < 32; n++) D[tid * 32 + n] = v[n];
  } else if (tid == 0) {
    *status = 1;
    umma::mbar_wait(bar, 0, 1LL << 26);
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) umma::tmem_dealloc(tmem, 32);
}

// The bounded mbarrier wait of the tensor-core kernels (umma::mbar_wait),
// made to run out: thread 0 waits for a phase of a barrier that nothing
// arrives at, with `polls` polls, and records the outcome in out[0] (1: it
// gave up); then it arrives itself and waits again, which must succeed
// (out[1] = 1).  The kernel returns normally either way.
__global__ void k_selftest_bounded_wait(long long polls, int *__restrict__ out)
{
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x != 0) return;
  umma::mbar_init(&bar, 1);
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  out[0] = umma::mbar_wait(&bar, 0u, polls) ? 0 : 1;
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(umma::smem_addr(&bar)) : "memory");
  out[1] = umma::mbar_wait(&bar, 0u, polls) ? 1 : 0;
}

extern "C" int thorin_selftest_bounded_wait(long long polls, int *timed_out, int *completed_after_arrival)
{
  if (polls < 1 || polls > (1LL << 20) || !timed_out || !completed_after_arrival) {
    g_last_error = "selftest_bounded_wait: 1 <= polls <= 2^20 and two output pointers required";
    return THORIN_ERR_ARG;
  }
  int *dev = nullptr, host[2] = {0, 0};
  cudaError_t e = cudaMalloc((void **)&dev, sizeof(host));
  if (e == cudaSuccess) e = cudaMemset(dev, 0, sizeof(host));
  if (e == cudaSuccess) {
    k_selftest_bounded_wait<<<1, 32>>>(polls, dev);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(host, dev, sizeof(host), cudaMemcpyDeviceToHost);
  if (dev) cudaFree(dev);
  if (e != cudaSuccess) {
    g_last_error = std::string("selftest_bounded_wait: ") + cudaGetErrorString(e);
    return THORIN_ERR_CUDA;
  }
  *timed_out = host[0];
  *completed_after_arrival = host[1];
  return THORIN_OK;
}

extern "C" int thorin_selftest_umma(const uint16_t *a, const uint16_t *b, float *d)
{
  if (!a || !b || !d) {
    g_last_error = "selftest_umma: buffers required";
    return THORIN_ERR_ARG;
  }
  uint16_t *dA = nullptr, *dB = nullptr;
  float *dD = nullptr;
  int *dS = nullptr, st = 0;
  const int smem = 200 * 1024;
  cudaError_t e = cudaMalloc((void **)&dA, 128 * 64 * 2);
  if (e == cudaSuccess) e = cudaMalloc((void **)&dB, 32 * 64 * 2);
  if (e == cudaSuccess) e = cudaMalloc((void **)&dD, 128 * 32 * 4);
  if (e == cudaSuccess) e = cudaMalloc((void **)&dS, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(dS, 0, sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpy(dA, a, 128 * 64 * 2, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dB, b, 32 * 64 * 2, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_selftest_umma, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess) {
    k_selftest_umma<<<1, 128, smem>>>(dA, dB, dD, dS);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(d, dD, 128 * 32 * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&st, dS, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(dA); cudaFree(dB); cudaFree(dD); cudaFree(dS);
  if (e != cudaSuccess) {
    g_last_error = std::string("selftest_umma: ") + cudaGetErrorString(e);
    return THORIN_ERR_CUDA;
  }
  if (st) {
    g_last_error = "selftest_umma: the MMA completion wait timed out";
    return THORIN_ERR_TIMEOUT;
  }
  return THORIN_OK;
}
