// thorin_selftest.cu -- on-device check of the kernels' division routine
// (div_fast) against IEEE division.
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
