// warmnet.cu -- the learned SOR warm start (include/thorin_warmnet.h).
//
// A polar-periodic convolutional encoder-decoder in BF16 with FP32
// accumulation.  Every 3x3 convolution of the forward pass, of the input
// gradient and of the weight gradient is an implicit GEMM on the tcgen05
// tensor cores: 128 cells per tile, operands staged from global memory into
// shared memory (im2col with the azimuthal wrap and the radial zero pad),
// one thread issues the MMAs into a TMEM accumulator, the warpgroup reads it
// back with tcgen05.ld for the epilogue.  Pooling, upsampling, ReLU masks,
// the loss, gradient reductions and Adam are plain kernels.  All reductions
// run in a fixed order, so results repeat bit for bit.
#include <cuda_bf16.h>
#include <cmath>
#include <string>
#include "thorin_kernels.cuh"
#include "tc_umma.cuh"
#include "../../include/thorin_warmnet.h"

extern thread_local std::string g_last_error;

typedef __nv_bfloat16 bf16;

namespace {

constexpr int WN_C = 32;          // feature channels
constexpr int WN_NL = 8;          // layers: e0 e1 e2 e3 d2 d1 d0 out
constexpr int WN_NIN = 7;         // input channels used
constexpr float WN_YSCALE = 32.f; // output unit, in residual scales
constexpr long long WN_WAIT = 1LL << 26;  // mbarrier polls before giving up
constexpr int WS_MAXORDER = THORIN_WS_MAX_ORDER;   // longest extrapolated start

struct LayerDef {
  int cin, cout, cinp, coutp;
};
__host__ __device__ constexpr LayerDef layer_def(int l)
{
  return l == 0 ? LayerDef{WN_NIN, WN_C, THORIN_WN_INPUTS, WN_C}
                : (l == WN_NL - 1 ? LayerDef{WN_C, 1, WN_C, 16} : LayerDef{WN_C, WN_C, WN_C, WN_C});
}
__host__ __device__ constexpr int layer_size(int l) { return layer_def(l).cout * 9 * layer_def(l).cin + layer_def(l).cout; }
__host__ __device__ constexpr int layer_off(int l) { return l == 0 ? 0 : layer_off(l - 1) + layer_size(l - 1); }
static_assert(layer_off(WN_NL) == THORIN_WN_NPARAMS, "parameter count");

__device__ __forceinline__ unsigned char *align128(unsigned char *p)
{
  return (unsigned char *)(((uintptr_t)p + 127) & ~(uintptr_t)127);
}

// ---------------------------------------------------------------------------
// Convolution, forward and input-gradient form.  out[p] = sum over taps and
// input channels of in[p + tap] * W, with in = 0 outside rings 0..H-1 and the
// azimuth periodic.  MODE 0: bf16 [P][N] = relu(acc + bias); MODE 1: float
// [P] = acc[0] + bias[0]; MODE 2: float [P][N] = acc.
//
// A tile is 128 consecutive cells of one ring.  The CTA stages the ring and
// its two neighbours over the tile's 128 cells plus one halo cell on each
// side (azimuth wrapped) once, as [c/8][ring r' = 0..2][cell p' = 0..129][16 B].
// Each tap (dr, dphi) is then the same tile seen through a shifted
// descriptor: rows m = cells p' = m + 1 + dphi of ring r' = 1 + dr, 8 cells
// per core matrix (SBO 128 B), channel groups 3 * 130 * 16 B apart (LBO).  No
// im2col copy: a tile stages 3 * 130 cells instead of 9 * 128.
// B: [kg][N][16 B] (LBO N*16, SBO 128); wk is [N][9*CIN] (K = tap*CIN + c).
struct ConvArgs {
  const bf16 *in;
  const bf16 *wk;
  const float *bias;
  int coutr;
  void *out;
  int B, H, W;
  int *err;
};

constexpr int WN_HALO_W = 130;                     // 128 cells + one halo cell each side

template <int CIN, int N>
constexpr int conv_smem() { return (CIN / 8) * 3 * WN_HALO_W * 16 + 9 * CIN * N * 2 + 128 + 128; }

template <int CIN, int N, int MODE>
__global__ void __launch_bounds__(128, 4) k_wn_conv(ConvArgs a)
{
  constexpr int K = 9 * CIN, KG = K / 8, C8 = CIN / 8;
  constexpr int A_BYTES = C8 * 3 * WN_HALO_W * 16, B_BYTES = KG * N * 16, LBO_A = 3 * WN_HALO_W * 16;
  constexpr uint32_t IDESC = umma::idesc_bf16(128, N);
  extern __shared__ unsigned char smem_raw[];
  unsigned char *sA = align128(smem_raw), *sB = sA + A_BYTES;
  uint64_t *bar = (uint64_t *)(sB + B_BYTES);
  uint32_t *tslot = (uint32_t *)(bar + 1);
  const int tid = threadIdx.x, warp = tid >> 5;

  for (int c = tid; c < N * KG; c += 128) {
    const int n = c / KG, kg = c - n * KG;
    *(uint4 *)(sB + kg * N * 16 + n * 16) = *(const uint4 *)(a.wk + (size_t)n * K + kg * 8);
  }
  if (tid == 0) umma::mbar_init(bar, 1);
  if (warp == 0) umma::tmem_alloc(tslot, 32);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *tslot;

  // the bias is read in the epilogue (L1-resident), not held in registers
  // beside the next tile's loads
  auto bias = [&](int n) { return (MODE != 2 && n < a.coutr) ? __ldg(a.bias + n) : 0.f; };

  const int tpr = (a.W + 127) / 128;                       // tiles per ring
  const long long ntiles = (long long)a.B * a.H * tpr;
  // A tile stages rings i-1, i, i+1 over cells p0-1 .. p0+128 (azimuth
  // wrapped).  The global loads of the next tile are issued into registers
  // as soon as this tile's MMAs are issued, so their latency overlaps the
  // MMA wait and the epilogue; every load of the thread is in flight before
  // the first store.
  constexpr int NCH = 3 * WN_HALO_W * C8, PER = (NCH + 127) / 128;
  uint4 val[PER];
  auto load_tile = [&](long long tile) {
    const long long ring = tile / tpr;
    const int p0 = (int)(tile - ring * tpr) * 128;
    const int i = (int)(ring % a.H);
    const long long rbase = ring - i;
#pragma unroll
    for (int k = 0; k < PER; k++) {
      const int ch = tid + 128 * k;
      val[k] = make_uint4(0u, 0u, 0u, 0u);
      if (ch < NCH) {
        const int c8 = ch % C8, rest = ch / C8, pp = rest % WN_HALO_W, rr = rest / WN_HALO_W;
        const int ii = i + rr - 1;
        int jj = p0 - 1 + pp;
        jj = jj < 0 ? jj + a.W : (jj >= a.W ? jj % a.W : jj);
        if (ii >= 0 && ii < a.H) val[k] = __ldg((const uint4 *)(a.in + ((rbase + ii) * a.W + jj) * CIN + c8 * 8));
      }
    }
  };
  uint32_t phase = 0;
  bool ok = true;
  if ((long long)blockIdx.x < ntiles) load_tile(blockIdx.x);
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long ring = tile / tpr;                     // b * H + i
    const int p0 = (int)(tile - ring * tpr) * 128;
#pragma unroll
    for (int k = 0; k < PER; k++) {
      const int ch = tid + 128 * k;
      if (ch < NCH) {
        const int c8 = ch % C8, rest = ch / C8, pp = rest % WN_HALO_W, rr = rest / WN_HALO_W;
        *(uint4 *)(sA + ((c8 * 3 + rr) * WN_HALO_W + pp) * 16) = val[k];
      }
    }
    umma::fence_smem_async();
    __syncthreads();
    if (tid == 0) {
      umma::fence_after_sync();
      const uint32_t a0 = umma::smem_addr(sA), b0 = umma::smem_addr(sB);
#pragma unroll
      for (int t = 0; t < 9; t++) {
        const int rr = t / 3, pp = t % 3;                  // ring 1 + dr, first cell 1 + dphi
#pragma unroll
        for (int ks = 0; ks < CIN / 16; ks++)
          umma::mma_bf16(tmem, umma::desc(a0 + ((2 * ks * 3 + rr) * WN_HALO_W + pp) * 16, LBO_A, 128),
                         umma::desc(b0 + (t * (CIN / 16) + ks) * 2 * N * 16, N * 16, 128), IDESC, t > 0 || ks > 0);
      }
      umma::mma_commit(bar);
    }
    __syncwarp();
    if (tile + gridDim.x < ntiles) load_tile(tile + gridDim.x);   // registers only: sA is the MMA's until the wait
    ok = umma::mbar_wait(bar, phase, WN_WAIT);
    ok = __syncthreads_and(ok);
    phase ^= 1u;
    if (!ok) break;
    umma::fence_after_sync();
    float v[N];
    umma::tmem_ld<N>(tmem + ((uint32_t)(warp * 32) << 16), v);
    const bool live = p0 + tid < a.W;
    const long long p = ring * a.W + p0 + tid;
    if (live) {
      if (MODE == 0) {
        uint4 *dst = (uint4 *)((bf16 *)a.out + p * N);
#pragma unroll
        for (int q = 0; q < N / 8; q++) {
          __nv_bfloat162 h[4];
#pragma unroll
          for (int e = 0; e < 4; e++)
            h[e] = __floats2bfloat162_rn(fmaxf(v[8 * q + 2 * e] + bias(8 * q + 2 * e), 0.f),
                                         fmaxf(v[8 * q + 2 * e + 1] + bias(8 * q + 2 * e + 1), 0.f));
          dst[q] = *(uint4 *)h;
        }
      } else if (MODE == 1) {
        ((float *)a.out)[p] = v[0] + bias(0);
      } else {
        float4 *dst = (float4 *)((float *)a.out + p * N);
#pragma unroll
        for (int q = 0; q < N / 4; q++) dst[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
      }
    }
    umma::fence_before_sync();
    __syncthreads();
  }
  if (!ok) {
    if (tid == 0) atomicExch(a.err, 1);
    umma::mbar_wait(bar, phase ^ 1u, WN_WAIT);   // let an MMA still in flight finish before freeing TMEM
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) umma::tmem_dealloc(tmem, 32);
}

// ---------------------------------------------------------------------------
// Weight gradient: D[(tap, ci)][co] = sum over cells p of in[p + tap][ci] *
// gout[p][co], K = cells (128 per chunk).  Rows 9*CIN are cut into M tiles of
// 128; each tile is [kg = cell/8][row][16 B] (LBO 2048, SBO 128), gout is
// [kg][co][16 B] (LBO N*16, SBO 128).  Each block accumulates its chunks in
// TMEM and writes its partial D and the partial bias gradient.
struct WgradArgs {
  const bf16 *in;
  const bf16 *gout;
  float *part;       // [grid][9*CIN][N], then [grid][N]
  int B, H, W;
  int *err;
};

template <int CIN, int N>
struct WgradShape {
  static constexpr int R = 9 * CIN, MT = (R + 127) / 128, A_TILE = 16 * 128 * 16, A_BYTES = MT * A_TILE,
                       B_BYTES = 16 * N * 16, COLS = MT * N <= 32 ? 32 : (MT * N <= 64 ? 64 : 128),
                       SMEM = A_BYTES + B_BYTES + 4 * N * 4 + 128 + 128;
};

template <int CIN, int N>
__global__ void __launch_bounds__(128) k_wn_wgrad(WgradArgs a)
{
  using S = WgradShape<CIN, N>;
  constexpr uint32_t IDESC = umma::idesc_bf16(128, N);
  extern __shared__ unsigned char smem_raw[];
  unsigned char *sA = align128(smem_raw), *sB = sA + S::A_BYTES;
  float *sred = (float *)(sB + S::B_BYTES);
  uint64_t *bar = (uint64_t *)(sred + 4 * N);
  uint32_t *tslot = (uint32_t *)(bar + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  for (int o = tid * 16; o < S::A_BYTES; o += 128 * 16) *(uint4 *)(sA + o) = make_uint4(0u, 0u, 0u, 0u);
  if (tid == 0) umma::mbar_init(bar, 1);
  if (warp == 0) umma::tmem_alloc(tslot, S::COLS);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *tslot;

  float db[N];
#pragma unroll
  for (int n = 0; n < N; n++) db[n] = 0.f;
  const long long HW = (long long)a.H * a.W, P = (long long)a.B * HW;
  const long long nchunks = (P + 127) / 128;
  uint32_t phase = 0;
  bool ok = true;
  int started = 0;
  for (long long ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
    const long long p = ch * 128 + tid;
    const bool live = p < P;
    int b = 0, i = 0, j = 0;
    if (live) {
      b = (int)(p / HW);
      const long long rem = p - (long long)b * HW;
      i = (int)(rem / a.W);
      j = (int)(rem - (long long)i * a.W);
    }
    const int kg = tid >> 3, kk = (tid & 7) * 2;
    {
      const uint4 *src = (const uint4 *)(a.gout + (live ? p : 0) * N);
#pragma unroll
      for (int q = 0; q < N / 8; q++) {
        uint4 val = live ? src[q] : make_uint4(0u, 0u, 0u, 0u);
        const bf16 *h = (const bf16 *)&val;
#pragma unroll
        for (int e = 0; e < 8; e++) {
          const int n = 8 * q + e;
          *(bf16 *)(sB + kg * N * 16 + n * 16 + kk) = h[e];
          db[n] += __bfloat162float(h[e]);
        }
      }
    }
#pragma unroll 1
    for (int t = 0; t < 9; t++) {
      const int ii = i + t / 3 - 1;
      int jj = j + t % 3 - 1;
      jj = jj < 0 ? jj + a.W : (jj >= a.W ? jj - a.W : jj);
      const bool v = live && ii >= 0 && ii < a.H;
      const uint4 *src = (const uint4 *)(a.in + (((long long)b * a.H + (v ? ii : 0)) * a.W + jj) * CIN);
#pragma unroll
      for (int q = 0; q < CIN / 8; q++) {
        uint4 val = v ? src[q] : make_uint4(0u, 0u, 0u, 0u);
        const bf16 *h = (const bf16 *)&val;
#pragma unroll
        for (int e = 0; e < 8; e++) {
          const int r = t * CIN + 8 * q + e;
          *(bf16 *)(sA + (r >> 7) * S::A_TILE + kg * 2048 + (r & 127) * 16 + kk) = h[e];
        }
      }
    }
    umma::fence_smem_async();
    __syncthreads();
    if (tid == 0) {
      umma::fence_after_sync();
      const uint32_t a0 = umma::smem_addr(sA), b0 = umma::smem_addr(sB);
#pragma unroll
      for (int q = 0; q < S::MT; q++)
#pragma unroll
        for (int ks = 0; ks < 8; ks++)
          umma::mma_bf16(tmem + q * N, umma::desc(a0 + q * S::A_TILE + ks * 4096, 2048, 128),
                         umma::desc(b0 + ks * 2 * N * 16, N * 16, 128), IDESC, started || ks > 0);
      umma::mma_commit(bar);
    }
    __syncwarp();
    ok = umma::mbar_wait(bar, phase, WN_WAIT);
    ok = __syncthreads_and(ok);
    phase ^= 1u;
    started = 1;
    if (!ok) break;
  }
  if (!ok) {
    if (tid == 0) atomicExch(a.err, 1);
    umma::mbar_wait(bar, phase ^ 1u, WN_WAIT);
  } else {
    umma::fence_after_sync();
    float *pd = a.part + (size_t)blockIdx.x * S::R * N;
#pragma unroll 1
    for (int q = 0; q < S::MT; q++) {
      float v[N];
      umma::tmem_ld<N>(tmem + q * N + ((uint32_t)(warp * 32) << 16), v);
      const int r = q * 128 + warp * 32 + lane;
      if (r < S::R) {
#pragma unroll
        for (int n = 0; n < N; n++) pd[(size_t)r * N + n] = started ? v[n] : 0.f;
      }
    }
  }
  // bias gradient: fixed-order reduction over the block
#pragma unroll
  for (int n = 0; n < N; n++) {
    float s = db[n];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) sred[warp * N + n] = s;
  }
  __syncthreads();
  if (tid < N)
    a.part[(size_t)gridDim.x * S::R * N + (size_t)blockIdx.x * N + tid] =
        ((sred[tid] + sred[N + tid]) + sred[2 * N + tid]) + sred[3 * N + tid];
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) umma::tmem_dealloc(tmem, S::COLS);
}

// Sum the block partials in block order and scatter into the FP32 gradient
// layout W[cout][tap][cin], bias[cout].
__global__ void k_wn_wgrad_reduce(const float *__restrict__ part, int nblk, int cin, int cinp, int cout, int n,
                                  float *__restrict__ gw)
{
  const int R = 9 * cinp;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx < R * n) {
    const int r = idx / n, co = idx - r * n, t = r / cinp, ci = r - t * cinp;
    if (ci >= cin || co >= cout) return;
    float s = 0.f;
    for (int k = 0; k < nblk; k++) s += part[(size_t)k * R * n + idx];
    gw[(co * 9 + t) * cin + ci] = s;
  } else if (idx < R * n + cout) {
    const int co = idx - R * n;
    float s = 0.f;
    const float *pb = part + (size_t)nblk * R * n;
    for (int k = 0; k < nblk; k++) s += pb[(size_t)k * n + co];
    gw[cout * 9 * cin + co] = s;
  }
}

// FP32 master W[cout][tap][cin] -> wk [coutp][9*cinp] and the flipped,
// transposed wt [cinp][9*coutp] (input-gradient convolution).
__global__ void k_wn_pack(const float *__restrict__ w, int cin, int cout, int cinp, int coutp, bf16 *__restrict__ wk,
                          bf16 *__restrict__ wt)
{
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  const int nk = coutp * 9 * cinp;
  if (idx < nk) {
    const int n = idx / (9 * cinp), k = idx - n * 9 * cinp, t = k / cinp, ci = k - t * cinp;
    wk[idx] = __float2bfloat16_rn((n < cout && ci < cin) ? w[(n * 9 + t) * cin + ci] : 0.f);
  } else if (idx < 2 * nk) {
    const int o = idx - nk;
    const int ci = o / (9 * coutp), k = o - ci * 9 * coutp, t = k / coutp, co = k - t * coutp;
    wt[o] = __float2bfloat16_rn((co < cout && ci < cin) ? w[(co * 9 + (8 - t)) * cin + ci] : 0.f);
  }
}

// 2x2 average pooling, bf16 [B][H][W][32] -> [B][H/2][W/2][32]; one thread
// per 8 channels of an output cell
__global__ void k_wn_pool(const bf16 *__restrict__ a, bf16 *__restrict__ p, int B, int H, int W)
{
  const long long n = (long long)B * (H / 2) * (W / 2) * (WN_C / 8);
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= n) return;
  const int c8 = (int)(idx % (WN_C / 8));
  long long q = idx / (WN_C / 8);
  const int j = (int)(q % (W / 2));
  q /= W / 2;
  const int i = (int)(q % (H / 2));
  const int b = (int)(q / (H / 2));
  const bf16 *s = a + (((long long)b * H + 2 * i) * W + 2 * j) * WN_C + 8 * c8;
  const uint4 u0 = *(const uint4 *)s, u1 = *(const uint4 *)(s + WN_C), u2 = *(const uint4 *)(s + (long long)W * WN_C),
              u3 = *(const uint4 *)(s + (long long)W * WN_C + WN_C);
  const bf16 *h0 = (const bf16 *)&u0, *h1 = (const bf16 *)&u1, *h2 = (const bf16 *)&u2, *h3 = (const bf16 *)&u3;
  uint4 out;
  bf16 *ho = (bf16 *)&out;
#pragma unroll
  for (int e = 0; e < 8; e++)
    ho[e] = __float2bfloat16_rn(0.25f * ((__bfloat162float(h0[e]) + __bfloat162float(h1[e])) +
                                         (__bfloat162float(h2[e]) + __bfloat162float(h3[e]))));
  *(uint4 *)(p + idx * 8) = out;
}

// u = up2(low) + skip, bf16 at the finer level [B][H][W][32]; one thread per
// 8 channels of a cell
__global__ void k_wn_upadd(const bf16 *__restrict__ low, const bf16 *__restrict__ skip, bf16 *__restrict__ u, int B,
                           int H, int W)
{
  const long long n = (long long)B * H * W * (WN_C / 8);
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= n) return;
  const int c8 = (int)(idx % (WN_C / 8));
  long long q = idx / (WN_C / 8);
  const int j = (int)(q % W);
  q /= W;
  const int i = (int)(q % H);
  const int b = (int)(q / H);
  const uint4 lo = *(const uint4 *)(low + (((long long)b * (H / 2) + i / 2) * (W / 2) + j / 2) * WN_C + 8 * c8);
  const uint4 sk = *(const uint4 *)(skip + idx * 8);
  const bf16 *hl = (const bf16 *)&lo, *hs = (const bf16 *)&sk;
  uint4 out;
  bf16 *ho = (bf16 *)&out;
#pragma unroll
  for (int e = 0; e < 8; e++) ho[e] = __float2bfloat16_rn(__bfloat162float(hl[e]) + __bfloat162float(hs[e]));
  *(uint4 *)(u + idx * 8) = out;
}

// bf16 gradient = g * (act > 0)
__global__ void k_wn_relu_mask(const float *__restrict__ g, const bf16 *__restrict__ act, bf16 *__restrict__ out,
                               long long n)
{
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= n) return;
  out[idx] = __float2bfloat16_rn(__bfloat162float(act[idx]) > 0.f ? g[idx] : 0.f);
}

// coarse gradient of up2: sum of the 4 fine children, then the ReLU mask of
// the coarse activation; bf16 out at the coarse level [B][H/2][W/2][32]
__global__ void k_wn_downsum_mask(const float *__restrict__ gu, const bf16 *__restrict__ act, bf16 *__restrict__ out,
                                  int B, int H, int W)
{
  const long long n = (long long)B * (H / 2) * (W / 2) * WN_C;
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= n) return;
  const int c = (int)(idx % WN_C);
  long long q = idx / WN_C;
  const int j = (int)(q % (W / 2));
  q /= W / 2;
  const int i = (int)(q % (H / 2));
  const int b = (int)(q / (H / 2));
  const float *s = gu + (((long long)b * H + 2 * i) * W + 2 * j) * WN_C + c;
  const float v = (s[0] + s[WN_C]) + (s[(long long)W * WN_C] + s[(long long)W * WN_C + WN_C]);
  out[idx] = __float2bfloat16_rn(__bfloat162float(act[idx]) > 0.f ? v : 0.f);
}

// fine gradient of the pooling: ga += 0.25 * gp(coarse); the result then
// gets the ReLU mask of the fine activation, bf16 out
__global__ void k_wn_unpool_mask(const float *__restrict__ ga, const float *__restrict__ gp, const bf16 *__restrict__ act,
                                 bf16 *__restrict__ out, int B, int H, int W)
{
  const long long n = (long long)B * H * W * WN_C;
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= n) return;
  const int c = (int)(idx % WN_C);
  long long q = idx / WN_C;
  const int j = (int)(q % W);
  q /= W;
  const int i = (int)(q % H);
  const int b = (int)(q / H);
  const float v = ga[idx] + 0.25f * gp[(((long long)b * (H / 2) + i / 2) * (W / 2) + j / 2) * WN_C + c];
  out[idx] = __float2bfloat16_rn(__bfloat162float(act[idx]) > 0.f ? v : 0.f);
}

// loss = sum over rings 1..H-2 of (y - t)^2 * inv_n; gy16[p][0] = dloss/dy
__global__ void k_wn_loss(const float *__restrict__ y, const float *__restrict__ t, int B, int H, int W, float inv_n,
                          bf16 *__restrict__ gy16, double *__restrict__ lpart)
{
  const long long P = (long long)B * H * W;
  const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  double l = 0.0;
  if (p < P) {
    const int i = (int)((p / W) % H);
    float g = 0.f;
    if (i >= 1 && i <= H - 2) {
      const float d = y[p] - t[p];
      l = (double)d * (double)d;
      g = 2.f * d * inv_n;
    }
    uint4 z[2] = {make_uint4(0u, 0u, 0u, 0u), make_uint4(0u, 0u, 0u, 0u)};
    ((bf16 *)z)[0] = __float2bfloat16_rn(g);
    uint4 *dst = (uint4 *)(gy16 + p * 16);
    dst[0] = z[0];
    dst[1] = z[1];
  }
  l = block_reduce(l, OpAdd(), 0.0);
  if (threadIdx.x == 0) lpart[blockIdx.x] = l;
}

// ordered sum of n partials times scale -> *out (one warp)
__global__ void k_wn_sum(const double *__restrict__ part, int n, double scale, double *__restrict__ out)
{
  double s = 0.0;
  for (int k = threadIdx.x; k < n; k += 32) s += part[k];
  s = warp_reduce(s, OpAdd());
  if (threadIdx.x == 0) *out = s * scale;
}

// the same with scale = 1 / (omega a b), omega read from the device (the
// device-resident DT's control block)
__global__ void k_wn_sum_omega(const double *__restrict__ part, int n, const double *__restrict__ omega, double a,
                               double b, double *__restrict__ out)
{
  double s = 0.0;
  for (int k = threadIdx.x; k < n; k += 32) s += part[k];
  s = warp_reduce(s, OpAdd());
  if (threadIdx.x == 0) *out = s * (1.0 / (*omega * a * b));
}

__global__ void k_wn_sqnorm(const float *__restrict__ g, int n, double *__restrict__ part)
{
  double s = 0.0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) s += (double)g[k] * g[k];
  s = block_reduce(s, OpAdd(), 0.0);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void k_wn_adam(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m,
                          float *__restrict__ v, int n, float lr, float b1, float b2, float eps, float bc1, float bc2,
                          const double *__restrict__ sqnorm, float max_norm)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const double nrm = sqrt(*sqnorm);
  const float clip = (max_norm > 0.f && nrm > (double)max_norm) ? (float)((double)max_norm / nrm) : 1.f;
  const float gk = g[k] * clip;
  const float mk = b1 * m[k] + (1.f - b1) * gk, vk = b2 * v[k] + (1.f - b2) * gk * gk;
  m[k] = mk;
  v[k] = vk;
  w[k] -= lr * (mk / bc1) / (sqrtf(vk / bc2) + eps);
}

// ---------------------------------------------------------------------------
// Coupling to the SOR system (rows 1..nr-2 are the unknowns).  T is in the
// grid layout (l = j + i*ns); the coefficients and the right-hand side are
// colour-packed (sor_pidx), as k_matrix writes them.
struct SorSys {
  const double *ml, *mlip, *mlim, *mljp, *mljm, *rhs;
};

// residual of cell (i, j), row l = j + i*ns, packed position q
__device__ __forceinline__ double sor_resid(const double *T, const SorSys &m, int ns, int i, int j, size_t q)
{
  const int l = j + i * ns;
  const int ljp = (j == ns - 1) ? i * ns : l + 1, ljm = (j == 0) ? i * ns + ns - 1 : l - 1;
  return T[l] * m.ml[q] + T[l + ns] * m.mlip[q] + T[l - ns] * m.mlim[q] + T[ljp] * m.mljp[q] + T[ljm] * m.mljm[q] -
         m.rhs[q];
}

// partial sums over the unknowns of |r / Ml| (part[block]) and |r|
// (part[grid + block]), grid-stride, block order
__global__ void k_wn_scale(int nr, int ns, const double *__restrict__ T, SorSys m, double *__restrict__ part)
{
  double s = 0.0, sr = 0.0;
  const long long n = (long long)(nr - 2) * ns;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    const int i = 1 + (int)(q / ns), j = (int)(q % ns);
    const size_t pq = sor_pidx(i, j, ns >> 1);
    const double r = sor_resid(T, m, ns, i, j, pq);
    s += (double)fabsf((float)r / (float)m.ml[pq]);      // a scale: FP32 is plenty
    sr += fabs(r);
  }
  s = block_reduce(s, OpAdd(), 0.0);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
  sr = block_reduce(sr, OpAdd(), 0.0);
  if (threadIdx.x == 0) part[gridDim.x + blockIdx.x] = sr;
}

// The network may run on a coarser grid than the disk: f x f disk cells
// (f = 1 or 2) make one network cell.  Its inputs are the averages of the
// fine cells' inputs, and its prediction is applied to each of them (nearest
// upsampling).  The Jacobi step stays per fine cell.

// One fine cell's inputs: the Jacobi-scaled residual over its mean
// (clipped), the four neighbour weights -M/Ml, the stiffness
// -log(1 - sum w) / 4 and the previous solve's update in the output's units
// (clipped; zero before the first solve).  Returns the Jacobi step -r/Ml.
// The residual needs FP64 (it cancels); the rest only feeds bf16 inputs and
// the start of the solve, so it runs in FP32.
__device__ __forceinline__ double wn_cell_inputs(int nr, int ns, int i, int j, const double *T, const SorSys &m,
                                                 float is, const double *prev, float (&f)[WN_NIN])
{
  if (i < 1 || i > nr - 2) return 0.0;
  const int l = j + i * ns;
  const size_t q = sor_pidx(i, j, ns >> 1);
  const double r = sor_resid(T, m, ns, i, j, q);
  const float iml = 1.0f / (float)m.ml[q];
  const float rj = (float)r * iml;
  f[0] += fminf(fmaxf(rj * is, -16.f), 16.f);
  const float w1 = -(float)m.mlip[q] * iml, w2 = -(float)m.mlim[q] * iml, w3 = -(float)m.mljp[q] * iml,
              w4 = -(float)m.mljm[q] * iml;
  f[1] += w1; f[2] += w2; f[3] += w3; f[4] += w4;
  f[5] += -logf(fmaxf(1.f - (((w1 + w2) + w3) + w4), 1e-6f)) * 0.25f;
  if (prev) f[6] += fminf(fmaxf((float)prev[l] * is * (1.f / WN_YSCALE), -16.f), 16.f);
  return -(double)rj;
}

// network input x[L][16] for each network cell L (the mean of its f x f
// fine cells' inputs) and the Jacobi step jac of every fine cell
__global__ void k_wn_features(int nr, int ns, int fc, const double *__restrict__ T, SorSys m,
                              const double *__restrict__ scale, const double *__restrict__ prev, bf16 *__restrict__ x,
                              double *__restrict__ jac)
{
  const int H = nr / fc, W = ns / fc;
  const long long n = (long long)H * W;
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int I = (int)(q / W), J = (int)(q % W);
  const double s = *scale;
  const float is = s > 1e-30 ? (float)(1.0 / s) : 0.f;
  float f[WN_NIN] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  for (int a = 0; a < fc; a++)
    for (int b = 0; b < fc; b++) {
      const int i = I * fc + a, j = J * fc + b;
      jac[j + (long long)i * ns] = wn_cell_inputs(nr, ns, i, j, T, m, is, prev, f);
    }
  const float inv = 1.f / (float)(fc * fc);
  uint4 z[2] = {make_uint4(0u, 0u, 0u, 0u), make_uint4(0u, 0u, 0u, 0u)};
  bf16 *h = (bf16 *)z;
#pragma unroll
  for (int c = 0; c < WN_NIN; c++) h[c] = __float2bfloat16_rn(f[c] * inv);
  uint4 *dst = (uint4 *)(x + q * THORIN_WN_INPUTS);
  dst[0] = z[0];
  dst[1] = z[1];
}

// Prolongation of the network's output to the disk's cells.  fc = 1: the
// same cell.  fc = 2: bilinear between network-cell centres.  Disk cell i
// sits at network coordinate (i - 1/2) / 2, so an even i takes 1/4 of
// network cell i/2 - 1 and 3/4 of i/2, and an odd i takes 3/4 of (i-1)/2
// and 1/4 of (i+1)/2.  Radially the index is clamped to the grid;
// azimuthally it wraps.
__device__ __forceinline__ void wn_up_1d(int i, int n, bool periodic, int (&k)[2], float (&w)[2])
{
  const int I = i >> 1;
  if (i & 1) { k[0] = I; k[1] = I + 1; w[0] = 0.75f; w[1] = 0.25f; }
  else       { k[0] = I - 1; k[1] = I; w[0] = 0.25f; w[1] = 0.75f; }
  for (int a = 0; a < 2; a++) {
    if (periodic) k[a] = (k[a] + n) % n;
    else k[a] = k[a] < 0 ? 0 : (k[a] >= n ? n - 1 : k[a]);
  }
}

__device__ __forceinline__ double wn_up(const float *y, int i, int j, int nr, int ns, int fc)
{
  if (fc == 1) return (double)y[(long long)i * ns + j];
  const int H = nr / 2, W = ns / 2;
  int ki[2], kj[2];
  float wi[2], wj[2];
  wn_up_1d(i, H, false, ki, wi);
  wn_up_1d(j, W, true, kj, wj);
  float v = 0.f;
  for (int a = 0; a < 2; a++)
    for (int b = 0; b < 2; b++) v += wi[a] * wj[b] * y[(long long)ki[a] * W + kj[b]];
  return (double)v;
}

// weight with which disk index i reaches network index I (the transpose of
// wn_up_1d)
__device__ __forceinline__ float wn_up_weight(int i, int I, int n, bool periodic)
{
  int k[2];
  float w[2];
  wn_up_1d(i, n, periodic, k, w);
  return (k[0] == I ? w[0] : 0.f) + (k[1] == I ? w[1] : 0.f);
}

// T += jac + scale * YSCALE * y (y of the cell's network cell) on the
// unknowns; a non-positive result keeps T
__global__ void k_wn_apply(int nr, int ns, int fc, double *__restrict__ T, const double *__restrict__ jac,
                           const float *__restrict__ y, const double *__restrict__ scale)
{
  const long long n = (long long)(nr - 2) * ns;
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= n) return;
  const long long l = q + ns;
  const int i = (int)(l / ns), j = (int)(l % ns);
  const double t = T[l] + jac[l] + (*scale) * (double)WN_YSCALE * wn_up(y, i, j, nr, ns, fc);
  if (t > 0.0) T[l] = t;
}

// training target of each network cell: the mean over its fine cells of
// (T_conv - T_k - jac) / (scale * YSCALE), unknowns only
__global__ void k_wn_target(int nr, int ns, int fc, const double *__restrict__ tconv, const double *__restrict__ tk,
                            const double *__restrict__ jac, const double *__restrict__ scale, float *__restrict__ tgt)
{
  const int H = nr / fc, W = ns / fc;
  const long long n = (long long)H * W;
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int I = (int)(q / W), J = (int)(q % W);
  const double s = *scale;
  double acc = 0.0;
  for (int a = 0; a < fc; a++)
    for (int b = 0; b < fc; b++) {
      const int i = I * fc + a, j = J * fc + b;
      const long long l = j + (long long)i * ns;
      if (i >= 1 && i <= nr - 2) acc += tconv[l] - tk[l] - jac[l];
    }
  tgt[q] = s > 0.0 ? (float)(acc / ((double)(fc * fc) * s * (double)WN_YSCALE)) : 0.f;
}

// predicted start temperature: tp = T_k + jac + scale * YSCALE * y on the
// unknowns, T_k on the boundary rings
__global__ void k_wn_tpred(int nr, int ns, int fc, const double *__restrict__ tk, const double *__restrict__ jac,
                           const float *__restrict__ y, const double *__restrict__ scale, double *__restrict__ tp)
{
  const long long n = (long long)nr * ns;
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int i = (int)(q / ns), j = (int)(q % ns);
  tp[q] = (i >= 1 && i <= nr - 2) ? tk[q] + jac[q] + (*scale) * (double)WN_YSCALE * wn_up(y, i, j, nr, ns, fc)
                                   : tk[q];
}

// rs = (A tp - rhs) / sr on the unknowns (zero elsewhere); partial sums of rs^2
__global__ void k_wn_res(int nr, int ns, const double *__restrict__ tp, SorSys m, const double *__restrict__ sr,
                         float *__restrict__ rs, double *__restrict__ part)
{
  const long long n = (long long)nr * ns;
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  double acc = 0.0;
  if (q < n) {
    const int i = (int)(q / ns), j = (int)(q % ns), l = (int)q;
    float v = 0.f;
    if (i >= 1 && i <= nr - 2 && *sr > 0.0) {
      const double r = sor_resid(tp, m, ns, i, j, sor_pidx(i, j, ns >> 1)) / *sr;
      v = (float)r;
      acc = r * r;
    }
    rs[l] = v;
  }
  acc = block_reduce(acc, OpAdd(), 0.0);
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

// gradient of wres * mean_fine(rs^2) with respect to each fine cell's
// predicted update: wres * 2/N * (scale * YSCALE / sr) * (A^T rs)
__global__ void k_wn_res_grad(int nr, int ns, const float *__restrict__ rs, SorSys m, const double *__restrict__ scale,
                              const double *__restrict__ sr, float wres, double inv_n, float *__restrict__ gf)
{
  const long long n = (long long)nr * ns;
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int i = (int)(q / ns), j = (int)(q % ns), l = (int)q;
  float g = 0.f;
  if (i >= 1 && i <= nr - 2 && *sr > 0.0) {
    // (A^T rs)_l: column l of A holds Ml of row l and the neighbour rows'
    // coefficients that point at l
    const int half = ns >> 1;
    const int jp = (j == ns - 1) ? 0 : j + 1, jm = (j == 0) ? ns - 1 : j - 1;
    const int ljp = jp + i * ns, ljm = jm + i * ns;
    double at = m.ml[sor_pidx(i, j, half)] * rs[l] + m.mljm[sor_pidx(i, jp, half)] * rs[ljp] +
                m.mljp[sor_pidx(i, jm, half)] * rs[ljm];
    if (i + 1 <= nr - 2) at += m.mlim[sor_pidx(i + 1, j, half)] * rs[l + ns];
    if (i - 1 >= 1) at += m.mlip[sor_pidx(i - 1, j, half)] * rs[l - ns];
    g = (float)(2.0 * inv_n * (double)wres * (*scale) * (double)WN_YSCALE / (*sr) * at);
  }
  gf[l] = g;
}

// output gradient of each network cell: its fine cells' residual gradients
// through the transpose of the prolongation, plus wsup * 2/Nc * (y - tgt),
// as channel 0 of gy16; partial sums of (y - tgt)^2
__global__ void k_wn_out_grad(int nr, int ns, int fc, const float *__restrict__ gf, const float *__restrict__ y,
                              const float *__restrict__ tgt, float wsup, double inv_nc, bf16 *__restrict__ gy16,
                              double *__restrict__ part)
{
  const int H = nr / fc, W = ns / fc;
  const long long n = (long long)H * W;
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  double acc = 0.0;
  if (q < n) {
    const int I = (int)(q / W), J = (int)(q % W);
    float g = 0.f;
    if (fc == 1) {
      g = gf[q];
    } else {
      for (int i = 2 * I - 1; i <= 2 * I + 2; i++) {
        if (i < 0 || i >= nr) continue;
        const float wi = wn_up_weight(i, I, H, false);
        if (wi == 0.f) continue;
        for (int jj = 2 * J - 1; jj <= 2 * J + 2; jj++) {
          const int j = (jj + ns) % ns;
          const float wj = wn_up_weight(j, J, W, true);
          if (wj != 0.f) g += wi * wj * gf[(long long)i * ns + j];
        }
      }
    }
    const double d = (double)y[q] - (double)tgt[q];
    acc = d * d;
    g += (float)(2.0 * inv_nc * (double)wsup * d);
    uint4 z[2] = {make_uint4(0u, 0u, 0u, 0u), make_uint4(0u, 0u, 0u, 0u)};
    ((bf16 *)z)[0] = __float2bfloat16_rn(g);
    uint4 *dst = (uint4 *)(gy16 + q * 16);
    dst[0] = z[0];
    dst[1] = z[1];
  }
  acc = block_reduce(acc, OpAdd(), 0.0);
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

// dscal[0] = wres * dscal[4] + wsup * dscal[5]
__global__ void k_wn_total(double *dscal, float wres, float wsup)
{
  dscal[0] = (double)wres * dscal[4] + (double)wsup * dscal[5];
}

// the solve's update tconv - tstart (the previous-update input of the next
// solve) into hist[0] and the time step it was made with into dts[0]; the
// older nh - 1 updates and time steps move one slot back first
__global__ void k_wn_record(long long n, const double *__restrict__ tconv, const double *__restrict__ tstart,
                            double *__restrict__ hist, int nh, const double *__restrict__ dt, double *__restrict__ dts)
{
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q < n) {
    for (int k = nh - 1; k > 0; k--) hist[k * n + q] = hist[(k - 1) * n + q];
    hist[q] = tconv[q] - tstart[q];
  }
  if (q == 0 && dts) {
    for (int k = nh - 1; k > 0; k--) dts[k] = dts[k - 1];
    dts[0] = *dt;
  }
}

// Coefficients of the backward-difference extrapolation to the next point of
// an evenly spaced sequence from its last m values (m = 1..WS_MAXORDER):
// c_k = (-1)^k binom(m, k+1), e.g. 2, -1 (linear) and 3, -3, 1 (quadratic).
struct WsCoef { double c[WS_MAXORDER][WS_MAXORDER]; };

// The extrapolated update u = dt r over all cells, r the update rate u_k /
// dt_k of the last m recorded solves extrapolated to this one (m = the
// order, fewer while fewer are recorded; u = 0 before the first).
__global__ void k_ws_delta(long long cells, const double *__restrict__ hist, int order, const double *__restrict__ dt,
                           const double *__restrict__ dts, WsCoef cf, double *__restrict__ u)
{
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= cells) return;
  int m = 0;
  while (m < order && dts[m] > 0.0) m++;
  double rate = 0.0;
  for (int k = 0; k < m; k++) rate += cf.c[m - 1][k] * (hist[k * cells + q] / dts[k]);
  u[q] = *dt * rate;
}

// Step length along u that minimises the L2 norm of the residual
// R(T + s u) = R(T) + s A u over the unknowns: block partials of
// sum R(T) (A u) and sum (A u)^2, grid-stride, fixed order.  Each unknown
// also gets what the start then needs for one Jacobi step from T + s u:
// with R(T + s u)/Ml = q0 + s qa (q = R cw / omega, cw = omega / Ml from the
// solve's own start pass), v = u - qa and q0 go to vq[0..cells) and
// vq[cells..2 cells).
__global__ void k_ws_line(int nr, int ns, const double *__restrict__ T, const double *__restrict__ u, SorSys m,
                          const double *__restrict__ cw, const double *__restrict__ omega, double *__restrict__ vq,
                          double *__restrict__ part)
{
  double ra = 0.0, aa = 0.0;
  const long long n = (long long)(nr - 2) * ns, cells = (long long)nr * ns;
  const double iw = 1.0 / *omega;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const int i = 1 + (int)(k / ns), j = (int)(k % ns);
    const size_t pq = sor_pidx(i, j, ns >> 1);
    const double r = sor_resid(T, m, ns, i, j, pq);
    const int l = j + i * ns;
    const int ljp = (j == ns - 1) ? i * ns : l + 1, ljm = (j == 0) ? i * ns + ns - 1 : l - 1;
    const double au = u[l] * m.ml[pq] + u[l + ns] * m.mlip[pq] + u[l - ns] * m.mlim[pq] + u[ljp] * m.mljp[pq] +
                      u[ljm] * m.mljm[pq];
    ra += r * au;
    aa += au * au;
    const double iml = cw[pq] * iw;                 // 1 / Ml
    vq[l] = u[l] - au * iml;
    vq[cells + l] = r * iml;
  }
  ra = block_reduce(ra, OpAdd(), 0.0);
  if (threadIdx.x == 0) part[blockIdx.x] = ra;
  aa = block_reduce(aa, OpAdd(), 0.0);
  if (threadIdx.x == 0) part[gridDim.x + blockIdx.x] = aa;
}

// s = -sum R (A u) / sum (A u)^2, kept in [0, 2] (0 when A u vanishes);
// out[0] = s, out[1] += s (a running sum for the statistics)
__global__ void k_ws_step(const double *__restrict__ part, int nb, double *__restrict__ out)
{
  double ra = 0.0, aa = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    ra += part[b];
    aa += part[nb + b];
  }
  ra = block_reduce(ra, OpAdd(), 0.0);
  __syncthreads();
  aa = block_reduce(aa, OpAdd(), 0.0);
  if (threadIdx.x == 0) {
    double st = aa > 0.0 ? -ra / aa : 0.0;
    st = st > 2.0 ? 2.0 : (st > 0.0 ? st : 0.0);     // also maps NaN to 0
    out[0] = st;
    out[1] += st;
  }
}

// T -> T + s u - R(T + s u) / Ml = T + s v - q0 on the unknowns, once a
// solve is recorded (the first solve after attaching starts from T); a
// non-positive result keeps T
__global__ void k_ws_apply(int nr, int ns, double *__restrict__ T, const double *__restrict__ vq,
                           const double *__restrict__ step, const double *__restrict__ dts)
{
  const long long n = (long long)(nr - 2) * ns, cells = (long long)nr * ns;
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= n || !(dts[0] > 0.0)) return;
  const long long l = q + ns;
  const double t = __fma_rn(*step, vq[l], T[l]) - vq[cells + l];
  if (t > 0.0) T[l] = t;
}

inline unsigned nblk(long long n, int bs = 256) { return (unsigned)((n + bs - 1) / bs); }

}  // namespace

// ---------------------------------------------------------------------------
struct thorin_warmnet {
  int nr, ns, maxb, nsm;
  cudaStream_t own;
  float *w, *g, *m, *v;                  // FP32 parameters, gradient, Adam moments
  bf16 *wk[WN_NL], *wt[WN_NL];
  bf16 *x;                               // [B][H][W][16]
  bf16 *act[14];                         // a0 p1 a1 p2 a2 p3 a3 u2 b2 u1 b1 u0 b0, gy16
  float *y, *tgt;
  float *gf[4], *ga[4];                  // FP32 gradient scratch per level
  bf16 *gb[4];                           // bf16 masked gradient per level
  float *part;                           // weight-gradient partials
  int part_blocks;
  double *dscal;                         // [0] loss, [1] grad sq-norm, [2] residual scale, partials from 8
  int *err;
  int adam_t;
  int B;                                 // batch of the last forward
};

enum { A0, P1, A1, P2, A2, P3, A3, U2, B2, U1, B1, U0, B0, GY16 };

static int wn_fail(const char *what, cudaError_t e)
{
  g_last_error = std::string("warmnet: ") + what + ": " + cudaGetErrorString(e);
  return THORIN_ERR_CUDA;
}
#define RCHK_WN(...)              \
  do {                            \
    const int r_ = (__VA_ARGS__); \
    if (r_) return r_;            \
  } while (0)
#define WNCHK(call)                                    \
  do {                                                 \
    cudaError_t e_ = (call);                           \
    if (e_ != cudaSuccess) return wn_fail(#call, e_);  \
  } while (0)

template <int CIN, int N, int MODE>
static int conv_launch(thorin_warmnet *n, const bf16 *in, const bf16 *wk, const float *bias, int coutr, void *out,
                       int B, int H, int W, cudaStream_t s)
{
  constexpr int SM = conv_smem<CIN, N>();
  static std::atomic<bool> attr{false};
  if (!attr.load()) {
    WNCHK(cudaFuncSetAttribute(k_wn_conv<CIN, N, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, SM));
    attr.store(true);
  }
  // Four persistent CTAs per SM (44 KB of shared memory and 32 TMEM columns
  // each): the occupancy calculator answers 1 for this kernel, and one CTA
  // per SM leaves the tile's load -> MMA -> epilogue chain unhidden (3x
  // slower measured); CTAs that do not fit simply start later.
  constexpr long long per_sm = 4;
  const long long tiles = (long long)B * H * ((W + 127) / 128);
  const long long wave = per_sm * n->nsm;
  const int grid = (int)(tiles < wave ? tiles : wave);
  ConvArgs a{in, wk, bias, coutr, out, B, H, W, n->err};
  k_wn_conv<CIN, N, MODE><<<grid, 128, SM, s>>>(a);
  g_thorin_launches++;
  return THORIN_OK;
}

template <int CIN, int N>
static int wgrad_launch(thorin_warmnet *n, int layer, const bf16 *in, const bf16 *gout, int B, int H, int W,
                        cudaStream_t s)
{
  using S = WgradShape<CIN, N>;
  static std::atomic<bool> attr{false};
  if (!attr.load()) {
    WNCHK(cudaFuncSetAttribute(k_wn_wgrad<CIN, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, S::SMEM));
    attr.store(true);
  }
  const long long chunks = ((long long)B * H * W + 127) / 128;
  const int grid = (int)(chunks < n->part_blocks ? chunks : n->part_blocks);
  WgradArgs a{in, gout, n->part, B, H, W, n->err};
  k_wn_wgrad<CIN, N><<<grid, 128, S::SMEM, s>>>(a);
  g_thorin_launches++;
  const LayerDef L = layer_def(layer);
  const int tot = 9 * L.cinp * N + L.cout;
  k_wn_wgrad_reduce<<<nblk(tot), 256, 0, s>>>(n->part, grid, L.cin, L.cinp, L.cout, N, n->g + layer_off(layer));
  g_thorin_launches++;
  return THORIN_OK;
}

static void pack_all(thorin_warmnet *n, cudaStream_t s)
{
  for (int l = 0; l < WN_NL; l++) {
    const LayerDef L = layer_def(l);
    k_wn_pack<<<nblk(2LL * L.coutp * 9 * L.cinp), 256, 0, s>>>(n->w + layer_off(l), L.cin, L.cout, L.cinp, L.coutp,
                                                              n->wk[l], n->wt[l]);
    g_thorin_launches++;
  }
}

static inline const float *bias_of(const thorin_warmnet *n, int l)
{
  const LayerDef L = layer_def(l);
  return n->w + layer_off(l) + L.cout * 9 * L.cin;
}

// forward pass of the batch in n->x -> n->y
static int wn_forward(thorin_warmnet *n, int B, cudaStream_t s)
{
  const int H = n->nr, W = n->ns;
  int h[4] = {H, H / 2, H / 4, H / 8}, w[4] = {W, W / 2, W / 4, W / 8};
  bf16 **A = n->act;
  auto pool = [&](const bf16 *a, bf16 *p, int lv) {
    k_wn_pool<<<nblk((long long)B * h[lv + 1] * w[lv + 1] * (WN_C / 8)), 256, 0, s>>>(a, p, B, h[lv], w[lv]);
    g_thorin_launches++;
  };
  auto upadd = [&](const bf16 *low, const bf16 *skip, bf16 *u, int lv) {
    k_wn_upadd<<<nblk((long long)B * h[lv] * w[lv] * (WN_C / 8)), 256, 0, s>>>(low, skip, u, B, h[lv], w[lv]);
    g_thorin_launches++;
  };
  RCHK_WN(conv_launch<16, 32, 0>(n, n->x, n->wk[0], bias_of(n, 0), 32, A[A0], B, h[0], w[0], s));
  pool(A[A0], A[P1], 0);
  RCHK_WN(conv_launch<32, 32, 0>(n, A[P1], n->wk[1], bias_of(n, 1), 32, A[A1], B, h[1], w[1], s));
  pool(A[A1], A[P2], 1);
  RCHK_WN(conv_launch<32, 32, 0>(n, A[P2], n->wk[2], bias_of(n, 2), 32, A[A2], B, h[2], w[2], s));
  pool(A[A2], A[P3], 2);
  RCHK_WN(conv_launch<32, 32, 0>(n, A[P3], n->wk[3], bias_of(n, 3), 32, A[A3], B, h[3], w[3], s));
  upadd(A[A3], A[A2], A[U2], 2);
  RCHK_WN(conv_launch<32, 32, 0>(n, A[U2], n->wk[4], bias_of(n, 4), 32, A[B2], B, h[2], w[2], s));
  upadd(A[B2], A[A1], A[U1], 1);
  RCHK_WN(conv_launch<32, 32, 0>(n, A[U1], n->wk[5], bias_of(n, 5), 32, A[B1], B, h[1], w[1], s));
  upadd(A[B1], A[A0], A[U0], 0);
  RCHK_WN(conv_launch<32, 32, 0>(n, A[U0], n->wk[6], bias_of(n, 6), 32, A[B0], B, h[0], w[0], s));
  RCHK_WN(conv_launch<32, 16, 1>(n, A[B0], n->wk[7], bias_of(n, 7), 1, n->y, B, h[0], w[0], s));
  n->B = B;
  return THORIN_OK;
}

// loss of n->y against n->tgt and the gradient into n->g (after wn_forward)
static int wn_backward(thorin_warmnet *n, int B, cudaStream_t s, bool mse_loss = true)
{
  const int H = n->nr, W = n->ns;
  int h[4] = {H, H / 2, H / 4, H / 8}, w[4] = {W, W / 2, W / 4, W / 8};
  bf16 **A = n->act;
  const long long P0 = (long long)B * H * W;
  const float inv_n = (float)(1.0 / ((double)B * (H - 2) * W));
  const unsigned lb = nblk(P0);
  double *lpart = n->dscal + 8;
  if (mse_loss) {       // otherwise the caller filled gy16 and the loss
    k_wn_loss<<<lb, 256, 0, s>>>(n->y, n->tgt, B, H, W, inv_n, A[GY16], lpart);
    g_thorin_launches++;
    k_wn_sum<<<1, 32, 0, s>>>(lpart, (int)lb, (double)inv_n, n->dscal);
    g_thorin_launches++;
  }
  auto cnt = [&](int lv) { return (long long)B * h[lv] * w[lv] * WN_C; };
  // out layer
  RCHK_WN(wgrad_launch<32, 16>(n, 7, A[B0], A[GY16], B, h[0], w[0], s));
  RCHK_WN(conv_launch<16, 32, 2>(n, A[GY16], n->wt[7], nullptr, 0, n->gf[0], B, h[0], w[0], s));
  k_wn_relu_mask<<<nblk(cnt(0)), 256, 0, s>>>(n->gf[0], A[B0], n->gb[0], cnt(0));
  g_thorin_launches++;
  // d0 (input u0 = up(b1) + a0)
  RCHK_WN(wgrad_launch<32, 32>(n, 6, A[U0], n->gb[0], B, h[0], w[0], s));
  RCHK_WN(conv_launch<32, 32, 2>(n, n->gb[0], n->wt[6], nullptr, 0, n->ga[0], B, h[0], w[0], s));
  k_wn_downsum_mask<<<nblk(cnt(1)), 256, 0, s>>>(n->ga[0], A[B1], n->gb[1], B, h[0], w[0]);
  g_thorin_launches++;
  // d1
  RCHK_WN(wgrad_launch<32, 32>(n, 5, A[U1], n->gb[1], B, h[1], w[1], s));
  RCHK_WN(conv_launch<32, 32, 2>(n, n->gb[1], n->wt[5], nullptr, 0, n->ga[1], B, h[1], w[1], s));
  k_wn_downsum_mask<<<nblk(cnt(2)), 256, 0, s>>>(n->ga[1], A[B2], n->gb[2], B, h[1], w[1]);
  g_thorin_launches++;
  // d2
  RCHK_WN(wgrad_launch<32, 32>(n, 4, A[U2], n->gb[2], B, h[2], w[2], s));
  RCHK_WN(conv_launch<32, 32, 2>(n, n->gb[2], n->wt[4], nullptr, 0, n->ga[2], B, h[2], w[2], s));
  k_wn_downsum_mask<<<nblk(cnt(3)), 256, 0, s>>>(n->ga[2], A[A3], n->gb[3], B, h[2], w[2]);
  g_thorin_launches++;
  // e3 (input p3 = pool(a2))
  RCHK_WN(wgrad_launch<32, 32>(n, 3, A[P3], n->gb[3], B, h[3], w[3], s));
  RCHK_WN(conv_launch<32, 32, 2>(n, n->gb[3], n->wt[3], nullptr, 0, n->gf[3], B, h[3], w[3], s));
  k_wn_unpool_mask<<<nblk(cnt(2)), 256, 0, s>>>(n->ga[2], n->gf[3], A[A2], n->gb[2], B, h[2], w[2]);
  g_thorin_launches++;
  // e2
  RCHK_WN(wgrad_launch<32, 32>(n, 2, A[P2], n->gb[2], B, h[2], w[2], s));
  RCHK_WN(conv_launch<32, 32, 2>(n, n->gb[2], n->wt[2], nullptr, 0, n->gf[2], B, h[2], w[2], s));
  k_wn_unpool_mask<<<nblk(cnt(1)), 256, 0, s>>>(n->ga[1], n->gf[2], A[A1], n->gb[1], B, h[1], w[1]);
  g_thorin_launches++;
  // e1
  RCHK_WN(wgrad_launch<32, 32>(n, 1, A[P1], n->gb[1], B, h[1], w[1], s));
  RCHK_WN(conv_launch<32, 32, 2>(n, n->gb[1], n->wt[1], nullptr, 0, n->gf[1], B, h[1], w[1], s));
  k_wn_unpool_mask<<<nblk(cnt(0)), 256, 0, s>>>(n->ga[0], n->gf[1], A[A0], n->gb[0], B, h[0], w[0]);
  g_thorin_launches++;
  // e0
  RCHK_WN(wgrad_launch<16, 32>(n, 0, n->x, n->gb[0], B, h[0], w[0], s));
  return THORIN_OK;
}

static int wn_adam(thorin_warmnet *n, float lr, float b1, float b2, float eps, float max_norm, cudaStream_t s)
{
  const int np = THORIN_WN_NPARAMS;
  double *part = n->dscal + 8;
  k_wn_sqnorm<<<64, 256, 0, s>>>(n->g, np, part);
  g_thorin_launches++;
  k_wn_sum<<<1, 32, 0, s>>>(part, 64, 1.0, n->dscal + 1);
  g_thorin_launches++;
  n->adam_t++;
  const float bc1 = 1.f - powf(b1, (float)n->adam_t), bc2 = 1.f - powf(b2, (float)n->adam_t);
  k_wn_adam<<<nblk(np), 256, 0, s>>>(n->w, n->g, n->m, n->v, np, lr, b1, b2, eps, bc1, bc2, n->dscal + 1, max_norm);
  g_thorin_launches++;
  pack_all(n, s);
  return THORIN_OK;
}

static int wn_check_err(thorin_warmnet *n)
{
  int e = 0;
  WNCHK(cudaMemcpy(&e, n->err, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) {
    g_last_error = "warmnet: a tensor-core wait timed out";
    return THORIN_ERR_TIMEOUT;
  }
  return THORIN_OK;
}

// ---------------------------------------------------------------------------
// Disk coupling, called from the SOR driver on the disk's stream.

// T (start of the solve) -> T + jac + network.  The network grid is
// (nr/fc) x (ns/fc); jac has the disk's nr x ns cells.
int wn_sor_predict(thorin_warmnet *n, int nr, int ns, int fc, double *T, const double *ml, const double *mlip,
                   const double *mlim, const double *mljp, const double *mljm, const double *rhs, const double *prev,
                   double *jac, const double *jscale, double omega, const double *omega_dev, cudaStream_t s)
{
  // dscal: [2] mean |r/Ml| of the start, [3] mean |r|, [4] residual loss,
  // [5] supervised loss, [0] total loss; partials from dscal + 8
  SorSys m{ml, mlip, mlim, mljp, mljm, rhs};
  double *part = n->dscal + 8;
  const int sb = 2 * n->nsm;
  if (jscale && omega_dev) {   // omega on the device (device-resident DT)
    k_wn_sum_omega<<<1, 32, 0, s>>>(jscale, 1, omega_dev, (double)(nr - 2), (double)ns, n->dscal + 2);
    g_thorin_launches += 1;
  } else if (jscale) {      // sum of omega |r / Ml| from the solve's own residual pass
    k_wn_sum<<<1, 32, 0, s>>>(jscale, 1, 1.0 / (omega * (double)(nr - 2) * ns), n->dscal + 2);
    g_thorin_launches += 1;
  } else {
    k_wn_scale<<<sb, 256, 0, s>>>(nr, ns, T, m, part);
    k_wn_sum<<<1, 32, 0, s>>>(part, sb, 1.0 / ((double)(nr - 2) * ns), n->dscal + 2);
    g_thorin_launches += 2;
  }
  k_wn_features<<<nblk((long long)(nr / fc) * (ns / fc)), 256, 0, s>>>(nr, ns, fc, T, m, n->dscal + 2, prev, n->x, jac);
  g_thorin_launches += 1;
  RCHK_WN(wn_forward(n, 1, s));
  k_wn_apply<<<nblk((long long)(nr - 2) * ns), 256, 0, s>>>(nr, ns, fc, T, jac, n->y, n->dscal + 2);
  g_thorin_launches++;
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? THORIN_OK : wn_fail("predict kernels", e);
}

// one training step on the solve that went from tk to tconv: loss = WRES *
// mean((A T_pred - rhs)^2) / mean|r_k|^2 over the disk's unknowns + WSUP *
// mean((y - target)^2) over the network cells, T_pred = tk + jac + scale *
// YSCALE * y, target the converged update beyond the Jacobi step in the same
// units (averaged over each network cell)
int wn_sor_train(thorin_warmnet *n, int nr, int ns, int fc, const double *tk, const double *tconv, const double *ml,
                 const double *mlip, const double *mlim, const double *mljp, const double *mljm, const double *rhs,
                 const double *prev, double *jac, float lr, double *scratch, cudaStream_t s)
{
  constexpr float WRES = 1.0f, WSUP = 0.1f;
  SorSys m{ml, mlip, mlim, mljp, mljm, rhs};
  double *part = n->dscal + 8;
  const int sb = 2 * n->nsm;
  const long long cells = (long long)nr * ns, ncells = (long long)(nr / fc) * (ns / fc);
  const double inv_n = 1.0 / ((double)(nr - 2) * ns), inv_nc = 1.0 / (double)ncells;
  k_wn_scale<<<sb, 256, 0, s>>>(nr, ns, tk, m, part);
  k_wn_sum<<<1, 32, 0, s>>>(part, sb, inv_n, n->dscal + 2);
  k_wn_sum<<<1, 32, 0, s>>>(part + sb, sb, inv_n, n->dscal + 3);
  k_wn_features<<<nblk(ncells), 256, 0, s>>>(nr, ns, fc, tk, m, n->dscal + 2, prev, n->x, jac);
  k_wn_target<<<nblk(ncells), 256, 0, s>>>(nr, ns, fc, tconv, tk, jac, n->dscal + 2, n->tgt);
  g_thorin_launches += 5;
  RCHK_WN(wn_forward(n, 1, s));
  float *rs = n->gf[0], *gfine = n->gf[0] + cells;    // free until the backward pass (>= 8 * cells floats)
  k_wn_tpred<<<nblk(cells), 256, 0, s>>>(nr, ns, fc, tk, jac, n->y, n->dscal + 2, scratch);
  k_wn_res<<<nblk(cells), 256, 0, s>>>(nr, ns, scratch, m, n->dscal + 3, rs, part);
  k_wn_sum<<<1, 32, 0, s>>>(part, (int)nblk(cells), inv_n, n->dscal + 4);
  k_wn_res_grad<<<nblk(cells), 256, 0, s>>>(nr, ns, rs, m, n->dscal + 2, n->dscal + 3, WRES, inv_n, gfine);
  k_wn_out_grad<<<nblk(ncells), 256, 0, s>>>(nr, ns, fc, gfine, n->y, n->tgt, WSUP, inv_nc, n->act[GY16], part);
  k_wn_sum<<<1, 32, 0, s>>>(part, (int)nblk(ncells), inv_nc, n->dscal + 5);
  k_wn_total<<<1, 1, 0, s>>>(n->dscal, WRES, WSUP);
  g_thorin_launches += 7;
  RCHK_WN(wn_backward(n, 1, s, false));
  RCHK_WN(wn_adam(n, lr, 0.9f, 0.999f, 1e-8f, 1.0f, s));
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? THORIN_OK : wn_fail("training kernels", e);
}

// hist[0] = tconv - tstart over nr x ns cells and dts[0] = *dt, after the
// older nh - 1 entries move one slot back
int wn_record_update(int nr, int ns, const double *tconv, const double *tstart, double *hist, int nh,
                     const double *dt, double *dts, cudaStream_t s)
{
  const long long cells = (long long)nr * ns;
  k_wn_record<<<nblk(cells), 256, 0, s>>>(cells, tconv, tstart, hist, nh, dt, dts);
  g_thorin_launches++;
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? THORIN_OK : wn_fail("record kernel", e);
}

extern "C" int thorin_warmstart_coefficients(int order, double *c)
{
  if (order < 1 || order > WS_MAXORDER || !c) return THORIN_ERR_ARG;
  double b = 1.0;                                   // binom(order, k + 1), built up along k
  for (int k = 0; k < order; k++) {
    b = b * (double)(order - k) / (double)(k + 1);
    c[k] = (k & 1) ? -b : b;
  }
  return THORIN_OK;
}

// T (start of the solve) -> T + s u followed by one Jacobi step: u the
// update extrapolated from the last `order` recorded solves (into scratch),
// s the step that minimises the L2 residual along u (part: 4 nsm + 2
// doubles; step: s and its running sum; vq: 2 nr ns doubles; cw = omega/Ml
// and omega of the solve).
int ws_extrapolate(int nr, int ns, double *T, const double *hist, int order, const double *dt, const double *dts,
                   const double *ml, const double *mlip, const double *mlim, const double *mljp, const double *mljm,
                   const double *rhs, const double *cw, const double *omega, double *scratch, double *vq,
                   double *part, double *step, int nsm, cudaStream_t s)
{
  if (order < 1 || order > WS_MAXORDER) return THORIN_ERR_ARG;
  WsCoef cf = {};
  for (int m = 1; m <= WS_MAXORDER; m++) thorin_warmstart_coefficients(m, cf.c[m - 1]);
  const long long cells = (long long)nr * ns;
  const SorSys m{ml, mlip, mlim, mljp, mljm, rhs};
  const int nb = 2 * nsm;
  k_ws_delta<<<nblk(cells), 256, 0, s>>>(cells, hist, order, dt, dts, cf, scratch);
  k_ws_line<<<nb, 256, 0, s>>>(nr, ns, T, scratch, m, cw, omega, vq, part);
  k_ws_step<<<1, 256, 0, s>>>(part, nb, step);
  k_ws_apply<<<nblk((long long)(nr - 2) * ns), 256, 0, s>>>(nr, ns, T, vq, step, dts);
  g_thorin_launches += 4;
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? THORIN_OK : wn_fail("extrapolation kernels", e);
}

// total, residual and supervised loss of the last training step
int wn_last_loss(thorin_warmnet *n, double *loss)
{
  double v[6];
  WNCHK(cudaMemcpy(v, n->dscal, sizeof(v), cudaMemcpyDeviceToHost));
  loss[0] = v[0];
  loss[1] = v[4];
  loss[2] = v[5];
  return wn_check_err(n);
}

int wn_dims(const thorin_warmnet *n, int *nr, int *ns)
{
  *nr = n->nr;
  *ns = n->ns;
  return THORIN_OK;
}

// ---------------------------------------------------------------------------
extern "C" int thorin_warmnet_create(int nrad, int nsec, int max_batch, thorin_warmnet **out)
{
  if (!out || nrad < 16 || nsec < 16 || nrad % 8 || nsec % 8 || max_batch < 1) {
    g_last_error = "warmnet_create: nrad, nsec multiples of 8 and >= 16, max_batch >= 1";
    return THORIN_ERR_ARG;
  }
  *out = nullptr;
  thorin_warmnet *n = new thorin_warmnet();
  n->nr = nrad;
  n->ns = nsec;
  n->maxb = max_batch;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n->nsm, cudaDevAttrMultiProcessorCount, dev);
  if (n->nsm < 1) n->nsm = 1;
  n->part_blocks = 2 * n->nsm;
  const long long P0 = (long long)max_batch * nrad * nsec;
  long long lv[4];
  for (int k = 0; k < 4; k++) lv[k] = P0 >> (2 * k);
  auto fail = [&](cudaError_t e) {
    thorin_warmnet_destroy(n);
    return wn_fail("allocation", e);
  };
  cudaError_t e = cudaStreamCreateWithFlags(&n->own, cudaStreamNonBlocking);
  if (e != cudaSuccess) return fail(e);
  const int np = THORIN_WN_NPARAMS;
  float **fp[] = {&n->w, &n->g, &n->m, &n->v};
  for (float **p : fp) {
    if ((e = cudaMalloc((void **)p, np * sizeof(float))) != cudaSuccess) return fail(e);
    cudaMemset(*p, 0, np * sizeof(float));
  }
  for (int l = 0; l < WN_NL; l++) {
    const LayerDef L = layer_def(l);
    const size_t nk = (size_t)L.coutp * 9 * L.cinp;
    if ((e = cudaMalloc((void **)&n->wk[l], nk * sizeof(bf16))) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc((void **)&n->wt[l], nk * sizeof(bf16))) != cudaSuccess) return fail(e);
  }
  if ((e = cudaMalloc((void **)&n->x, P0 * THORIN_WN_INPUTS * sizeof(bf16))) != cudaSuccess) return fail(e);
  const int lvl[14] = {0, 1, 1, 2, 2, 3, 3, 2, 2, 1, 1, 0, 0, 0};
  for (int k = 0; k < 14; k++) {
    const size_t cnt = (size_t)lv[lvl[k]] * (k == GY16 ? 16 : WN_C);
    if ((e = cudaMalloc((void **)&n->act[k], cnt * sizeof(bf16))) != cudaSuccess) return fail(e);
  }
  if ((e = cudaMalloc((void **)&n->y, P0 * sizeof(float))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc((void **)&n->tgt, P0 * sizeof(float))) != cudaSuccess) return fail(e);
  for (int k = 0; k < 4; k++) {
    if ((e = cudaMalloc((void **)&n->gf[k], lv[k] * WN_C * sizeof(float))) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc((void **)&n->ga[k], lv[k] * WN_C * sizeof(float))) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc((void **)&n->gb[k], lv[k] * WN_C * sizeof(bf16))) != cudaSuccess) return fail(e);
  }
  const size_t part = (size_t)n->part_blocks * (9 * WN_C * WN_C + WN_C);
  if ((e = cudaMalloc((void **)&n->part, part * sizeof(float))) != cudaSuccess) return fail(e);
  // reduction partials: one per 256 cells of the largest grid a pass runs
  // over, which for a disk coupled at half resolution is 4x the network's
  const size_t nd = 8 + (size_t)(nblk(4 * P0) > 4096 ? nblk(4 * P0) : 4096);
  if ((e = cudaMalloc((void **)&n->dscal, nd * sizeof(double))) != cudaSuccess) return fail(e);
  cudaMemset(n->dscal, 0, nd * sizeof(double));
  if ((e = cudaMalloc((void **)&n->err, sizeof(int))) != cudaSuccess) return fail(e);
  cudaMemset(n->err, 0, sizeof(int));
  pack_all(n, n->own);
  if ((e = cudaStreamSynchronize(n->own)) != cudaSuccess) return fail(e);
  *out = n;
  return THORIN_OK;
}

extern "C" int thorin_warmnet_destroy(thorin_warmnet *n)
{
  if (!n) return THORIN_OK;
  if (n->own) cudaStreamSynchronize(n->own);
  void *ptrs[] = {n->w, n->g, n->m, n->v, n->x, n->y, n->tgt, n->part, n->dscal, n->err};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  for (int l = 0; l < WN_NL; l++) {
    if (n->wk[l]) cudaFree(n->wk[l]);
    if (n->wt[l]) cudaFree(n->wt[l]);
  }
  for (bf16 *p : n->act)
    if (p) cudaFree(p);
  for (int k = 0; k < 4; k++) {
    if (n->gf[k]) cudaFree(n->gf[k]);
    if (n->ga[k]) cudaFree(n->ga[k]);
    if (n->gb[k]) cudaFree(n->gb[k]);
  }
  if (n->own) cudaStreamDestroy(n->own);
  delete n;
  return THORIN_OK;
}

extern "C" int thorin_warmnet_set_params(thorin_warmnet *n, const float *host, int count)
{
  if (!n || !host || count != THORIN_WN_NPARAMS) {
    g_last_error = "warmnet_set_params: count must be THORIN_WN_NPARAMS";
    return THORIN_ERR_ARG;
  }
  WNCHK(cudaMemcpyAsync(n->w, host, count * sizeof(float), cudaMemcpyHostToDevice, n->own));
  WNCHK(cudaMemsetAsync(n->m, 0, count * sizeof(float), n->own));
  WNCHK(cudaMemsetAsync(n->v, 0, count * sizeof(float), n->own));
  n->adam_t = 0;
  pack_all(n, n->own);
  WNCHK(cudaStreamSynchronize(n->own));
  return THORIN_OK;
}

extern "C" int thorin_warmnet_get_params(thorin_warmnet *n, float *host, int count)
{
  if (!n || !host || count != THORIN_WN_NPARAMS) {
    g_last_error = "warmnet_get_params: count must be THORIN_WN_NPARAMS";
    return THORIN_ERR_ARG;
  }
  WNCHK(cudaDeviceSynchronize());
  WNCHK(cudaMemcpy(host, n->w, count * sizeof(float), cudaMemcpyDeviceToHost));
  return THORIN_OK;
}

extern "C" int thorin_warmnet_forward(thorin_warmnet *n, int batch, const uint16_t *x, float *y)
{
  if (!n || !x || !y || batch < 1 || batch > n->maxb) {
    g_last_error = "warmnet_forward: 1 <= batch <= max_batch and buffers required";
    return THORIN_ERR_ARG;
  }
  const size_t P = (size_t)batch * n->nr * n->ns;
  WNCHK(cudaMemcpyAsync(n->x, x, P * THORIN_WN_INPUTS * sizeof(bf16), cudaMemcpyHostToDevice, n->own));
  RCHK_WN(wn_forward(n, batch, n->own));
  WNCHK(cudaMemcpyAsync(y, n->y, P * sizeof(float), cudaMemcpyDeviceToHost, n->own));
  WNCHK(cudaStreamSynchronize(n->own));
  return wn_check_err(n);
}

extern "C" int thorin_warmnet_gradient(thorin_warmnet *n, int batch, const uint16_t *x, const float *target,
                                       float *loss, float *grad)
{
  if (!n || !x || !target || batch < 1 || batch > n->maxb) {
    g_last_error = "warmnet_gradient: 1 <= batch <= max_batch and buffers required";
    return THORIN_ERR_ARG;
  }
  const size_t P = (size_t)batch * n->nr * n->ns;
  WNCHK(cudaMemcpyAsync(n->x, x, P * THORIN_WN_INPUTS * sizeof(bf16), cudaMemcpyHostToDevice, n->own));
  WNCHK(cudaMemcpyAsync(n->tgt, target, P * sizeof(float), cudaMemcpyHostToDevice, n->own));
  RCHK_WN(wn_forward(n, batch, n->own));
  RCHK_WN(wn_backward(n, batch, n->own));
  double l = 0.0;
  WNCHK(cudaMemcpyAsync(&l, n->dscal, sizeof(double), cudaMemcpyDeviceToHost, n->own));
  if (grad) WNCHK(cudaMemcpyAsync(grad, n->g, THORIN_WN_NPARAMS * sizeof(float), cudaMemcpyDeviceToHost, n->own));
  WNCHK(cudaStreamSynchronize(n->own));
  if (loss) *loss = (float)l;
  return wn_check_err(n);
}

extern "C" int thorin_warmnet_adam(thorin_warmnet *n, float lr, float beta1, float beta2, float eps, float max_norm)
{
  if (!n || !(lr > 0.f) || !(beta1 >= 0.f && beta1 < 1.f) || !(beta2 >= 0.f && beta2 < 1.f) || !(eps > 0.f)) {
    g_last_error = "warmnet_adam: lr > 0, 0 <= beta < 1, eps > 0";
    return THORIN_ERR_ARG;
  }
  RCHK_WN(wn_adam(n, lr, beta1, beta2, eps, max_norm, n->own));
  WNCHK(cudaStreamSynchronize(n->own));
  return THORIN_OK;
}
