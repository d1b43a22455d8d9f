// Learned surrogate: the 5 -> 128 -> 128 -> 128 -> 4 GELU network of
// spss_surrogate.h, trained and evaluated by hand-written tcgen05 kernels.
//
// Tensor-core scheme (one CTA = 128 rows of a batch, 4 warps):
//   * operands live in shared memory in the K-major, no-swizzle canonical
//     layout: core matrices of 8 rows x 16 bytes (8 BF16), adjacent along K at
//     128 bytes (leading byte offset), row groups at K/8 * 128 bytes (stride
//     byte offset);
//   * one thread issues tcgen05.mma.cta_group::1.kind::f16 (BF16 x BF16 ->
//     FP32, M = 128, N = 128 or 16, K = 16 per instruction) into a 128-column
//     tensor-memory accumulator and commits to an mbarrier (bounded wait);
//   * after the wait every thread reads its own row of the accumulator with
//     tcgen05.ld (warp w owns lanes 32w .. 32w + 31), applies bias and GELU in
//     FP32 and writes the BF16 activation back into shared memory as the next
//     layer's A operand.
// Backward: dZ_l = dA_l * GELU'(Z_l) with dA_{l-1} = dZ_l W_l (tensor cores,
// W_l^T staged as the K-major B operand), and dW_l = dZ_l^T A_{l-1} over
// 128-row batch chunks (both operands staged transposed, accumulated in tensor
// memory), reduced over CTAs in a fixed order; Adam on FP32 master weights.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <random>
#include <vector>

#include "spss_internal.cuh"
#include "spss_surrogate.h"

namespace spss
{
namespace mlp
{

constexpr int IN = SPSS_MLP_INPUTS, H = SPSS_MLP_HIDDEN, OUT = SPSS_MLP_OUTPUTS;
constexpr int INP = 16, OUTP = 16;  // input and output widths padded to the MMA granularity
constexpr int TR = 128;             // rows per CTA (MMA M)
constexpr int NP = SPSS_MLP_PARAMS;
constexpr int oW1 = 0, ob1 = oW1 + H * IN, oW2 = ob1 + H, ob2 = oW2 + H * H, oW3 = ob2 + H, ob3 = oW3 + H * H,
              oW4 = ob3 + H, ob4 = oW4 + OUT * H, oEnd = ob4 + OUT;
static_assert(oEnd == NP, "parameter count");
constexpr long long kWaitCycles = 1ll << 31;  // about one second at the SM clock
constexpr int kMaxPartials = 2 * 152;         // CTAs of the weight-gradient kernel

typedef __nv_bfloat16 bf16;

// ---------------------------------------------------------------- tcgen05

__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
  return (uint32_t) __cvta_generic_to_shared(p);
}

// Byte offset of element (r, k) of a K-major operand with K columns.
__device__ __forceinline__ uint32_t canon(int r, int k, int K)
{
  return (uint32_t) ((r >> 3) * (K >> 3) * 128 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// Shared-memory matrix descriptor: start address, leading and stride byte
// offsets (16-byte units), descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
  return (uint64_t) ((addr >> 4) & 0x3FFFu) | ((uint64_t) ((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t) ((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t) 1 << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N >> 3 and M >> 4.
__device__ __forceinline__ uint32_t instr_desc(int M, int N)
{
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t) (N >> 3) << 17) | ((uint32_t) (M >> 4) << 24);
}

// D[128 x N] (+)= A[128 x K] B[N x K]^T, both operands K-major in shared memory.
__device__ __forceinline__ void mma_issue(uint32_t tmem, const void *a, const void *b, int K, int N, bool accumulate)
{
  const uint32_t idesc = instr_desc(TR, N);
  const uint32_t sbo = (uint32_t) (K >> 3) * 128u;
  for (int kk = 0; kk < K / 16; ++kk)
  {
    const uint64_t ad = smem_desc(smem_addr(a) + kk * 256, 128, sbo);
    const uint64_t bd = smem_desc(smem_addr(b) + kk * 256, 128, sbo);
    const uint32_t acc = (accumulate || kk > 0) ? 1u : 0u;
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(
            tmem),
        "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
  }
}

__device__ __forceinline__ void mma_commit(const unsigned long long *mbar)
{
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(mbar))
               : "memory");
}

__device__ __forceinline__ uint32_t wait_phase(const unsigned long long *mbar, uint32_t phase)
{
  uint32_t done = 0;
  const long long t0 = clock64();
  while (!done && clock64() - t0 < kWaitCycles)
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                 : "=r"(done)
                 : "r"(smem_addr(mbar)), "r"(phase)
                 : "memory");
  return done;
}

__device__ __forceinline__ void fence_before_sync()
{
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void fence_after_sync()
{
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Operands written by threads become visible to the tensor cores, then a barrier.
__device__ __forceinline__ void publish_operands()
{
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
}

// 32 (or 16) consecutive accumulator columns of this thread's row.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float v[32])
{
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
      "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float v[16])
{
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// Tensor memory: 128 columns (FP32 128 x 128 accumulator), one warp.
__device__ __forceinline__ void tmem_alloc(uint32_t *dst)
{
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst)), "r"(128));
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t tmem)
{
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(128));
}

__device__ __forceinline__ void mbar_init(unsigned long long *mbar)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(mbar)));
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// ---------------------------------------------------------------- staging

// rows x K BF16 matrix (row-major, `valid` rows present, the rest zero) into
// the canonical layout, 16 bytes at a time.
__device__ __forceinline__ void stage_rows(unsigned char *dst, const bf16 *src, int rows, int valid, int K)
{
  const int chunks = rows * (K / 8);
  for (int c = threadIdx.x; c < chunks; c += blockDim.x)
  {
    const int r = c / (K / 8), k = (c - r * (K / 8)) * 8;
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (r < valid) v = *reinterpret_cast<const uint4 *>(src + (long) r * K + k);
    *reinterpret_cast<uint4 *>(dst + canon(r, k, K)) = v;
  }
}

// Eight consecutive columns c8 .. c8 + 7 of row r of a K-major operand.
__device__ __forceinline__ void put8(unsigned char *dst, int r, int c8, int K, const float v[8])
{
  __nv_bfloat162 h[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) h[j] = __floats2bfloat162_rn(v[2 * j], v[2 * j + 1]);
  *reinterpret_cast<uint4 *>(dst + canon(r, c8, K)) = *reinterpret_cast<const uint4 *>(h);
}

__device__ __forceinline__ float gelu(float x)
{
  return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f));
}

__device__ __forceinline__ float gelu_grad(float x)
{
  return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

struct Weights
{
  const float *p;                     // FP32 master parameters (flat order)
  const bf16 *w1, *w2, *w3, *w4;      // forward B operands: [128][16], [128][128], [128][128], [16][128]
  const bf16 *w4t, *w3t, *w2t;        // backward B operands (transposes): [128][16], [128][128], [128][128]
};

struct Acts
{
  bf16 *a[3];   // GELU outputs of the hidden layers, [rows][128]
  float *z[3];  // pre-activations, [rows][128]
};

constexpr int kFwdSmem = TR * H * 2 + H * INP * 2 + 2 * H * H * 2 + OUTP * H * 2;   // 104 KiB
constexpr int kBwdSmem = TR * H * 2 + H * OUTP * 2 + 2 * H * H * 2;                // 100 KiB
constexpr int kGradSmem = TR * TR * 2 + H * TR * 2;                                 // 64 KiB

// ---------------------------------------------------------------- forward

// Rows [128 b, 128 b + 128) of x (BF16 [n][16], inputs zero-padded): output
// y [n][4] (FP32); with `acts`, the hidden activations and pre-activations.
__global__ void __launch_bounds__(TR, 1) mlp_forward_kernel(Weights W, const bf16 *__restrict__ x, int n,
                                                            float *__restrict__ y, Acts acts, int save, int *status)
{
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char *sA = smem;
  unsigned char *sW1 = sA + TR * H * 2;
  unsigned char *sW2 = sW1 + H * INP * 2;
  unsigned char *sW3 = sW2 + H * H * 2;
  unsigned char *sW4 = sW3 + H * H * 2;
  __shared__ __align__(8) unsigned long long mbar;
  __shared__ uint32_t tmem_base;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int row0 = blockIdx.x * TR;
  const int valid = min(TR, n - row0);
  const int row = row0 + tid;
  stage_rows(sA, x + (long) row0 * INP, TR, valid, INP);
  stage_rows(sW1, W.w1, H, H, INP);
  stage_rows(sW2, W.w2, H, H, H);
  stage_rows(sW3, W.w3, H, H, H);
  stage_rows(sW4, W.w4, OUTP, OUTP, H);
  if (warp == 0) tmem_alloc(&tmem_base);
  if (tid == 0) mbar_init(&mbar);
  publish_operands();
  const uint32_t tmem = tmem_base;
  const uint32_t trow = tmem + ((uint32_t) (warp * 32) << 16);
  uint32_t phase = 0;
  bool ok = true;
  for (int l = 0; l < 4 && ok; ++l)
  {
    const unsigned char *sB = l == 0 ? sW1 : (l == 1 ? sW2 : (l == 2 ? sW3 : sW4));
    if (tid == 0)
    {
      mma_issue(tmem, sA, sB, l == 0 ? INP : H, l == 3 ? OUTP : H, false);
      mma_commit(&mbar);
    }
    ok = __syncthreads_and(wait_phase(&mbar, phase));
    if (!ok) break;
    phase ^= 1u;
    fence_after_sync();
    if (l < 3)
    {
      const float *b = W.p + (l == 0 ? ob1 : (l == 1 ? ob2 : ob3));
      for (int c0 = 0; c0 < H; c0 += 32)
      {
        float v[32];
        tmem_ld32(trow + c0, v);
#pragma unroll
        for (int j = 0; j < 32; ++j)
        {
          const float z = v[j] + __ldg(b + c0 + j);
          if (save && tid < valid) acts.z[l][(long) row * H + c0 + j] = z;
          v[j] = gelu(z);
        }
#pragma unroll
        for (int j = 0; j < 32; j += 8)
        {
          put8(sA, tid, c0 + j, H, v + j);
          if (save && tid < valid)
          {
            __nv_bfloat162 h[4];
            for (int u = 0; u < 4; ++u) h[u] = __floats2bfloat162_rn(v[j + 2 * u], v[j + 2 * u + 1]);
            *reinterpret_cast<uint4 *>(acts.a[l] + (long) row * H + c0 + j) = *reinterpret_cast<const uint4 *>(h);
          }
        }
      }
      publish_operands();
    } else
    {
      float v[16];
      tmem_ld16(trow, v);
      if (tid < valid)
        for (int o = 0; o < OUT; ++o) y[(long) row * OUT + o] = v[o] + __ldg(W.p + ob4 + o);
    }
  }
  if (!ok)
  {
    // the accumulator did not complete in time: report and give the MMAs a
    // second bounded wait before the tensor memory is released
    if (tid == 0) atomicOr(status, 1);
    wait_phase(&mbar, phase);
  }
  fence_before_sync();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem);
}

// ---------------------------------------------------------------- backward

// Loss gradient dZ4 = 2 w (y - t) / n_batch and the back-propagated dZ3, dZ2,
// dZ1 (BF16, the operands of the weight gradients); loss partial per CTA.
__global__ void __launch_bounds__(TR, 1) mlp_backward_kernel(Weights W, const float *__restrict__ y,
                                                             const float *__restrict__ t, float4 wl, float scale,
                                                             int n, Acts acts, bf16 *__restrict__ dz4,
                                                             bf16 *dz3, bf16 *dz2, bf16 *dz1,
                                                             float *__restrict__ loss_partial, int *status)
{
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char *sA = smem;
  unsigned char *sW4t = sA + TR * H * 2;
  unsigned char *sW3t = sW4t + H * OUTP * 2;
  unsigned char *sW2t = sW3t + H * H * 2;
  __shared__ __align__(8) unsigned long long mbar;
  __shared__ uint32_t tmem_base;
  __shared__ float red[TR / 32];
  const int tid = threadIdx.x, warp = tid >> 5;
  const int row0 = blockIdx.x * TR;
  const int valid = min(TR, n - row0);
  const int row = row0 + tid;
  const bool live = tid < valid;
  stage_rows(sW4t, W.w4t, H, H, OUTP);
  stage_rows(sW3t, W.w3t, H, H, H);
  stage_rows(sW2t, W.w2t, H, H, H);
  // output layer
  {
    const float w4[4] = {wl.x, wl.y, wl.z, wl.w};
    float g[16], loss = 0.0f;
#pragma unroll
    for (int o = 0; o < 16; ++o) g[o] = 0.0f;
    if (live)
      for (int o = 0; o < OUT; ++o)
      {
        const float d = y[(long) row * OUT + o] - t[(long) row * OUT + o];
        loss += w4[o] * d * d;
        g[o] = 2.0f * w4[o] * d * scale;
      }
    put8(sA, tid, 0, OUTP, g);
    put8(sA, tid, 8, OUTP, g + 8);
    if (live)
    {
      __nv_bfloat162 h[8];
      for (int u = 0; u < 8; ++u) h[u] = __floats2bfloat162_rn(g[2 * u], g[2 * u + 1]);
      *reinterpret_cast<uint4 *>(dz4 + (long) row * OUTP) = *reinterpret_cast<const uint4 *>(h);
      *reinterpret_cast<uint4 *>(dz4 + (long) row * OUTP + 8) = *reinterpret_cast<const uint4 *>(h + 4);
    }
    for (int off = 16; off > 0; off >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, off);
    if ((tid & 31) == 0) red[warp] = loss;
  }
  if (warp == 0) tmem_alloc(&tmem_base);
  if (tid == 0) mbar_init(&mbar);
  publish_operands();
  if (tid == 0) loss_partial[blockIdx.x] = red[0] + red[1] + red[2] + red[3];
  const uint32_t tmem = tmem_base;
  const uint32_t trow = tmem + ((uint32_t) (warp * 32) << 16);
  uint32_t phase = 0;
  bool ok = true;
  // dA_{l} = dZ_{l+1} W_{l+1}, l = 2, 1, 0 (hidden layers 3, 2, 1)
  for (int l = 2; l >= 0 && ok; --l)
  {
    const unsigned char *sB = l == 2 ? sW4t : (l == 1 ? sW3t : sW2t);
    if (tid == 0)
    {
      mma_issue(tmem, sA, sB, l == 2 ? OUTP : H, H, false);
      mma_commit(&mbar);
    }
    ok = __syncthreads_and(wait_phase(&mbar, phase));
    if (!ok) break;
    phase ^= 1u;
    fence_after_sync();
    bf16 *dz = l == 2 ? dz3 : (l == 1 ? dz2 : dz1);
    for (int c0 = 0; c0 < H; c0 += 32)
    {
      float v[32];
      tmem_ld32(trow + c0, v);
#pragma unroll
      for (int j = 0; j < 32; ++j)
        v[j] = live ? v[j] * gelu_grad(acts.z[l][(long) row * H + c0 + j]) : 0.0f;
#pragma unroll
      for (int j = 0; j < 32; j += 8)
      {
        put8(sA, tid, c0 + j, H, v + j);
        if (live)
        {
          __nv_bfloat162 h[4];
          for (int u = 0; u < 4; ++u) h[u] = __floats2bfloat162_rn(v[j + 2 * u], v[j + 2 * u + 1]);
          *reinterpret_cast<uint4 *>(dz + (long) row * H + c0 + j) = *reinterpret_cast<const uint4 *>(h);
        }
      }
    }
    publish_operands();
  }
  if (!ok)
  {
    if (tid == 0) atomicOr(status, 1);
    wait_phase(&mbar, phase);
  }
  fence_before_sync();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem);
}

// dW = dZ^T A_prev over 128-row chunks of the batch (CTA c takes chunks c,
// c + gridDim.x, ...), accumulated in tensor memory: A operand [m = out][k =
// row] and B operand [n = in][k = row] staged transposed.  dz: [n][zp] (zp
// outputs, zero rows above), ap: [n][kin].  Partials: pw[cta][128][kin],
// pb[cta][128].
__global__ void __launch_bounds__(TR, 1) mlp_weight_grad_kernel(const bf16 *__restrict__ dz, int zp,
                                                                const bf16 *__restrict__ ap, int kin, int n,
                                                                float *__restrict__ pw, float *__restrict__ pb,
                                                                int *status)
{
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char *sA = smem;               // [128 out][128 rows]
  unsigned char *sB = sA + TR * TR * 2;   // [kin][128 rows]
  __shared__ __align__(8) unsigned long long mbar;
  __shared__ uint32_t tmem_base;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int chunks = (n + TR - 1) / TR;
  // rows of the A operand beyond the layer's outputs stay zero
  for (int c = tid; c < TR * TR / 8; c += TR)
  {
    const int r = c / (TR / 8), k = (c - r * (TR / 8)) * 8;
    if (r >= zp) *reinterpret_cast<uint4 *>(sA + canon(r, k, TR)) = make_uint4(0u, 0u, 0u, 0u);
  }
  if (warp == 0) tmem_alloc(&tmem_base);
  if (tid == 0) mbar_init(&mbar);
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = tmem_base;
  uint32_t phase = 0;
  bool ok = true, any = false;
  float db = 0.0f;
  for (int c = blockIdx.x; c < chunks && ok; c += gridDim.x)
  {
    // thread = row of the chunk
    const int r = c * TR + tid;
    const bool live = r < n;
    for (int m8 = 0; m8 < zp; m8 += 8)
    {
      uint4 raw = make_uint4(0u, 0u, 0u, 0u);
      if (live) raw = *reinterpret_cast<const uint4 *>(dz + (long) r * zp + m8);
      const bf16 *h = reinterpret_cast<const bf16 *>(&raw);
      for (int u = 0; u < 8; ++u) *reinterpret_cast<bf16 *>(sA + canon(m8 + u, tid, TR)) = h[u];
    }
    for (int k8 = 0; k8 < kin; k8 += 8)
    {
      uint4 raw = make_uint4(0u, 0u, 0u, 0u);
      if (live) raw = *reinterpret_cast<const uint4 *>(ap + (long) r * kin + k8);
      const bf16 *h = reinterpret_cast<const bf16 *>(&raw);
      for (int u = 0; u < 8; ++u) *reinterpret_cast<bf16 *>(sB + canon(k8 + u, tid, TR)) = h[u];
    }
    publish_operands();
    // bias gradient: thread m sums row m of the staged dZ^T
    if (tid < zp)
      for (int k = 0; k < TR; ++k) db += __bfloat162float(*reinterpret_cast<const bf16 *>(sA + canon(tid, k, TR)));
    if (tid == 0)
    {
      mma_issue(tmem, sA, sB, TR, kin, any);
      mma_commit(&mbar);
    }
    ok = __syncthreads_and(wait_phase(&mbar, phase));
    phase ^= 1u;
    any = true;
    fence_after_sync();
  }
  const int m = tid;
  float *out = pw + ((long) blockIdx.x * TR + m) * kin;
  if (ok && any)
  {
    const uint32_t trow = tmem + ((uint32_t) (warp * 32) << 16);
    for (int c0 = 0; c0 < kin; c0 += 16)
    {
      float v[16];
      tmem_ld16(trow + c0, v);
      for (int j = 0; j < 16; ++j) out[c0 + j] = v[j];
    }
  } else
  {
    for (int j = 0; j < kin; ++j) out[j] = 0.0f;
  }
  pb[(long) blockIdx.x * TR + m] = db;
  if (!ok)
  {
    if (tid == 0) atomicOr(status, 1);
    wait_phase(&mbar, phase ^ 1u);
  }
  fence_before_sync();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem);
}

// ---------------------------------------------------------------- optimiser

struct Grads
{
  const float *pw[4], *pb[4];  // partials of the four layers
  int parts[4];                // partial count per layer
};

struct Adam
{
  float *p, *m1, *m2;
  bf16 *w1, *w2, *w3, *w4, *w4t, *w3t, *w2t;
  float lr, c1, c2;  // learning rate, 1 - beta1^t, 1 - beta2^t
};

// Layer, row and column of flat parameter i (col -1: bias).
__device__ __forceinline__ void locate(int i, int &layer, int &m, int &c)
{
  if (i < ob1)
  {
    layer = 0;
    m = i / IN;
    c = i - m * IN;
  } else if (i < oW2)
  {
    layer = 0;
    m = i - ob1;
    c = -1;
  } else if (i < ob2)
  {
    layer = 1;
    m = (i - oW2) / H;
    c = (i - oW2) - m * H;
  } else if (i < oW3)
  {
    layer = 1;
    m = i - ob2;
    c = -1;
  } else if (i < ob3)
  {
    layer = 2;
    m = (i - oW3) / H;
    c = (i - oW3) - m * H;
  } else if (i < oW4)
  {
    layer = 2;
    m = i - ob3;
    c = -1;
  } else if (i < ob4)
  {
    layer = 3;
    m = (i - oW4) / H;
    c = (i - oW4) - m * H;
  } else
  {
    layer = 3;
    m = i - ob4;
    c = -1;
  }
}

// Sum the partial gradients (fixed order), optionally take an Adam step, and
// refresh the BF16 operand copies of every weight.
__global__ void mlp_update_kernel(Adam A, Grads G, int update, float *__restrict__ grad_out)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NP) return;
  int layer, m, c;
  locate(i, layer, m, c);
  const int kin = layer == 0 ? INP : H;
  float g = 0.0f;
  for (int q = 0; q < G.parts[layer]; ++q)
    g += c >= 0 ? G.pw[layer][((long) q * TR + m) * kin + c] : G.pb[layer][(long) q * TR + m];
  if (grad_out) grad_out[i] = g;
  float p = A.p[i];
  if (update)
  {
    const float m1 = 0.9f * A.m1[i] + 0.1f * g;
    const float m2 = 0.999f * A.m2[i] + 0.001f * g * g;
    A.m1[i] = m1;
    A.m2[i] = m2;
    p -= A.lr * (m1 / A.c1) / (sqrtf(m2 / A.c2) + 1e-8f);
    A.p[i] = p;
  }
  if (c < 0) return;
  const bf16 h = __float2bfloat16_rn(p);
  switch (layer)
  {
    case 0: A.w1[m * INP + c] = h; break;
    case 1:
      A.w2[m * H + c] = h;
      A.w2t[c * H + m] = h;
      break;
    case 2:
      A.w3[m * H + c] = h;
      A.w3t[c * H + m] = h;
      break;
    default:
      A.w4[m * H + c] = h;
      A.w4t[c * OUTP + m] = h;
      break;
  }
}

// FP32 inputs [n][5] -> BF16 [n][16] (zero padding), optionally gathered
// through a permutation; targets [n][4] gathered alongside.
__global__ void mlp_pack_kernel(const float *__restrict__ x, const float *__restrict__ t, const int *__restrict__ perm,
                                long n, bf16 *__restrict__ xb, float *__restrict__ tout)
{
  const long i = (long) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const long s = perm ? perm[i] : i;
  bf16 v[INP];
  for (int k = 0; k < INP; ++k) v[k] = __float2bfloat16_rn(k < IN ? x[s * IN + k] : 0.0f);
  *reinterpret_cast<uint4 *>(xb + i * INP) = *reinterpret_cast<const uint4 *>(v);
  *reinterpret_cast<uint4 *>(xb + i * INP + 8) = *reinterpret_cast<const uint4 *>(v + 8);
  if (t && tout)
    for (int o = 0; o < OUT; ++o) tout[i * OUT + o] = t[s * OUT + o];
}

}  // namespace mlp
}  // namespace spss

using namespace spss;
using namespace spss::mlp;

struct spss_mlp
{
  cudaStream_t stream = nullptr;
  DeviceArray<float> p, m1, m2, grad;
  DeviceArray<bf16> w1, w2, w3, w4, w4t, w3t, w2t;
  // resident training set and its shuffled copy
  DeviceArray<float> x_raw, t_raw, t_shuf;
  DeviceArray<bf16> x_shuf;
  DeviceArray<int> perm;
  long n_data = 0;
  // batch workspace
  DeviceArray<bf16> xb, a[3], dz4, dz[3];
  DeviceArray<float> xin, tin, y, z[3], pw[4], pb[4], loss_partial;
  DeviceArray<int> status;
  long rows_cap = 0;
  long step = 0;
  unsigned long long launches = 0;
};

namespace
{

int reserve_rows(spss_mlp *m, long rows)
{
  rows = (rows + TR - 1) / TR * TR;
  if (rows <= m->rows_cap) return SPSS_OK;
  SPSS_TRY(m->xb.reserve((size_t) rows * INP));
  SPSS_TRY(m->y.reserve((size_t) rows * OUT));
  SPSS_TRY(m->tin.reserve((size_t) rows * OUT));
  SPSS_TRY(m->dz4.reserve((size_t) rows * OUTP));
  for (int l = 0; l < 3; ++l)
  {
    SPSS_TRY(m->a[l].reserve((size_t) rows * H));
    SPSS_TRY(m->dz[l].reserve((size_t) rows * H));
    SPSS_TRY(m->z[l].reserve((size_t) rows * H));
  }
  SPSS_TRY(m->loss_partial.reserve((size_t) rows / TR));
  m->rows_cap = rows;
  return SPSS_OK;
}

Weights weights(spss_mlp *m)
{
  return Weights{m->p.ptr, m->w1.ptr, m->w2.ptr, m->w3.ptr, m->w4.ptr, m->w4t.ptr, m->w3t.ptr, m->w2t.ptr};
}

Acts acts(spss_mlp *m)
{
  return Acts{{m->a[0].ptr, m->a[1].ptr, m->a[2].ptr}, {m->z[0].ptr, m->z[1].ptr, m->z[2].ptr}};
}

int check_status(spss_mlp *m)
{
  int st = 0;
  SPSS_CUDA_TRY(cudaMemcpyAsync(&st, m->status.ptr, sizeof(int), cudaMemcpyDeviceToHost, m->stream));
  SPSS_CUDA_TRY(cudaStreamSynchronize(m->stream));
  return st ? SPSS_ERR_CUDA : SPSS_OK;
}

int forward_rows(spss_mlp *m, const bf16 *xb, long rows, float *y, int save)
{
  const int blocks = (int) ((rows + TR - 1) / TR);
  mlp_forward_kernel<<<blocks, TR, kFwdSmem, m->stream>>>(weights(m), xb, (int) rows, y, acts(m), save,
                                                          m->status.ptr);
  ++m->launches;
  return check_launch("mlp_forward_kernel");
}

// Gradient of the batch held in xb / tin (rows rows): partials, then the
// update kernel (with or without an Adam step).
int backward_rows(spss_mlp *m, long rows, const float w[4], float lr, int update, float *grad_out)
{
  const int blocks = (int) ((rows + TR - 1) / TR);
  const float4 wl = make_float4(w[0], w[1], w[2], w[3]);
  mlp_backward_kernel<<<blocks, TR, kBwdSmem, m->stream>>>(weights(m), m->y.ptr, m->tin.ptr, wl,
                                                           1.0f / (float) rows, (int) rows, acts(m), m->dz4.ptr,
                                                           m->dz[2].ptr, m->dz[1].ptr, m->dz[0].ptr,
                                                           m->loss_partial.ptr, m->status.ptr);
  ++m->launches;
  SPSS_TRY(check_launch("mlp_backward_kernel"));
  const int parts = std::min(blocks, kMaxPartials);
  Grads G;
  // layer l: dZ_l [rows][zp] and its input A_{l-1} [rows][kin]
  const bf16 *dzs[4] = {m->dz[0].ptr, m->dz[1].ptr, m->dz[2].ptr, m->dz4.ptr};
  const bf16 *ins[4] = {m->xb.ptr, m->a[0].ptr, m->a[1].ptr, m->a[2].ptr};
  for (int l = 0; l < 4; ++l)
  {
    const int zp = l == 3 ? OUTP : H, kin = l == 0 ? INP : H;
    mlp_weight_grad_kernel<<<parts, TR, kGradSmem, m->stream>>>(dzs[l], zp, ins[l], kin, (int) rows, m->pw[l].ptr,
                                                                m->pb[l].ptr, m->status.ptr);
    ++m->launches;
    SPSS_TRY(check_launch("mlp_weight_grad_kernel"));
    G.pw[l] = m->pw[l].ptr;
    G.pb[l] = m->pb[l].ptr;
    G.parts[l] = parts;
  }
  Adam A;
  A.p = m->p.ptr;
  A.m1 = m->m1.ptr;
  A.m2 = m->m2.ptr;
  A.w1 = m->w1.ptr;
  A.w2 = m->w2.ptr;
  A.w3 = m->w3.ptr;
  A.w4 = m->w4.ptr;
  A.w4t = m->w4t.ptr;
  A.w3t = m->w3t.ptr;
  A.w2t = m->w2t.ptr;
  A.lr = 0.0f;
  A.c1 = A.c2 = 1.0f;
  if (update)
  {
    m->step += 1;
    A.lr = lr;
    A.c1 = (float) (1.0 - std::pow(0.9, (double) m->step));
    A.c2 = (float) (1.0 - std::pow(0.999, (double) m->step));
  }
  mlp_update_kernel<<<(NP + 255) / 256, 256, 0, m->stream>>>(A, G, update, grad_out);
  return check_launch("mlp_update_kernel");
}

// BF16 operand copies from the master parameters.
int refresh_copies(spss_mlp *m)
{
  Grads G;
  for (int l = 0; l < 4; ++l)
  {
    G.pw[l] = nullptr;
    G.pb[l] = nullptr;
    G.parts[l] = 0;
  }
  Adam A;
  std::memset(&A, 0, sizeof(A));
  A.p = m->p.ptr;
  A.w1 = m->w1.ptr;
  A.w2 = m->w2.ptr;
  A.w3 = m->w3.ptr;
  A.w4 = m->w4.ptr;
  A.w4t = m->w4t.ptr;
  A.w3t = m->w3t.ptr;
  A.w2t = m->w2t.ptr;
  A.c1 = A.c2 = 1.0f;
  mlp_update_kernel<<<(NP + 255) / 256, 256, 0, m->stream>>>(A, G, 0, nullptr);
  return check_launch("mlp_update_kernel");
}

int upload_batch(spss_mlp *m, const float *x, const float *t, long n)
{
  SPSS_TRY(reserve_rows(m, n));
  SPSS_TRY(m->xin.reserve((size_t) n * IN));
  SPSS_CUDA_TRY(cudaMemcpyAsync(m->xin.ptr, x, sizeof(float) * n * IN, cudaMemcpyHostToDevice, m->stream));
  float *traw = nullptr;
  if (t)
  {
    SPSS_TRY(m->t_raw.reserve((size_t) n * OUT));
    SPSS_CUDA_TRY(cudaMemcpyAsync(m->t_raw.ptr, t, sizeof(float) * n * OUT, cudaMemcpyHostToDevice, m->stream));
    traw = m->t_raw.ptr;
  }
  mlp_pack_kernel<<<(int) ((n + 255) / 256), 256, 0, m->stream>>>(m->xin.ptr, traw, nullptr, n, m->xb.ptr,
                                                                   t ? m->tin.ptr : nullptr);
  return check_launch("mlp_pack_kernel");
}

}  // namespace

extern "C" {

int spss_mlp_create(unsigned long long seed, spss_mlp **out)
{
  if (!out) return SPSS_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  spss_mlp *m = new (std::nothrow) spss_mlp();
  if (!m) return SPSS_ERR_OUT_OF_MEMORY;
  int rc = SPSS_OK;
  auto fail = [&](int code) {
    spss_mlp_destroy(m);
    return code;
  };
  if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess)
  {
    cudaGetLastError();
    return fail(SPSS_ERR_CUDA);
  }
  if ((rc = m->p.reserve(NP)) || (rc = m->m1.reserve(NP)) || (rc = m->m2.reserve(NP)) || (rc = m->grad.reserve(NP)) ||
      (rc = m->w1.reserve(H * INP)) || (rc = m->w2.reserve(H * H)) || (rc = m->w3.reserve(H * H)) ||
      (rc = m->w4.reserve(OUTP * H)) || (rc = m->w4t.reserve(H * OUTP)) || (rc = m->w3t.reserve(H * H)) ||
      (rc = m->w2t.reserve(H * H)) || (rc = m->status.reserve(1)))
    return fail(rc);
  for (int l = 0; l < 4; ++l)
  {
    const int kin = l == 0 ? INP : H;
    if ((rc = m->pw[l].reserve((size_t) kMaxPartials * TR * kin)) || (rc = m->pb[l].reserve((size_t) kMaxPartials * TR)))
      return fail(rc);
  }
  if (cudaFuncSetAttribute(mlp_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kFwdSmem) != cudaSuccess ||
      cudaFuncSetAttribute(mlp_backward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kBwdSmem) != cudaSuccess ||
      cudaFuncSetAttribute(mlp_weight_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kGradSmem) !=
          cudaSuccess)
  {
    cudaGetLastError();
    return fail(SPSS_ERR_CUDA);
  }
  // padding of the operand copies stays zero
  cudaMemsetAsync(m->w1.ptr, 0, sizeof(bf16) * H * INP, m->stream);
  cudaMemsetAsync(m->w4.ptr, 0, sizeof(bf16) * OUTP * H, m->stream);
  cudaMemsetAsync(m->w4t.ptr, 0, sizeof(bf16) * H * OUTP, m->stream);
  cudaMemsetAsync(m->m1.ptr, 0, sizeof(float) * NP, m->stream);
  cudaMemsetAsync(m->m2.ptr, 0, sizeof(float) * NP, m->stream);
  cudaMemsetAsync(m->status.ptr, 0, sizeof(int), m->stream);
  std::vector<float> h(NP, 0.0f);
  std::mt19937_64 gen(seed);
  auto fill = [&](int off, int count, int fan_in) {
    std::uniform_real_distribution<float> U(-1.0f / std::sqrt((float) fan_in), 1.0f / std::sqrt((float) fan_in));
    for (int i = 0; i < count; ++i) h[off + i] = U(gen);
  };
  fill(oW1, H * IN, IN);
  fill(oW2, H * H, H);
  fill(oW3, H * H, H);
  fill(oW4, OUT * H, H);
  *out = m;
  rc = spss_mlp_set_params(m, h.data(), NP);
  if (rc != SPSS_OK)
  {
    *out = nullptr;
    return fail(rc);
  }
  return SPSS_OK;
}

int spss_mlp_destroy(spss_mlp *m)
{
  if (!m) return SPSS_ERR_INVALID_ARGUMENT;
  if (m->stream) cudaStreamSynchronize(m->stream);
  m->p.release();
  m->m1.release();
  m->m2.release();
  m->grad.release();
  m->w1.release();
  m->w2.release();
  m->w3.release();
  m->w4.release();
  m->w4t.release();
  m->w3t.release();
  m->w2t.release();
  m->x_raw.release();
  m->t_raw.release();
  m->t_shuf.release();
  m->x_shuf.release();
  m->perm.release();
  m->xb.release();
  m->dz4.release();
  m->xin.release();
  m->tin.release();
  m->y.release();
  m->loss_partial.release();
  m->status.release();
  for (int l = 0; l < 3; ++l)
  {
    m->a[l].release();
    m->dz[l].release();
    m->z[l].release();
  }
  for (int l = 0; l < 4; ++l)
  {
    m->pw[l].release();
    m->pb[l].release();
  }
  if (m->stream) cudaStreamDestroy(m->stream);
  cudaGetLastError();
  delete m;
  return SPSS_OK;
}

int spss_mlp_set_params(spss_mlp *m, const float *params, long len)
{
  if (!m || !params) return SPSS_ERR_INVALID_ARGUMENT;
  if (len != NP) return SPSS_ERR_SIZE;
  SPSS_CUDA_TRY(cudaMemcpyAsync(m->p.ptr, params, sizeof(float) * NP, cudaMemcpyHostToDevice, m->stream));
  SPSS_CUDA_TRY(cudaMemsetAsync(m->m1.ptr, 0, sizeof(float) * NP, m->stream));
  SPSS_CUDA_TRY(cudaMemsetAsync(m->m2.ptr, 0, sizeof(float) * NP, m->stream));
  m->step = 0;
  SPSS_TRY(refresh_copies(m));
  SPSS_CUDA_TRY(cudaStreamSynchronize(m->stream));
  return SPSS_OK;
}

int spss_mlp_get_params(spss_mlp *m, float *params, long len)
{
  if (!m || !params) return SPSS_ERR_INVALID_ARGUMENT;
  if (len != NP) return SPSS_ERR_SIZE;
  SPSS_CUDA_TRY(cudaMemcpyAsync(params, m->p.ptr, sizeof(float) * NP, cudaMemcpyDeviceToHost, m->stream));
  SPSS_CUDA_TRY(cudaStreamSynchronize(m->stream));
  return SPSS_OK;
}

int spss_mlp_forward(spss_mlp *m, const float *x, long n, float *y)
{
  if (!m || !x || !y || n <= 0) return SPSS_ERR_INVALID_ARGUMENT;
  if (n > 0x7fffff00L) return SPSS_ERR_SIZE;
  SPSS_TRY(upload_batch(m, x, nullptr, n));
  SPSS_TRY(forward_rows(m, m->xb.ptr, n, m->y.ptr, 0));
  SPSS_CUDA_TRY(cudaMemcpyAsync(y, m->y.ptr, sizeof(float) * n * OUT, cudaMemcpyDeviceToHost, m->stream));
  return check_status(m);
}

int spss_mlp_gradient(spss_mlp *m, const float *x, const float *t, const float *w, long n, float *grad, double *loss)
{
  if (!m || !x || !t || !grad || n <= 0) return SPSS_ERR_INVALID_ARGUMENT;
  if (n > 0x7fffff00L) return SPSS_ERR_SIZE;
  const float ones[4] = {1.0f, 1.0f, 1.0f, 1.0f};
  float wl[4];
  std::memcpy(wl, w ? w : ones, 4 * sizeof(float));
  SPSS_TRY(upload_batch(m, x, t, n));
  SPSS_TRY(forward_rows(m, m->xb.ptr, n, m->y.ptr, 1));
  SPSS_TRY(backward_rows(m, n, wl, 0.0f, 0, m->grad.ptr));
  SPSS_CUDA_TRY(cudaMemcpyAsync(grad, m->grad.ptr, sizeof(float) * NP, cudaMemcpyDeviceToHost, m->stream));
  const int blocks = (int) ((n + TR - 1) / TR);
  std::vector<float> lp(blocks);
  SPSS_CUDA_TRY(cudaMemcpyAsync(lp.data(), m->loss_partial.ptr, sizeof(float) * blocks, cudaMemcpyDeviceToHost,
                                m->stream));
  SPSS_TRY(check_status(m));
  if (loss)
  {
    double s = 0.0;
    for (float v : lp) s += v;
    *loss = s / (double) n;
  }
  return SPSS_OK;
}

int spss_mlp_set_data(spss_mlp *m, const float *x, const float *t, long n)
{
  if (!m || !x || !t || n <= 0) return SPSS_ERR_INVALID_ARGUMENT;
  if (n > 0x7fffff00L) return SPSS_ERR_SIZE;
  SPSS_TRY(m->x_raw.reserve((size_t) n * IN));
  SPSS_TRY(m->t_raw.reserve((size_t) n * OUT));
  SPSS_TRY(m->x_shuf.reserve((size_t) ((n + TR - 1) / TR * TR) * INP));
  SPSS_TRY(m->t_shuf.reserve((size_t) ((n + TR - 1) / TR * TR) * OUT));
  SPSS_TRY(m->perm.reserve((size_t) n));
  SPSS_CUDA_TRY(cudaMemcpyAsync(m->x_raw.ptr, x, sizeof(float) * n * IN, cudaMemcpyHostToDevice, m->stream));
  SPSS_CUDA_TRY(cudaMemcpyAsync(m->t_raw.ptr, t, sizeof(float) * n * OUT, cudaMemcpyHostToDevice, m->stream));
  SPSS_CUDA_TRY(cudaStreamSynchronize(m->stream));
  m->n_data = n;
  return SPSS_OK;
}

int spss_mlp_train(spss_mlp *m, int epochs, int batch, float lr, const float *w, unsigned long long shuffle_seed,
                   float *loss_per_epoch)
{
  if (!m || epochs < 0 || batch < TR || batch % TR || !(lr > 0.0f)) return SPSS_ERR_INVALID_ARGUMENT;
  if (m->n_data <= 0) return SPSS_ERR_INVALID_ARGUMENT;
  const long n = m->n_data;
  SPSS_TRY(reserve_rows(m, batch));
  float wl[4] = {1.0f, 1.0f, 1.0f, 1.0f};
  if (w) std::memcpy(wl, w, 4 * sizeof(float));
  std::vector<int> perm((size_t) n);
  const long nb = (n + batch - 1) / batch;
  std::vector<float> lp((size_t) nb * (batch / TR));
  for (int e = 0; e < epochs; ++e)
  {
    for (long i = 0; i < n; ++i) perm[i] = (int) i;
    std::mt19937_64 gen(shuffle_seed + (unsigned long long) e);
    std::shuffle(perm.begin(), perm.end(), gen);
    SPSS_CUDA_TRY(cudaMemcpyAsync(m->perm.ptr, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, m->stream));
    mlp_pack_kernel<<<(int) ((n + 255) / 256), 256, 0, m->stream>>>(m->x_raw.ptr, m->t_raw.ptr, m->perm.ptr, n,
                                                                     m->x_shuf.ptr, m->t_shuf.ptr);
    SPSS_TRY(check_launch("mlp_pack_kernel"));
    double epoch_loss = 0.0;
    for (long b = 0; b < nb; ++b)
    {
      const long r0 = b * batch, rows = std::min<long>(batch, n - r0);
      // the batch views the shuffled set in place
      SPSS_CUDA_TRY(cudaMemcpyAsync(m->xb.ptr, m->x_shuf.ptr + r0 * INP, sizeof(bf16) * rows * INP,
                                    cudaMemcpyDeviceToDevice, m->stream));
      SPSS_CUDA_TRY(cudaMemcpyAsync(m->tin.ptr, m->t_shuf.ptr + r0 * OUT, sizeof(float) * rows * OUT,
                                    cudaMemcpyDeviceToDevice, m->stream));
      SPSS_TRY(forward_rows(m, m->xb.ptr, rows, m->y.ptr, 1));
      SPSS_TRY(backward_rows(m, rows, wl, lr, 1, nullptr));
      const int blocks = (int) ((rows + TR - 1) / TR);
      SPSS_CUDA_TRY(cudaMemcpyAsync(lp.data() + b * (batch / TR), m->loss_partial.ptr, sizeof(float) * blocks,
                                    cudaMemcpyDeviceToHost, m->stream));
      SPSS_CUDA_TRY(cudaStreamSynchronize(m->stream));
      double s = 0.0;
      for (int q = 0; q < blocks; ++q) s += lp[b * (batch / TR) + q];
      epoch_loss += s / (double) rows;
    }
    if (loss_per_epoch) loss_per_epoch[e] = (float) (epoch_loss / (double) nb);
  }
  return check_status(m);
}

int spss_mlp_kernel_launches(spss_mlp *m, unsigned long long *count)
{
  if (!m || !count) return SPSS_ERR_INVALID_ARGUMENT;
  *count = m->launches;
  return SPSS_OK;
}

}  // extern "C"
