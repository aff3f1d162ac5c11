// Surrogate network for the Newton initial guess: an MLP
//   (x, y, z, t, p, D) -> 256 -> 256 -> 256 -> 256 -> 18,   SiLU on the hidden layers,
// BF16 weights and activations, FP32 accumulation, FP32 master weights (Adam).
//
// Every dense layer, forward and backward, is one call of k_gemm_tc: a hand-written
// tcgen05 GEMM for sm_103a.  A CTA owns a 128 x NT output tile whose FP32 accumulator
// lives in tensor memory (TMEM, NT columns); K is staged through shared memory in 64-wide
// chunks in the canonical no-swizzle K-major layout (8-row x 16-byte core matrices),
// one elected thread issues tcgen05.mma (kind::f16, BF16 inputs) per 16-wide K step and
// commits to an mbarrier; the epilogue reads TMEM with tcgen05.ld and fuses the layer's
// elementwise work (bias, SiLU, SiLU', loss gradient) before writing.
//
//   forward : Z_l = H_{l-1} W_l^T + b_l,  H_l = SiLU(Z_l)        (GEMM M = points)
//   backward: dH_{l-1} = delta_l W_l,  delta_{l-1} = dH_{l-1} * SiLU'(Z_{l-1})
//             dW_l^T = H_{l-1}^T delta_l                          (GEMM M = fan-in, K = points, split-K)
//
// All mbarrier waits are bounded: on timeout the kernel raises an error flag, waits
// again (bounded) for its own MMAs, frees its TMEM and returns.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "glgpu.h"
#include "glgpu_internal.h"

namespace glgpu
{
namespace mlp
{
constexpr int kIn = 6, kInPad = 16, kHid = 256, kOut = 18, kOutPad = 32, kLayers = 5;
constexpr int kTileM = 128, kKChunk = 64, kGemmThreads = 256;
constexpr int kSplitMax = 64;
constexpr uint32_t kWaitLimit = 1u << 26;

enum Epi
{
  EPI_HIDDEN = 0, // z = acc + b; store z (f32), SiLU(z) (bf16, row-major and transposed)
  EPI_OUTPUT = 1, // y = acc + b (f32)
  EPI_DELTA = 2,  // delta = acc * SiLU'(z) (bf16 row-major and transposed)
  EPI_PARTIAL = 3 // split-K partial of a weight gradient (f32)
};

struct GemmArgs
{
  const __nv_bfloat16 *A; // [M][lda]
  const __nv_bfloat16 *B; // [N][ldb]
  int M, N, K, lda, ldb;
  int k_per_split;        // K range of one split (multiple of 16)
  const float *bias;      // [N]
  float *out_f32;         // [M][ldo] (EPI_HIDDEN: z, EPI_OUTPUT: y, EPI_PARTIAL: [split][M][ldo])
  int ldo;
  __nv_bfloat16 *out_h;   // [M][ldh]
  int ldh;
  __nv_bfloat16 *out_t;   // [N][ldt] transposed copy
  int ldt;
  const float *z_in;      // [M][ldz] pre-activations for EPI_DELTA
  int ldz;
  int *err;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

// tcgen05 shared-memory matrix descriptor: start, leading (K) and stride (M/N) byte
// offsets, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
  uint64_t d = static_cast<uint64_t>((saddr & 0x3FFFF) >> 4);
  d |= static_cast<uint64_t>((lbo & 0x3FFFF) >> 4) << 16;
  d |= static_cast<uint64_t>((sbo & 0x3FFFF) >> 4) << 32;
  d |= static_cast<uint64_t>(1) << 46;
  return d;
}

// instruction descriptor: BF16 x BF16 -> FP32, both K-major, M = 128, N = n
__host__ __device__ constexpr uint32_t idesc_bf16(int n)
{
  return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(n >> 3) << 17) | (static_cast<uint32_t>(128 >> 4) << 24);
}

__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity)
{
  uint32_t done = 0;
  for (uint32_t it = 0; it < kWaitLimit && !done; ++it)
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(done)
                 : "r"(mbar), "r"(parity));
  return done != 0;
}

__device__ __forceinline__ float silu(float z) { return z / (1.f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z)
{
  const float s = 1.f / (1.f + __expf(-z));
  return s * (1.f + z * (1.f - s));
}

// operand bytes of one K chunk: A 128 x 64 and B NT x 64 (BF16)
template <int NT> __host__ __device__ constexpr int stage_bytes() { return (kTileM + NT) * kKChunk * 2; }

// one 16-byte unit global -> shared, asynchronously; zero-filled when !valid
__device__ __forceinline__ void cp16(void *dst, const void *src, bool valid)
{
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(valid ? 16 : 0));
}

// K chunk [k0, k0 + kc) of A (128 rows from m0) and B (NT rows from n0) into one stage, in
// the no-swizzle K-major core-matrix layout: 16-byte unit (row r, k group kg) at
// ((r / 8) kgc + kg) 128 + (r % 8) 16
template <int NT>
__device__ __forceinline__ void stage_chunk(const GemmArgs &g, unsigned char *st, int m0, int n0, int k0, int kc, int tid)
{
  const int kgc = kc / 8;
  unsigned char *sA = st, *sB = st + kTileM * kKChunk * 2;
  for (int u = tid; u < kTileM * kgc; u += kGemmThreads)
    {
      const int r = u / kgc, kg = u % kgc;
      const bool ok = m0 + r < g.M;
      const __nv_bfloat16 *src = g.A + (ok ? static_cast<int64_t>(m0 + r) * g.lda + k0 + kg * 8 : 0);
      cp16(sA + ((r >> 3) * kgc + kg) * 128 + (r & 7) * 16, src, ok);
    }
  for (int u = tid; u < NT * kgc; u += kGemmThreads)
    {
      const int r = u / kgc, kg = u % kgc;
      const bool ok = n0 + r < g.N;
      const __nv_bfloat16 *src = g.B + (ok ? static_cast<int64_t>(n0 + r) * g.ldb + k0 + kg * 8 : 0);
      cp16(sB + ((r >> 3) * kgc + kg) * 128 + (r & 7) * 16, src, ok);
    }
  asm volatile("cp.async.commit_group;");
}

// Two operand stages: the copies of chunk i + 1 run while the tensor core works on chunk i;
// a stage is refilled only after the MMAs that read it have committed (one mbarrier per
// stage).
template <int NT, int EPI>
__global__ void __launch_bounds__(kGemmThreads) k_gemm_tc(GemmArgs g)
{
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ uint32_t tmem_base;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * kTileM, n0 = blockIdx.y * NT;
  const int split = blockIdx.z;
  const int kb = split * g.k_per_split;
  const int ke = min(g.K, kb + g.k_per_split);
  const int nchunks = ke > kb ? (ke - kb + kKChunk - 1) / kKChunk : 0;
  constexpr uint32_t kCols = NT < 32 ? 32 : NT;
  if (warp == 0)
    {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                   "r"(kCols));
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
  if (tid == 0)
    {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&mbar[0])), "r"(1));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&mbar[1])), "r"(1));
      asm volatile("fence.mbarrier_init.release.cluster;");
    }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_base;
  bool ok = true;
  int committed = 0; // chunks whose MMAs were committed
  if (nchunks > 0) stage_chunk<NT>(g, smem, m0, n0, kb, min(kKChunk, ke - kb), tid);
  for (int i = 0; i < nchunks && ok; ++i)
    {
      const int k0 = kb + i * kKChunk;
      const int kc = min(kKChunk, ke - k0); // multiple of 16
      const int kgc = kc / 8;
      unsigned char *st = smem + (i & 1) * stage_bytes<NT>();
      if (i + 1 < nchunks)
        {
          // the other stage was read by the MMAs of chunk i - 1: wait for their commit
          if (i >= 1 && !mbar_wait(smem_u32(&mbar[(i - 1) & 1]), static_cast<uint32_t>(((i - 1) >> 1) & 1)))
            {
              ok = false;
              break;
            }
          const int k1 = k0 + kKChunk;
          stage_chunk<NT>(g, smem + ((i + 1) & 1) * stage_bytes<NT>(), m0, n0, k1, min(kKChunk, ke - k1), tid);
          asm volatile("cp.async.wait_group 1;"); // chunk i has landed; chunk i + 1 may be in flight
        }
      else
        asm volatile("cp.async.wait_group 0;");
      asm volatile("fence.proxy.async.shared::cta;");
      asm volatile("tcgen05.fence::before_thread_sync;");
      __syncthreads();
      asm volatile("tcgen05.fence::after_thread_sync;");
      if (tid == 0)
        {
          constexpr uint32_t idesc = idesc_bf16(NT);
          const uint32_t sa = smem_u32(st), sb = smem_u32(st + kTileM * kKChunk * 2);
          for (int ks = 0; ks < kc / 16; ++ks)
            {
              const uint64_t ad = smem_desc(sa + ks * 256, 128, kgc * 128);
              const uint64_t bd = smem_desc(sb + ks * 256, 128, kgc * 128);
              const uint32_t acc = (i > 0 || ks > 0) ? 1u : 0u;
              asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                           "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                           "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
            }
          asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(&mbar[i & 1])));
        }
      committed = i + 1;
    }
  asm volatile("cp.async.wait_group 0;");
  // every MMA is tracked by the last commit: wait for it before reading the accumulator
  if (committed > 0)
    {
      const int j = committed - 1;
      if (!mbar_wait(smem_u32(&mbar[j & 1]), static_cast<uint32_t>((j >> 1) & 1)))
        {
          ok = false;
          mbar_wait(smem_u32(&mbar[j & 1]), static_cast<uint32_t>((j >> 1) & 1)); // bounded second wait
        }
    }
  if (!ok && lane == 0) atomicExch(g.err, 1);
  asm volatile("tcgen05.fence::after_thread_sync;");
  // epilogue: warps w and w + 4 own accumulator rows 32 (w % 4) .. + 31 (the TMEM lane
  // quarter a warp may read) and one half of the columns each, 16 columns per load; a
  // thread's 16 consecutive outputs of its row are written as 16-byte vectors
  const int quarter = warp & 3, half = warp >> 2;
  const int row = quarter * 32 + lane;
  const int m = m0 + row;
  constexpr int kHalfCols = NT / 2 < 16 ? 16 : NT / 2;
  if (ok && committed > 0)
    for (int c0 = half * kHalfCols; c0 < NT && c0 < (half + 1) * kHalfCols; c0 += 16)
      {
        uint32_t r[16];
        const uint32_t taddr = tmem + (static_cast<uint32_t>(quarter * 32) << 16) + c0;
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                     "[%16];"
                     : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                       "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                       "=r"(r[14]), "=r"(r[15])
                     : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;");
        if (m >= g.M) continue;
        const int nb = n0 + c0;
        const bool full = nb + 16 <= g.N;
        if (EPI == EPI_HIDDEN && full)
          {
            float z[16];
            __nv_bfloat16 h[16];
#pragma unroll
            for (int j = 0; j < 16; ++j)
              {
                z[j] = __uint_as_float(r[j]) + g.bias[nb + j];
                h[j] = __float2bfloat16(silu(z[j]));
              }
            if (g.out_f32) // pre-activations only when a backward pass follows
              {
                float4 *zo = reinterpret_cast<float4 *>(g.out_f32 + static_cast<int64_t>(m) * g.ldo + nb);
#pragma unroll
                for (int q = 0; q < 4; ++q) zo[q] = make_float4(z[4 * q], z[4 * q + 1], z[4 * q + 2], z[4 * q + 3]);
              }
            uint4 *ho = reinterpret_cast<uint4 *>(g.out_h + static_cast<int64_t>(m) * g.ldh + nb);
            ho[0] = *reinterpret_cast<const uint4 *>(&h[0]);
            ho[1] = *reinterpret_cast<const uint4 *>(&h[8]);
            if (g.out_t)
#pragma unroll
              for (int j = 0; j < 16; ++j) g.out_t[static_cast<int64_t>(nb + j) * g.ldt + m] = h[j];
            continue;
          }
        if (EPI == EPI_DELTA && full)
          {
            __nv_bfloat16 d[16];
            const float4 *zi = reinterpret_cast<const float4 *>(g.z_in + static_cast<int64_t>(m) * g.ldz + nb);
#pragma unroll
            for (int q = 0; q < 4; ++q)
              {
                const float4 zz = zi[q];
                d[4 * q] = __float2bfloat16(__uint_as_float(r[4 * q]) * dsilu(zz.x));
                d[4 * q + 1] = __float2bfloat16(__uint_as_float(r[4 * q + 1]) * dsilu(zz.y));
                d[4 * q + 2] = __float2bfloat16(__uint_as_float(r[4 * q + 2]) * dsilu(zz.z));
                d[4 * q + 3] = __float2bfloat16(__uint_as_float(r[4 * q + 3]) * dsilu(zz.w));
              }
            uint4 *ho = reinterpret_cast<uint4 *>(g.out_h + static_cast<int64_t>(m) * g.ldh + nb);
            ho[0] = *reinterpret_cast<const uint4 *>(&d[0]);
            ho[1] = *reinterpret_cast<const uint4 *>(&d[8]);
            if (g.out_t)
#pragma unroll
              for (int j = 0; j < 16; ++j) g.out_t[static_cast<int64_t>(nb + j) * g.ldt + m] = d[j];
            continue;
          }
#pragma unroll
        for (int j = 0; j < 16; ++j)
          {
            const int n = nb + j;
            if (n >= g.N) continue;
            const float acc = __uint_as_float(r[j]);
            if (EPI == EPI_HIDDEN)
              {
                const float z = acc + g.bias[n];
                if (g.out_f32) g.out_f32[static_cast<int64_t>(m) * g.ldo + n] = z;
                const __nv_bfloat16 h = __float2bfloat16(silu(z));
                g.out_h[static_cast<int64_t>(m) * g.ldh + n] = h;
                if (g.out_t) g.out_t[static_cast<int64_t>(n) * g.ldt + m] = h;
              }
            else if (EPI == EPI_OUTPUT)
              g.out_f32[static_cast<int64_t>(m) * g.ldo + n] = acc + g.bias[n];
            else if (EPI == EPI_DELTA)
              {
                const __nv_bfloat16 dl = __float2bfloat16(acc * dsilu(g.z_in[static_cast<int64_t>(m) * g.ldz + n]));
                g.out_h[static_cast<int64_t>(m) * g.ldh + n] = dl;
                if (g.out_t) g.out_t[static_cast<int64_t>(n) * g.ldt + m] = dl;
              }
            else
              g.out_f32[(static_cast<int64_t>(split) * g.M + m) * g.ldo + n] = acc;
          }
      }
  else if (EPI == EPI_PARTIAL && m < g.M && half == 0)
    for (int n = n0; n < min(g.N, n0 + NT); ++n) g.out_f32[(static_cast<int64_t>(split) * g.M + m) * g.ldo + n] = 0.f;
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols));
}

// ---------------------------------------------------------------------------------
// elementwise kernels
// ---------------------------------------------------------------------------------
// rows of inputs in FP32 -> BF16 [P][16] row-major and [16 -> padded to 128][P] transposed
__global__ void k_prep_inputs(const float *__restrict__ in, int P, int ldp, __nv_bfloat16 *__restrict__ X,
                              __nv_bfloat16 *__restrict__ XT, const float *__restrict__ shift,
                              const float *__restrict__ scale)
{
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= static_cast<int64_t>(ldp) * kInPad) return;
  const int p = static_cast<int>(i / kInPad), c = static_cast<int>(i % kInPad);
  float v = 0.f;
  if (p < P && c < kIn) v = (in[static_cast<int64_t>(p) * kIn + c] - shift[c]) * scale[c];
  const __nv_bfloat16 b = __float2bfloat16(v);
  X[static_cast<int64_t>(p) * kInPad + c] = b;
  if (XT) XT[static_cast<int64_t>(c) * ldp + p] = b;
}

// delta_out = (y - target) * w / P on the 18 outputs (0 on padding); loss partials per row
__global__ void k_loss_grad(const float *__restrict__ Y, const float *__restrict__ T, int P, int ldp,
                            __nv_bfloat16 *__restrict__ D, __nv_bfloat16 *__restrict__ DT, float *__restrict__ row_loss)
{
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= ldp) return;
  float l = 0.f;
  for (int c = 0; c < kOutPad; ++c)
    {
      float d = 0.f;
      if (p < P && c < kOut)
        {
          const float e = Y[static_cast<int64_t>(p) * kOutPad + c] - T[static_cast<int64_t>(p) * kOut + c];
          l += e * e;
          d = e / static_cast<float>(P);
        }
      const __nv_bfloat16 b = __float2bfloat16(d);
      D[static_cast<int64_t>(p) * kOutPad + c] = b;
      DT[static_cast<int64_t>(c) * ldp + p] = b;
    }
  row_loss[p] = 0.5f * l / static_cast<float>(P > 0 ? P : 1);
}

// grad[n][k] (= dW_l) from split partials of dW_l^T [split][fan_in_pad][ld]
__global__ void k_reduce_grad(const float *__restrict__ part, int splits, int Mpad, int ld, int fan_in, int fan_out,
                              float *__restrict__ grad)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= fan_in * fan_out) return;
  const int n = i / fan_in, k = i % fan_in;
  float s = 0.f;
  for (int sp = 0; sp < splits; ++sp) s += part[(static_cast<int64_t>(sp) * Mpad + k) * ld + n];
  grad[i] = s;
}

// bias gradient: sum over points of the layer's delta (bf16 [P][ld])
__global__ void k_bias_grad(const __nv_bfloat16 *__restrict__ D, int P, int ld, int n_out, float *__restrict__ gb)
{
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= n_out) return;
  float s = 0.f;
  for (int p = 0; p < P; ++p) s += __bfloat162float(D[static_cast<int64_t>(p) * ld + n]);
  gb[n] = s;
}

// Adam on FP32 master weights; refreshes the BF16 copies W [fan_out_pad][fan_in_pad] and
// W^T [fan_in_pad][fan_out_pad] used by the GEMMs
__global__ void k_adam(float *__restrict__ w, float *__restrict__ mom, float *__restrict__ vel,
                       const float *__restrict__ g, int n, float lr, float b1, float b2, float eps, float c1, float c2)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * mom[i] + (1.f - b1) * gi;
  const float vi = b2 * vel[i] + (1.f - b2) * gi * gi;
  mom[i] = mi;
  vel[i] = vi;
  w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

__global__ void k_pack_weights(const float *__restrict__ w, int fan_out, int fan_in, int out_pad, int in_pad,
                               __nv_bfloat16 *__restrict__ W, __nv_bfloat16 *__restrict__ WT)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= out_pad * in_pad) return;
  const int o = i / in_pad, k = i % in_pad;
  const float v = (o < fan_out && k < fan_in) ? w[o * fan_in + k] : 0.f;
  const __nv_bfloat16 b = __float2bfloat16(v);
  W[i] = b;
  WT[static_cast<int64_t>(k) * out_pad + o] = b;
}

// ---------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------
struct LayerShape
{
  int fan_in, fan_out, in_pad, out_pad;
};
constexpr LayerShape kShape[kLayers] = {
  {kIn, kHid, kInPad, kHid}, {kHid, kHid, kHid, kHid}, {kHid, kHid, kHid, kHid}, {kHid, kHid, kHid, kHid},
  {kHid, kOut, kHid, kOutPad}};

} // namespace mlp
} // namespace glgpu

using namespace glgpu;
using namespace glgpu::mlp;

struct glgpu_surrogate
{
  cudaStream_t st = nullptr;
  std::vector<void *> allocs;
  // parameters (FP32 master), Adam moments, gradients
  float *w[kLayers] = {}, *b[kLayers] = {}, *mw[kLayers] = {}, *vw[kLayers] = {}, *mb[kLayers] = {},
        *vb[kLayers] = {}, *gw[kLayers] = {}, *gb[kLayers] = {};
  __nv_bfloat16 *W[kLayers] = {}, *WT[kLayers] = {};
  float *shift = nullptr, *scale = nullptr;
  int adam_t = 0;
  // activations for a batch capacity
  int cap = 0;
  __nv_bfloat16 *X = nullptr, *XT = nullptr, *H[4] = {}, *HT[4] = {}, *Dl[5] = {}, *DT[5] = {};
  float *Z[4] = {}, *Y = nullptr, *Tg = nullptr, *In = nullptr, *rowloss = nullptr, *part = nullptr;
  int *err = nullptr;
  int64_t launches = 0;
};

namespace
{
template <typename T> glgpu_status salloc(glgpu_surrogate *s, T **p, size_t n)
{
  *p = nullptr;
  const cudaError_t e = cudaMalloc(reinterpret_cast<void **>(p), (n ? n : 1) * sizeof(T));
  if (e != cudaSuccess) return set_error(GLGPU_ERR_NOMEM, std::string("surrogate: cudaMalloc: ") + cudaGetErrorString(e));
  s->allocs.push_back(*p);
  return GLGPU_OK;
}

#define SCK(call)                                                                                                    \
  do                                                                                                                 \
    {                                                                                                                \
      cudaError_t e_ = (call);                                                                                       \
      if (e_ != cudaSuccess) return set_error(GLGPU_ERR_CUDA, std::string("surrogate: ") + cudaGetErrorString(e_));  \
    }                                                                                                                \
  while (0)
#define SCKS(call)                                                                                                   \
  do                                                                                                                 \
    {                                                                                                                \
      glgpu_status s_ = (call);                                                                                      \
      if (s_ != GLGPU_OK) return s_;                                                                                 \
    }                                                                                                                \
  while (0)

constexpr size_t kGemmSmem = 100 * 1024; // two operand stages (96 KB at NT = 256); at most two CTAs share an SM (TMEM <= 512 columns)

template <int NT, int EPI> glgpu_status gemm(glgpu_surrogate *s, GemmArgs g, int splits)
{
  static bool attr = false;
  if (!attr)
    {
      SCK(cudaFuncSetAttribute(k_gemm_tc<NT, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kGemmSmem)));
      attr = true;
    }
  g.err = s->err;
  dim3 grid((g.M + kTileM - 1) / kTileM, (g.N + NT - 1) / NT, splits);
  k_gemm_tc<NT, EPI><<<grid, kGemmThreads, kGemmSmem, s->st>>>(g);
  s->launches++;
  SCK(cudaGetLastError());
  return GLGPU_OK;
}

int round_up(int v, int a) { return (v + a - 1) / a * a; }

glgpu_status ensure_capacity(glgpu_surrogate *s, int P)
{
  const int ldp = round_up(P, kTileM);
  if (ldp <= s->cap) return GLGPU_OK;
  // grow: free the old activation buffers (they are tracked in allocs; release them there too)
  auto release = [&](void *p) {
    if (!p) return;
    for (auto &a : s->allocs)
      if (a == p)
        {
          cudaFree(a);
          a = nullptr;
        }
  };
  release(s->X);
  release(s->XT);
  for (int l = 0; l < 4; ++l)
    {
      release(s->H[l]);
      release(s->HT[l]);
      release(s->Z[l]);
    }
  for (int l = 0; l < 5; ++l)
    {
      release(s->Dl[l]);
      release(s->DT[l]);
    }
  release(s->Y);
  release(s->Tg);
  release(s->In);
  release(s->rowloss);
  release(s->part);
  SCKS(salloc(s, &s->X, static_cast<size_t>(ldp) * kInPad));
  SCKS(salloc(s, &s->XT, static_cast<size_t>(kTileM) * ldp)); // 16 rows used, padded to one M tile
  SCK(cudaMemset(s->XT, 0, sizeof(__nv_bfloat16) * static_cast<size_t>(kTileM) * ldp));
  for (int l = 0; l < 4; ++l)
    {
      SCKS(salloc(s, &s->H[l], static_cast<size_t>(ldp) * kHid));
      SCKS(salloc(s, &s->HT[l], static_cast<size_t>(kHid) * ldp));
      SCKS(salloc(s, &s->Z[l], static_cast<size_t>(ldp) * kHid));
    }
  for (int l = 0; l < 5; ++l)
    {
      const int w = (l == 4) ? kOutPad : kHid;
      SCKS(salloc(s, &s->Dl[l], static_cast<size_t>(ldp) * w));
      SCKS(salloc(s, &s->DT[l], static_cast<size_t>(w) * ldp));
    }
  SCKS(salloc(s, &s->Y, static_cast<size_t>(ldp) * kOutPad));
  SCKS(salloc(s, &s->Tg, static_cast<size_t>(ldp) * kOut));
  SCKS(salloc(s, &s->In, static_cast<size_t>(ldp) * kIn));
  SCKS(salloc(s, &s->rowloss, static_cast<size_t>(ldp)));
  SCKS(salloc(s, &s->part, static_cast<size_t>(kSplitMax) * kHid * kHid));
  s->cap = ldp;
  return GLGPU_OK;
}

glgpu_status pack_all(glgpu_surrogate *s)
{
  for (int l = 0; l < kLayers; ++l)
    {
      const LayerShape &L = kShape[l];
      const int n = L.out_pad * L.in_pad;
      k_pack_weights<<<(n + 255) / 256, 256, 0, s->st>>>(s->w[l], L.fan_out, L.fan_in, L.out_pad, L.in_pad, s->W[l],
                                                         s->WT[l]);
      s->launches++;
    }
  SCK(cudaGetLastError());
  return GLGPU_OK;
}

// forward over P rows already in s->In; outputs Y [P][32] f32
glgpu_status forward(glgpu_surrogate *s, int P, bool want_transposes)
{
  const int ldp = round_up(P, kTileM);
  const int n = ldp * kInPad;
  k_prep_inputs<<<(n + 255) / 256, 256, 0, s->st>>>(s->In, P, ldp, s->X, want_transposes ? s->XT : nullptr, s->shift,
                                                     s->scale);
  s->launches++;
  const __nv_bfloat16 *in = s->X;
  int ld_in = kInPad;
  for (int l = 0; l < 4; ++l)
    {
      GemmArgs g{};
      g.A = in;
      g.lda = ld_in;
      g.B = s->W[l];
      g.ldb = kShape[l].in_pad;
      g.M = ldp;
      g.N = kHid;
      g.K = kShape[l].in_pad;
      g.k_per_split = g.K;
      g.bias = s->b[l];
      g.out_f32 = want_transposes ? s->Z[l] : nullptr; // the backward pass reads them
      g.ldo = kHid;
      g.out_h = s->H[l];
      g.ldh = kHid;
      g.out_t = want_transposes ? s->HT[l] : nullptr;
      g.ldt = ldp;
      SCKS((gemm<256, EPI_HIDDEN>(s, g, 1)));
      in = s->H[l];
      ld_in = kHid;
    }
  GemmArgs g{};
  g.A = s->H[3];
  g.lda = kHid;
  g.B = s->W[4];
  g.ldb = kHid;
  g.M = ldp;
  g.N = kOutPad;
  g.K = kHid;
  g.k_per_split = g.K;
  g.bias = s->b[4];
  g.out_f32 = s->Y;
  g.ldo = kOutPad;
  return gemm<32, EPI_OUTPUT>(s, g, 1);
}

// backward after forward(..., true) and k_loss_grad: fills gw[l], gb[l]
glgpu_status backward(glgpu_surrogate *s, int P)
{
  const int ldp = round_up(P, kTileM);
  // delta_l for l = 4 .. 1 (index of the layer whose pre-activation it multiplies)
  for (int l = 4; l >= 1; --l)
    {
      GemmArgs g{};
      g.A = s->Dl[l];                      // delta of layer l: [P][out_pad(l)]
      g.lda = kShape[l].out_pad;
      g.B = s->WT[l];                      // W_l^T: [in_pad(l)][out_pad(l)]
      g.ldb = kShape[l].out_pad;
      g.M = ldp;
      g.N = kHid;
      g.K = kShape[l].out_pad;
      g.k_per_split = g.K;
      g.z_in = s->Z[l - 1];
      g.ldz = kHid;
      g.out_h = s->Dl[l - 1];
      g.ldh = kHid;
      g.out_t = s->DT[l - 1];
      g.ldt = ldp;
      SCKS((gemm<256, EPI_DELTA>(s, g, 1)));
    }
  // weight gradients dW_l^T = H_{l-1}^T delta_l, split over the points
  const int splits = std::min(kSplitMax, std::max(1, ldp / 512));
  const int kps = round_up((ldp + splits - 1) / splits, 16);
  for (int l = 0; l < kLayers; ++l)
    {
      const LayerShape &L = kShape[l];
      GemmArgs g{};
      g.A = (l == 0) ? s->XT : s->HT[l - 1];
      g.lda = ldp;
      g.B = s->DT[l];
      g.ldb = ldp;
      g.M = (l == 0) ? kTileM : kHid; // fan-in rows (16 inputs padded to one tile)
      g.N = L.out_pad;
      g.K = ldp;
      g.k_per_split = kps;
      g.out_f32 = s->part;
      g.ldo = L.out_pad;
      const int nsp = (ldp + kps - 1) / kps;
      if (L.out_pad == kHid)
        SCKS((gemm<256, EPI_PARTIAL>(s, g, nsp)));
      else
        SCKS((gemm<32, EPI_PARTIAL>(s, g, nsp)));
      const int nw = L.fan_in * L.fan_out;
      k_reduce_grad<<<(nw + 255) / 256, 256, 0, s->st>>>(s->part, nsp, g.M, L.out_pad, L.fan_in, L.fan_out, s->gw[l]);
      k_bias_grad<<<(L.fan_out + 127) / 128, 128, 0, s->st>>>(s->Dl[l], P, L.out_pad, L.fan_out, s->gb[l]);
      s->launches += 2;
    }
  SCK(cudaGetLastError());
  return GLGPU_OK;
}

glgpu_status check_err(glgpu_surrogate *s)
{
  int h = 0;
  SCK(cudaMemcpyAsync(&h, s->err, sizeof(int), cudaMemcpyDeviceToHost, s->st));
  SCK(cudaStreamSynchronize(s->st));
  if (h) return set_error(GLGPU_ERR_TIMEOUT, "surrogate: a tensor-core wait timed out");
  return GLGPU_OK;
}

// splitmix-based uniform for reproducible initialisation
double unif(uint64_t seed, uint64_t i)
{
  uint64_t z = seed * 0x9E3779B97F4A7C15ull + i + 1;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (static_cast<double>(z >> 11) + 0.5) / 9007199254740992.0;
}
} // namespace

extern "C" glgpu_status glgpu_surrogate_create(uint64_t seed, glgpu_surrogate **out)
{
  if (!out) return set_error(GLGPU_ERR_ARG, "glgpu_surrogate_create: out is NULL");
  *out = nullptr;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return set_error(GLGPU_ERR_CUDA, "glgpu_surrogate_create: no device");
  glgpu_surrogate *s = new glgpu_surrogate();
  auto fail = [&](glgpu_status st) {
    std::string msg = glgpu_last_error();
    glgpu_surrogate_destroy(s);
    set_error(st, msg);
    return st;
  };
  if (cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking) != cudaSuccess)
    return fail(set_error(GLGPU_ERR_CUDA, "glgpu_surrogate_create: stream"));
  glgpu_status st;
  for (int l = 0; l < kLayers; ++l)
    {
      const LayerShape &L = kShape[l];
      const size_t nw = static_cast<size_t>(L.fan_in) * L.fan_out;
      if ((st = salloc(s, &s->w[l], nw)) || (st = salloc(s, &s->mw[l], nw)) || (st = salloc(s, &s->vw[l], nw)) ||
          (st = salloc(s, &s->gw[l], nw)) || (st = salloc(s, &s->b[l], L.out_pad)) ||
          (st = salloc(s, &s->mb[l], L.out_pad)) || (st = salloc(s, &s->vb[l], L.out_pad)) ||
          (st = salloc(s, &s->gb[l], L.out_pad)) ||
          (st = salloc(s, &s->W[l], static_cast<size_t>(L.out_pad) * L.in_pad)) ||
          (st = salloc(s, &s->WT[l], static_cast<size_t>(L.out_pad) * L.in_pad)))
        return fail(st);
      // Glorot-uniform weights, zero biases
      std::vector<float> hw(nw);
      const double a = std::sqrt(6.0 / (L.fan_in + L.fan_out));
      for (size_t i = 0; i < nw; ++i) hw[i] = static_cast<float>((2.0 * unif(seed, l * 1000003ull + i) - 1.0) * a);
      if (cudaMemcpy(s->w[l], hw.data(), nw * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
          cudaMemset(s->mw[l], 0, nw * 4) != cudaSuccess || cudaMemset(s->vw[l], 0, nw * 4) != cudaSuccess ||
          cudaMemset(s->b[l], 0, L.out_pad * 4) != cudaSuccess || cudaMemset(s->mb[l], 0, L.out_pad * 4) != cudaSuccess ||
          cudaMemset(s->vb[l], 0, L.out_pad * 4) != cudaSuccess)
        return fail(set_error(GLGPU_ERR_CUDA, "glgpu_surrogate_create: initialisation"));
    }
  if ((st = salloc(s, &s->shift, kIn)) || (st = salloc(s, &s->scale, kIn)) || (st = salloc(s, &s->err, 1)))
    return fail(st);
  const float sh[kIn] = {0, 0, 0, 0, 0, 0}, sc[kIn] = {1, 1, 1, 1, 1, 1};
  cudaMemcpy(s->shift, sh, sizeof sh, cudaMemcpyHostToDevice);
  cudaMemcpy(s->scale, sc, sizeof sc, cudaMemcpyHostToDevice);
  cudaMemset(s->err, 0, sizeof(int));
  if ((st = pack_all(s)) != GLGPU_OK) return fail(st);
  if (cudaStreamSynchronize(s->st) != cudaSuccess) return fail(set_error(GLGPU_ERR_CUDA, "glgpu_surrogate_create: sync"));
  *out = s;
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_surrogate_destroy(glgpu_surrogate *s)
{
  if (!s) return GLGPU_OK;
  if (s->st) cudaStreamSynchronize(s->st);
  for (void *p : s->allocs)
    if (p) cudaFree(p);
  if (s->st) cudaStreamDestroy(s->st);
  delete s;
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_surrogate_set_normalization(glgpu_surrogate *s, const float *shift, const float *scale)
{
  if (!s || !shift || !scale) return set_error(GLGPU_ERR_ARG, "glgpu_surrogate_set_normalization: NULL argument");
  SCK(cudaMemcpy(s->shift, shift, sizeof(float) * kIn, cudaMemcpyHostToDevice));
  SCK(cudaMemcpy(s->scale, scale, sizeof(float) * kIn, cudaMemcpyHostToDevice));
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_surrogate_param_count(int64_t *n)
{
  if (!n) return set_error(GLGPU_ERR_ARG, "glgpu_surrogate_param_count: NULL");
  int64_t t = 0;
  for (int l = 0; l < kLayers; ++l) t += static_cast<int64_t>(kShape[l].fan_in) * kShape[l].fan_out + kShape[l].fan_out;
  *n = t;
  return GLGPU_OK;
}

// parameter order: for each layer, W [fan_out][fan_in] then b [fan_out]
extern "C" glgpu_status glgpu_surrogate_get_params(glgpu_surrogate *s, float *p)
{
  if (!s || !p) return set_error(GLGPU_ERR_ARG, "glgpu_surrogate_get_params: NULL");
  SCK(cudaStreamSynchronize(s->st));
  for (int l = 0; l < kLayers; ++l)
    {
      const size_t nw = static_cast<size_t>(kShape[l].fan_in) * kShape[l].fan_out;
      SCK(cudaMemcpy(p, s->w[l], nw * 4, cudaMemcpyDeviceToHost));
      p += nw;
      SCK(cudaMemcpy(p, s->b[l], kShape[l].fan_out * 4, cudaMemcpyDeviceToHost));
      p += kShape[l].fan_out;
    }
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_surrogate_set_params(glgpu_surrogate *s, const float *p)
{
  if (!s || !p) return set_error(GLGPU_ERR_ARG, "glgpu_surrogate_set_params: NULL");
  SCK(cudaStreamSynchronize(s->st));
  for (int l = 0; l < kLayers; ++l)
    {
      const size_t nw = static_cast<size_t>(kShape[l].fan_in) * kShape[l].fan_out;
      SCK(cudaMemcpy(s->w[l], p, nw * 4, cudaMemcpyHostToDevice));
      p += nw;
      SCK(cudaMemcpy(s->b[l], p, kShape[l].fan_out * 4, cudaMemcpyHostToDevice));
      p += kShape[l].fan_out;
    }
  SCKS(pack_all(s));
  SCK(cudaStreamSynchronize(s->st));
  return GLGPU_OK;
}

extern "C" glgpu_status glgpu_surrogate_predict(glgpu_surrogate *s, const float *inputs, int P, float *outputs)
{
  if (!s || !inputs || !outputs || P < 0) return set_error(GLGPU_ERR_ARG, "glgpu_surrogate_predict: bad argument");
  if (P == 0) return GLGPU_OK;
  SCKS(ensure_capacity(s, P));
  SCK(cudaMemcpyAsync(s->In, inputs, sizeof(float) * P * kIn, cudaMemcpyHostToDevice, s->st));
  SCKS(forward(s, P, false));
  SCK(cudaMemcpy2DAsync(outputs, sizeof(float) * kOut, s->Y, sizeof(float) * kOutPad, sizeof(float) * kOut, P,
                        cudaMemcpyDeviceToHost, s->st));
  return check_err(s);
}

// one forward + backward without an update: loss and gradients in parameter order
extern "C" glgpu_status glgpu_surrogate_gradient(glgpu_surrogate *s, const float *inputs, const float *targets, int P,
                                                 float *loss, float *grad)
{
  if (!s || !inputs || !targets || P <= 0) return set_error(GLGPU_ERR_ARG, "glgpu_surrogate_gradient: bad argument");
  SCKS(ensure_capacity(s, P));
  const int ldp = round_up(P, kTileM);
  SCK(cudaMemcpyAsync(s->In, inputs, sizeof(float) * P * kIn, cudaMemcpyHostToDevice, s->st));
  SCK(cudaMemcpyAsync(s->Tg, targets, sizeof(float) * P * kOut, cudaMemcpyHostToDevice, s->st));
  SCKS(forward(s, P, true));
  k_loss_grad<<<(ldp + 127) / 128, 128, 0, s->st>>>(s->Y, s->Tg, P, ldp, s->Dl[4], s->DT[4], s->rowloss);
  s->launches++;
  SCKS(backward(s, P));
  SCKS(check_err(s));
  if (loss)
    {
      std::vector<float> rl(ldp);
      SCK(cudaMemcpy(rl.data(), s->rowloss, sizeof(float) * ldp, cudaMemcpyDeviceToHost));
      double t = 0;
      for (float v : rl) t += v;
      *loss = static_cast<float>(t);
    }
  if (grad)
    for (int l = 0; l < kLayers; ++l)
      {
        const size_t nw = static_cast<size_t>(kShape[l].fan_in) * kShape[l].fan_out;
        SCK(cudaMemcpy(grad, s->gw[l], nw * 4, cudaMemcpyDeviceToHost));
        grad += nw;
        SCK(cudaMemcpy(grad, s->gb[l], kShape[l].fan_out * 4, cudaMemcpyDeviceToHost));
        grad += kShape[l].fan_out;
      }
  return GLGPU_OK;
}

// Adam training on (inputs, targets): `steps` minibatches of `batch` rows drawn in a
// fixed shuffled order (seeded).  loss_out (may be NULL) receives the loss of the last
// `report` steps averaged.
extern "C" glgpu_status glgpu_surrogate_train(glgpu_surrogate *s, const float *inputs, const float *targets, int n_rows,
                                              int steps, int batch, float lr, uint64_t seed, float *loss_out)
{
  if (!s || !inputs || !targets || n_rows <= 0 || steps < 0 || batch <= 0)
    return set_error(GLGPU_ERR_ARG, "glgpu_surrogate_train: bad argument");
  batch = std::min(batch, n_rows);
  SCKS(ensure_capacity(s, batch));
  const int ldp = round_up(batch, kTileM);
  // minibatches are gathered on the host from a seeded shuffle and copied per step
  std::vector<int> order(n_rows);
  for (int i = 0; i < n_rows; ++i) order[i] = i;
  int pos = n_rows;
  double loss_acc = 0;
  int loss_n = 0;
  std::vector<float> rl(ldp);
  glgpu_status result = GLGPU_OK;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  std::vector<float> hin(static_cast<size_t>(batch) * kIn), htg(static_cast<size_t>(batch) * kOut);
  for (int step = 0; step < steps && result == GLGPU_OK; ++step)
    {
      if (pos + batch > n_rows)
        {
          for (int i = n_rows - 1; i > 0; --i)
            {
              const int j = static_cast<int>(unif(seed, static_cast<uint64_t>(step) * 7919u + i) * (i + 1));
              std::swap(order[i], order[j < i + 1 ? j : i]);
            }
          pos = 0;
        }
      for (int r = 0; r < batch; ++r)
        {
          std::memcpy(&hin[static_cast<size_t>(r) * kIn], inputs + static_cast<size_t>(order[pos + r]) * kIn, sizeof(float) * kIn);
          std::memcpy(&htg[static_cast<size_t>(r) * kOut], targets + static_cast<size_t>(order[pos + r]) * kOut,
                      sizeof(float) * kOut);
        }
      pos += batch;
      if (cudaMemcpyAsync(s->In, hin.data(), sizeof(float) * hin.size(), cudaMemcpyHostToDevice, s->st) != cudaSuccess ||
          cudaMemcpyAsync(s->Tg, htg.data(), sizeof(float) * htg.size(), cudaMemcpyHostToDevice, s->st) != cudaSuccess)
        {
          result = set_error(GLGPU_ERR_CUDA, "glgpu_surrogate_train: copy");
          break;
        }
      if ((result = forward(s, batch, true)) != GLGPU_OK) break;
      k_loss_grad<<<(ldp + 127) / 128, 128, 0, s->st>>>(s->Y, s->Tg, batch, ldp, s->Dl[4], s->DT[4], s->rowloss);
      s->launches++;
      if ((result = backward(s, batch)) != GLGPU_OK) break;
      ++s->adam_t;
      const float c1 = 1.f - std::pow(b1, static_cast<float>(s->adam_t));
      const float c2 = 1.f - std::pow(b2, static_cast<float>(s->adam_t));
      for (int l = 0; l < kLayers; ++l)
        {
          const int nw = kShape[l].fan_in * kShape[l].fan_out, nb = kShape[l].fan_out;
          k_adam<<<(nw + 255) / 256, 256, 0, s->st>>>(s->w[l], s->mw[l], s->vw[l], s->gw[l], nw, lr, b1, b2, eps, c1, c2);
          k_adam<<<(nb + 255) / 256, 256, 0, s->st>>>(s->b[l], s->mb[l], s->vb[l], s->gb[l], nb, lr, b1, b2, eps, c1, c2);
          s->launches += 2;
        }
      if ((result = pack_all(s)) != GLGPU_OK) break;
      if (step >= steps - 20)
        {
          if (cudaMemcpyAsync(rl.data(), s->rowloss, sizeof(float) * ldp, cudaMemcpyDeviceToHost, s->st) != cudaSuccess ||
              cudaStreamSynchronize(s->st) != cudaSuccess)
            {
              result = set_error(GLGPU_ERR_CUDA, "glgpu_surrogate_train: loss copy");
              break;
            }
          double t = 0;
          for (float v : rl) t += v;
          loss_acc += t;
          ++loss_n;
        }
    }
  cudaStreamSynchronize(s->st);
  if (result != GLGPU_OK) return result;
  SCKS(check_err(s));
  if (loss_out) *loss_out = loss_n ? static_cast<float>(loss_acc / loss_n) : 0.f;
  return GLGPU_OK;
}

extern "C" int64_t glgpu_surrogate_launch_count(const glgpu_surrogate *s) { return s ? s->launches : 0; }
