// Multigrid kernels (sm_103a): inter-level transfers and the coarsest-level dense solve.
//
// Transfers are node-level CSR gathers applied to all B components of a node:
//   prolongation   z_fine[n][c]  += sum_j w_j z_coarse[idx_j][c]   (trilinear, P)
//   restriction    r_coarse[i][c] = sum_j w_j r_fine[idx_j][c]     (P^T, transposed CSR)
// Constrained components (zero-Dirichlet, hanging) are left alone on the way up and
// zeroed on the way down, so every Krylov vector keeps zeros there.
// Coarse Jacobians are Galerkin products P^T J P, one warp per coarse block.  The
// coarsest level (1 cell per axis, 8 nodes, 144 unknowns per instance) is inverted
// densely once per Newton step: one CTA per instance, Gauss-Jordan in shared memory.
#include <cstdint>
#include <cuda_runtime.h>

#include <cuda_fp16.h>

#include "device.h"

namespace glgpu
{
// sum over row n's fixed slots of w * v[idx * B + c], in slot (list) order
template <typename T, int S>
__device__ __forceinline__ T slot_sum(const int32_t *__restrict__ sidx, const T *__restrict__ sw, int64_t n,
                                      const T *__restrict__ v, int B, int c)
{
  static_assert(S % 4 == 0, "slots in 16-byte groups");
  int id[S];
  const int4 *ip = reinterpret_cast<const int4 *>(sidx + n * S);
#pragma unroll
  for (int q = 0; q < S / 4; ++q)
    {
      const int4 t = __ldg(ip + q);
      id[4 * q] = t.x;
      id[4 * q + 1] = t.y;
      id[4 * q + 2] = t.z;
      id[4 * q + 3] = t.w;
    }
  T s = 0;
#pragma unroll
  for (int k = 0; k < S; ++k)
    if (id[k] >= 0) s += __ldg(sw + n * S + k) * v[static_cast<int64_t>(id[k]) * B + c];
  return s;
}

// zf = base + P zc (base == nullptr: zf += P zc); constrained components keep base
template <typename T>
__global__ void k_prolong_add(int64_t nn_f, int B, const int32_t *__restrict__ ptr, const int32_t *__restrict__ idx,
                              const T *__restrict__ w, const T *__restrict__ zc, T *__restrict__ zf,
                              const uint32_t *__restrict__ mask_f, const int32_t *__restrict__ hptr_f,
                              const int32_t *__restrict__ node_inst, const uint8_t *__restrict__ act,
                              const T *__restrict__ base, const int32_t *__restrict__ sidx, const T *__restrict__ sw)
{
  pdl_wait();
  pdl_trigger();
  const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= nn_f * B) return;
  const int64_t n = t / B;
  const int c = static_cast<int>(t % B);
  if (act && !act[node_inst[n]]) return;
  const T b0 = base ? base[t] : zf[t];
  if (hptr_f[n + 1] > hptr_f[n] || ((mask_f[n] >> c) & 1u))
    {
      if (base) zf[t] = b0;
      return;
    }
  T s = 0;
  if (sidx)
    s = slot_sum<T, kProlongSlots>(sidx, sw, n, zc, B, c);
  else
    for (int k = ptr[n]; k < ptr[n + 1]; ++k) s += w[k] * zc[static_cast<int64_t>(idx[k]) * B + c];
  zf[t] = b0 + s;
}

template <typename T>
__global__ void k_restrict(int64_t nn_c, int B, const int32_t *__restrict__ ptr, const int32_t *__restrict__ idx,
                           const T *__restrict__ w, const T *__restrict__ rf, T *__restrict__ rc,
                           const uint32_t *__restrict__ mask_c, const int32_t *__restrict__ node_inst,
                           const uint8_t *__restrict__ act, const int32_t *__restrict__ sidx, const T *__restrict__ sw)
{
  pdl_wait();
  pdl_trigger();
  const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= nn_c * B) return;
  const int64_t n = t / B;
  const int c = static_cast<int>(t % B);
  if (act && !act[node_inst[n]]) return;
  T s = 0;
  if (!((mask_c[n] >> c) & 1u))
    {
      if (sidx)
        s = slot_sum<T, kRestrictSlots>(sidx, sw, n, rf, B, c);
      else
        for (int k = ptr[n]; k < ptr[n + 1]; ++k) s += w[k] * rf[static_cast<int64_t>(idx[k]) * B + c];
    }
  rc[t] = s;
}

// Restriction fused with the first smoothing sweep of the coarse level, which starts from
// zero: rc = P^T rf (zero on zero-Dirichlet components) and z = omega D^-1 rc.  Thread
// (coarse node, component), 16 nodes per CTA; the node's 18 restricted values meet in
// shared memory for the 18 x 18 inverse block (18x18 blocks only).
constexpr int kRsNodes = 16;

template <typename T>
__global__ void __launch_bounds__(kRsNodes * 18)
  k_restrict_smooth(int64_t nn_c, const int32_t *__restrict__ ptr, const int32_t *__restrict__ idx,
                    const T *__restrict__ w, const T *__restrict__ rf, T *__restrict__ rc,
                    const uint32_t *__restrict__ mask_c, const int32_t *__restrict__ node_inst,
                    const uint8_t *__restrict__ act, const T *__restrict__ dinv, T omega, T *__restrict__ z,
                    const int32_t *__restrict__ sidx, const T *__restrict__ sw)
{
  pdl_wait();
  pdl_trigger();
  __shared__ T t_s[kRsNodes][18];
  const int ln = threadIdx.x / 18, c = threadIdx.x - 18 * (threadIdx.x / 18);
  const int64_t n = static_cast<int64_t>(blockIdx.x) * kRsNodes + ln;
  const bool on = n < nn_c && !(act && !act[node_inst[n]]);
  T s = 0;
  if (on && !((mask_c[n] >> c) & 1u))
    {
      if (sidx)
        s = slot_sum<T, kRestrictSlots>(sidx, sw, n, rf, 18, c);
      else
        for (int k = ptr[n]; k < ptr[n + 1]; ++k) s += w[k] * rf[static_cast<int64_t>(idx[k]) * 18 + c];
    }
  if (on) rc[n * 18 + c] = s;
  t_s[ln][c] = s;
  __syncthreads();
  if (!on) return;
  const T *row = dinv + n * 324 + c * 18;
  T u = 0;
#pragma unroll
  for (int d = 0; d < 18; ++d) u += row[d] * t_s[ln][d];
  z[n * 18 + c] = omega * u;
}

__device__ __forceinline__ float to_f(float v) { return v; }
__device__ __forceinline__ float to_f(double v) { return static_cast<float>(v); }
__device__ __forceinline__ float to_f(__half v) { return __half2float(v); }

// Galerkin product: one warp per coarse block (I, J).  The block is
//   J_c(I, J) = sum over fine blocks (i, j) with P(i, I) P(j, J) != 0 of P(i, I) P(j, J) J_f(i, j),
// a weighted sum of whole fine blocks whose (block index, weight) list is built on the
// host once per mesh.  Each fine block is streamed with 128-bit loads; lane l owns the
// same scalars of every block (the SpMV lane map), so the sum stays in registers.
constexpr int kGalWarps = 8;

template <typename T> struct GVec;
template <> struct GVec<float>
{
  using type = float4;
  static constexpr int n = 4;
};
template <> struct GVec<double>
{
  using type = double2;
  static constexpr int n = 2;
};
__device__ __forceinline__ void gfma(float4 &a, float w, const float4 &v)
{
  a.x = fmaf(w, v.x, a.x);
  a.y = fmaf(w, v.y, a.y);
  a.z = fmaf(w, v.z, a.z);
  a.w = fmaf(w, v.w, a.w);
}
__device__ __forceinline__ void gfma(double2 &a, double w, const double2 &v)
{
  a.x = fma(w, v.x, a.x);
  a.y = fma(w, v.y, a.y);
}
__device__ __forceinline__ float &gcomp(float4 &v, int k) { return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w; }
__device__ __forceinline__ double &gcomp(double2 &v, int k) { return k == 0 ? v.x : v.y; }

// chunk ch of a stored block (FP32 / FP64: 16-byte loads; FP16: 8-byte loads of four halves)
__device__ __forceinline__ float4 gload(const float *blk, int ch) { return __ldg(reinterpret_cast<const float4 *>(blk) + ch); }
__device__ __forceinline__ double2 gload(const double *blk, int ch)
{
  return __ldg(reinterpret_cast<const double2 *>(blk) + ch);
}
__device__ __forceinline__ float4 gload(const __half *blk, int ch)
{
  const uint2 u = __ldg(reinterpret_cast<const uint2 *>(blk) + ch);
  const float2 a = __half22float2(*reinterpret_cast<const __half2 *>(&u.x));
  const float2 b = __half22float2(*reinterpret_cast<const __half2 *>(&u.y));
  return make_float4(a.x, a.y, b.x, b.y);
}
__device__ __forceinline__ void gstore(float *blk, int ch, const float4 &v) { reinterpret_cast<float4 *>(blk)[ch] = v; }
__device__ __forceinline__ void gstore(double *blk, int ch, const double2 &v) { reinterpret_cast<double2 *>(blk)[ch] = v; }
__device__ __forceinline__ void gstore(__half *blk, int ch, const float4 &v)
{
  const __half2 a = __floats2half2_rn(v.x, v.y), b = __floats2half2_rn(v.z, v.w);
  uint2 u;
  u.x = *reinterpret_cast<const unsigned *>(&a);
  u.y = *reinterpret_cast<const unsigned *>(&b);
  reinterpret_cast<uint2 *>(blk)[ch] = u;
}

// T: accumulation type; IN / OUT: storage of the fine and coarse blocks (FP16 on the coarse
// levels of a mixed context, summed in FP32)
template <typename T, typename IN, typename OUT>
__global__ void __launch_bounds__(kGalWarps * 32)
  k_galerkin(int64_t n_up, const int32_t *__restrict__ up, const int32_t *__restrict__ g_row,
             const int32_t *__restrict__ cols_c, const uint32_t *__restrict__ mask_c, const int32_t *__restrict__ hptr_c,
             OUT *__restrict__ vals_c, const int64_t *__restrict__ g_toff, const int32_t *__restrict__ g_blk,
             const T *__restrict__ g_w, const IN *__restrict__ vals_f, const int32_t *__restrict__ node_inst_c,
             const uint8_t *__restrict__ act)
{
  pdl_wait();
  pdl_trigger();
  using V = typename GVec<T>::type;
  constexpr int NV = GVec<T>::n;
  constexpr int NCH = 324 / NV;
  constexpr int NIT = (NCH + 31) / 32;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t u = static_cast<int64_t>(blockIdx.x) * kGalWarps + warp;
  if (u >= n_up) return;
  const int64_t cb = up[u];
  const int32_t I = g_row[cb];
  if (act && !act[node_inst_c[I]]) return;
  V acc[NIT];
#pragma unroll
  for (int k = 0; k < NIT; ++k)
#pragma unroll
    for (int q = 0; q < NV; ++q) gcomp(acc[k], q) = T(0);
  const int64_t t1 = g_toff[cb + 1];
#pragma unroll 2
  for (int64_t t = g_toff[cb]; t < t1; ++t)
    {
      const IN *bp = vals_f + static_cast<int64_t>(__ldg(g_blk + t)) * 324;
      const T w = __ldg(g_w + t);
#pragma unroll
      for (int k = 0; k < NIT; ++k)
        {
          const int ch = lane + 32 * k;
          if (ch < NCH) gfma(acc[k], w, gload(bp, ch));
        }
    }
  // zero-Dirichlet components and constrained (periodic image) nodes of the coarse level:
  // identity rows, zero columns
  const int32_t J = cols_c[cb];
  constexpr uint32_t kAll = (1u << 18) - 1u;
  const uint32_t mI = (hptr_c[I + 1] > hptr_c[I]) ? kAll : mask_c[I];
  const uint32_t mJ = (hptr_c[J + 1] > hptr_c[J]) ? kAll : mask_c[J];
  OUT *dst = vals_c + cb * 324;
#pragma unroll
  for (int k = 0; k < NIT; ++k)
    {
      const int ch = lane + 32 * k;
      if (ch >= NCH) continue;
      V o = acc[k];
      if (mI | mJ)
#pragma unroll
        for (int q = 0; q < NV; ++q)
          {
            const int el = ch * NV + q, a = el / 18, bb = el - 18 * (el / 18);
            if (((mI >> a) & 1u) || ((mJ >> bb) & 1u)) gcomp(o, q) = (J == I && a == bb) ? T(1) : T(0);
          }
      gstore(dst, ch, o);
    }
}

// the blocks below the diagonal: block lo[2 i] = transpose of block lo[2 i + 1], warp per block
template <typename OUT>
__global__ void __launch_bounds__(kGalWarps * 32)
  k_galerkin_mirror(int64_t n_lo, const int32_t *__restrict__ lo, const int32_t *__restrict__ g_row,
                    OUT *__restrict__ vals_c, const int32_t *__restrict__ node_inst_c, const uint8_t *__restrict__ act)
{
  pdl_wait();
  pdl_trigger();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t i = static_cast<int64_t>(blockIdx.x) * kGalWarps + warp;
  if (i >= n_lo) return;
  const int64_t dst = lo[2 * i], src = lo[2 * i + 1];
  if (act && !act[node_inst_c[g_row[dst]]]) return;
  const OUT *s = vals_c + src * 324;
  OUT *d = vals_c + dst * 324;
  for (int e = lane; e < 324; e += 32)
    {
      const int a = e / 18, b = e - 18 * (e / 18);
      d[e] = s[b * 18 + a];
    }
}

template <typename T>
cudaError_t launch_prolong_add(int64_t nn_f, int B, const int32_t *ptr, const int32_t *idx, const void *w,
                               const void *zc, void *zf, const uint32_t *mask_f, const int32_t *hptr_f,
                               const int32_t *node_inst, const uint8_t *act, const void *base, cudaStream_t s,
                               TransferSlots sl)
{
  const int64_t n = nn_f * B;
  pdl_launch(k_prolong_add<T>, static_cast<unsigned>((n + 255) / 256), 256, 0, s, nn_f, B, ptr, idx,
             static_cast<const T *>(w), static_cast<const T *>(zc), static_cast<T *>(zf), mask_f, hptr_f, node_inst, act,
             static_cast<const T *>(base), sl.idx, static_cast<const T *>(sl.w));
  return cudaGetLastError();
}

cudaError_t launch_prolong(bool fp32, int64_t nn_f, int B, const int32_t *ptr, const int32_t *idx, const void *w,
                           const void *zc, void *zf, const uint32_t *mask_f, const int32_t *hptr_f,
                           const int32_t *node_inst, const uint8_t *act, cudaStream_t s, const void *base,
                           TransferSlots sl)
{
  return fp32 ? launch_prolong_add<float>(nn_f, B, ptr, idx, w, zc, zf, mask_f, hptr_f, node_inst, act, base, s, sl)
              : launch_prolong_add<double>(nn_f, B, ptr, idx, w, zc, zf, mask_f, hptr_f, node_inst, act, base, s, sl);
}

cudaError_t launch_restrict(bool fp32, int64_t nn_c, int B, const int32_t *ptr, const int32_t *idx, const void *w,
                            const void *rf, void *rc, const uint32_t *mask_c, const int32_t *node_inst,
                            const uint8_t *act, cudaStream_t s, TransferSlots sl)
{
  const int64_t n = nn_c * B;
  const unsigned g = static_cast<unsigned>((n + 255) / 256);
  if (fp32)
    pdl_launch(k_restrict<float>, g, 256, 0, s, nn_c, B, ptr, idx, static_cast<const float *>(w),
               static_cast<const float *>(rf), static_cast<float *>(rc), mask_c, node_inst, act, sl.idx,
               static_cast<const float *>(sl.w));
  else
    pdl_launch(k_restrict<double>, g, 256, 0, s, nn_c, B, ptr, idx, static_cast<const double *>(w),
               static_cast<const double *>(rf), static_cast<double *>(rc), mask_c, node_inst, act, sl.idx,
               static_cast<const double *>(sl.w));
  return cudaGetLastError();
}

cudaError_t launch_restrict_smooth(bool fp32, int64_t nn_c, const int32_t *ptr, const int32_t *idx, const void *w,
                                   const void *rf, void *rc, const uint32_t *mask_c, const int32_t *node_inst,
                                   const uint8_t *act, const void *dinv, double omega, void *z, cudaStream_t s,
                                   TransferSlots sl)
{
  const unsigned g = static_cast<unsigned>((nn_c + kRsNodes - 1) / kRsNodes);
  if (fp32)
    pdl_launch(k_restrict_smooth<float>, g, kRsNodes * 18, 0, s, nn_c, ptr, idx, static_cast<const float *>(w),
               static_cast<const float *>(rf), static_cast<float *>(rc), mask_c, node_inst, act,
               static_cast<const float *>(dinv), static_cast<float>(omega), static_cast<float *>(z), sl.idx,
               static_cast<const float *>(sl.w));
  else
    pdl_launch(k_restrict_smooth<double>, g, kRsNodes * 18, 0, s, nn_c, ptr, idx, static_cast<const double *>(w),
               static_cast<const double *>(rf), static_cast<double *>(rc), mask_c, node_inst, act,
               static_cast<const double *>(dinv), omega, static_cast<double *>(z), sl.idx,
               static_cast<const double *>(sl.w));
  return cudaGetLastError();
}

cudaError_t launch_galerkin(bool fp32, int64_t n_up, const int32_t *up, int64_t n_lo, const int32_t *lo,
                            const int32_t *g_row, const int32_t *cols_c, const uint32_t *mask_c, const int32_t *hptr_c,
                            void *vals_c, const int64_t *g_toff, const int32_t *g_blk, const void *g_w,
                            const void *vals_f, const int32_t *node_inst_c, const uint8_t *act, cudaStream_t s,
                            bool half_in, bool half_out)
{
  if (n_up == 0) return cudaSuccess;
  const int64_t grid = (n_up + kGalWarps - 1) / kGalWarps, grid_lo = (n_lo + kGalWarps - 1) / kGalWarps;
  if (grid > 0x7fffffff || grid_lo > 0x7fffffff) return cudaErrorInvalidValue;
  const unsigned g = static_cast<unsigned>(grid), gl = static_cast<unsigned>(grid_lo);
  const float *wf = static_cast<const float *>(g_w);
  if (fp32 && half_in && half_out)
    pdl_launch(k_galerkin<float, __half, __half>, g, kGalWarps * 32, 0, s, n_up, up, g_row, cols_c, mask_c, hptr_c,
               static_cast<__half *>(vals_c), g_toff, g_blk, wf, static_cast<const __half *>(vals_f), node_inst_c, act);
  else if (fp32 && half_out)
    pdl_launch(k_galerkin<float, float, __half>, g, kGalWarps * 32, 0, s, n_up, up, g_row, cols_c, mask_c, hptr_c,
               static_cast<__half *>(vals_c), g_toff, g_blk, wf, static_cast<const float *>(vals_f), node_inst_c, act);
  else if (fp32 && half_in)
    pdl_launch(k_galerkin<float, __half, float>, g, kGalWarps * 32, 0, s, n_up, up, g_row, cols_c, mask_c, hptr_c,
               static_cast<float *>(vals_c), g_toff, g_blk, wf, static_cast<const __half *>(vals_f), node_inst_c, act);
  else if (fp32)
    pdl_launch(k_galerkin<float, float, float>, g, kGalWarps * 32, 0, s, n_up, up, g_row, cols_c, mask_c, hptr_c,
               static_cast<float *>(vals_c), g_toff, g_blk, wf, static_cast<const float *>(vals_f), node_inst_c, act);
  else if (!fp32 && !half_in && !half_out)
    pdl_launch(k_galerkin<double, double, double>, g, kGalWarps * 32, 0, s, n_up, up, g_row, cols_c, mask_c, hptr_c,
               static_cast<double *>(vals_c), g_toff, g_blk, static_cast<const double *>(g_w),
               static_cast<const double *>(vals_f), node_inst_c, act);
  else
    return cudaErrorInvalidValue;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || n_lo == 0) return e;
  if (fp32 && half_out)
    pdl_launch(k_galerkin_mirror<__half>, gl, kGalWarps * 32, 0, s, n_lo, lo, g_row, static_cast<__half *>(vals_c),
               node_inst_c, act);
  else if (fp32)
    pdl_launch(k_galerkin_mirror<float>, gl, kGalWarps * 32, 0, s, n_lo, lo, g_row, static_cast<float *>(vals_c),
               node_inst_c, act);
  else
    pdl_launch(k_galerkin_mirror<double>, gl, kGalWarps * 32, 0, s, n_lo, lo, g_row, static_cast<double *>(vals_c),
               node_inst_c, act);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------------
// coarsest level (one cell per axis: 8 nodes, 144 unknowns per instance): dense inverse
// of the slightly shifted matrix in shared memory, FP32, one CTA per instance.  It is a preconditioner component, so
// FP32 suffices in both precision modes (the outer flexible GMRES is exact).
// ---------------------------------------------------------------------------------
constexpr int kGjThreads = 864;       // (column, row chunk) pairs: 6 chunks of the 144 columns
constexpr int kMaxDense = 144;        // largest coarsest system (unknowns per instance): 8 nodes x 18
constexpr int kGjRows = 24;           // register rows per thread: a multiple of 4, >= every chunk
constexpr int kGjPad = kMaxDense + kGjRows; // pivot-column length: chunks x rows < nd + rows
// rows per chunk for nd unknowns: at least kGjThreads / nd >= 6 chunks, so at most 24 rows;
// 864 threads leave 72 registers each, which hold 24 rows without spilling
__host__ __device__ constexpr int gj_rows(int nd)
{
  return ((nd + (kGjThreads / nd) - 1) / (kGjThreads / nd) + 3) & ~3;
}
// every system size fits: its rows in registers, its chunks in the block, its padded pivot
// column in shared memory
__host__ __device__ constexpr bool gj_chunks_fit()
{
  for (int nd = 1; nd <= kMaxDense; ++nd)
    {
      const int r = gj_rows(nd), nch = (nd + r - 1) / r;
      if (r > kGjRows || nch * nd > kGjThreads || nch * r > kGjPad) return false;
    }
  return true;
}
static_assert(gj_chunks_fit(), "Gauss-Jordan chunking");

// Gauss-Jordan on A + shift I with implicit partial pivoting, in place: column k is replaced in
// step k by the column of the inverse's row-permuted form that the augmented scheme [A | I]
// would build in its right half for the unit vector of the pivot row, so every step updates
// exactly nd columns.  Thread (column c, chunk) holds a 4-aligned run of rows of column c in
// registers; shared memory carries only the pivot column and the pivot row.  Step k:
//  * every warp picks the same pivot p_k (largest unused |entry| of column k, lowest index on a
//    tie) from the published column; the threads holding row p_k publish it; one barrier;
//  * every entry takes W -= colk * wp, wp = W[p][c] / pivot, and row p receives wp (the same
//    floating-point operations as the augmented scheme, entry for entry); the holders of column
//    k + 1 publish it into the other buffer; one barrier.
// Afterwards row p_k holds row k of the inverse with its columns in pivot order (column j of
// the inverse sits in the column of the step whose pivot row was j).
template <typename T>
__global__ void __launch_bounds__(kGjThreads, 1) k_dense_invert(DevMesh m, const T *__restrict__ vals,
                                                                const int64_t *__restrict__ dense_off,
                                                                float *__restrict__ inv, int *__restrict__ singular,
                                                                float shift)
{
  pdl_wait();
  pdl_trigger();
  extern __shared__ float W[]; // column-major [nd][ld]: load and write-back staging
  __shared__ __align__(16) float colk[2][kGjPad];
  __shared__ float prowv[2][kMaxDense];
  __shared__ int prow[kMaxDense];
  __shared__ int pinv[kMaxDense];
  __shared__ float s_shift;
  const int inst = blockIdx.x;
  const int64_t n0 = m.node_off_ptr[inst], n1 = m.node_off_ptr[inst + 1];
  const int B = m.B;
  const int nd = static_cast<int>((n1 - n0) * B);
  const int ld = nd | 1; // odd: a warp's lanes (consecutive columns) hit distinct banks
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (nd > kMaxDense || nd == 0) return; // rejected by the host before launch
  // chunks of rows_per rows (a multiple of 4 for the float4 reads of the pivot column)
  const int rows_per = gj_rows(nd);
  const int nch = (nd + rows_per - 1) / rows_per;
  const int my_c = tid % nd, my_ch = tid / nd;
  const bool worker = my_ch < nch;
  const int r0 = worker ? my_ch * rows_per : 0;
  for (int e = tid; e < nd * ld; e += kGjThreads) W[e] = 0.f;
  for (int e = tid; e < 2 * kGjPad; e += kGjThreads) (&colk[0][0])[e] = 0.f;
  __syncthreads();
  const int64_t b0 = m.rowptr[n0], b1 = m.rowptr[n1];
  for (int64_t i = tid; i < (b1 - b0) * B * B; i += kGjThreads)
    {
      const int64_t blk = b0 + i / (B * B);
      const int e = static_cast<int>(i % (B * B)), cr = e / B, cd = e % B;
      int64_t lo = n0, hi = n1 - 1;
      while (lo < hi)
        {
          const int64_t mid = (lo + hi + 1) / 2;
          if (m.rowptr[mid] <= blk) lo = mid;
          else hi = mid - 1;
        }
      const int row = static_cast<int>((lo - n0) * B + cr), col = static_cast<int>((m.cols[blk] - n0) * B + cd);
      W[col * ld + row] = to_f(vals[blk * B * B + e]);
    }
  __syncthreads();
  if (warp == 0)
    {
      float sd = 0.f;
      for (int i = lane; i < nd; i += 32) sd += fabsf(W[i * ld + i]);
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) sd += __shfl_xor_sync(0xffffffffu, sd, off);
      if (lane == 0) s_shift = shift * sd / static_cast<float>(nd);
    }
  __syncthreads();
  // near-null modes (global phase and spin rotations near a solution) would be amplified
  // without bound by an exact inverse: invert A + shift * mean|diag| * I instead
  float w[kGjRows];
  const float *wc = W + my_c * ld + r0; // this thread's rows, contiguous
#pragma unroll
  for (int j = 0; j < kGjRows; ++j)
    {
      const int r = r0 + j;
      w[j] = 0.f;
      if (worker && j < rows_per && r < nd) w[j] = wc[j] + (r == my_c ? s_shift : 0.f);
    }
  if (worker && my_c == 0)
#pragma unroll
    for (int j = 0; j < kGjRows; ++j)
      if (j < rows_per) colk[0][r0 + j] = w[j];
  unsigned used = 0; // bit j: row lane + 32 j is a pivot row already
  bool sing = false;
  int b = 0;
  for (int k = 0; k < nd; ++k)
    {
      __syncthreads(); // column k published; the other buffers are free again
      float best = -1.f;
      int bi = nd;
#pragma unroll
      for (int j = 0; j < (kMaxDense + 31) / 32; ++j)
        {
          const int i = lane + 32 * j;
          if (i < nd)
            {
              const float v = colk[b][i];
              if (!((used >> j) & 1u) && fabsf(v) > best)
                {
                  best = fabsf(v);
                  bi = i;
                }
            }
        }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1)
        {
          const float ob = __shfl_xor_sync(0xffffffffu, best, off);
          const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
          if (ob > best || (ob == best && oi < bi))
            {
              best = ob;
              bi = oi;
            }
        }
      if (!(best > 1e-30f) || bi >= nd)
        {
          sing = true; // every warp reads the same column: the whole block leaves here
          break;
        }
      const int p = bi;
      const float piv = colk[b][p];
      if ((p & 31) == lane) used |= 1u << (p >> 5);
      if (worker && p >= r0 && p < r0 + rows_per)
        {
          float v = 0.f;
#pragma unroll
          for (int j = 0; j < kGjRows; ++j)
            if (r0 + j == p) v = w[j];
          prowv[b][my_c] = v;
        }
      if (tid == 0) prow[k] = p;
      __syncthreads(); // row p published
      if (worker)
        {
          // column k stands for the unit vector of row p: zero except 1 in row p
          const bool pc = my_c == k;
          const float wp = (pc ? 1.f : prowv[b][my_c]) * (1.f / piv);
          const float *ck = colk[b] + r0;
#pragma unroll
          for (int j = 0; j < kGjRows; j += 4)
            if (j < rows_per)
              {
                const float4 c4 = *reinterpret_cast<const float4 *>(ck + j);
                const float cv[4] = {c4.x, c4.y, c4.z, c4.w};
#pragma unroll
                for (int t = 0; t < 4; ++t)
                  w[j + t] = (r0 + j + t == p) ? wp : fmaf(-cv[t], wp, pc ? 0.f : w[j + t]);
              }
          if (my_c == k + 1)
#pragma unroll
            for (int j = 0; j < kGjRows; ++j)
              if (j < rows_per) colk[b ^ 1][r0 + j] = w[j];
        }
      b ^= 1;
    }
  if (worker)
#pragma unroll
    for (int j = 0; j < kGjRows; ++j)
      if (j < rows_per && r0 + j < nd) W[my_c * ld + r0 + j] = w[j];
  __syncthreads();
  if (!sing)
    for (int k = tid; k < nd; k += kGjThreads) pinv[prow[k]] = k;
  __syncthreads();
  float *out = inv + dense_off[inst];
  for (int e = tid; e < nd * nd; e += kGjThreads)
    {
      const int i = e / nd, c = e - i * nd;
      out[e] = sing ? (i == c ? 1.f : 0.f) : W[pinv[c] * ld + prow[i]];
    }
  if (tid == 0 && sing) singular[inst] = 1;
}

// z = inv r per instance: one warp per row
template <typename T>
__global__ void k_dense_apply(DevMesh m, const int64_t *__restrict__ dense_off, const float *__restrict__ inv,
                              const T *__restrict__ r, T *__restrict__ z, const uint8_t *__restrict__ act)
{
  pdl_wait();
  pdl_trigger();
  const int inst = blockIdx.y;
  if (act && !act[inst]) return;
  const int64_t n0 = m.node_off_ptr[inst], n1 = m.node_off_ptr[inst + 1];
  const int nd = static_cast<int>((n1 - n0) * m.B);
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= nd) return;
  const float *A = inv + dense_off[inst] + static_cast<int64_t>(warp) * nd;
  const T *rv = r + n0 * m.B;
  float s = 0.f;
  for (int j = lane; j < nd; j += 32) s += A[j] * static_cast<float>(rv[j]);
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  if (lane == 0) z[n0 * m.B + warp] = static_cast<T>(s);
}

template <typename T>
static cudaError_t launch_dense_invert(const DevMesh &m, const void *vals, const int64_t *dense_off, float *inv,
                                      int *singular, float shift, size_t sm, cudaStream_t s)
{
  cudaError_t e =
      cudaFuncSetAttribute(k_dense_invert<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sm));
  if (e != cudaSuccess) return e;
  pdl_launch(k_dense_invert<T>, m.n_inst, kGjThreads, sm, s, m, static_cast<const T *>(vals), dense_off, inv, singular,
             shift);
  return cudaGetLastError();
}

cudaError_t launch_dense_setup(const DevMesh &m, bool fp32, const void *vals, const int64_t *dense_off, int max_nd,
                               float *inv, int *singular, float shift, cudaStream_t s)
{
  const size_t sm = static_cast<size_t>(max_nd) * (max_nd | 1) * sizeof(float);
  if (max_nd > kMaxDense || max_nd < 1) return cudaErrorInvalidValue;
  if (fp32 && m.half_vals) return launch_dense_invert<__half>(m, vals, dense_off, inv, singular, shift, sm, s);
  if (fp32) return launch_dense_invert<float>(m, vals, dense_off, inv, singular, shift, sm, s);
  return launch_dense_invert<double>(m, vals, dense_off, inv, singular, shift, sm, s);
}

cudaError_t launch_dense_apply(const DevMesh &m, bool fp32, int max_nd, const int64_t *dense_off, const float *inv,
                               const void *r, void *z, const uint8_t *act, cudaStream_t s)
{
  dim3 g((max_nd * 32 + 255) / 256, m.n_inst);
  if (fp32)
    pdl_launch(k_dense_apply<float>, g, 256, 0, s, m, dense_off, inv, static_cast<const float *>(r), static_cast<float *>(z),
                                           act);
  else
    pdl_launch(k_dense_apply<double>, g, 256, 0, s, m, dense_off, inv, static_cast<const double *>(r),
                                            static_cast<double *>(z), act);
  return cudaGetLastError();
}

} // namespace glgpu
