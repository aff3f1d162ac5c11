// Linear-algebra kernels (sm_103a): block-CSR SpMV, block-Jacobi, per-instance
// segmented reductions and vector updates, the GMRES small dense work, the
// line-search trial update and constraint distribution.
//
// Vectors are scalar arrays of length nn*B, node-major.  A context may hold several
// instances; every reduction and every per-instance scalar goes through "segments":
// contiguous ranges of at most seg_len scalars that never straddle two instances, one
// CTA per segment.  Reductions are two-pass (per-segment partials, then an ordered
// per-instance sum), so results are deterministic run to run.
#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>

#include <cuda_fp16.h>

#include "device.h"

namespace glgpu
{
template <typename T> struct Vec16;
template <> struct Vec16<float>
{
  using type = float4;
  static constexpr int n = 4;
};
template <> struct Vec16<double>
{
  using type = double2;
  static constexpr int n = 2;
};
// FP16 storage (the coarse multigrid matrices in mixed mode): four halves per 8-byte load, so
// a 324-entry block is 81 chunks like the FP32 float4 chunks (648-byte blocks are 8-byte aligned)
template <> struct Vec16<__half>
{
  using type = uint2;
  static constexpr int n = 4;
};
template <typename V, typename T> __device__ __forceinline__ T vget(const V &v, int k);
template <> __device__ __forceinline__ float vget<float4, float>(const float4 &v, int k)
{
  return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w;
}
template <> __device__ __forceinline__ double vget<double2, double>(const double2 &v, int k) { return k == 0 ? v.x : v.y; }
template <> __device__ __forceinline__ float vget<uint2, float>(const uint2 &v, int k)
{
  const unsigned w = (k < 2) ? v.x : v.y;
  const unsigned short b = static_cast<unsigned short>((k & 1) ? (w >> 16) : (w & 0xffffu));
  return __half2float(__ushort_as_half(b));
}
// scalar read of a stored matrix entry as T
template <typename T> __device__ __forceinline__ T mval(const T *p) { return *p; }
__device__ __forceinline__ float mval(const __half *p) { return __half2float(*p); }

// ---------------------------------------------------------------------------------
// SpMV, 18x18 blocks: one warp per block row.  Each block (324 scalars, 16-byte
// aligned) is streamed with 128-bit loads; lane l always owns the same scalars e of
// every block, so it accumulates sum_blocks J[e] x[col][e % 18] in registers; the 18
// row sums are formed once per row through shared memory.  x[col] is loaded once per
// block (lanes 0..17) and broadcast with shuffles.
// ---------------------------------------------------------------------------------
constexpr int kSpmvWarps = 8;

// Row n's products: acc[it][v] = sum over the row's blocks b = kw, kw + WPR, ... of
// block[e] * x[col][e % 18] for the scalars e = (lane + 32 it) * NV + v this lane owns.  The
// row's column ids are loaded once, one per lane, and broadcast by shuffle, and the block
// loop is unrolled, so the loads of several blocks are in flight together.  With WPR > 1
// warps per row (small coarse levels, where one warp per 27-block row would leave the
// GPU latency-bound) warp kw of the row takes every WPR-th block.  With CG, x is read from L2
// (ld.global.cg): inside one launch it was written by other CTAs.
template <typename T, typename MT, int WPR, bool CG = false>
__device__ __forceinline__ void row_products(const DevMesh &m, const MT *__restrict__ vals, const T *__restrict__ x,
                                             int64_t n, int lane, int kw,
                                             T (&acc)[(324 / Vec16<MT>::n + 31) / 32][Vec16<MT>::n])
{
  using V = typename Vec16<MT>::type;
  constexpr int NV = Vec16<MT>::n;
  constexpr int NCH = 324 / NV;
  constexpr int NIT = (NCH + 31) / 32;
#pragma unroll
  for (int it = 0; it < NIT; ++it)
#pragma unroll
    for (int v = 0; v < NV; ++v) acc[it][v] = T(0);
  // column ids from the fixed 27-slot table where the level has one: the load does not wait
  // for the row bounds (such rows have at most 27 blocks: one pass of the loop below)
  const int fixed_col = (m.cols27 && lane < 27) ? m.cols27[n * 27 + lane] : 0;
  const int b0 = m.rowptr[n], b1 = m.rowptr[n + 1];
  for (int base = b0; base < b1; base += 32)
    {
      const int nbk = (b1 - base) < 32 ? (b1 - base) : 32;
      const int mycol = m.cols27 ? fixed_col : ((lane < nbk) ? m.cols[base + lane] : 0);
#pragma unroll 4
      for (int k = kw; k < nbk; k += WPR)
        {
          const int64_t col = __shfl_sync(0xffffffffu, mycol, k);
          const T xv = (lane < 18) ? (CG ? __ldcg(x + col * 18 + lane) : x[col * 18 + lane]) : T(0);
          const V *bp = reinterpret_cast<const V *>(vals + static_cast<int64_t>(base + k) * 324);
#pragma unroll
          for (int it = 0; it < NIT; ++it)
            {
              const int ch = lane + 32 * it;
              const V w = (ch < NCH) ? __ldg(bp + ch) : V{};
#pragma unroll
              for (int v = 0; v < NV; ++v)
                {
                  const int e = (ch < NCH) ? ch * NV + v : 0;
                  acc[it][v] += vget<V, T>(w, v) * __shfl_sync(0xffffffffu, xv, e % 18);
                }
            }
        }
    }
}

// the row sums of red[w0 .. w0 + WPR - 1] for component `lane` (< 18)
template <typename T, int WPR>
__device__ __forceinline__ T row_sum(const T (*red)[324], int w0, int lane)
{
  T s = 0;
#pragma unroll
  for (int j = 0; j < WPR; ++j)
#pragma unroll
    for (int d = 0; d < 18; ++d) s += red[w0 + j][lane * 18 + d];
  return s;
}

// spill a warp's products into its red row
template <typename T, typename MT = T>
__device__ __forceinline__ void store_products(T *red_w, const T (&acc)[(324 / Vec16<MT>::n + 31) / 32][Vec16<MT>::n],
                                               int lane)
{
  constexpr int NV = Vec16<MT>::n;
  constexpr int NCH = 324 / NV;
  constexpr int NIT = (NCH + 31) / 32;
#pragma unroll
  for (int it = 0; it < NIT; ++it)
    {
      const int ch = lane + 32 * it;
      if (ch < NCH)
#pragma unroll
        for (int v = 0; v < NV; ++v) red_w[ch * NV + v] = acc[it][v];
    }
}

// y = A x (RES: y = b - A x); kSpmvWarps / WPR rows per CTA
template <typename T, typename MT, bool RES, int WPR>
__global__ void __launch_bounds__(kSpmvWarps * 32) k_spmv18(DevMesh m, const MT *__restrict__ vals,
                                                            const T *__restrict__ x, T *__restrict__ y,
                                                            const uint8_t *__restrict__ act, const T *__restrict__ b)
{
  pdl_wait();
  pdl_trigger();
  constexpr int NV = Vec16<MT>::n;
  constexpr int NIT = (324 / NV + 31) / 32;
  __shared__ T red[kSpmvWarps][324];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int kw = warp % WPR, w0 = warp - kw;
  const int64_t n = static_cast<int64_t>(blockIdx.x) * (kSpmvWarps / WPR) + warp / WPR;
  const bool on = n < m.nn && !(act && !act[m.node_inst[n]]);
  if (WPR == 1 && !on) return;
  T bv = T(0);
  if (on && RES && kw == 0 && lane < 18) bv = b[n * 18 + lane];
  if (on)
    {
      T acc[NIT][NV];
      row_products<T, MT, WPR>(m, vals, x, n, lane, kw, acc);
      store_products<T, MT>(red[warp], acc, lane);
    }
  if (WPR > 1)
    __syncthreads();
  else
    __syncwarp();
  if (on && kw == 0 && lane < 18)
    {
      const T s = row_sum<T, WPR>(red, w0, lane);
      y[n * 18 + lane] = RES ? bv - s : s; // A x, or the residual b - A x
    }
}

// One damped block-Jacobi sweep, fused: y = z + omega D^-1 (b - A z) (z == nullptr: the
// sweep from zero, y = omega D^-1 b).  The row's SpMV as in k_spmv18 (WPR warps per row),
// then the 18x18 inverse block applied by the row's first warp with the same lane map.
// y must not alias z (neighbouring rows read z).
template <typename T, typename MT, int WPR>
__global__ void __launch_bounds__(kSpmvWarps * 32) k_smooth18(DevMesh m, const MT *__restrict__ vals,
                                                              const T *__restrict__ dinv, const T *__restrict__ b,
                                                              const T *__restrict__ z, T *__restrict__ y, T omega,
                                                              const uint8_t *__restrict__ act)
{
  pdl_wait();
  pdl_trigger();
  using V = typename Vec16<T>::type;
  constexpr int NV = Vec16<T>::n;
  constexpr int NCH = 324 / NV;
  constexpr int NIT = (NCH + 31) / 32;
  constexpr int MNV = Vec16<MT>::n;
  constexpr int MNIT = (324 / MNV + 31) / 32;
  __shared__ T red[kSpmvWarps][324];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int kw = warp % WPR, w0 = warp - kw;
  const int64_t n = static_cast<int64_t>(blockIdx.x) * (kSpmvWarps / WPR) + warp / WPR;
  const bool on = n < m.nn && !(act && !act[m.node_inst[n]]);
  if (WPR == 1 && !on) return;
  T t = (on && lane < 18) ? b[n * 18 + lane] : T(0);
  if (z)
    {
      if (on)
        {
          T acc[MNIT][MNV];
          row_products<T, MT, WPR>(m, vals, z, n, lane, kw, acc);
          store_products<T, MT>(red[warp], acc, lane);
        }
      if (WPR > 1)
        __syncthreads();
      else
        __syncwarp();
      if (lane < 18 && on) t -= row_sum<T, WPR>(red, w0, lane);
      if (WPR > 1)
        __syncthreads();
      else
        __syncwarp();
    }
  if (!on || kw != 0) return;
  // u = D^-1 t
  {
    T acc[NIT][NV];
    const V *bp = reinterpret_cast<const V *>(dinv + n * 324);
#pragma unroll
    for (int it = 0; it < NIT; ++it)
      {
        const int ch = lane + 32 * it;
        const V w = (ch < NCH) ? __ldg(bp + ch) : V{};
#pragma unroll
        for (int v = 0; v < NV; ++v)
          {
            const int e = (ch < NCH) ? ch * NV + v : 0;
            acc[it][v] = vget<V, T>(w, v) * __shfl_sync(0xffffffffu, t, e % 18);
          }
      }
    store_products<T>(red[warp], acc, lane);
    __syncwarp();
  }
  if (lane < 18)
    {
      const T u = row_sum<T, 1>(red, warp, lane);
      y[n * 18 + lane] = (z ? z[n * 18 + lane] : T(0)) + omega * u;
    }
}

template <typename T>
__global__ void k_spmv2(DevMesh m, const T *__restrict__ vals, const T *__restrict__ x, T *__restrict__ y,
                        const uint8_t *__restrict__ act)
{
  pdl_wait();
  pdl_trigger();
  const int64_t n = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (n >= m.nn) return;
  if (act && !act[m.node_inst[n]]) return;
  T y0 = 0, y1 = 0;
  for (int blk = m.rowptr[n]; blk < m.rowptr[n + 1]; ++blk)
    {
      const int64_t col = m.cols[blk];
      const T *B = vals + static_cast<int64_t>(blk) * 4;
      const T x0 = x[2 * col], x1 = x[2 * col + 1];
      y0 += B[0] * x0 + B[1] * x1;
      y1 += B[2] * x0 + B[3] * x1;
    }
  y[2 * n] = y0;
  y[2 * n + 1] = y1;
}

// Rows below these counts (coarse multigrid levels) get 4 / 8 warps per row.
constexpr int64_t kSmallRows = 20000;
constexpr int64_t kTinyRows = 2000;

template <typename T, typename MT, bool RES, int WPR>
static void spmv18_t(const DevMesh &m, const void *vals, const void *x, void *y, const uint8_t *act, const void *b,
                     cudaStream_t s)
{
  constexpr int rows = kSpmvWarps / WPR;
  const unsigned grid = static_cast<unsigned>((m.nn + rows - 1) / rows);
  pdl_launch(k_spmv18<T, MT, RES, WPR>, grid, kSpmvWarps * 32, 0, s, m, static_cast<const MT *>(vals),
                                                              static_cast<const T *>(x), static_cast<T *>(y), act,
                                                              static_cast<const T *>(b));
}

template <typename T, typename MT>
static void spmv18_dispatch(const DevMesh &m, const void *vals, const void *x, void *y, const uint8_t *act,
                            const void *b, cudaStream_t s)
{
  if (b)
    m.nn < kTinyRows    ? spmv18_t<T, MT, true, 8>(m, vals, x, y, act, b, s)
    : m.nn < kSmallRows ? spmv18_t<T, MT, true, 4>(m, vals, x, y, act, b, s)
                        : spmv18_t<T, MT, true, 1>(m, vals, x, y, act, b, s);
  else
    m.nn < kTinyRows    ? spmv18_t<T, MT, false, 8>(m, vals, x, y, act, b, s)
    : m.nn < kSmallRows ? spmv18_t<T, MT, false, 4>(m, vals, x, y, act, b, s)
                        : spmv18_t<T, MT, false, 1>(m, vals, x, y, act, b, s);
}

cudaError_t launch_spmv(const DevMesh &m, bool fp32, const void *vals, const void *x, void *y, const uint8_t *act,
                        cudaStream_t s, const void *b)
{
  if (m.B == 18)
    {
      if (fp32 && m.half_vals)
        spmv18_dispatch<float, __half>(m, vals, x, y, act, b, s);
      else if (fp32)
        spmv18_dispatch<float, float>(m, vals, x, y, act, b, s);
      else
        spmv18_dispatch<double, double>(m, vals, x, y, act, b, s);
    }
  else
    {
      if (b) return cudaErrorInvalidValue; // the residual form exists for 18x18 blocks only
      const unsigned grid = static_cast<unsigned>((m.nn + 255) / 256);
      if (fp32)
        pdl_launch(k_spmv2<float>, grid, 256, 0, s, m, static_cast<const float *>(vals), static_cast<const float *>(x),
                                            static_cast<float *>(y), act);
      else
        pdl_launch(k_spmv2<double>, grid, 256, 0, s, m, static_cast<const double *>(vals), static_cast<const double *>(x),
                                             static_cast<double *>(y), act);
    }
  return cudaGetLastError();
}

// The sweep from zero, y = omega D^-1 b: thread (node, component), 16 nodes per CTA; the
// node's 18 values of b meet in shared memory and thread c reads row c of the inverse block
// (the node's 18 threads read the block's 1296 contiguous bytes)
constexpr int kSzNodes = 16;

template <typename T, typename DT = T>
__global__ void __launch_bounds__(kSzNodes * 18) k_smooth_zero18(DevMesh m, const DT *__restrict__ dinv,
                                                                 const T *__restrict__ b, T *__restrict__ y, T omega,
                                                                 const uint8_t *__restrict__ act)
{
  pdl_wait();
  pdl_trigger();
  __shared__ T b_s[kSzNodes][18];
  const int ln = threadIdx.x / 18, c = threadIdx.x - 18 * (threadIdx.x / 18);
  const int64_t n = static_cast<int64_t>(blockIdx.x) * kSzNodes + ln;
  const bool on = n < m.nn && !(act && !act[m.node_inst[n]]);
  b_s[ln][c] = on ? b[n * 18 + c] : T(0);
  __syncthreads();
  if (!on) return;
  const DT *row = dinv + n * 324 + c * 18;
  T u = 0;
  if constexpr (sizeof(DT) == 2)
    {
      // FP16 row: 36 bytes at a 4-byte boundary, nine half2 loads
      const __half2 *r2 = reinterpret_cast<const __half2 *>(row);
#pragma unroll
      for (int d = 0; d < 9; ++d)
        {
          const float2 w = __half22float2(__ldg(r2 + d));
          u += w.x * b_s[ln][2 * d];
          u += w.y * b_s[ln][2 * d + 1];
        }
    }
  else
#pragma unroll
    for (int d = 0; d < 18; ++d) u += mval(row + d) * b_s[ln][d];
  y[n * 18 + c] = omega * u;
}

template <typename T, typename MT, int WPR>
static void smooth18_t(const DevMesh &m, const void *vals, const void *dinv, const void *b, const void *z, void *y,
                       double omega, const uint8_t *act, cudaStream_t s)
{
  constexpr int rows = kSpmvWarps / WPR;
  const unsigned grid = static_cast<unsigned>((m.nn + rows - 1) / rows);
  pdl_launch(k_smooth18<T, MT, WPR>, grid, kSpmvWarps * 32, 0, s, m, static_cast<const MT *>(vals),
                                                           static_cast<const T *>(dinv), static_cast<const T *>(b),
                                                           static_cast<const T *>(z), static_cast<T *>(y),
                                                           static_cast<T>(omega), act);
}

template <typename T, typename MT>
static void smooth18_dispatch(const DevMesh &m, const void *vals, const void *dinv, const void *b, const void *z,
                              void *y, double omega, const uint8_t *act, cudaStream_t s)
{
  m.nn < kTinyRows    ? smooth18_t<T, MT, 8>(m, vals, dinv, b, z, y, omega, act, s)
  : m.nn < kSmallRows ? smooth18_t<T, MT, 4>(m, vals, dinv, b, z, y, omega, act, s)
                      : smooth18_t<T, MT, 1>(m, vals, dinv, b, z, y, omega, act, s);
}

cudaError_t launch_smooth_zero_half(const DevMesh &m, const __half *dinv, const float *b, float *y, double omega,
                                    const uint8_t *act, cudaStream_t s)
{
  if (m.B != 18) return cudaErrorInvalidValue;
  const unsigned grid = static_cast<unsigned>((m.nn + kSzNodes - 1) / kSzNodes);
  pdl_launch(k_smooth_zero18<float, __half>, grid, kSzNodes * 18, 0, s, m, dinv, b, y, static_cast<float>(omega), act);
  return cudaGetLastError();
}

cudaError_t launch_smooth(const DevMesh &m, bool fp32, const void *vals, const void *dinv, const void *b, const void *z,
                          void *y, double omega, const uint8_t *act, cudaStream_t s)
{
  if (m.B != 18) return cudaErrorInvalidValue;
  if (!z)
    {
      const unsigned grid = static_cast<unsigned>((m.nn + kSzNodes - 1) / kSzNodes);
      if (fp32)
        pdl_launch(k_smooth_zero18<float>, grid, kSzNodes * 18, 0, s, m, static_cast<const float *>(dinv),
                                                             static_cast<const float *>(b), static_cast<float *>(y),
                                                             static_cast<float>(omega), act);
      else
        pdl_launch(k_smooth_zero18<double>, grid, kSzNodes * 18, 0, s, m, static_cast<const double *>(dinv),
                                                              static_cast<const double *>(b), static_cast<double *>(y),
                                                              omega, act);
      return cudaGetLastError();
    }
  if (fp32 && m.half_vals)
    smooth18_dispatch<float, __half>(m, vals, dinv, b, z, y, omega, act, s);
  else if (fp32)
    smooth18_dispatch<float, float>(m, vals, dinv, b, z, y, omega, act, s);
  else
    smooth18_dispatch<double, double>(m, vals, dinv, b, z, y, omega, act, s);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------------
// block-Jacobi: invert each node's diagonal block (Gauss-Jordan, partial pivoting,
// FP64 arithmetic), one warp per node for 18x18.  A singular block falls back to
// the identity so the preconditioner stays defined.
// ---------------------------------------------------------------------------------
constexpr int kBjWarps = 4;

// OUT: storage of the inverse blocks (FP16 for the finest level's smoother in mixed mode)
template <typename T, typename MT = T, typename OUT = T>
__global__ void __launch_bounds__(kBjWarps * 32) k_bj_setup18(DevMesh m, const MT *__restrict__ vals,
                                                              OUT *__restrict__ dinv, int l1)
{
  pdl_wait();
  pdl_trigger();
  __shared__ T M[kBjWarps][18][37];
  __shared__ T L1s[kBjWarps][324]; // l1: per-entry absolute sums of the row's off-diagonal blocks
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t n = static_cast<int64_t>(blockIdx.x) * kBjWarps + warp;
  if (n >= m.nn) return;
  const MT *D = vals + static_cast<int64_t>(m.diag[n]) * 324;
  for (int i = lane; i < 18 * 36; i += 32)
    {
      const int r = i / 36, c = i % 36;
      M[warp][r][c] = (c < 18) ? static_cast<T>(mval(D + r * 18 + c)) : ((c - 18 == r) ? T(1) : T(0));
    }
  __syncwarp();
  if (l1)
    {
      // l1 block-Jacobi: row r's diagonal grows by the absolute sum of its entries outside
      // the diagonal block (with the diagonal's sign), which makes the smoother convergent
      // for every symmetric positive definite matrix, mass-dominated ones included.  The
      // warp streams the row's blocks with the SpMV lane map (lane l owns entries
      // e = (l + 32 it) NV + v of every block, 16- or 8-byte loads); the per-entry sums then
      // meet per row in shared memory.
      using V = typename Vec16<MT>::type;
      constexpr int NV = Vec16<MT>::n;
      constexpr int NCH = 324 / NV;
      constexpr int NIT = (NCH + 31) / 32;
      T acc[NIT][NV];
#pragma unroll
      for (int it = 0; it < NIT; ++it)
#pragma unroll
        for (int v = 0; v < NV; ++v) acc[it][v] = T(0);
      const int32_t rb0 = m.rowptr[n], rb1 = m.rowptr[n + 1], rd = m.diag[n];
#pragma unroll 4
      for (int32_t b = rb0; b < rb1; ++b)
        {
          if (b == rd) continue;
          const V *bp = reinterpret_cast<const V *>(vals + static_cast<int64_t>(b) * 324);
#pragma unroll
          for (int it = 0; it < NIT; ++it)
            {
              const int ch = lane + 32 * it;
              const V w = (ch < NCH) ? __ldg(bp + ch) : V{};
#pragma unroll
              for (int v = 0; v < NV; ++v) acc[it][v] += fabs(static_cast<T>(vget<V, T>(w, v)));
            }
        }
      T *l1s = L1s[warp];
#pragma unroll
      for (int it = 0; it < NIT; ++it)
        {
          const int ch = lane + 32 * it;
          if (ch < NCH)
#pragma unroll
            for (int v = 0; v < NV; ++v) l1s[ch * NV + v] = acc[it][v];
        }
      __syncwarp();
      if (lane < 18)
        {
          T sum = 0;
#pragma unroll
          for (int c = 0; c < 18; ++c) sum += l1s[lane * 18 + c];
          const T d = M[warp][lane][lane];
          M[warp][lane][lane] = d + (d < T(0) ? -sum : sum);
        }
      __syncwarp();
    }
  bool singular = false;
  for (int k = 0; k < 18; ++k)
    {
      T best = (lane >= k && lane < 18) ? fabs(M[warp][lane][k]) : T(-1);
      int bi = lane;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1)
        {
          const T ob = __shfl_xor_sync(0xffffffffu, best, off);
          const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
          if (ob > best || (ob == best && oi < bi))
            {
              best = ob;
              bi = oi;
            }
        }
      if (!(best > (sizeof(T) == 4 ? T(1e-30) : T(1e-300))))
        {
          singular = true;
          break;
        }
      if (bi != k)
        for (int c = lane; c < 36; c += 32)
          {
            const T t = M[warp][k][c];
            M[warp][k][c] = M[warp][bi][c];
            M[warp][bi][c] = t;
          }
      __syncwarp();
      const T piv = M[warp][k][k];
      __syncwarp();
      for (int c = lane; c < 36; c += 32) M[warp][k][c] /= piv;
      __syncwarp();
      T f[18];
#pragma unroll
      for (int r = 0; r < 18; ++r) f[r] = M[warp][r][k];
      __syncwarp();
      for (int c = lane; c < 36; c += 32)
        {
          const T pk = M[warp][k][c];
#pragma unroll
          for (int r = 0; r < 18; ++r)
            if (r != k) M[warp][r][c] -= f[r] * pk;
        }
      __syncwarp();
    }
  OUT *out = dinv + n * 324;
  for (int i = lane; i < 324; i += 32)
    {
      const int r = i / 18, c = i % 18;
      out[i] = static_cast<OUT>(singular ? T(r == c ? 1 : 0) : M[warp][r][18 + c]);
    }
}

template <typename T>
__global__ void k_bj_setup2(DevMesh m, const T *__restrict__ vals, T *__restrict__ dinv)
{
  pdl_wait();
  pdl_trigger();
  const int64_t n = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (n >= m.nn) return;
  const T *D = vals + static_cast<int64_t>(m.diag[n]) * 4;
  const double a = D[0], b = D[1], c = D[2], d = D[3];
  const double det = a * d - b * c;
  T *o = dinv + n * 4;
  if (fabs(det) > 1e-300)
    {
      o[0] = static_cast<T>(d / det);
      o[1] = static_cast<T>(-b / det);
      o[2] = static_cast<T>(-c / det);
      o[3] = static_cast<T>(a / det);
    }
  else
    {
      o[0] = T(1);
      o[1] = T(0);
      o[2] = T(0);
      o[3] = T(1);
    }
}

cudaError_t launch_bj_setup_half(const DevMesh &m, const void *vals, __half *dinv, cudaStream_t s)
{
  if (m.B != 18) return cudaErrorInvalidValue;
  const unsigned grid = static_cast<unsigned>((m.nn + kBjWarps - 1) / kBjWarps);
  if (m.half_vals)
    pdl_launch(k_bj_setup18<float, __half, __half>, grid, kBjWarps * 32, 0, s, m, static_cast<const __half *>(vals),
               dinv, 1);
  else
    pdl_launch(k_bj_setup18<float, float, __half>, grid, kBjWarps * 32, 0, s, m, static_cast<const float *>(vals), dinv,
               1);
  return cudaGetLastError();
}

cudaError_t launch_bj_setup(const DevMesh &m, bool fp32, const void *vals, void *dinv, cudaStream_t s, bool l1)
{
  if (m.B == 18)
    {
      const unsigned grid = static_cast<unsigned>((m.nn + kBjWarps - 1) / kBjWarps);
      if (fp32 && m.half_vals)
        pdl_launch(k_bj_setup18<float, __half>, grid, kBjWarps * 32, 0, s, m, static_cast<const __half *>(vals),
                                                                   static_cast<float *>(dinv), l1 ? 1 : 0);
      else if (fp32)
        pdl_launch(k_bj_setup18<float>, grid, kBjWarps * 32, 0, s, m, static_cast<const float *>(vals), static_cast<float *>(dinv),
                                                           l1 ? 1 : 0);
      else
        pdl_launch(k_bj_setup18<double>, grid, kBjWarps * 32, 0, s, m, static_cast<const double *>(vals),
                                                            static_cast<double *>(dinv), l1 ? 1 : 0);
    }
  else
    {
      const unsigned grid = static_cast<unsigned>((m.nn + 255) / 256);
      if (fp32)
        pdl_launch(k_bj_setup2<float>, grid, 256, 0, s, m, static_cast<const float *>(vals), static_cast<float *>(dinv));
      else
        pdl_launch(k_bj_setup2<double>, grid, 256, 0, s, m, static_cast<const double *>(vals), static_cast<double *>(dinv));
    }
  return cudaGetLastError();
}

// z[n] = Dinv[n] r[n]: the SpMV kernel over a diagonal-only pattern
template <typename T>
__global__ void __launch_bounds__(kSpmvWarps * 32) k_bj_apply18(DevMesh m, const T *__restrict__ dinv,
                                                                const T *__restrict__ x, T *__restrict__ y,
                                                                const uint8_t *__restrict__ act)
{
  pdl_wait();
  pdl_trigger();
  using V = typename Vec16<T>::type;
  constexpr int NV = Vec16<T>::n;
  constexpr int NCH = 324 / NV;
  constexpr int NIT = (NCH + 31) / 32;
  __shared__ T red[kSpmvWarps][324];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t n = static_cast<int64_t>(blockIdx.x) * kSpmvWarps + warp;
  if (n >= m.nn) return;
  if (act && !act[m.node_inst[n]]) return;
  const T xv = (lane < 18) ? x[n * 18 + lane] : T(0);
  const V *bp = reinterpret_cast<const V *>(dinv + n * 324);
#pragma unroll
  for (int it = 0; it < NIT; ++it)
    {
      const int ch = lane + 32 * it;
      V w;
      if (ch < NCH)
        w = __ldg(bp + ch);
      else
        w = V{};
#pragma unroll
      for (int v = 0; v < NV; ++v)
        {
          const int e = (ch < NCH) ? ch * NV + v : 0;
          const T xd = __shfl_sync(0xffffffffu, xv, e % 18);
          if (ch < NCH) red[warp][e] = vget<V, T>(w, v) * xd;
        }
    }
  __syncwarp();
  if (lane < 18)
    {
      T s = 0;
#pragma unroll
      for (int d = 0; d < 18; ++d) s += red[warp][lane * 18 + d];
      y[n * 18 + lane] = s;
    }
}

template <typename T>
__global__ void k_bj_apply2(DevMesh m, const T *__restrict__ dinv, const T *__restrict__ x, T *__restrict__ y,
                            const uint8_t *__restrict__ act)
{
  pdl_wait();
  pdl_trigger();
  const int64_t n = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (n >= m.nn) return;
  if (act && !act[m.node_inst[n]]) return;
  const T *D = dinv + n * 4;
  const T x0 = x[2 * n], x1 = x[2 * n + 1];
  y[2 * n] = D[0] * x0 + D[1] * x1;
  y[2 * n + 1] = D[2] * x0 + D[3] * x1;
}

cudaError_t launch_bj_apply(const DevMesh &m, bool fp32, const void *dinv, const void *x, void *y,
                            const uint8_t *act, cudaStream_t s)
{
  if (m.B == 18)
    {
      const unsigned grid = static_cast<unsigned>((m.nn + kSpmvWarps - 1) / kSpmvWarps);
      if (fp32)
        pdl_launch(k_bj_apply18<float>, grid, kSpmvWarps * 32, 0, s, m, static_cast<const float *>(dinv),
                                                            static_cast<const float *>(x), static_cast<float *>(y), act);
      else
        pdl_launch(k_bj_apply18<double>, grid, kSpmvWarps * 32, 0, s, m, static_cast<const double *>(dinv),
                                                             static_cast<const double *>(x), static_cast<double *>(y),
                                                             act);
    }
  else
    {
      const unsigned grid = static_cast<unsigned>((m.nn + 255) / 256);
      if (fp32)
        pdl_launch(k_bj_apply2<float>, grid, 256, 0, s, m, static_cast<const float *>(dinv), static_cast<const float *>(x),
                                                static_cast<float *>(y), act);
      else
        pdl_launch(k_bj_apply2<double>, grid, 256, 0, s, m, static_cast<const double *>(dinv), static_cast<const double *>(x),
                                                 static_cast<double *>(y), act);
    }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------------
// segmented reductions
// ---------------------------------------------------------------------------------
__device__ __forceinline__ double block_sum(double v, double *sh)
{
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  double s = 0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (kSegThreads >> 5); ++w) s += sh[w];
  return s; // valid in thread 0
}

// Multi-dot partials: the segment of y is staged in shared memory once, then each warp
// takes basis vectors v = warp, warp + 8, ... and reduces with shuffles only.
template <typename TX, typename TY>
__global__ void __launch_bounds__(kSegThreads) k_seg_mdot(DevMesh m, const TX *__restrict__ X, int64_t ld, int nvec,
                                                          const TY *__restrict__ y, double *__restrict__ partial,
                                                          const uint8_t *__restrict__ act)
{
  pdl_wait();
  pdl_trigger();
  __shared__ TY ys[kSegMax];
  const int s = blockIdx.x;
  const int64_t b = m.seg_begin[s];
  const int len = static_cast<int>(m.seg_end[s] - b);
  const bool on = !act || act[m.seg_inst[s]];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (on)
    for (int i = threadIdx.x; i < len; i += kSegThreads) ys[i] = y[b + i];
  __syncthreads();
  for (int v = warp; v < nvec; v += kSegThreads / 32)
    {
      double acc = 0.0;
      if (on)
        {
          const TX *xv = X + v * ld + b;
          float facc0 = 0.f, facc1 = 0.f;
          double dacc0 = 0.0, dacc1 = 0.0;
          int i = lane;
          for (; i + 32 < len; i += 64)
            {
              if (sizeof(TX) == 4)
                {
                  facc0 += static_cast<float>(xv[i]) * static_cast<float>(ys[i]);
                  facc1 += static_cast<float>(xv[i + 32]) * static_cast<float>(ys[i + 32]);
                }
              else
                {
                  dacc0 += static_cast<double>(xv[i]) * static_cast<double>(ys[i]);
                  dacc1 += static_cast<double>(xv[i + 32]) * static_cast<double>(ys[i + 32]);
                }
            }
          if (i < len)
            {
              if (sizeof(TX) == 4)
                facc0 += static_cast<float>(xv[i]) * static_cast<float>(ys[i]);
              else
                dacc0 += static_cast<double>(xv[i]) * static_cast<double>(ys[i]);
            }
          acc = static_cast<double>(facc0) + static_cast<double>(facc1) + dacc0 + dacc1;
        }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
      if (lane == 0) partial[static_cast<int64_t>(s) * nvec + v] = acc;
    }
}

cudaError_t launch_seg_mdot(const DevMesh &m, bool fp32, const void *X, int64_t ld, int nvec, const void *y,
                            double *partial, const uint8_t *act, cudaStream_t s)
{
  if (fp32)
    pdl_launch(k_seg_mdot<float, float>, m.n_seg, kSegThreads, 0, s, m, static_cast<const float *>(X), ld, nvec,
                                                             static_cast<const float *>(y), partial, act);
  else
    pdl_launch(k_seg_mdot<double, double>, m.n_seg, kSegThreads, 0, s, m, static_cast<const double *>(X), ld, nvec,
                                                               static_cast<const double *>(y), partial, act);
  return cudaGetLastError();
}

// one warp per (instance, vector): lanes take segments lane, lane + 32, ... into four
// interleaved sums (four loads in flight) in a fixed order, then a fixed shuffle tree:
// deterministic
__global__ void k_seg_finalize(DevMesh m, const double *__restrict__ partial, int nvec, double *__restrict__ out,
                               int ld_out, int take_sqrt)
{
  pdl_wait();
  pdl_trigger();
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= m.n_inst * nvec) return;
  const int inst = w / nvec, v = w % nvec;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
  const int g1 = m.inst_seg_off[inst + 1];
  int g = m.inst_seg_off[inst] + lane;
  for (; g + 96 < g1; g += 128)
    {
      s0 += partial[static_cast<int64_t>(g) * nvec + v];
      s1 += partial[static_cast<int64_t>(g + 32) * nvec + v];
      s2 += partial[static_cast<int64_t>(g + 64) * nvec + v];
      s3 += partial[static_cast<int64_t>(g + 96) * nvec + v];
    }
  for (; g < g1; g += 32) s0 += partial[static_cast<int64_t>(g) * nvec + v];
  double s = (s0 + s1) + (s2 + s3);
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  if (lane == 0) out[inst * ld_out + v] = take_sqrt ? sqrt(s) : s;
}

cudaError_t launch_seg_finalize(const DevMesh &m, const double *partial, int nvec, double *out, int ld_out,
                                int take_sqrt, cudaStream_t s)
{
  const int nw = m.n_inst * nvec;
  pdl_launch(k_seg_finalize, (nw + 3) / 4, 128, 0, s, m, partial, nvec, out, ld_out, take_sqrt);
  return cudaGetLastError();
}

// y_seg -= sum_v coef[inst][v] X[v]_seg (arithmetic in T), then, in the same pass,
// the partial dots of the updated y_seg with X[0..nvec2) and with itself: the second
// Gram-Schmidt projection and the norm of the new basis vector need no extra read of y.
template <typename T>
__global__ void __launch_bounds__(kSegThreads) k_seg_update(DevMesh m, const T *__restrict__ X, int64_t ld, int nvec,
                                                            const double *__restrict__ coef, int ldc,
                                                            T *__restrict__ y, int nvec2, double *__restrict__ partial2,
                                                            double *__restrict__ partial_norm,
                                                            const uint8_t *__restrict__ act)
{
  pdl_wait();
  pdl_trigger();
  __shared__ T cf[64];
  __shared__ T ys[kSegMax];
  const int s = blockIdx.x;
  const int inst = m.seg_inst[s];
  const bool on = !act || act[inst];
  const int64_t b = m.seg_begin[s];
  const int len = static_cast<int>(m.seg_end[s] - b);
  for (int v = threadIdx.x; v < nvec; v += kSegThreads) cf[v] = on ? static_cast<T>(coef[inst * ldc + v]) : T(0);
  __syncthreads();
  if (on)
    for (int i = threadIdx.x; i < len; i += kSegThreads)
      {
        T acc = y[b + i];
        const T *xp = X + b + i;
        int v = 0;
        for (; v + 4 <= nvec; v += 4)
          {
            const T x0 = xp[(v + 0) * ld], x1 = xp[(v + 1) * ld], x2 = xp[(v + 2) * ld], x3 = xp[(v + 3) * ld];
            acc -= cf[v] * x0;
            acc -= cf[v + 1] * x1;
            acc -= cf[v + 2] * x2;
            acc -= cf[v + 3] * x3;
          }
        for (; v < nvec; ++v) acc -= cf[v] * xp[v * ld];
        y[b + i] = acc;
        ys[i] = acc;
      }
  if (nvec2 <= 0 && !partial_norm) return;
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntot = nvec2 + (partial_norm ? 1 : 0);
  for (int v = warp; v < ntot; v += kSegThreads / 32)
    {
      T a0 = 0, a1 = 0;
      if (on)
        {
          const T *xv = (v < nvec2) ? X + v * ld + b : nullptr;
          int i = lane;
          for (; i + 32 < len; i += 64)
            {
              const T y0 = ys[i], y1 = ys[i + 32];
              a0 += (xv ? xv[i] : y0) * y0;
              a1 += (xv ? xv[i + 32] : y1) * y1;
            }
          if (i < len) a0 += (xv ? xv[i] : ys[i]) * ys[i];
        }
      double acc = static_cast<double>(a0) + static_cast<double>(a1);
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
      if (lane == 0)
        {
          if (v < nvec2)
            partial2[static_cast<int64_t>(s) * nvec2 + v] = acc;
          else
            partial_norm[s] = acc;
        }
    }
}

cudaError_t launch_seg_update(const DevMesh &m, bool fp32, const void *X, int64_t ld, int nvec, const double *coef,
                              int ldc, void *y, int nvec2, double *partial2, double *partial_norm, const uint8_t *act,
                              cudaStream_t s)
{
  if (nvec > 64) return cudaErrorInvalidValue;
  if (fp32)
    pdl_launch(k_seg_update<float>, m.n_seg, kSegThreads, 0, s, m, static_cast<const float *>(X), ld, nvec, coef, ldc,
                                                        static_cast<float *>(y), nvec2, partial2, partial_norm, act);
  else
    pdl_launch(k_seg_update<double>, m.n_seg, kSegThreads, 0, s, m, static_cast<const double *>(X), ld, nvec, coef, ldc,
                                                         static_cast<double *>(y), nvec2, partial2, partial_norm, act);
  return cudaGetLastError();
}

cudaError_t launch_seg_maxpy(const DevMesh &m, bool fp32, const void *X, int64_t ld, int nvec, const double *coef,
                             int ldc, void *y, const uint8_t *act, cudaStream_t s)
{
  return launch_seg_update(m, fp32, X, ld, nvec, coef, ldc, y, 0, nullptr, nullptr, act, s);
}

template <typename TX, typename TY, typename TZ>
__global__ void __launch_bounds__(kSegThreads) k_seg_axpby(DevMesh m, const TX *__restrict__ x, TY *__restrict__ y,
                                                           const TZ *__restrict__ z, Axpby k,
                                                           const uint8_t *__restrict__ act)
{
  pdl_wait();
  pdl_trigger();
  const int s = blockIdx.x;
  const int inst = m.seg_inst[s];
  if (act && !act[inst]) return;
  const double a = k.a ? k.a[inst * k.sa] : k.a0;
  const double b = k.b ? k.b[inst * k.sb] : k.b0;
  const double c = k.c ? k.c[inst * k.sc] : k.c0;
  const int64_t b0 = m.seg_begin[s], e = m.seg_end[s];
  // arithmetic in FP32 when every operand is FP32, else FP64
  using C = typename std::conditional<(sizeof(TX) == 4 && sizeof(TY) == 4 && sizeof(TZ) == 4), float, double>::type;
  const C ca = static_cast<C>(a), cb = static_cast<C>(b), cc = static_cast<C>(c);
  for (int64_t i = b0 + threadIdx.x; i < e; i += kSegThreads)
    {
      C v = (a != 0.0 && x) ? ca * static_cast<C>(x[i]) : C(0);
      if (b != 0.0) v += cb * static_cast<C>(y[i]);
      if (z && c != 0.0) v += cc * static_cast<C>(z[i]);
      y[i] = static_cast<TY>(v);
    }
}

template <typename TX, typename TY>
static void axpby_z(const DevMesh &m, const void *x, void *y, bool z32, const void *z, const Axpby &k,
                    const uint8_t *act, cudaStream_t s)
{
  if (z32)
    pdl_launch(k_seg_axpby<TX, TY, float>, m.n_seg, kSegThreads, 0, s, m, static_cast<const TX *>(x), static_cast<TY *>(y),
                                                               static_cast<const float *>(z), k, act);
  else
    pdl_launch(k_seg_axpby<TX, TY, double>, m.n_seg, kSegThreads, 0, s, m, static_cast<const TX *>(x), static_cast<TY *>(y),
                                                                static_cast<const double *>(z), k, act);
}

cudaError_t launch_seg_axpby(const DevMesh &m, bool x32, const void *x, bool y32, void *y, bool z32, const void *z,
                             const Axpby &k, const uint8_t *act, cudaStream_t s)
{
  if (x32 && y32) axpby_z<float, float>(m, x, y, z32, z, k, act, s);
  else if (x32) axpby_z<float, double>(m, x, y, z32, z, k, act, s);
  else if (y32) axpby_z<double, float>(m, x, y, z32, z, k, act, s);
  else axpby_z<double, double>(m, x, y, z32, z, k, act, s);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------------
// constraints: line-search trial and distribute
// ---------------------------------------------------------------------------------
__global__ void k_trial(DevMesh m, const double *__restrict__ x, const double *__restrict__ dl,
                        const double *__restrict__ a, double *__restrict__ xt, const uint8_t *__restrict__ act)
{
  pdl_wait();
  pdl_trigger();
  const int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= m.nn * m.B) return;
  const int64_t n = idx / m.B;
  const int c = static_cast<int>(idx % m.B);
  const int inst = m.node_inst[n];
  if (act && !act[inst]) return;
  const double al = a[inst];
  double v;
  if (m.hptr[n + 1] > m.hptr[n])
    {
      v = 0.0;
      for (int k = m.hptr[n]; k < m.hptr[n + 1]; ++k)
        {
          const int64_t p = m.hpar[k];
          if (!((m.mask[p] >> c) & 1u)) v += m.hw[k] * (x[p * m.B + c] + al * dl[p * m.B + c]);
        }
    }
  else if ((m.mask[n] >> c) & 1u)
    v = 0.0;
  else
    v = x[idx] + al * dl[idx];
  xt[idx] = v;
}

cudaError_t launch_trial(const DevMesh &m, const double *x, const double *delta, const double *a, double *xt,
                         const uint8_t *act, cudaStream_t s)
{
  const int64_t n = m.nn * m.B;
  pdl_launch(k_trial, static_cast<unsigned>((n + 255) / 256), 256, 0, s, m, x, delta, a, xt, act);
  return cudaGetLastError();
}

// two passes: Dirichlet zeros on regular nodes, then hanging nodes from parents
__global__ void k_dist_regular(DevMesh m, double *__restrict__ v)
{
  pdl_wait();
  pdl_trigger();
  const int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= m.nn * m.B) return;
  const int64_t n = idx / m.B;
  const int c = static_cast<int>(idx % m.B);
  if (m.hptr[n + 1] == m.hptr[n] && ((m.mask[n] >> c) & 1u)) v[idx] = 0.0;
}

__global__ void k_dist_hanging(DevMesh m, double *__restrict__ v)
{
  pdl_wait();
  pdl_trigger();
  const int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= m.nn * m.B) return;
  const int64_t n = idx / m.B;
  const int c = static_cast<int>(idx % m.B);
  if (m.hptr[n + 1] == m.hptr[n]) return;
  double s = 0.0;
  for (int k = m.hptr[n]; k < m.hptr[n + 1]; ++k) s += m.hw[k] * v[static_cast<int64_t>(m.hpar[k]) * m.B + c];
  v[idx] = s;
}

cudaError_t launch_distribute(const DevMesh &m, double *v, cudaStream_t s)
{
  const int64_t n = m.nn * m.B;
  const unsigned grid = static_cast<unsigned>((n + 255) / 256);
  pdl_launch(k_dist_regular, grid, 256, 0, s, m, v);
  pdl_launch(k_dist_hanging, grid, 256, 0, s, m, v);
  return cudaGetLastError();
}

// ordered per-instance sum of per-cell values
__global__ void __launch_bounds__(kSegThreads) k_cell_sum(DevMesh m, const double *__restrict__ ec,
                                                          double *__restrict__ out)
{
  pdl_wait();
  pdl_trigger();
  __shared__ double sh[kSegThreads / 32];
  const int inst = blockIdx.x;
  const int64_t b = m.cell_off[inst], e = m.cell_off[inst + 1];
  double acc = 0.0;
  for (int64_t i = b + threadIdx.x; i < e; i += kSegThreads) acc += ec[i];
  const double tot = block_sum(acc, sh);
  if (threadIdx.x == 0) out[inst] = tot;
}

cudaError_t launch_cell_sum(const DevMesh &m, const double *e_cell, double *out, cudaStream_t s)
{
  pdl_launch(k_cell_sum, m.n_inst, kSegThreads, 0, s, m, e_cell, out);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------------
// GMRES small dense work (one thread per instance)
// ---------------------------------------------------------------------------------
__global__ void k_gmres_start(GmresDev g, int n_inst, const uint8_t *__restrict__ solve_active)
{
  pdl_wait();
  pdl_trigger();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_inst) return;
  const double beta = g.beta[k];
  for (int i = 0; i <= g.m; ++i) g.g[k * (g.m + 1) + i] = 0.0;
  g.g[k * (g.m + 1)] = beta;
  g.its[k] = 0;
  g.res_est[k] = beta;
  const bool on = (!solve_active || solve_active[k]) && beta > g.tol[k] && isfinite(beta);
  g.active[k] = on ? 1 : 0;
  g.inv_scale[k] = (on && beta > 0.0) ? 1.0 / beta : 0.0;
}

cudaError_t launch_gmres_start(const GmresDev &g, int n_inst, const uint8_t *solve_active, cudaStream_t s)
{
  pdl_launch(k_gmres_start, (n_inst + 127) / 128, 128, 0, s, g, n_inst, solve_active);
  return cudaGetLastError();
}

// hcol[k][0..j] + hcol2[k][0..j]: projections; hcol[k][j+1]: norm of the new vector
__global__ void k_gmres_column(GmresDev g, int n_inst, int j)
{
  pdl_wait();
  pdl_trigger();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_inst) return;
  if (!g.active[k])
    {
      g.inv_scale[k] = 0.0;
      return;
    }
  const int m = g.m;
  double *h = g.hcol + k * (m + 2);
  const double *h2 = g.hcol2 + k * (m + 2);
  double col[64 + 2];
  for (int i = 0; i <= j; ++i) col[i] = h[i] + h2[i];
  col[j + 1] = h[j + 1];
  double *cs = g.cs + k * m, *sn = g.sn + k * m, *gg = g.g + k * (m + 1);
  for (int i = 0; i < j; ++i)
    {
      const double t = cs[i] * col[i] + sn[i] * col[i + 1];
      col[i + 1] = -sn[i] * col[i] + cs[i] * col[i + 1];
      col[i] = t;
    }
  const double a = col[j], b = col[j + 1];
  const double r = hypot(a, b);
  double c1 = 1.0, s1 = 0.0;
  if (r > 0.0)
    {
      c1 = a / r;
      s1 = b / r;
    }
  cs[j] = c1;
  sn[j] = s1;
  col[j] = r;
  gg[j + 1] = -s1 * gg[j];
  gg[j] = c1 * gg[j];
  double *Hc = g.H + static_cast<int64_t>(k) * (m + 1) * m + static_cast<int64_t>(j) * (m + 1);
  for (int i = 0; i <= j; ++i) Hc[i] = col[i];
  const double nrm = h[j + 1];
  g.inv_scale[k] = (nrm > 0.0 && isfinite(nrm)) ? 1.0 / nrm : 0.0;
  g.its[k] = j + 1;
  const double est = fabs(gg[j + 1]);
  g.res_est[k] = est;
  if (!(est > g.tol[k]) || !(nrm > 0.0) || !isfinite(est)) g.active[k] = 0;
}

cudaError_t launch_gmres_column(const GmresDev &g, int n_inst, int j, cudaStream_t s)
{
  if (g.m > 64) return cudaErrorInvalidValue;
  pdl_launch(k_gmres_column, (n_inst + 127) / 128, 128, 0, s, g, n_inst, j);
  return cudaGetLastError();
}

// y = H(0:its,0:its)^-1 g(0:its); stored negated so that maxpy (y -= sum c_v V_v) adds V y
__global__ void k_gmres_solve_y(GmresDev g, int n_inst)
{
  pdl_wait();
  pdl_trigger();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_inst) return;
  const int m = g.m, nk = g.its[k];
  const double *H = g.H + static_cast<int64_t>(k) * (m + 1) * m;
  const double *gg = g.g + k * (m + 1);
  double *y = g.y + k * m;
  for (int i = 0; i < m; ++i) y[i] = 0.0;
  for (int i = nk - 1; i >= 0; --i)
    {
      double s = gg[i];
      for (int c = i + 1; c < nk; ++c) s -= H[c * (m + 1) + i] * y[c];
      const double d = H[i * (m + 1) + i];
      y[i] = (d != 0.0) ? s / d : 0.0;
    }
  for (int i = 0; i < nk; ++i) y[i] = -y[i];
}

cudaError_t launch_gmres_solve_y(const GmresDev &g, int n_inst, cudaStream_t s)
{
  pdl_launch(k_gmres_solve_y, (n_inst + 127) / 128, 128, 0, s, g, n_inst);
  return cudaGetLastError();
}

__global__ void k_inv(const double *__restrict__ in, double *__restrict__ out, int n)
{
  pdl_wait();
  pdl_trigger();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const double v = in[k];
  out[k] = (v > 0.0 && isfinite(v)) ? 1.0 / v : 0.0;
}

cudaError_t launch_inv(const double *in, double *out, int n, cudaStream_t s)
{
  pdl_launch(k_inv, (n + 127) / 128, 128, 0, s, in, out, n);
  return cudaGetLastError();
}

} // namespace glgpu

namespace glgpu
{
// =================================================================================
// Arnoldi step kernels with in-kernel finalization.
//
// Every CTA writes its per-segment partial sums, then takes a ticket on a per-instance
// counter (atomicAdd after __threadfence).  The CTA that draws the last ticket of its
// instance sums all partials of the instance in segment order (fixed shuffle tree, so
// results are deterministic), writes the per-instance result and resets the counter.
// Nothing waits on another CTA: the last CTA only runs after every other CTA of the
// instance has published its partials.
// =================================================================================
__device__ __forceinline__ bool take_last_ticket(unsigned int *cnt, int inst, int nseg_inst)
{
  __shared__ bool s_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0)
    {
      const unsigned int t = atomicAdd(cnt + inst, 1u);
      s_last = (t == static_cast<unsigned int>(nseg_inst - 1));
    }
  __syncthreads();
  if (s_last) __threadfence();
  return s_last;
}

// sum partial[g][v] over the instance's segments for v < nv into out[v] (one warp per v)
__device__ __forceinline__ void instance_sums(const DevMesh &m, int inst, const double *partial, int nv, double *out,
                                              int take_sqrt)
{
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g0 = m.inst_seg_off[inst], g1 = m.inst_seg_off[inst + 1];
  for (int v = warp; v < nv; v += kSegThreads / 32)
    {
      // four independent partial sums per lane keep four loads in flight; the order of the
      // additions is fixed, so the result is deterministic
      double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
      int g = g0 + lane;
      for (; g + 96 < g1; g += 128)
        {
          s0 += __ldcg(partial + static_cast<int64_t>(g) * nv + v);
          s1 += __ldcg(partial + static_cast<int64_t>(g + 32) * nv + v);
          s2 += __ldcg(partial + static_cast<int64_t>(g + 64) * nv + v);
          s3 += __ldcg(partial + static_cast<int64_t>(g + 96) * nv + v);
        }
      for (; g < g1; g += 32) s0 += __ldcg(partial + static_cast<int64_t>(g) * nv + v);
      double s = (s0 + s1) + (s2 + s3);
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
      if (lane == 0) out[v] = take_sqrt ? sqrt(s) : s;
    }
}

// h[inst][0..nvec) = V[0..nvec)^T w
template <typename T>
__global__ void __launch_bounds__(kSegThreads) k_arnoldi_dot(DevMesh m, const T *__restrict__ X, int64_t ld, int nvec,
                                                             const T *__restrict__ w, double *__restrict__ partial,
                                                             double *__restrict__ hout, int ldh,
                                                             unsigned int *__restrict__ cnt,
                                                             const uint8_t *__restrict__ act)
{
  pdl_wait();
  pdl_trigger();
  __shared__ T ys[kSegMax];
  const int s = blockIdx.x;
  const int inst = m.seg_inst[s];
  if (act && !act[inst]) return;
  const int64_t b = m.seg_begin[s];
  const int len = static_cast<int>(m.seg_end[s] - b);
  for (int i = threadIdx.x; i < len; i += kSegThreads) ys[i] = w[b + i];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int v = warp; v < nvec; v += kSegThreads / 32)
    {
      const T *xv = X + v * ld + b;
      T a0 = 0, a1 = 0, a2 = 0, a3 = 0;
      int i = lane;
      for (; i + 96 < len; i += 128)
        {
          a0 += xv[i] * ys[i];
          a1 += xv[i + 32] * ys[i + 32];
          a2 += xv[i + 64] * ys[i + 64];
          a3 += xv[i + 96] * ys[i + 96];
        }
      for (; i < len; i += 32) a0 += xv[i] * ys[i];
      double acc = static_cast<double>(a0) + static_cast<double>(a1) + static_cast<double>(a2) + static_cast<double>(a3);
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
      if (lane == 0) partial[static_cast<int64_t>(s) * nvec + v] = acc;
    }
  const int nseg = m.inst_seg_off[inst + 1] - m.inst_seg_off[inst];
  if (take_last_ticket(cnt, inst, nseg))
    {
      instance_sums(m, inst, partial, nvec, hout + inst * ldh, 0);
      if (threadIdx.x == 0) cnt[inst] = 0u;
    }
}

// Givens update of column j for one instance (same arithmetic as k_gmres_column); with
// reorth the column is the sum of both Gram-Schmidt projections
__device__ void givens_column(GmresDev &g, int k, int j, bool reorth = true)
{
  const int m = g.m;
  double *h = g.hcol + k * (m + 2);
  const double *h2 = g.hcol2 + k * (m + 2);
  double col[64 + 2];
  for (int i = 0; i <= j; ++i) col[i] = reorth ? h[i] + h2[i] : h[i];
  col[j + 1] = h[j + 1];
  double *cs = g.cs + k * m, *sn = g.sn + k * m, *gg = g.g + k * (m + 1);
  for (int i = 0; i < j; ++i)
    {
      const double t = cs[i] * col[i] + sn[i] * col[i + 1];
      col[i + 1] = -sn[i] * col[i] + cs[i] * col[i + 1];
      col[i] = t;
    }
  const double a = col[j], b = col[j + 1];
  const double r = hypot(a, b);
  double c1 = 1.0, s1 = 0.0;
  if (r > 0.0)
    {
      c1 = a / r;
      s1 = b / r;
    }
  cs[j] = c1;
  sn[j] = s1;
  col[j] = r;
  gg[j + 1] = -s1 * gg[j];
  gg[j] = c1 * gg[j];
  double *Hc = g.H + static_cast<int64_t>(k) * (m + 1) * m + static_cast<int64_t>(j) * (m + 1);
  for (int i = 0; i <= j; ++i) Hc[i] = col[i];
  const double nrm = h[j + 1];
  g.inv_scale[k] = (nrm > 0.0 && isfinite(nrm)) ? 1.0 / nrm : 0.0;
  g.its[k] = j + 1;
  const double est = fabs(gg[j + 1]);
  g.res_est[k] = est;
  if (!(est > g.tol[k]) || !(nrm > 0.0) || !isfinite(est)) g.active[k] = 0;
}

// w -= V h (h = hcol or hcol2 of the instance); then
//   mode 1: hcol2 = V^T w                     (second Gram-Schmidt projection)
//   mode 2: hcol[j+1] = |w|, then the Givens update of column j
//   mode 3: as mode 2 with h = hcol: one projection, no reorthogonalization
template <typename T>
__global__ void __launch_bounds__(kSegThreads) k_arnoldi_update(DevMesh m, const T *__restrict__ X, int64_t ld,
                                                                int nvec, T *__restrict__ w, int mode, int j,
                                                                double *__restrict__ partial, GmresDev g,
                                                                unsigned int *__restrict__ cnt)
{
  pdl_wait();
  pdl_trigger();
  __shared__ T cf[64];
  __shared__ T ys[kSegMax];
  const int s = blockIdx.x;
  const int inst = m.seg_inst[s];
  if (!g.active[inst]) return;
  const int mr = g.m;
  const double *h = (mode == 2 ? g.hcol2 : g.hcol) + inst * (mr + 2);
  for (int v = threadIdx.x; v < nvec; v += kSegThreads) cf[v] = static_cast<T>(__ldcg(h + v));
  __syncthreads();
  const int64_t b = m.seg_begin[s];
  const int len = static_cast<int>(m.seg_end[s] - b);
  // update: four elements per thread in flight, basis vectors in the outer loop
  for (int i0 = threadIdx.x; i0 < len; i0 += 4 * kSegThreads)
    {
      T acc[4];
      const T *xp = X + b;
#pragma unroll
      for (int u = 0; u < 4; ++u)
        {
          const int i = i0 + u * kSegThreads;
          acc[u] = (i < len) ? w[b + i] : T(0);
        }
      for (int v = 0; v < nvec; ++v)
        {
          const T c = cf[v];
#pragma unroll
          for (int u = 0; u < 4; ++u)
            {
              const int i = i0 + u * kSegThreads;
              if (i < len) acc[u] -= c * xp[v * ld + i];
            }
        }
#pragma unroll
      for (int u = 0; u < 4; ++u)
        {
          const int i = i0 + u * kSegThreads;
          if (i < len)
            {
              w[b + i] = acc[u];
              ys[i] = acc[u];
            }
        }
    }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nout = (mode == 1) ? nvec : 1;
  for (int v = warp; v < nout; v += kSegThreads / 32)
    {
      const T *xv = (mode == 1) ? X + v * ld + b : nullptr;
      T a0 = 0, a1 = 0;
      int i = lane;
      for (; i + 32 < len; i += 64)
        {
          a0 += (xv ? xv[i] : ys[i]) * ys[i];
          a1 += (xv ? xv[i + 32] : ys[i + 32]) * ys[i + 32];
        }
      if (i < len) a0 += (xv ? xv[i] : ys[i]) * ys[i];
      double acc = static_cast<double>(a0) + static_cast<double>(a1);
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
      if (lane == 0) partial[static_cast<int64_t>(s) * nout + v] = acc;
    }
  const int nseg = m.inst_seg_off[inst + 1] - m.inst_seg_off[inst];
  if (take_last_ticket(cnt, inst, nseg))
    {
      if (mode == 1)
        instance_sums(m, inst, partial, nvec, g.hcol2 + inst * (mr + 2), 0);
      else
        instance_sums(m, inst, partial, 1, g.hcol + inst * (mr + 2) + j + 1, 1);
      __syncthreads();
      if (threadIdx.x == 0)
        {
          cnt[inst] = 0u;
          if (mode >= 2)
            {
              __threadfence();
              givens_column(g, inst, j, mode == 2);
            }
        }
    }
}

// z = D^-1 (s v) and, when rescale is set, v <- s v, with s = scale[inst] (the
// normalisation of the previous Arnoldi vector, folded into this pass)
template <typename T>
__global__ void __launch_bounds__(kSpmvWarps * 32) k_bj_apply_scale18(DevMesh m, const T *__restrict__ dinv,
                                                                      T *__restrict__ x, T *__restrict__ y,
                                                                      const double *__restrict__ scale,
                                                                      const uint8_t *__restrict__ act)
{
  pdl_wait();
  pdl_trigger();
  using V = typename Vec16<T>::type;
  constexpr int NV = Vec16<T>::n;
  constexpr int NCH = 324 / NV;
  constexpr int NIT = (NCH + 31) / 32;
  __shared__ T red[kSpmvWarps][324];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t n = static_cast<int64_t>(blockIdx.x) * kSpmvWarps + warp;
  if (n >= m.nn) return;
  const int inst = m.node_inst[n];
  if (act && !act[inst]) return;
  const T sc = scale ? static_cast<T>(scale[inst]) : T(1);
  T xv = (lane < 18) ? x[n * 18 + lane] * sc : T(0);
  if (scale && lane < 18) x[n * 18 + lane] = xv;
  const V *bp = reinterpret_cast<const V *>(dinv + n * 324);
#pragma unroll
  for (int it = 0; it < NIT; ++it)
    {
      const int ch = lane + 32 * it;
      V wv;
      if (ch < NCH)
        wv = __ldg(bp + ch);
      else
        wv = V{};
#pragma unroll
      for (int v = 0; v < NV; ++v)
        {
          const int e = (ch < NCH) ? ch * NV + v : 0;
          const T xd = __shfl_sync(0xffffffffu, xv, e % 18);
          if (ch < NCH) red[warp][e] = vget<V, T>(wv, v) * xd;
        }
    }
  __syncwarp();
  if (lane < 18)
    {
      T s = 0;
#pragma unroll
      for (int d = 0; d < 18; ++d) s += red[warp][lane * 18 + d];
      y[n * 18 + lane] = s;
    }
}

cudaError_t launch_arnoldi_dot(const DevMesh &m, bool fp32, const void *X, int64_t ld, int nvec, const void *w,
                               double *partial, double *hout, int ldh, unsigned int *cnt, const uint8_t *act,
                               cudaStream_t s)
{
  if (fp32)
    pdl_launch(k_arnoldi_dot<float>, m.n_seg, kSegThreads, 0, s, m, static_cast<const float *>(X), ld, nvec,
                                                         static_cast<const float *>(w), partial, hout, ldh, cnt, act);
  else
    pdl_launch(k_arnoldi_dot<double>, m.n_seg, kSegThreads, 0, s, m, static_cast<const double *>(X), ld, nvec,
                                                          static_cast<const double *>(w), partial, hout, ldh, cnt, act);
  return cudaGetLastError();
}

cudaError_t launch_arnoldi_update(const DevMesh &m, bool fp32, const void *X, int64_t ld, int nvec, void *w, int mode,
                                  int j, double *partial, const GmresDev &g, unsigned int *cnt, cudaStream_t s)
{
  if (nvec > 64 || g.m > 64) return cudaErrorInvalidValue;
  if (fp32)
    pdl_launch(k_arnoldi_update<float>, m.n_seg, kSegThreads, 0, s, m, static_cast<const float *>(X), ld, nvec,
                                                            static_cast<float *>(w), mode, j, partial, g, cnt);
  else
    pdl_launch(k_arnoldi_update<double>, m.n_seg, kSegThreads, 0, s, m, static_cast<const double *>(X), ld, nvec,
                                                             static_cast<double *>(w), mode, j, partial, g, cnt);
  return cudaGetLastError();
}

cudaError_t launch_bj_apply_scale(const DevMesh &m, bool fp32, const void *dinv, void *x, void *y,
                                  const double *scale, const uint8_t *act, cudaStream_t s)
{
  if (m.B != 18) return cudaErrorInvalidValue;
  const unsigned grid = static_cast<unsigned>((m.nn + kSpmvWarps - 1) / kSpmvWarps);
  if (fp32)
    pdl_launch(k_bj_apply_scale18<float>, grid, kSpmvWarps * 32, 0, s, m, static_cast<const float *>(dinv),
                                                               static_cast<float *>(x), static_cast<float *>(y), scale,
                                                               act);
  else
    pdl_launch(k_bj_apply_scale18<double>, grid, kSpmvWarps * 32, 0, s, m, static_cast<const double *>(dinv),
                                                                static_cast<double *>(x), static_cast<double *>(y),
                                                                scale, act);
  return cudaGetLastError();
}
// ---------------------------------------------------------------------------------
// The small coarse levels of a V-cycle in one cooperative launch.  Below a few thousand
// nodes a level's sweep, residual, restriction or prolongation is a short launch whose time
// is mostly launch latency and ramp; here all CTAs stay resident and walk the levels phase
// by phase, with a grid-wide barrier between phases.  The phases compute exactly what the
// separate kernels compute (the same row map: the 8 warps of a CTA share a block row).
// ---------------------------------------------------------------------------------
constexpr int kSmallThreads = 256;
constexpr unsigned kBarrierSpins = 20u * 1000u * 1000u; // with 64 ns naps: about a second

// Grid-wide barrier (every CTA of the launch is resident: cooperative launch).  The last
// CTA to arrive resets the count and advances the generation; the others wait for the
// generation to move, at most kBarrierSpins polls, after which they record the failure in
// *err and go on (the results are then invalid and the host reports a timeout).
__device__ __forceinline__ void grid_barrier(unsigned int *bar, int *err)
{
  __syncthreads();
  if (threadIdx.x == 0)
    {
      volatile unsigned int *gen = bar + 1;
      const unsigned int g = *gen;
      __threadfence();
      if (atomicAdd(bar, 1u) == gridDim.x - 1)
        {
          atomicExch(bar, 0u);
          __threadfence();
          atomicAdd(bar + 1, 1u);
        }
      else
        {
          unsigned int spins = 0;
          while (*gen == g)
            {
              if (++spins > kBarrierSpins)
                {
                  atomicExch(err, 1);
                  break;
                }
              __nanosleep(64);
            }
        }
      __threadfence();
    }
  __syncthreads();
}

// y = zin + omega D^-1 (r - A zin) (zin == nullptr: y = omega D^-1 r), or, with RES, the
// residual y = r - A zin; one block row per CTA iteration, its blocks split over 8 warps
template <typename T, bool RES>
__device__ void small_rows(const SmallLevel<T> &L, const T *zin, T *y, T omega, const uint8_t *act,
                           T (*red)[324])
{
  using V = typename Vec16<T>::type;
  constexpr int NV = Vec16<T>::n;
  constexpr int NCH = 324 / NV;
  constexpr int NIT = (NCH + 31) / 32;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int64_t n = blockIdx.x; n < L.m.nn; n += gridDim.x)
    {
      const bool on = !(act && !act[L.m.node_inst[n]]); // uniform over the CTA
      if (!on) continue;
      T t = (lane < 18) ? L.r[n * 18 + lane] : T(0);
      if (zin)
        {
          T acc[NIT][NV];
          row_products<T, T, kSpmvWarps>(L.m, L.vals, zin, n, lane, warp, acc);
          store_products<T, T>(red[warp], acc, lane);
          __syncthreads();
          if (warp == 0 && lane < 18) t -= row_sum<T, kSpmvWarps>(red, 0, lane);
          __syncthreads();
        }
      if (RES)
        {
          if (warp == 0 && lane < 18) y[n * 18 + lane] = t;
          continue;
        }
      if (warp == 0)
        {
          T acc[NIT][NV];
          const V *bp = reinterpret_cast<const V *>(L.dinv + n * 324);
#pragma unroll
          for (int it = 0; it < NIT; ++it)
            {
              const int ch = lane + 32 * it;
              const V w = (ch < NCH) ? __ldg(bp + ch) : V{};
#pragma unroll
              for (int v = 0; v < NV; ++v)
                {
                  const int e = (ch < NCH) ? ch * NV + v : 0;
                  acc[it][v] = vget<V, T>(w, v) * __shfl_sync(0xffffffffu, t, e % 18);
                }
            }
          store_products<T>(red[0], acc, lane);
          __syncwarp();
          if (lane < 18) y[n * 18 + lane] = (zin ? zin[n * 18 + lane] : T(0)) + omega * row_sum<T, 1>(red, 0, lane);
        }
      __syncthreads(); // red is reused by the next row
    }
}

// rc = P^T rf on the coarse level C (zero on its zero-Dirichlet components); with `smooth`
// also C.z = omega D_c^-1 rc, the coarse level's first sweep from zero.  Warp per coarse node.
template <typename T>
__device__ void small_restrict(const SmallLevel<T> &F, const SmallLevel<T> &C, bool smooth, T omega,
                               const uint8_t *act)
{
  const int lane = threadIdx.x & 31;
  const int64_t gw = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  for (int64_t n = gw; n < C.m.nn; n += nw)
    {
      if (act && !act[C.m.node_inst[n]]) continue;
      T s = T(0);
      if (lane < 18 && !((C.m.mask[n] >> lane) & 1u))
        for (int k = F.r_ptr[n]; k < F.r_ptr[n + 1]; ++k) s += F.r_w[k] * F.t[static_cast<int64_t>(F.r_idx[k]) * 18 + lane];
      if (lane < 18) C.r[n * 18 + lane] = s;
      if (smooth)
        {
          const T *row = C.dinv + n * 324 + (lane < 18 ? lane : 0) * 18;
          T u = T(0);
#pragma unroll
          for (int d = 0; d < 18; ++d) u += row[d] * __shfl_sync(0xffffffffu, s, d);
          if (lane < 18) C.z[n * 18 + lane] = omega * u;
        }
    }
}

// out = base + P zc on level F (constrained components keep base); thread per (node, component)
template <typename T>
__device__ void small_prolong(const SmallLevel<T> &F, const T *zc, const T *base, T *out, const uint8_t *act)
{
  const int64_t total = F.m.nn * 18;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    {
      const int64_t n = i / 18;
      const int c = static_cast<int>(i - n * 18);
      if (act && !act[F.m.node_inst[n]]) continue;
      const T b0 = base[i];
      if (F.m.hptr[n + 1] > F.m.hptr[n] || ((F.m.mask[n] >> c) & 1u))
        {
          out[i] = b0;
          continue;
        }
      T s = T(0);
      for (int k = F.p_ptr[n]; k < F.p_ptr[n + 1]; ++k) s += F.p_w[k] * zc[static_cast<int64_t>(F.p_idx[k]) * 18 + c];
      out[i] = b0 + s;
    }
}

template <typename T>
__global__ void __launch_bounds__(kSmallThreads) k_vcycle_small(const SmallLevel<T> *__restrict__ lev, SmallCycle<T> cy,
                                                                const uint8_t *__restrict__ act)
{
  pdl_wait();
  __shared__ T red[kSpmvWarps][324];
  constexpr int kMaxSmall = 16;
  T *curs[kMaxSmall];
  // descent: every level entered with r and its first sweep from the restriction
  for (int i = 0; i < cy.n_small; ++i)
    {
      const SmallLevel<T> &L = lev[i];
      T *cur = L.z, *oth = L.t2;
      for (int sw = 1; sw < cy.pre; ++sw)
        {
          small_rows<T, false>(L, cur, oth, cy.omega, act, red);
          grid_barrier(cy.bar, cy.err);
          T *tmp = cur;
          cur = oth;
          oth = tmp;
        }
      small_rows<T, true>(L, cur, L.t, cy.omega, act, red);
      grid_barrier(cy.bar, cy.err);
      small_restrict<T>(L, lev[i + 1], i + 1 < cy.n_small, cy.omega, act);
      grid_barrier(cy.bar, cy.err);
      curs[i] = cur;
    }
  // coarsest level: z = inverse r per instance, warp per row
  {
    const SmallLevel<T> &D = lev[cy.n_small];
    const int lane = threadIdx.x & 31;
    const int64_t gw = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    const int64_t units = static_cast<int64_t>(D.m.n_inst) * cy.max_nd;
    for (int64_t u = gw; u < units; u += nw)
      {
        const int inst = static_cast<int>(u / cy.max_nd), row = static_cast<int>(u - inst * static_cast<int64_t>(cy.max_nd));
        if (act && !act[inst]) continue;
        const int64_t n0 = D.m.node_off_ptr[inst], n1 = D.m.node_off_ptr[inst + 1];
        const int nd = static_cast<int>((n1 - n0) * 18);
        if (row >= nd) continue;
        const float *A = cy.inv + cy.dense_off[inst] + static_cast<int64_t>(row) * nd;
        const T *rv = D.r + n0 * 18;
        float s = 0.f;
        for (int j = lane; j < nd; j += 32) s += A[j] * static_cast<float>(rv[j]);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        if (lane == 0) D.z[n0 * 18 + row] = static_cast<T>(s);
      }
    grid_barrier(cy.bar, cy.err);
  }
  // ascent: prolongation into the other buffer, post-sweeps, result in z
  for (int i = cy.n_small - 1; i >= 0; --i)
    {
      const SmallLevel<T> &L = lev[i];
      T *cur = curs[i];
      T *oth = (cur == L.z) ? L.t2 : L.z;
      small_prolong<T>(L, lev[i + 1].z, cur, oth, act);
      grid_barrier(cy.bar, cy.err);
      T *tmp = cur;
      cur = oth;
      oth = tmp;
      for (int sw = 0; sw < cy.post; ++sw)
        {
          small_rows<T, false>(L, cur, oth, cy.omega, act, red);
          grid_barrier(cy.bar, cy.err);
          tmp = cur;
          cur = oth;
          oth = tmp;
        }
      if (cur != L.z)
        {
          const int64_t total = L.m.nn * 18;
          for (int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; k < total;
               k += static_cast<int64_t>(gridDim.x) * blockDim.x)
            if (!(act && !act[L.m.node_inst[k / 18]])) L.z[k] = cur[k];
          grid_barrier(cy.bar, cy.err);
        }
    }
}

int vcycle_small_blocks_per_sm(bool fp32)
{
  int nb = 0;
  const cudaError_t e =
    fp32 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_vcycle_small<float>, kSmallThreads, 0)
         : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_vcycle_small<double>, kSmallThreads, 0);
  if (e != cudaSuccess) return 0;
  return nb < 4 ? nb : 4;
}

cudaError_t launch_vcycle_small(bool fp32, const void *levels, const void *cycle, int grid, const uint8_t *act,
                                cudaStream_t s)
{
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(static_cast<unsigned>(grid));
  cfg.blockDim = dim3(kSmallThreads);
  cfg.stream = s;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  if (fp32)
    return cudaLaunchKernelEx(&cfg, k_vcycle_small<float>, static_cast<const SmallLevel<float> *>(levels),
                              *static_cast<const SmallCycle<float> *>(cycle), act);
  return cudaLaunchKernelEx(&cfg, k_vcycle_small<double>, static_cast<const SmallLevel<double> *>(levels),
                            *static_cast<const SmallCycle<double> *>(cycle), act);
}

// ---------------------------------------------------------------------------------
// The V-cycle's tail (the smallest levels and the dense solve) as one launch of one
// thread-block cluster per instance.  Each of those levels is a few hundred nodes at most,
// so a separate launch per sweep, residual and transfer is almost all latency; here the
// cluster's CTAs split each phase's rows and wait for each other at the cluster barrier
// (barrier.cluster, release / acquire: a hardware barrier over co-scheduled CTAs, no
// polling).  Vectors written in one phase and read in the next by other CTAs are read
// from L2 (ld.global.cg).  The phases compute what the separate kernels compute, row for
// row: the same lane maps, the same summation orders.
// ---------------------------------------------------------------------------------
constexpr int kTailThreads = 512;
constexpr int kTailWarps = kTailThreads / 32;
constexpr int kTailWpr = 2;                      // warps per block row
constexpr int kTailRows = kTailWarps / kTailWpr; // block rows per CTA and pass
constexpr int kTailNodes = kTailThreads / 18;    // nodes per CTA and pass, thread per component
constexpr int kMaxTail = 8;                      // smoothing levels in a tail

template <typename T> constexpr size_t tail_smem_bytes() { return sizeof(T) * (kTailWarps * 324 + kTailNodes * 18); }

__device__ __forceinline__ unsigned tail_rank()
{
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ unsigned tail_csize()
{
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
  return r;
}
// all threads of the cluster: the writes before are visible to the reads after
__device__ __forceinline__ void tail_sync()
{
  asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}

// rows [n0, n1) of level L: RES: y = r - A zin; otherwise y = zin + omega D^-1 (r - A zin)
// (zin == nullptr: y = omega D^-1 r).  The loop is uniform over the CTA (it depends on the
// rank only), so the CTA barriers inside are reached by every thread.
template <typename T, bool RES>
__device__ void tail_rows(const SmallLevel<T> &L, int64_t n0, int64_t n1, const T *zin, T *y, T omega, unsigned rank,
                          unsigned cs, T (*red)[324])
{
  using V = typename Vec16<T>::type;
  constexpr int NV = Vec16<T>::n;
  constexpr int NCH = 324 / NV;
  constexpr int NIT = (NCH + 31) / 32;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int kw = warp % kTailWpr, w0 = warp - kw;
  for (int64_t base = n0 + static_cast<int64_t>(rank) * kTailRows; base < n1;
       base += static_cast<int64_t>(cs) * kTailRows)
    {
      const int64_t n = base + warp / kTailWpr;
      const bool on = n < n1; // uniform over the warp
      T t = (on && lane < 18) ? __ldcg(L.r + n * 18 + lane) : T(0);
      if (zin)
        {
          T acc[NIT][NV];
          if (on)
            row_products<T, T, kTailWpr, true>(L.m, L.vals, zin, n, lane, kw, acc);
          else
#pragma unroll
            for (int it = 0; it < NIT; ++it)
#pragma unroll
              for (int v = 0; v < NV; ++v) acc[it][v] = T(0);
          store_products<T, T>(red[warp], acc, lane);
          __syncthreads();
          if (on && lane < 18) t -= row_sum<T, kTailWpr>(red, w0, lane);
          __syncthreads();
        }
      if (RES)
        {
          if (on && kw == 0 && lane < 18) y[n * 18 + lane] = t;
          continue;
        }
      if (on && kw == 0)
        {
          T acc[NIT][NV];
          const V *bp = reinterpret_cast<const V *>(L.dinv + n * 324);
#pragma unroll
          for (int it = 0; it < NIT; ++it)
            {
              const int ch = lane + 32 * it;
              const V w = (ch < NCH) ? __ldg(bp + ch) : V{};
#pragma unroll
              for (int v = 0; v < NV; ++v)
                {
                  const int e = (ch < NCH) ? ch * NV + v : 0;
                  acc[it][v] = vget<V, T>(w, v) * __shfl_sync(0xffffffffu, t, e % 18);
                }
            }
          store_products<T>(red[warp], acc, lane);
          __syncwarp();
          if (lane < 18)
            y[n * 18 + lane] = (zin ? __ldcg(zin + n * 18 + lane) : T(0)) + omega * row_sum<T, 1>(red, warp, lane);
        }
      __syncthreads(); // red is reused by the next pass
    }
}

// rc = P^T rf on the coarse rows [c0, c1) of C (zero on zero-Dirichlet components); with
// SMOOTH also C.z = omega D^-1 rc, the coarse level's first sweep from zero
template <typename T, bool SMOOTH>
__device__ void tail_restrict(const SmallLevel<T> &F, const T *rf, const SmallLevel<T> &C, int64_t c0, int64_t c1,
                              T omega, unsigned rank, unsigned cs, T (*ts)[18])
{
  const int ln = threadIdx.x / 18, c = threadIdx.x - 18 * (threadIdx.x / 18);
  for (int64_t base = c0 + static_cast<int64_t>(rank) * kTailNodes; base < c1;
       base += static_cast<int64_t>(cs) * kTailNodes)
    {
      const int64_t n = base + ln;
      const bool on = ln < kTailNodes && n < c1;
      T s = T(0);
      if (on && !((C.m.mask[n] >> c) & 1u))
        for (int k = F.r_ptr[n]; k < F.r_ptr[n + 1]; ++k)
          s += F.r_w[k] * __ldcg(rf + static_cast<int64_t>(F.r_idx[k]) * 18 + c);
      if (on) C.r[n * 18 + c] = s;
      if (SMOOTH)
        {
          if (ln < kTailNodes) ts[ln][c] = s;
          __syncthreads();
          if (on)
            {
              const T *row = C.dinv + n * 324 + c * 18;
              T u = T(0);
#pragma unroll
              for (int d = 0; d < 18; ++d) u += __ldg(row + d) * ts[ln][d];
              C.z[n * 18 + c] = omega * u;
            }
          __syncthreads();
        }
    }
}

// out = base + P zc on the rows [f0, f1) of F (hanging nodes and constrained components keep base)
template <typename T>
__device__ void tail_prolong(const SmallLevel<T> &F, int64_t f0, int64_t f1, const T *zc, const T *base, T *out,
                             unsigned rank, unsigned cs)
{
  const int64_t total = (f1 - f0) * 18;
  for (int64_t i = static_cast<int64_t>(rank) * kTailThreads + threadIdx.x; i < total;
       i += static_cast<int64_t>(cs) * kTailThreads)
    {
      const int64_t g = f0 * 18 + i;
      const int64_t n = g / 18;
      const int c = static_cast<int>(g - n * 18);
      const T b0 = __ldcg(base + g);
      if (F.m.hptr[n + 1] > F.m.hptr[n] || ((F.m.mask[n] >> c) & 1u))
        {
          out[g] = b0;
          continue;
        }
      T s = T(0);
      for (int k = F.p_ptr[n]; k < F.p_ptr[n + 1]; ++k)
        s += F.p_w[k] * __ldcg(zc + static_cast<int64_t>(F.p_idx[k]) * 18 + c);
      out[g] = b0 + s;
    }
}

template <typename T>
__global__ void __launch_bounds__(kTailThreads, 1)
  k_vcycle_tail(const SmallLevel<T> *__restrict__ lev, TailCycle<T> cy, const T *__restrict__ p_res,
                const T *__restrict__ p_cur, T *__restrict__ p_out, const uint8_t *__restrict__ act)
{
  pdl_wait();
  pdl_trigger();
  extern __shared__ __align__(16) unsigned char tail_smem[];
  T(*red)[324] = reinterpret_cast<T(*)[324]>(tail_smem);
  T(*ts)[18] = reinterpret_cast<T(*)[18]>(tail_smem + sizeof(T) * kTailWarps * 324);
  const unsigned rank = tail_rank(), cs = tail_csize();
  const int inst = static_cast<int>(blockIdx.x / cs);
  if (act && !act[inst]) return; // the whole cluster: the flag is per instance
  const int nt = cy.n_tail;
  const T om = cy.omega;
  T *curs[kMaxTail + 1];
  // descent: level 1's right-hand side and first sweep from the parent's residual
  tail_restrict<T, true>(lev[0], p_res, lev[1], lev[1].m.node_off_ptr[inst], lev[1].m.node_off_ptr[inst + 1], om, rank,
                         cs, ts);
  tail_sync();
  for (int i = 1; i <= nt; ++i)
    {
      const SmallLevel<T> &L = lev[i];
      const int64_t a = L.m.node_off_ptr[inst], b = L.m.node_off_ptr[inst + 1];
      T *cur = L.z, *oth = L.t2;
      for (int sw = 1; sw < cy.pre; ++sw)
        {
          tail_rows<T, false>(L, a, b, cur, oth, om, rank, cs, red);
          tail_sync();
          T *tmp = cur;
          cur = oth;
          oth = tmp;
        }
      tail_rows<T, true>(L, a, b, cur, L.t, om, rank, cs, red);
      tail_sync();
      const SmallLevel<T> &C = lev[i + 1];
      const int64_t ca = C.m.node_off_ptr[inst], cb = C.m.node_off_ptr[inst + 1];
      if (i < nt)
        tail_restrict<T, true>(L, L.t, C, ca, cb, om, rank, cs, ts);
      else
        tail_restrict<T, false>(L, L.t, C, ca, cb, om, rank, cs, ts);
      tail_sync();
      curs[i] = cur;
    }
  // the dense coarsest level: z = inverse r, warp per row (FP32 inverse and accumulation)
  {
    const SmallLevel<T> &D = lev[nt + 1];
    const int64_t d0 = D.m.node_off_ptr[inst], d1 = D.m.node_off_ptr[inst + 1];
    const int nd = static_cast<int>((d1 - d0) * 18);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const float *Ai = cy.inv + cy.dense_off[inst];
    const T *rv = D.r + d0 * 18;
    for (int row = static_cast<int>(rank) * kTailWarps + warp; row < nd; row += static_cast<int>(cs) * kTailWarps)
      {
        const float *A = Ai + static_cast<int64_t>(row) * nd;
        float s = 0.f;
        for (int j = lane; j < nd; j += 32) s += __ldg(A + j) * static_cast<float>(__ldcg(rv + j));
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        if (lane == 0) D.z[d0 * 18 + row] = static_cast<T>(s);
      }
  }
  tail_sync();
  // ascent: prolongation into the other buffer, post-sweeps
  const T *zc = lev[nt + 1].z;
  for (int i = nt; i >= 1; --i)
    {
      const SmallLevel<T> &L = lev[i];
      const int64_t a = L.m.node_off_ptr[inst], b = L.m.node_off_ptr[inst + 1];
      T *cur = curs[i];
      T *oth = (cur == L.z) ? L.t2 : L.z;
      tail_prolong<T>(L, a, b, zc, cur, oth, rank, cs);
      tail_sync();
      T *tmp = cur;
      cur = oth;
      oth = tmp;
      for (int sw = 0; sw < cy.post; ++sw)
        {
          tail_rows<T, false>(L, a, b, cur, oth, om, rank, cs, red);
          tail_sync();
          tmp = cur;
          cur = oth;
          oth = tmp;
        }
      zc = cur;
    }
  // the parent's coarse correction (read by the next launch)
  tail_prolong<T>(lev[0], lev[0].m.node_off_ptr[inst], lev[0].m.node_off_ptr[inst + 1], zc, p_cur, p_out, rank, cs);
}

template <typename T> static cudaError_t tail_attributes(int cs)
{
  cudaError_t e = cudaFuncSetAttribute(k_vcycle_tail<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(tail_smem_bytes<T>()));
  if (e == cudaSuccess && cs > 8) e = cudaFuncSetAttribute(k_vcycle_tail<T>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  return e;
}

template <typename T> static int tail_cluster_t(int n_inst)
{
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    {
      cudaGetLastError();
      return 0;
    }
  // at least 4 CTAs per instance (fewer leave each phase's rows to too few SMs), and all
  // clusters co-resident in about two waves
  for (int cs = 16; cs >= 4; cs /= 2)
    {
      if (static_cast<int64_t>(n_inst) * cs > 2 * static_cast<int64_t>(sms)) continue;
      if (tail_attributes<T>(cs) != cudaSuccess)
        {
          cudaGetLastError();
          continue;
        }
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = static_cast<unsigned>(cs);
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(static_cast<unsigned>(cs * n_inst));
      cfg.blockDim = dim3(kTailThreads);
      cfg.dynamicSmemBytes = tail_smem_bytes<T>();
      cfg.attrs = at;
      cfg.numAttrs = 1;
      int nc = 0;
      if (cudaOccupancyMaxActiveClusters(&nc, k_vcycle_tail<T>, &cfg) == cudaSuccess && nc > 0) return cs;
      cudaGetLastError();
    }
  return 0;
}

int vcycle_tail_cluster(bool fp32, int n_inst) { return fp32 ? tail_cluster_t<float>(n_inst) : tail_cluster_t<double>(n_inst); }

cudaError_t launch_vcycle_tail(bool fp32, const void *levels, const void *cycle, int n_inst, int cluster,
                               const void *p_res, const void *p_cur, void *p_out, const uint8_t *act, cudaStream_t s)
{
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = static_cast<unsigned>(cluster);
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(static_cast<unsigned>(cluster * n_inst));
  cfg.blockDim = dim3(kTailThreads);
  cfg.stream = s;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  if (fp32)
    {
      cfg.dynamicSmemBytes = tail_smem_bytes<float>();
      return cudaLaunchKernelEx(&cfg, k_vcycle_tail<float>, static_cast<const SmallLevel<float> *>(levels),
                                *static_cast<const TailCycle<float> *>(cycle), static_cast<const float *>(p_res),
                                static_cast<const float *>(p_cur), static_cast<float *>(p_out), act);
    }
  cfg.dynamicSmemBytes = tail_smem_bytes<double>();
  return cudaLaunchKernelEx(&cfg, k_vcycle_tail<double>, static_cast<const SmallLevel<double> *>(levels),
                            *static_cast<const TailCycle<double> *>(cycle), static_cast<const double *>(p_res),
                            static_cast<const double *>(p_cur), static_cast<double *>(p_out), act);
}

} // namespace glgpu
