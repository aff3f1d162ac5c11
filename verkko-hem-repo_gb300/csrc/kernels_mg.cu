// Multigrid kernels (sm_103a): inter-level transfers and the coarsest-level dense solve.
//
// Transfers are node-level CSR gathers applied to all B components of a node:
//   prolongation   z_fine[n][c]  += sum_j w_j z_coarse[idx_j][c]   (trilinear, P)
//   restriction    r_coarse[i][c] = sum_j w_j r_fine[idx_j][c]     (P^T, transposed CSR)
// Constrained components (zero-Dirichlet, hanging) are left alone on the way up and
// zeroed on the way down, so every Krylov vector keeps zeros there.
// Coarse Jacobians are Galerkin products P^T J P, one CTA per coarse block row.  The
// coarsest level (1 cell per axis, 8 nodes, 144 unknowns per instance) is inverted
// densely once per Newton step: one CTA per instance, Gauss-Jordan in shared memory.
#include <cstdint>
#include <cuda_runtime.h>

#include "device.h"

namespace glgpu
{
template <typename T>
__global__ void k_prolong_add(int64_t nn_f, int B, const int32_t *__restrict__ ptr, const int32_t *__restrict__ idx,
                              const T *__restrict__ w, const T *__restrict__ zc, T *__restrict__ zf,
                              const uint32_t *__restrict__ mask_f, const int32_t *__restrict__ hptr_f,
                              const int32_t *__restrict__ node_inst, const uint8_t *__restrict__ act)
{
  const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= nn_f * B) return;
  const int64_t n = t / B;
  const int c = static_cast<int>(t % B);
  if (act && !act[node_inst[n]]) return;
  if (hptr_f[n + 1] > hptr_f[n] || ((mask_f[n] >> c) & 1u)) return;
  T s = 0;
  for (int k = ptr[n]; k < ptr[n + 1]; ++k) s += w[k] * zc[static_cast<int64_t>(idx[k]) * B + c];
  zf[t] += s;
}

template <typename T>
__global__ void k_restrict(int64_t nn_c, int B, const int32_t *__restrict__ ptr, const int32_t *__restrict__ idx,
                           const T *__restrict__ w, const T *__restrict__ rf, T *__restrict__ rc,
                           const uint32_t *__restrict__ mask_c, const int32_t *__restrict__ node_inst,
                           const uint8_t *__restrict__ act)
{
  const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= nn_c * B) return;
  const int64_t n = t / B;
  const int c = static_cast<int>(t % B);
  if (act && !act[node_inst[n]]) return;
  T s = 0;
  if (!((mask_c[n] >> c) & 1u))
    for (int k = ptr[n]; k < ptr[n + 1]; ++k) s += w[k] * rf[static_cast<int64_t>(idx[k]) * B + c];
  rc[t] = s;
}

constexpr int kBlk = 324;         // 18 x 18 block
constexpr int kGalThreads = 352; // 11 warps: thread e owns entry e of every block

template <typename T>
__global__ void __launch_bounds__(kGalThreads)
  k_galerkin(const int32_t *__restrict__ rowptr_c, const int32_t *__restrict__ cols_c,
             const uint32_t *__restrict__ mask_c, T *__restrict__ vals_c, const int32_t *__restrict__ r_ptr,
             const int32_t *__restrict__ r_idx, const T *__restrict__ r_w, const int32_t *__restrict__ rowptr_f,
             const int32_t *__restrict__ cols_f, const T *__restrict__ vals_f, const int32_t *__restrict__ p_ptr,
             const T *__restrict__ p_w, const int64_t *__restrict__ g_ptr, const uint8_t *__restrict__ g_slot,
             const int32_t *__restrict__ node_inst_c, const uint8_t *__restrict__ act)
{
  extern __shared__ __align__(16) unsigned char g_smem[];
  T *acc = reinterpret_cast<T *>(g_smem); // [row blocks][324]
  const int64_t I = blockIdx.x;
  if (act && !act[node_inst_c[I]]) return;
  const int e = threadIdx.x;
  const int32_t b0 = rowptr_c[I];
  const int ns = rowptr_c[I + 1] - b0;
  for (int t = e; t < ns * kBlk; t += kGalThreads) acc[t] = T(0);
  __syncthreads();
  if (e < kBlk)
    {
      const uint8_t *slot = g_slot + g_ptr[I];
      int t = 0;
      for (int32_t k = r_ptr[I]; k < r_ptr[I + 1]; ++k)
        {
          const int32_t i = r_idx[k];
          const T wi = r_w[k];
          for (int32_t b = rowptr_f[i]; b < rowptr_f[i + 1]; ++b)
            {
              const int32_t j = cols_f[b];
              const T v = wi * vals_f[static_cast<int64_t>(b) * kBlk + e];
              for (int32_t q = p_ptr[j]; q < p_ptr[j + 1]; ++q, ++t) acc[slot[t] * kBlk + e] += p_w[q] * v;
            }
        }
    }
  __syncthreads();
  const uint32_t mI = mask_c[I];
  for (int t = e; t < ns * kBlk; t += kGalThreads)
    {
      const int s = t / kBlk, el = t - s * kBlk, a = el / 18, bb = el - a * 18;
      const int32_t J = cols_c[b0 + s];
      T v = acc[t];
      if (((mI >> a) & 1u) || ((mask_c[J] >> bb) & 1u)) v = (J == I && a == bb) ? T(1) : T(0);
      vals_c[static_cast<int64_t>(b0 + s) * kBlk + el] = v;
    }
}

template <typename T>
cudaError_t launch_prolong_add(int64_t nn_f, int B, const int32_t *ptr, const int32_t *idx, const void *w,
                               const void *zc, void *zf, const uint32_t *mask_f, const int32_t *hptr_f,
                               const int32_t *node_inst, const uint8_t *act, cudaStream_t s)
{
  const int64_t n = nn_f * B;
  k_prolong_add<T><<<static_cast<unsigned>((n + 255) / 256), 256, 0, s>>>(
    nn_f, B, ptr, idx, static_cast<const T *>(w), static_cast<const T *>(zc), static_cast<T *>(zf), mask_f, hptr_f,
    node_inst, act);
  return cudaGetLastError();
}

cudaError_t launch_prolong(bool fp32, int64_t nn_f, int B, const int32_t *ptr, const int32_t *idx, const void *w,
                           const void *zc, void *zf, const uint32_t *mask_f, const int32_t *hptr_f,
                           const int32_t *node_inst, const uint8_t *act, cudaStream_t s)
{
  return fp32 ? launch_prolong_add<float>(nn_f, B, ptr, idx, w, zc, zf, mask_f, hptr_f, node_inst, act, s)
              : launch_prolong_add<double>(nn_f, B, ptr, idx, w, zc, zf, mask_f, hptr_f, node_inst, act, s);
}

cudaError_t launch_restrict(bool fp32, int64_t nn_c, int B, const int32_t *ptr, const int32_t *idx, const void *w,
                            const void *rf, void *rc, const uint32_t *mask_c, const int32_t *node_inst,
                            const uint8_t *act, cudaStream_t s)
{
  const int64_t n = nn_c * B;
  const unsigned g = static_cast<unsigned>((n + 255) / 256);
  if (fp32)
    k_restrict<float><<<g, 256, 0, s>>>(nn_c, B, ptr, idx, static_cast<const float *>(w),
                                        static_cast<const float *>(rf), static_cast<float *>(rc), mask_c, node_inst, act);
  else
    k_restrict<double><<<g, 256, 0, s>>>(nn_c, B, ptr, idx, static_cast<const double *>(w),
                                         static_cast<const double *>(rf), static_cast<double *>(rc), mask_c, node_inst,
                                         act);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_galerkin_t(int64_t nn_c, const int32_t *rowptr_c, const int32_t *cols_c, const uint32_t *mask_c,
                              void *vals_c, const int32_t *r_ptr, const int32_t *r_idx, const void *r_w,
                              const int32_t *rowptr_f, const int32_t *cols_f, const void *vals_f, const int32_t *p_ptr,
                              const void *p_w, const int64_t *g_ptr, const uint8_t *g_slot, int max_row_blocks_c,
                              const int32_t *node_inst_c, const uint8_t *act, cudaStream_t s)
{
  const size_t sm = static_cast<size_t>(max_row_blocks_c) * kBlk * sizeof(T);
  if (sm > 200 * 1024 || nn_c > 0x7fffffff) return cudaErrorInvalidValue;
  if (nn_c == 0) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(k_galerkin<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sm));
  if (e != cudaSuccess) return e;
  k_galerkin<T><<<static_cast<unsigned>(nn_c), kGalThreads, sm, s>>>(
    rowptr_c, cols_c, mask_c, static_cast<T *>(vals_c), r_ptr, r_idx, static_cast<const T *>(r_w), rowptr_f, cols_f,
    static_cast<const T *>(vals_f), p_ptr, static_cast<const T *>(p_w), g_ptr, g_slot, node_inst_c, act);
  return cudaGetLastError();
}

cudaError_t launch_galerkin(bool fp32, int64_t nn_c, const int32_t *rowptr_c, const int32_t *cols_c,
                            const uint32_t *mask_c, void *vals_c, const int32_t *r_ptr, const int32_t *r_idx,
                            const void *r_w, const int32_t *rowptr_f, const int32_t *cols_f, const void *vals_f,
                            const int32_t *p_ptr, const void *p_w, const int64_t *g_ptr, const uint8_t *g_slot,
                            int max_row_blocks_c, const int32_t *node_inst_c, const uint8_t *act, cudaStream_t s)
{
  return fp32 ? launch_galerkin_t<float>(nn_c, rowptr_c, cols_c, mask_c, vals_c, r_ptr, r_idx, r_w, rowptr_f, cols_f,
                                         vals_f, p_ptr, p_w, g_ptr, g_slot, max_row_blocks_c, node_inst_c, act, s)
              : launch_galerkin_t<double>(nn_c, rowptr_c, cols_c, mask_c, vals_c, r_ptr, r_idx, r_w, rowptr_f, cols_f,
                                          vals_f, p_ptr, p_w, g_ptr, g_slot, max_row_blocks_c, node_inst_c, act, s);
}

// ---------------------------------------------------------------------------------
// coarsest level (one cell per axis: 8 nodes, 144 unknowns per instance): dense inverse
// of the slightly shifted matrix in shared memory, FP32, one CTA per instance.  It is a preconditioner component, so
// FP32 suffices in both precision modes (the outer flexible GMRES is exact).
// ---------------------------------------------------------------------------------
constexpr int kGjThreads = 512;
constexpr float kCoarseShift = 1e-4f; // relative diagonal shift of the coarsest solve

template <typename T>
__global__ void __launch_bounds__(kGjThreads) k_dense_invert(DevMesh m, const T *__restrict__ vals,
                                                             const int64_t *__restrict__ dense_off,
                                                             float *__restrict__ inv, int *__restrict__ singular)
{
  extern __shared__ float W[]; // [nd][2 nd]
  __shared__ float s_val[kGjThreads / 32];
  __shared__ int s_idx[kGjThreads / 32];
  __shared__ int s_piv;
  __shared__ int s_sing;
  __shared__ float s_shift;
  const int inst = blockIdx.x;
  const int64_t n0 = m.node_off_ptr[inst], n1 = m.node_off_ptr[inst + 1];
  const int B = m.B;
  const int nd = static_cast<int>((n1 - n0) * B);
  const int ld = 2 * nd;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int e = tid; e < nd * ld; e += kGjThreads)
    {
      const int r = e / ld, c = e % ld;
      W[e] = (c >= nd && c - nd == r) ? 1.f : 0.f;
    }
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
      W[row * ld + col] = static_cast<float>(vals[blk * B * B + e]);
    }
  if (tid == 0)
    {
      s_sing = 0;
      float sd = 0.f;
      for (int i = 0; i < nd; ++i) sd += fabsf(W[i * ld + i]);
      s_shift = nd > 0 ? kCoarseShift * sd / static_cast<float>(nd) : 0.f;
    }
  __syncthreads();
  // near-null modes (global phase and spin rotations near a solution) would be amplified
  // without bound by an exact inverse: invert A + shift * mean|diag| * I instead
  for (int i = tid; i < nd; i += kGjThreads) W[i * ld + i] += s_shift;
  __syncthreads();
  for (int k = 0; k < nd; ++k)
    {
      float best = -1.f;
      int bi = k;
      for (int i = k + tid; i < nd; i += kGjThreads)
        {
          const float v = fabsf(W[i * ld + k]);
          if (v > best)
            {
              best = v;
              bi = i;
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
      if (lane == 0)
        {
          s_val[warp] = best;
          s_idx[warp] = bi;
        }
      __syncthreads();
      if (tid == 0)
        {
          float bv = -1.f;
          int bidx = k;
          for (int w = 0; w < kGjThreads / 32; ++w)
            if (s_val[w] > bv || (s_val[w] == bv && s_idx[w] < bidx))
              {
                bv = s_val[w];
                bidx = s_idx[w];
              }
          s_piv = bidx;
          if (!(bv > 1e-30f)) s_sing = 1;
        }
      __syncthreads();
      if (s_sing) break;
      const int p = s_piv;
      if (p != k)
        for (int c = tid; c < ld; c += kGjThreads)
          {
            const float t = W[k * ld + c];
            W[k * ld + c] = W[p * ld + c];
            W[p * ld + c] = t;
          }
      __syncthreads();
      const float pinv = 1.f / W[k * ld + k];
      __syncthreads();
      for (int c = tid; c < ld; c += kGjThreads) W[k * ld + c] *= pinv;
      __syncthreads();
      for (int e = tid; e < nd * ld; e += kGjThreads)
        {
          const int i = e / ld, c = e - i * ld;
          if (i == k || c == k) continue;
          const float f = W[i * ld + k];
          if (f != 0.f) W[e] -= f * W[k * ld + c];
        }
      __syncthreads();
      for (int i = tid; i < nd; i += kGjThreads)
        if (i != k) W[i * ld + k] = 0.f;
      __syncthreads();
    }
  float *out = inv + dense_off[inst];
  for (int e = tid; e < nd * nd; e += kGjThreads)
    {
      const int i = e / nd, c = e % nd;
      out[e] = s_sing ? (i == c ? 1.f : 0.f) : W[i * ld + nd + c];
    }
  if (tid == 0 && s_sing) singular[inst] = 1;
}

// z = inv r per instance: one warp per row
template <typename T>
__global__ void k_dense_apply(DevMesh m, const int64_t *__restrict__ dense_off, const float *__restrict__ inv,
                              const T *__restrict__ r, T *__restrict__ z, const uint8_t *__restrict__ act)
{
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

cudaError_t launch_dense_setup(const DevMesh &m, bool fp32, const void *vals, const int64_t *dense_off, int max_nd,
                               float *inv, int *singular, cudaStream_t s)
{
  const size_t sm = static_cast<size_t>(max_nd) * 2 * max_nd * sizeof(float);
  if (sm > 200 * 1024) return cudaErrorInvalidValue;
  if (fp32)
    {
      cudaError_t e = cudaFuncSetAttribute(k_dense_invert<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           static_cast<int>(sm));
      if (e != cudaSuccess) return e;
      k_dense_invert<float><<<m.n_inst, kGjThreads, sm, s>>>(m, static_cast<const float *>(vals), dense_off, inv,
                                                             singular);
    }
  else
    {
      cudaError_t e = cudaFuncSetAttribute(k_dense_invert<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           static_cast<int>(sm));
      if (e != cudaSuccess) return e;
      k_dense_invert<double><<<m.n_inst, kGjThreads, sm, s>>>(m, static_cast<const double *>(vals), dense_off, inv,
                                                              singular);
    }
  return cudaGetLastError();
}

cudaError_t launch_dense_apply(const DevMesh &m, bool fp32, int max_nd, const int64_t *dense_off, const float *inv,
                               const void *r, void *z, const uint8_t *act, cudaStream_t s)
{
  dim3 g((max_nd * 32 + 255) / 256, m.n_inst);
  if (fp32)
    k_dense_apply<float><<<g, 256, 0, s>>>(m, dense_off, inv, static_cast<const float *>(r), static_cast<float *>(z),
                                           act);
  else
    k_dense_apply<double><<<g, 256, 0, s>>>(m, dense_off, inv, static_cast<const double *>(r),
                                            static_cast<double *>(z), act);
  return cudaGetLastError();
}

} // namespace glgpu
