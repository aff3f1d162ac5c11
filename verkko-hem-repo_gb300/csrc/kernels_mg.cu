// Multigrid kernels (sm_103a): inter-level transfers and the coarsest-level dense solve.
//
// Transfers are node-level CSR gathers applied to all B components of a node:
//   prolongation   z_fine[n][c]  += sum_j w_j z_coarse[idx_j][c]   (trilinear, P)
//   restriction    r_coarse[i][c] = sum_j w_j r_fine[idx_j][c]     (P^T, transposed CSR)
//   state transfer x_coarse[i][c] = sum_j w_j x_fine[idx_j][c]     (trilinear from the finer grid)
// Constrained components (zero-Dirichlet, hanging) are left alone on the way up and
// zeroed on the way down, so every Krylov vector keeps zeros there.
// The coarsest level (1 cell per axis, 8 nodes, 144 unknowns per instance) is inverted
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

__global__ void k_interp_state(int64_t nn_c, int B, const int32_t *__restrict__ ptr, const int32_t *__restrict__ idx,
                               const double *__restrict__ w, const double *__restrict__ xf, double *__restrict__ xc)
{
  const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= nn_c * B) return;
  const int64_t n = t / B;
  const int c = static_cast<int>(t % B);
  double s = 0;
  for (int k = ptr[n]; k < ptr[n + 1]; ++k) s += w[k] * xf[static_cast<int64_t>(idx[k]) * B + c];
  xc[t] = s;
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

cudaError_t launch_interp_state(int64_t nn_c, int B, const int32_t *ptr, const int32_t *idx, const double *w,
                                const double *xf, double *xc, cudaStream_t s)
{
  const int64_t n = nn_c * B;
  k_interp_state<<<static_cast<unsigned>((n + 255) / 256), 256, 0, s>>>(nn_c, B, ptr, idx, w, xf, xc);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------------
// coarsest level (one cell per axis: 8 nodes, 144 unknowns per instance): dense inverse
// in shared memory, FP32, one CTA per instance.  It is a preconditioner component, so
// FP32 suffices in both precision modes (the outer flexible GMRES is exact).
// ---------------------------------------------------------------------------------
constexpr int kGjThreads = 512;

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
  if (tid == 0) s_sing = 0;
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
