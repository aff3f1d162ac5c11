// GPU Kelly error estimator and fixed-number refinement flags (the reference calls deal.II's
// KellyErrorEstimator::estimate with QGauss<2>(2) faces, no Neumann boundaries, all 18
// components, then refine_and_coarsen_fixed_number: femgl/src/refine.cc:147-157).
//
//   eta_K^2 = (diam_K / 24) sum over the interior faces F of K of int_F |[d u / d n]|^2 dS
//
// Boundary faces contribute nothing; faces identified by periodicity are interior.  On a
// coarse-fine interface the integral runs over each fine face (a quarter of the coarse
// face) and counts for both the fine cell and the coarse cell.  Face integrals are FP64, the
// per-cell estimate is returned in FP32 (deal.II's Vector<float>).
//
// Flags: with n_K cells in an instance, the floor(top * n_K) cells of largest eta are flagged
// for refinement (eta >= the k-th largest value) and the floor(bottom * n_K) of smallest eta
// for coarsening (eta <= the k-th smallest).  The k-th value is found exactly by a radix
// select over the float bit patterns (eta >= 0, so bit order is value order): four 8-bit
// histogram passes per selection, all instances at once.
#include <cstdint>

#include "device.h"

namespace glgpu
{
namespace
{
constexpr int kKellyWarps = 8;
constexpr double kG0 = 0.21132486540518711775; // 1/2 - sqrt(3)/6: 2-point Gauss abscissa on [0, 1]

// normal derivative along `ax` of the Q1 field with vertex values xv at the face point with
// tangential reference coordinates (s1, s2) along (t1, t2); it does not depend on the
// coordinate along `ax`
__device__ __forceinline__ double normal_derivative(const double (&xv)[8], int ax, int t1, int t2, double s1, double s2,
                                                    double inv_h)
{
  double d = 0.0;
#pragma unroll
  for (int v = 0; v < 8; ++v)
    {
      const double l1 = ((v >> t1) & 1) ? s1 : 1.0 - s1;
      const double l2 = ((v >> t2) & 1) ? s2 : 1.0 - s2;
      d += (((v >> ax) & 1) ? xv[v] : -xv[v]) * l1 * l2;
    }
  return d * inv_h;
}

// one warp per face pair, lane = component
__global__ void __launch_bounds__(kKellyWarps * 32)
  k_kelly_face(DevMesh m, const double *__restrict__ x, const int32_t *__restrict__ pa, const int32_t *__restrict__ pb,
               const int8_t *__restrict__ fa, const int8_t *__restrict__ ob, const int8_t *__restrict__ sub, int64_t np,
               double *__restrict__ I)
{
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t k = static_cast<int64_t>(blockIdx.x) * kKellyWarps + warp;
  if (k >= np) return;
  const int64_t ea = pa[k], eb = pb[k];
  const int ax = fa[k] / 2;
  const int t1 = (ax == 0) ? 1 : 0, t2 = (ax == 2) ? 1 : 2;
  const int o = ob[k];
  const bool half = sub[k] != 0;
  double acc = 0.0;
  if (lane < 18)
    {
      double xa[8], xb[8];
#pragma unroll
      for (int v = 0; v < 8; ++v)
        {
          xa[v] = x[static_cast<int64_t>(m.cells[ea * 8 + v]) * 18 + lane];
          xb[v] = x[static_cast<int64_t>(m.cells[eb * 8 + v]) * 18 + lane];
        }
      const double iha = 1.0 / m.cell_h[3 * ea + ax], ihb = 1.0 / m.cell_h[3 * eb + ax];
      const double gp[2] = {kG0, 1.0 - kG0};
#pragma unroll
      for (int q = 0; q < 4; ++q)
        {
          const double s1 = gp[q & 1], s2 = gp[q >> 1];
          const double u1 = half ? 0.5 * ((o & 1) + s1) : s1, u2 = half ? 0.5 * (((o >> 1) & 1) + s2) : s2;
          const double j = normal_derivative(xa, ax, t1, t2, s1, s2, iha) - normal_derivative(xb, ax, t1, t2, u1, u2, ihb);
          acc += j * j;
        }
      acc *= 0.25 * m.cell_h[3 * ea + t1] * m.cell_h[3 * ea + t2];
    }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
  if (lane == 0) I[k] = acc;
}

__global__ void k_kelly_cell(DevMesh m, const int32_t *__restrict__ cptr, const int32_t *__restrict__ cpair,
                             const double *__restrict__ I, float *__restrict__ eta)
{
  const int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= m.nc) return;
  double s = 0.0;
  for (int32_t j = cptr[e]; j < cptr[e + 1]; ++j) s += I[cpair[j]];
  const double hx = m.cell_h[3 * e], hy = m.cell_h[3 * e + 1], hz = m.cell_h[3 * e + 2];
  eta[e] = static_cast<float>(sqrt(s * sqrt(hx * hx + hy * hy + hz * hz) / 24.0));
}

// histogram of bits [shift, shift + 8) of the cells whose higher bits equal prefix[inst]
__global__ void k_radix_hist(DevMesh m, const float *__restrict__ eta, const uint32_t *__restrict__ prefix, int shift,
                             uint32_t *__restrict__ hist)
{
  const int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= m.nc) return;
  const int inst = m.cell_inst[e];
  const uint32_t bits = __float_as_uint(eta[e]);
  const uint32_t hi_mask = (shift >= 24) ? 0u : (0xffffffffu << (shift + 8));
  if ((bits & hi_mask) != (prefix[inst] & hi_mask)) return;
  atomicAdd(&hist[inst * 256 + ((bits >> shift) & 255u)], 1u);
}

// flags: 1 refine (eta >= refine threshold), -1 coarsen (eta <= coarsen threshold), else 0;
// an instance with no refine (coarsen) cells has the bit pattern 0xffffffff as its threshold
__global__ void k_flags(DevMesh m, const float *__restrict__ eta, const uint32_t *__restrict__ thr_refine,
                        const uint32_t *__restrict__ thr_coarsen, int8_t *__restrict__ flags)
{
  const int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= m.nc) return;
  const int inst = m.cell_inst[e];
  const uint32_t b = __float_as_uint(eta[e]), tr = thr_refine[inst], tc = thr_coarsen[inst];
  int8_t f = 0;
  if (tr != 0xffffffffu && b >= tr)
    f = 1;
  else if (tc != 0xffffffffu && b <= tc)
    f = -1;
  flags[e] = f;
}
} // namespace

cudaError_t launch_kelly(const DevMesh &m, const double *x, const int32_t *pa, const int32_t *pb, const int8_t *fa,
                         const int8_t *ob, const int8_t *sub, int64_t np, const int32_t *cptr, const int32_t *cpair,
                         double *I, float *eta, cudaStream_t s)
{
  if (m.dim != 3 || m.B != 18 || m.nv != 8) return cudaErrorInvalidValue;
  if (np > 0)
    {
      const int64_t g = (np + kKellyWarps - 1) / kKellyWarps;
      k_kelly_face<<<static_cast<unsigned>(g), kKellyWarps * 32, 0, s>>>(m, x, pa, pb, fa, ob, sub, np, I);
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return e;
    }
  k_kelly_cell<<<static_cast<unsigned>((m.nc + 255) / 256), 256, 0, s>>>(m, cptr, cpair, I, eta);
  return cudaGetLastError();
}

cudaError_t launch_radix_hist(const DevMesh &m, const float *eta, const uint32_t *prefix, int shift, uint32_t *hist,
                              cudaStream_t s)
{
  cudaError_t e = cudaMemsetAsync(hist, 0, sizeof(uint32_t) * 256 * static_cast<size_t>(m.n_inst), s);
  if (e != cudaSuccess) return e;
  k_radix_hist<<<static_cast<unsigned>((m.nc + 255) / 256), 256, 0, s>>>(m, eta, prefix, shift, hist);
  return cudaGetLastError();
}

cudaError_t launch_flags(const DevMesh &m, const float *eta, const uint32_t *thr_refine, const uint32_t *thr_coarsen,
                         int8_t *flags, cudaStream_t s)
{
  k_flags<<<static_cast<unsigned>((m.nc + 255) / 256), 256, 0, s>>>(m, eta, thr_refine, thr_coarsen, flags);
  return cudaGetLastError();
}

} // namespace glgpu
