// Matrix-free application of the FP32 Jacobian (mixed mode, 3D Q1, 18 components).
//
// The assembled block row of a node holds 27 x 324 scalars; the cell data it is built from
// is 171 x 8 quadrature Hessian entries per cell plus the cell geometry, about 6.6x less.
// So the Krylov operator y = J z is applied cell by cell from the Hessians H that the
// assembly already wrote, and summed per node by a gather over the plan's (cell, vertex,
// weight) contributions (the same lists that condense the residual: hanging vertices pass
// to their parents, no atomics):
//
//   (J z)_a = jxw sum_q [ val_q(a) H_q Z_q + sum_k dval_q(a)/dx_k F_k(q) ],
//   F_k = K1 dZ/dx_k + [k == j(c)] (K2+K3) div_pm(c) Z,
//
// the same bilinear form as the assembled block (a, b) = vol sum_q S_abq H_q + gradient
// terms.  Interpolation to the 2x2x2 Gauss points and the transposed contraction are
// sum-factorised along the axes.  Constrained rows (hanging nodes, zero-Dirichlet
// components) act as the identity, and constrained components of z are read as zero;
// Krylov vectors are zero there.
#include <cstdint>
#include <cuda_runtime.h>

#include "device.h"

namespace glgpu
{
// cells per CTA (NC = 4, 8 or 16, a run-time choice): 8 NC (cell, point) pairs and 24 NC
// threads (3 per point in the Hessian product)
constexpr float kGaF = 0.21132486540518711775f; // Gauss point 1/2 - sqrt(3)/6 on [0, 1]
constexpr float kGbF = 0.78867513459481288225f;

template <int NC> struct MfSmem
{
  union
  {
    float zs[NC][8][18];       // nodal values (gather -> interpolation)
    float part[3][NC * 8][18]; // H Z per point, in three partial sums (product -> contraction)
  } u;
  float Z[NC * 8][19];
  float gZ[NC * 8][3][18];
  float ih[NC][3];
  float jxw[NC];
  float K1[NC], K23[NC];
};

__device__ __forceinline__ void gauss2f(float f0, float f1, float &q0, float &q1)
{
  q0 = kGbF * f0 + kGaF * f1;
  q1 = kGaF * f0 + kGbF * f1;
}

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

// offset (times 8 points) of the symmetric pair (c, d) in the upper-triangle enumeration of
// an 18x18 block: 8 * (18 lo - lo (lo - 1) / 2 + hi - lo), lo = min(c, d), hi = max(c, d)
struct SymTable
{
  unsigned short off[18][18];
};
constexpr SymTable make_sym_table()
{
  SymTable t{};
  for (int c = 0; c < 18; ++c)
    for (int d = 0; d < 18; ++d)
      {
        const int lo = c < d ? c : d, hi = c < d ? d : c;
        t.off[c][d] = static_cast<unsigned short>(8 * (18 * lo - (lo * (lo - 1)) / 2 + (hi - lo)));
      }
  return t;
}
__constant__ SymTable c_sym = make_sym_table();

// the t-th pair (c, d), c <= d, of the upper-triangle enumeration (t = 0..170)
__host__ __device__ constexpr int pair_c(int t)
{
  int c = 0;
  while (t >= 18 - c)
    {
      t -= 18 - c;
      ++c;
    }
  return c;
}
__host__ __device__ constexpr int pair_d(int t)
{
  int c = 0;
  while (t >= 18 - c)
    {
      t -= 18 - c;
      ++c;
    }
  return c + t;
}
static_assert(pair_c(170) == 17 && pair_d(170) == 17 && pair_c(17) == 0 && pair_d(18) == 1, "pair enumeration");

// entries T .. END-1 of H_q Z_q, each loaded once and applied to both w_c and w_d (H is
// symmetric); a compile-time recursion, so every (c, d) is a constant register index
template <int T, int END>
__device__ __forceinline__ void hz_terms(const float *__restrict__ Hc, const float (&zq)[18], float (&acc)[18])
{
  if constexpr (T < END)
    {
      constexpr int c = pair_c(T), d = pair_d(T);
      const float h = __ldg(Hc + T * 8);
      acc[c] = fmaf(h, zq[d], acc[c]);
      if constexpr (c != d) acc[d] = fmaf(h, zq[c], acc[d]);
      hz_terms<T + 1, END>(Hc, zq, acc);
    }
}

// one third of H_q Z_q: entries G*57 .. G*57+56
template <int G>
__device__ __forceinline__ void hz_part(const float *__restrict__ Hc, const float (&zq)[18], float (&acc)[18])
{
#pragma unroll
  for (int i = 0; i < 18; ++i) acc[i] = 0.f;
  hz_terms<G * 57, G * 57 + 57>(Hc, zq, acc);
}

// r[a] = sum_q val_q(a) w[q] + sum_k sum_q dval_q(a)/dxi_k F_k[q] (reference cube), a = ax + 2 ay + 4 az:
// the transposed interpolation, sum-factorised axis by axis
__device__ __forceinline__ void mf_contract(const float (&w)[8], const float (&F)[3][8], float (&r)[8])
{
      {
    float tx[2][4];
#pragma unroll
    for (int t = 0; t < 4; ++t)
      {
        tx[0][t] = kGbF * w[2 * t] + kGaF * w[2 * t + 1];
        tx[1][t] = kGaF * w[2 * t] + kGbF * w[2 * t + 1];
      }
    float ty[2][2][2];
#pragma unroll
    for (int ax = 0; ax < 2; ++ax)
#pragma unroll
      for (int qz = 0; qz < 2; ++qz)
        {
          ty[ax][0][qz] = kGbF * tx[ax][2 * qz] + kGaF * tx[ax][2 * qz + 1];
          ty[ax][1][qz] = kGaF * tx[ax][2 * qz] + kGbF * tx[ax][2 * qz + 1];
        }
#pragma unroll
    for (int ax = 0; ax < 2; ++ax)
#pragma unroll
      for (int ay = 0; ay < 2; ++ay)
        {
          r[ax + 2 * ay] = kGbF * ty[ax][ay][0] + kGaF * ty[ax][ay][1];
          r[ax + 2 * ay + 4] = kGaF * ty[ax][ay][0] + kGbF * ty[ax][ay][1];
        }
  }
  {
    float sx[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) sx[t] = F[0][2 * t] + F[0][2 * t + 1];
    float uy[2][2];
#pragma unroll
    for (int qz = 0; qz < 2; ++qz)
      {
        uy[0][qz] = kGbF * sx[2 * qz] + kGaF * sx[2 * qz + 1];
        uy[1][qz] = kGaF * sx[2 * qz] + kGbF * sx[2 * qz + 1];
      }
#pragma unroll
    for (int ay = 0; ay < 2; ++ay)
#pragma unroll
      for (int az = 0; az < 2; ++az)
        {
          const float v = az ? kGaF * uy[ay][0] + kGbF * uy[ay][1] : kGbF * uy[ay][0] + kGaF * uy[ay][1];
          r[1 + 2 * ay + 4 * az] += v;
          r[2 * ay + 4 * az] -= v;
        }
  }
  {
    float sy[4];
#pragma unroll
    for (int qz = 0; qz < 2; ++qz)
#pragma unroll
      for (int qx = 0; qx < 2; ++qx) sy[qx + 2 * qz] = F[1][qx + 4 * qz] + F[1][qx + 2 + 4 * qz];
    float ux[2][2];
#pragma unroll
    for (int qz = 0; qz < 2; ++qz)
      {
        ux[0][qz] = kGbF * sy[2 * qz] + kGaF * sy[2 * qz + 1];
        ux[1][qz] = kGaF * sy[2 * qz] + kGbF * sy[2 * qz + 1];
      }
#pragma unroll
    for (int ax = 0; ax < 2; ++ax)
#pragma unroll
      for (int az = 0; az < 2; ++az)
        {
          const float v = az ? kGaF * ux[ax][0] + kGbF * ux[ax][1] : kGbF * ux[ax][0] + kGaF * ux[ax][1];
          r[ax + 2 + 4 * az] += v;
          r[ax + 4 * az] -= v;
        }
  }
  {
    float sz[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) sz[t] = F[2][t] + F[2][t + 4];
    float ux[2][2];
#pragma unroll
    for (int qy = 0; qy < 2; ++qy)
      {
        ux[0][qy] = kGbF * sz[2 * qy] + kGaF * sz[2 * qy + 1];
        ux[1][qy] = kGaF * sz[2 * qy] + kGbF * sz[2 * qy + 1];
      }
#pragma unroll
    for (int ax = 0; ax < 2; ++ax)
#pragma unroll
      for (int ay = 0; ay < 2; ++ay)
        {
          const float v = ay ? kGaF * ux[ax][0] + kGbF * ux[ax][1] : kGbF * ux[ax][0] + kGaF * ux[ax][1];
          r[ax + 2 * ay + 4] += v;
          r[ax + 2 * ay] -= v;
        }
  }
}

template <int NC>
__global__ void __launch_bounds__(24 * NC) k_mf_cell(DevMesh m, const float *__restrict__ H,
                                                     const float *__restrict__ z, float *__restrict__ ycell,
                                                     const uint8_t *__restrict__ act, int *__restrict__ err)
{
  constexpr int kMCells = NC, kMPts = 8 * NC, kMThreads = 24 * NC;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  MfSmem<NC> &S = *reinterpret_cast<MfSmem<NC> *>(smem_raw);
  const int tid = threadIdx.x;
  const int64_t e0 = static_cast<int64_t>(blockIdx.x) * kMCells;
  const int ncb = static_cast<int>((m.nc - e0) < kMCells ? (m.nc - e0) : kMCells);
  const float *Hb = H + e0 * static_cast<int64_t>(kNS3) * 8;
  if (tid == 0)
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(Hb),
                 "r"(static_cast<uint32_t>(ncb) * kNS3 * 8 * static_cast<uint32_t>(sizeof(float)))
                 : "memory");
  if (tid < kMCells)
    {
      float4 g = make_float4(0.f, 0.f, 0.f, 0.f);
      float K1 = 0.f, K23 = 0.f;
      if (tid < ncb)
        {
          const int64_t e = e0 + tid;
          const int inst = m.cell_inst[e];
          g = m.geo_f[e];
          K1 = m.coef_f[inst * kCoef + 0];
          K23 = m.coef_f[inst * kCoef + 1];
        }
      S.ih[tid][0] = g.x;
      S.ih[tid][1] = g.y;
      S.ih[tid][2] = g.z;
      S.jxw[tid] = 0.125f * g.w;
      S.K1[tid] = K1;
      S.K23[tid] = K23;
    }
  for (int idx = tid; idx < kMCells * 144; idx += kMThreads)
    {
      const int cl = idx / 144, rem = idx - 144 * cl, v = rem / 18, c = rem - 18 * v;
      float val = 0.f;
      if (cl < ncb)
        {
          // the node's value, its constraint range and mask are independent loads
          const int node = m.cells[(e0 + cl) * 8 + v];
          const float zv = z[static_cast<int64_t>(node) * 18 + c];
          const int h0 = m.hptr[node], h1 = m.hptr[node + 1];
          const uint32_t mk = m.mask[node];
          if (h1 > h0)
            for (int k = h0; k < h1; ++k)
              {
                const int par = m.hpar[k]; // a parent's zero-Dirichlet components do not enter
                if (!((m.mask[par] >> c) & 1u)) val += static_cast<float>(m.hw[k]) * z[static_cast<int64_t>(par) * 18 + c];
              }
          else if (!((mk >> c) & 1u))
            val = zv;
        }
      S.u.zs[cl][v][c] = val;
    }
  __syncthreads();
  // Z and its physical gradient at the points: thread (cell, component)
  if (tid < kMCells * 18)
    {
      const int cl = tid / 18, c = tid - 18 * cl;
      const float *xv = &S.u.zs[cl][0][c]; // xv[18 v], v = vx + 2 vy + 4 vz
      float zq[2][4], zd[4];
#pragma unroll
      for (int t = 0; t < 4; ++t)
        {
          const float f0 = xv[18 * t], f1 = xv[18 * (t + 4)];
          gauss2f(f0, f1, zq[0][t], zq[1][t]);
          zd[t] = f1 - f0;
        }
      float yq[2][2][2], ydy[2][2], zdq[2][2];
#pragma unroll
      for (int vx = 0; vx < 2; ++vx)
        {
#pragma unroll
          for (int qz = 0; qz < 2; ++qz)
            {
              gauss2f(zq[qz][vx], zq[qz][2 + vx], yq[qz][0][vx], yq[qz][1][vx]);
              ydy[qz][vx] = zq[qz][2 + vx] - zq[qz][vx];
            }
          gauss2f(zd[vx], zd[2 + vx], zdq[0][vx], zdq[1][vx]);
        }
      const float i0 = S.ih[cl][0], i1 = S.ih[cl][1], i2 = S.ih[cl][2];
#pragma unroll
      for (int qz = 0; qz < 2; ++qz)
#pragma unroll
        for (int qy = 0; qy < 2; ++qy)
          {
            float v0, v1;
            gauss2f(yq[qz][qy][0], yq[qz][qy][1], v0, v1);
            const float dx = (yq[qz][qy][1] - yq[qz][qy][0]) * i0;
            const int p0 = cl * 8 + 2 * qy + 4 * qz;
            S.Z[p0][c] = v0;
            S.Z[p0 + 1][c] = v1;
            S.gZ[p0][0][c] = dx;
            S.gZ[p0 + 1][0][c] = dx;
          }
#pragma unroll
      for (int qz = 0; qz < 2; ++qz)
        {
          float d0, d1;
          gauss2f(ydy[qz][0], ydy[qz][1], d0, d1);
#pragma unroll
          for (int qy = 0; qy < 2; ++qy)
            {
              const int p0 = cl * 8 + 2 * qy + 4 * qz;
              S.gZ[p0][1][c] = d0 * i1;
              S.gZ[p0 + 1][1][c] = d1 * i1;
            }
        }
#pragma unroll
      for (int qy = 0; qy < 2; ++qy)
        {
          float d0, d1;
          gauss2f(zdq[qy][0], zdq[qy][1], d0, d1);
#pragma unroll
          for (int qz = 0; qz < 2; ++qz)
            {
              const int p0 = cl * 8 + 2 * qy + 4 * qz;
              S.gZ[p0][2][c] = d0 * i2;
              S.gZ[p0 + 1][2][c] = d1 * i2;
            }
        }
    }
  __syncthreads(); // Z, gZ complete
  // w = H_q Z_q in three partial sums: thread (point, third of the 171 entries); a warp's
  // lanes read the same entry for the 8 points of 4 cells (4 x 32 contiguous bytes, L2)
  {
    const int pq = tid & (kMPts - 1), g = tid / kMPts, cl = pq >> 3, q = pq & 7;
    float zq[18], acc[18];
#pragma unroll
    for (int i = 0; i < 18; ++i) zq[i] = S.Z[pq][i];
    __syncthreads(); // zs (aliased by the partial sums) is no longer read
    if (cl < ncb)
      {
        const float *Hc = Hb + cl * kNS3 * 8 + q;
        if (g == 0)
          hz_part<0>(Hc, zq, acc);
        else if (g == 1)
          hz_part<1>(Hc, zq, acc);
        else
          hz_part<2>(Hc, zq, acc);
#pragma unroll
        for (int i = 0; i < 18; ++i) S.u.part[g][pq][i] = acc[i];
      }
  }
  __syncthreads();
  // contraction with the test functions: thread (cell, component)
  if (tid < kMCells * 18)
    {
      const int cl = tid / 18, c = tid - 18 * cl;
      const int part = c / 9, mu = (c % 9) / 3, jc = c % 3;
      const float K1 = S.K1[cl], K23 = S.K23[cl];
      const float ih[3] = {S.ih[cl][0], S.ih[cl][1], S.ih[cl][2]};
      float w[8], F[3][8];
#pragma unroll
      for (int q = 0; q < 8; ++q)
        {
          const int pq = cl * 8 + q;
          w[q] = S.u.part[0][pq][c] + S.u.part[1][pq][c] + S.u.part[2][pq][c];
          const int base = 9 * part + 3 * mu;
          const float dterm = K23 * (S.gZ[pq][0][base] + S.gZ[pq][1][base + 1] + S.gZ[pq][2][base + 2]);
#pragma unroll
          for (int k = 0; k < 3; ++k) F[k][q] = ih[k] * (K1 * S.gZ[pq][k][c] + (k == jc ? dterm : 0.f));
        }
      float r[8];
      mf_contract(w, F, r);
      if (cl < ncb)
        {
          const float jxw = S.jxw[cl];
          float *out = ycell + (e0 + cl) * 144 + c;
#pragma unroll
          for (int a = 0; a < 8; ++a) out[18 * a] = r[a] * jxw;
        }
    }
  (void)act;
  (void)err;
}

// Node gather, one warp per node: s = sum of the row's cell contributions (the identity on
// constrained rows and components), then by mode
//   0: y = s,  1: y = b - s,  2: y = z + omega D^-1 (b - s)  (D^-1 [Nn][324], one sweep).
constexpr int kMgWarps = 8;

__global__ void __launch_bounds__(kMgWarps * 32) k_mf_gather(DevMesh m, const float *__restrict__ ycell,
                                                             const float *__restrict__ z, const float *__restrict__ b,
                                                             const float *__restrict__ dinv, float *__restrict__ y,
                                                             float omega, int mode, const uint8_t *__restrict__ act)
{
  __shared__ float red[kMgWarps][324];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t n = static_cast<int64_t>(blockIdx.x) * kMgWarps + warp;
  if (n >= m.nn) return;
  if (act && !act[m.node_inst[n]]) return;
  // the row's contributions: indices and weights loaded once, one per lane, then the
  // cell values of all of them requested together
  float s = 0.f;
  const bool hang = m.hptr[n + 1] > m.hptr[n];
  const int k0 = m.rc_ptr[n], k1 = m.rc_ptr[n + 1];
  for (int base = k0; base < k1; base += 32)
    {
      const int nk = (k1 - base) < 32 ? (k1 - base) : 32;
      int cell = 0, vtx = 0;
      float wt = 0.f;
      if (lane < nk)
        {
          cell = m.rc_cell[base + lane];
          vtx = m.rc_a[base + lane];
          wt = m.rc_wf[base + lane];
        }
#pragma unroll 4
      for (int k = 0; k < nk; ++k)
        {
          const int ck = __shfl_sync(0xffffffffu, cell, k), ak = __shfl_sync(0xffffffffu, vtx, k);
          const float w = __shfl_sync(0xffffffffu, wt, k);
          if (lane < 18) s += w * ycell[static_cast<int64_t>(ck) * 144 + ak * 18 + lane];
        }
    }
  if (lane < 18 && (hang || ((m.mask[n] >> lane) & 1u))) s = z[n * 18 + lane];
  if (mode == 0)
    {
      if (lane < 18) y[n * 18 + lane] = s;
      return;
    }
  const float t = (lane < 18) ? b[n * 18 + lane] - s : 0.f;
  if (mode == 1)
    {
      if (lane < 18) y[n * 18 + lane] = t;
      return;
    }
  // u = D^-1 t with the SpMV lane map: lane owns float4 chunks lane, lane + 32, lane + 64
  const float4 *bp = reinterpret_cast<const float4 *>(dinv + n * 324);
#pragma unroll
  for (int it = 0; it < 3; ++it)
    {
      const int ch = lane + 32 * it;
      const float4 wv = (ch < 81) ? __ldg(bp + ch) : make_float4(0.f, 0.f, 0.f, 0.f);
      const int e = (ch < 81) ? ch * 4 : 0;
      const float p0 = wv.x * __shfl_sync(0xffffffffu, t, (e + 0) % 18);
      const float p1 = wv.y * __shfl_sync(0xffffffffu, t, (e + 1) % 18);
      const float p2 = wv.z * __shfl_sync(0xffffffffu, t, (e + 2) % 18);
      const float p3 = wv.w * __shfl_sync(0xffffffffu, t, (e + 3) % 18);
      if (ch < 81)
        {
          red[warp][e + 0] = p0;
          red[warp][e + 1] = p1;
          red[warp][e + 2] = p2;
          red[warp][e + 3] = p3;
        }
    }
  __syncwarp();
  if (lane < 18)
    {
      float u = 0.f;
#pragma unroll
      for (int d = 0; d < 18; ++d) u += red[warp][lane * 18 + d];
      y[n * 18 + lane] = z[n * 18 + lane] + omega * u;
    }
}

// Robin faces in the matrix-free operator: ycell[e] += W z_e for the Robin cells, z_e the
// cell's vertex values expanded through the constraints and column masks exactly as
// k_mf_cell reads them (one CTA per Robin cell, thread = (vertex, component)).
constexpr int kRobinMfThreads = 160;

__global__ void __launch_bounds__(kRobinMfThreads) k_robin_mf(DevMesh m, const float *__restrict__ z,
                                                              float *__restrict__ ycell, const uint8_t *__restrict__ act)
{
  __shared__ float zs[144];
  const int64_t e = m.robin_cells[blockIdx.x];
  const int inst = m.cell_inst[e];
  if (act && !act[inst]) return; // uniform over the CTA
  const int tid = threadIdx.x;
  if (tid < 144)
    {
      const int v = tid / 18, c = tid - 18 * v;
      const int node = m.cells[e * 8 + v];
      const int h0 = m.hptr[node], h1 = m.hptr[node + 1];
      float val = 0.f;
      if (h1 > h0)
        for (int k = h0; k < h1; ++k)
          {
            const int par = m.hpar[k];
            if (!((m.mask[par] >> c) & 1u)) val += static_cast<float>(m.hw[k]) * z[static_cast<int64_t>(par) * 18 + c];
          }
      else if (!((m.mask[node] >> c) & 1u))
        val = z[static_cast<int64_t>(node) * 18 + c];
      zs[tid] = val;
    }
  __syncthreads();
  if (tid >= 144) return;
  const int a = tid / 18, c = tid - 18 * a;
  const float4 g = m.geo_f[e];
  const float wR = m.coef_f[inst * kCoef + 8];
  const int bits = m.robin[e];
  float y = 0.f;
  for (int b = 0; b < 8; ++b) y += robin_weight<float>(bits, a, b, c % 3, wR, g.w, g.x, g.y, g.z) * zs[18 * b + c];
  ycell[e * 144 + tid] += y;
}

cudaError_t launch_robin_mf(const DevMesh &m, const float *z, float *ycell, const uint8_t *act, cudaStream_t s)
{
  if (m.n_robin == 0) return cudaSuccess;
  if (m.dim != 3 || m.B != 18 || !m.robin || !m.robin_cells) return cudaErrorInvalidValue;
  k_robin_mf<<<static_cast<unsigned>(m.n_robin), kRobinMfThreads, 0, s>>>(m, z, ycell, act);
  return cudaGetLastError();
}

template <int NC>
static cudaError_t launch_mf_cell(const DevMesh &m, const float *H, const float *z, float *ycell, const uint8_t *act,
                                  int *err, cudaStream_t s)
{
  static bool attr = false;
  if (!attr)
    {
      cudaError_t e = cudaFuncSetAttribute(k_mf_cell<NC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           static_cast<int>(sizeof(MfSmem<NC>)));
      if (e != cudaSuccess) return e;
      attr = true;
    }
  const int64_t gc = (m.nc + NC - 1) / NC;
  k_mf_cell<NC><<<static_cast<unsigned>(gc), 24 * NC, sizeof(MfSmem<NC>), s>>>(m, H, z, ycell, act, err);
  return cudaGetLastError();
}

cudaError_t launch_mf(const DevMesh &m, const float *H, const float *z, float *ycell, float *y, const float *b,
                      const float *dinv, float omega, int mode, const uint8_t *act, cudaStream_t s, int *err,
                      int cells_per_cta)
{
  if (m.dim != 3 || m.B != 18 || m.nv != 8) return cudaErrorInvalidValue;
  if (mode == 2 && !dinv) return cudaErrorInvalidValue;
  if (mode >= 1 && !b) return cudaErrorInvalidValue;
  cudaError_t e = cells_per_cta == 4    ? launch_mf_cell<4>(m, H, z, ycell, act, err, s)
                  : cells_per_cta == 16 ? launch_mf_cell<16>(m, H, z, ycell, act, err, s)
                                        : launch_mf_cell<8>(m, H, z, ycell, act, err, s);
  if (e != cudaSuccess) return e;
  if ((e = launch_robin_mf(m, z, ycell, act, s)) != cudaSuccess) return e;
  const int64_t gn = (m.nn + kMgWarps - 1) / kMgWarps;
  k_mf_gather<<<static_cast<unsigned>(gn), kMgWarps * 32, 0, s>>>(m, ycell, z, b, dinv, y, omega, mode, act);
  return cudaGetLastError();
}

} // namespace glgpu
