// Matrix-free application of the FP32 Jacobian (mixed mode, 3D Q1, 18 components).
//
// The assembled block row of a node holds 27 x 324 scalars.  Here the Krylov operator
// y = J z is applied cell by cell from the state itself: the state A and the direction Z
// are interpolated to the 2x2x2 Gauss points, the bulk Hessian is applied to Z at each
// point in closed form (complex 3x3 algebra, hvp_part) without being formed, and the
// gradient terms act on the interpolated derivatives:
//
//   (J z)_a = jxw sum_q [ val_q(a) (H(A_q) Z_q) + sum_k dval_q(a)/dx_k F_k(q) ],
//   F_k = K1 dZ/dx_k + [k == j(c)] (K2+K3) div_pm(c) Z,
//
// the same bilinear form as the assembled block (a, b) = vol sum_q S_abq H_q + gradient
// terms.  The cell results are summed per node by a gather over the plan's (cell, vertex,
// weight) contributions (the lists that condense the residual: hanging vertices pass to
// their parents, no atomics).  Interpolation and the transposed contraction are
// sum-factorised along the axes.  Constrained rows (hanging nodes, zero-Dirichlet
// components) act as the identity, and constrained components of z are read as zero.
// Per apply the operator reads the two nodal vectors and writes / reads the cell results,
// instead of the 171 x 8 Hessian entries per cell.
#include <cstdint>
#include <cuda_runtime.h>

#include "device.h"

namespace glgpu
{
// cells per CTA (NC = 4, 8 or 16, a run-time choice): 8 NC (cell, point) pairs and 24 NC
// threads (3 per point in the Hessian-vector product)
constexpr float kGaF = 0.21132486540518711775f; // Gauss point 1/2 - sqrt(3)/6 on [0, 1]
constexpr float kGbF = 0.78867513459481288225f;

template <int NC> struct MfSmem
{
  union
  {
    struct
    {
      float zs[NC][8][18]; // nodal values of the direction (gather -> interpolation)
      float xs[NC][8][18]; // nodal values of the state
    } g;
    float part[3][NC * 8][18]; // H Z per point, in three partial sums (product -> contraction)
  } u;
  float Z[NC * 8][19];
  float X[NC * 8][19]; // the state A at the points
  float gZ[NC * 8][3][18];
  float ih[NC][3];
  float jxw[NC];
  float K1[NC], K23[NC];
  float bulk[NC][6]; // alpha, beta1..beta5
};

__device__ __forceinline__ void gauss2f(float f0, float f1, float &q0, float &q1)
{
  q0 = kGbF * f0 + kGaF * f1;
  q1 = kGaF * f0 + kGbF * f1;
}

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

// ---------------------------------------------------------------------------------
// The bulk Hessian applied to a direction without forming it.  With A = u + i v the 3x3
// complex order parameter at a point (component c < 9: u(c/3, c%3), else v), P = A A^T,
// Q = A A^+, p = tr P, q = tr Q and the direction F (packed like A), the product is
//   H F = alpha F + 2 sum_t beta_t dG_t[F],
//   dG_1 = dp A^* + p F^*,  dp = 2 sum A_ij F_ij
//   dG_2 = dq A + q F,      dq = 2 Re sum conj(A_ij) F_ij
//   dG_3 = (S + S^T) A^* + P F^*,   S = A F^T
//   dG_4 = (S + S^+) A + Q F,       S = F A^+
//   dG_5 = (S + S^+) A + Q^* F,     S = F^* A^T
// (G_t = (1/2) d I_t / dA^*, I_1 = |tr A A^T|^2, I_2 = (tr A A^+)^2, I_3 = tr(A A^T (A A^T)^*),
// I_4 = tr((A A^+)^2), I_5 = tr(A A^+ (A A^+)^*): femgl/src/cell_mat_vec/cell_mat_lhs_beta*.cc).
// FP32 complex 3x3 algebra in registers; every index is a compile-time constant.
// ---------------------------------------------------------------------------------
struct Cf
{
  float r, i;
};
__device__ __forceinline__ Cf cm(Cf a, Cf b) { return {a.r * b.r - a.i * b.i, a.r * b.i + a.i * b.r}; }
__device__ __forceinline__ Cf cma(Cf a, Cf b, Cf acc) // acc + a b
{
  return {fmaf(a.r, b.r, fmaf(-a.i, b.i, acc.r)), fmaf(a.r, b.i, fmaf(a.i, b.r, acc.i))};
}
__device__ __forceinline__ Cf cj(Cf a) { return {a.r, -a.i}; }
using M3 = Cf[3][3];

__device__ __forceinline__ void load_m3(const float *a, M3 &A)
{
#pragma unroll
  for (int k = 0; k < 9; ++k) A[k / 3][k % 3] = {a[k], a[9 + k]};
}
// out += w D
__device__ __forceinline__ void acc_m3(const M3 &D, float w, float (&out)[18])
{
#pragma unroll
  for (int k = 0; k < 9; ++k)
    {
      out[k] = fmaf(w, D[k / 3][k % 3].r, out[k]);
      out[9 + k] = fmaf(w, D[k / 3][k % 3].i, out[9 + k]);
    }
}
// C = op_a(X) op_b(Y) with op: 0 plain, 1 transpose, 2 conjugate, 3 conjugate transpose
template <int OA, int OB> __device__ __forceinline__ void mm3(const M3 &X, const M3 &Y, M3 &C)
{
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      {
        Cf acc = {0.f, 0.f};
#pragma unroll
        for (int k = 0; k < 3; ++k)
          {
            Cf x = (OA & 1) ? X[k][i] : X[i][k];
            if (OA & 2) x = cj(x);
            Cf y = (OB & 1) ? Y[j][k] : Y[k][j];
            if (OB & 2) y = cj(y);
            acc = cma(x, y, acc);
          }
        C[i][j] = acc;
      }
}

// out += w op_a(X) op_b(Y), packed like A (no 3x3 temporary)
template <int OA, int OB> __device__ __forceinline__ void mm3_acc(const M3 &X, const M3 &Y, float w, float (&out)[18])
{
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      {
        Cf acc = {0.f, 0.f};
#pragma unroll
        for (int k = 0; k < 3; ++k)
          {
            Cf x = (OA & 1) ? X[k][i] : X[i][k];
            if (OA & 2) x = cj(x);
            Cf y = (OB & 1) ? Y[j][k] : Y[k][j];
            if (OB & 2) y = cj(y);
            acc = cma(x, y, acc);
          }
        out[3 * i + j] = fmaf(w, acc.r, out[3 * i + j]);
        out[9 + 3 * i + j] = fmaf(w, acc.i, out[9 + 3 * i + j]);
      }
}

// terms of thread group G for the point with state a and direction f: out = the group's
// share of alpha f + sum_t 2 beta_t dG_t[f].  dG_4 and dG_5 are evaluated together: with
// S = F A^+ the matrix of dG_5 is conj(S) (F^* A^T = conj(F A^+)), and both terms multiply A and
// F from the right, so
//   w4 dG_4 + w5 dG_5 = [w4 (S + S^+) + w5 (conj(S) + S^T)] A + (w4 Q + w5 Q^*) F.
// G = 0: alpha f + dG_3;  G = 1: dG_1 and the A-product of dG_4, dG_5;  G = 2: dG_2 and their
// F-product.
template <int G>
__device__ __forceinline__ void hvp_part(const float (&a)[18], const float (&f)[18], const float *cf, float (&out)[18])
{
  M3 A, F, S, X;
  load_m3(a, A);
  load_m3(f, F);
  if constexpr (G == 0)
    {
#pragma unroll
      for (int k = 0; k < 18; ++k) out[k] = cf[0] * f[k];
      // dG_3 = (S + S^T) A^* + P F^*, S = A F^T, P = A A^T
      const float w3 = 2.f * cf[3];
      mm3<0, 1>(A, F, S);
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) X[i][j] = {S[i][j].r + S[j][i].r, S[i][j].i + S[j][i].i};
      mm3_acc<0, 2>(X, A, w3, out);
      mm3<0, 1>(A, A, S); // P
      mm3_acc<0, 2>(S, F, w3, out);
    }
  else
    {
#pragma unroll
      for (int k = 0; k < 18; ++k) out[k] = 0.f;
      const float w4 = 2.f * cf[4], w5 = 2.f * cf[5];
      if constexpr (G == 1)
        {
          // dG_1 = dp A^* + p F^*, p = tr A A^T, dp = 2 sum A_ij F_ij
          Cf p = {0.f, 0.f}, dp = {0.f, 0.f};
#pragma unroll
          for (int k = 0; k < 9; ++k)
            {
              const Cf x = A[k / 3][k % 3], y = F[k / 3][k % 3];
              p = cma(x, x, p);
              dp = cma(x, y, dp);
            }
          dp = {2.f * dp.r, 2.f * dp.i};
#pragma unroll
          for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) X[i][j] = cma(p, cj(F[i][j]), cm(dp, cj(A[i][j])));
          acc_m3(X, 2.f * cf[1], out);
          // [w4 (S + S^+) + w5 (conj(S) + S^T)] A, S = F A^+
          mm3<0, 3>(F, A, S);
#pragma unroll
          for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j)
              {
                const Cf sij = S[i][j], sji = S[j][i];
                // S + S^+ = (s_ij + conj s_ji); conj(S) + S^T = (conj s_ij + s_ji)
                X[i][j] = {(w4 + w5) * (sij.r + sji.r), w4 * (sij.i - sji.i) + w5 * (sji.i - sij.i)};
              }
          mm3_acc<0, 0>(X, A, 1.f, out);
        }
      else
        {
          // dG_2 = dq A + q F, q = tr A A^+, dq = 2 Re sum conj(A_ij) F_ij
          float q = 0.f, dq = 0.f;
#pragma unroll
          for (int k = 0; k < 9; ++k)
            {
              const Cf x = A[k / 3][k % 3], y = F[k / 3][k % 3];
              q = fmaf(x.r, x.r, fmaf(x.i, x.i, q));
              dq = fmaf(x.r, y.r, fmaf(x.i, y.i, dq));
            }
          dq *= 2.f;
#pragma unroll
          for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j)
              X[i][j] = {fmaf(dq, A[i][j].r, q * F[i][j].r), fmaf(dq, A[i][j].i, q * F[i][j].i)};
          acc_m3(X, 2.f * cf[2], out);
          // (w4 Q + w5 Q^*) F, Q = A A^+
          mm3<0, 3>(A, A, S);
#pragma unroll
          for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) X[i][j] = {(w4 + w5) * S[i][j].r, (w4 - w5) * S[i][j].i};
          mm3_acc<0, 0>(X, F, 1.f, out);
        }
    }
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
__global__ void __launch_bounds__(24 * NC, 32 / NC) k_mf_cell(DevMesh m, const float *__restrict__ xs,
                                                     const float *__restrict__ z, float *__restrict__ ycell,
                                                     const uint8_t *__restrict__ act)
{
  constexpr int kMCells = NC, kMPts = 8 * NC, kMThreads = 24 * NC;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  MfSmem<NC> &S = *reinterpret_cast<MfSmem<NC> *>(smem_raw);
  const int tid = threadIdx.x;
  const int64_t e0 = static_cast<int64_t>(blockIdx.x) * kMCells;
  const int ncb = static_cast<int>((m.nc - e0) < kMCells ? (m.nc - e0) : kMCells);
  if (tid < kMCells)
    {
      float4 g = make_float4(0.f, 0.f, 0.f, 0.f);
      float K1 = 0.f, K23 = 0.f;
      float bk[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      if (tid < ncb)
        {
          const int64_t e = e0 + tid;
          const int inst = m.cell_inst[e];
          g = m.geo_f[e];
          K1 = m.coef_f[inst * kCoef + 0];
          K23 = m.coef_f[inst * kCoef + 1];
#pragma unroll
          for (int k = 0; k < 6; ++k) bk[k] = m.coef_f[inst * kCoef + 2 + k];
        }
      S.ih[tid][0] = g.x;
      S.ih[tid][1] = g.y;
      S.ih[tid][2] = g.z;
      S.jxw[tid] = 0.125f * g.w;
      S.K1[tid] = K1;
      S.K23[tid] = K23;
#pragma unroll
      for (int k = 0; k < 6; ++k) S.bulk[tid][k] = bk[k];
    }
  // nodal values: thread entries idx = tid + k kMThreads, k < 6 (144 NC entries over 24 NC
  // threads); node ids, then values, ranges and masks are requested together
  {
    constexpr int kPer = 6;
    static_assert(kMCells * 144 == kPer * kMThreads, "six entries per thread");
    int node[kPer];
#pragma unroll
    for (int k = 0; k < kPer; ++k)
      {
        const int idx = tid + k * kMThreads, cl = idx / 144, v = (idx - 144 * cl) / 18;
        node[k] = (cl < ncb) ? m.cells[(e0 + cl) * 8 + v] : -1;
      }
    float zv[kPer], xv[kPer];
    int h0[kPer], h1[kPer];
    uint32_t mk[kPer];
#pragma unroll
    for (int k = 0; k < kPer; ++k)
      {
        const int idx = tid + k * kMThreads, c = (idx % 144) % 18;
        const bool ok = node[k] >= 0;
        const int64_t b = ok ? static_cast<int64_t>(node[k]) * 18 + c : 0;
        zv[k] = ok ? z[b] : 0.f;
        xv[k] = ok ? xs[b] : 0.f;
        h0[k] = ok ? m.hptr[node[k]] : 0;
        h1[k] = ok ? m.hptr[node[k] + 1] : 0;
        mk[k] = ok ? m.mask[node[k]] : ~0u;
      }
#pragma unroll
    for (int k = 0; k < kPer; ++k)
      {
        const int idx = tid + k * kMThreads, cl = idx / 144, rem = idx - 144 * cl, v = rem / 18, c = rem - 18 * v;
        float val = 0.f;
        if (h1[k] > h0[k])
          for (int j = h0[k]; j < h1[k]; ++j)
            {
              const int par = m.hpar[j]; // a parent's zero-Dirichlet components do not enter
              if (!((m.mask[par] >> c) & 1u)) val += static_cast<float>(m.hw[j]) * z[static_cast<int64_t>(par) * 18 + c];
            }
        else if (!((mk[k] >> c) & 1u))
          val = zv[k];
        S.u.g.zs[cl][v][c] = val;
        S.u.g.xs[cl][v][c] = xv[k]; // the state is stored distributed: vertex values as they are
      }
  }
  __syncthreads();
  // Z and its physical gradient at the points: thread (cell, component)
  if (tid < kMCells * 18)
    {
      const int cl = tid / 18, c = tid - 18 * cl;
      const float *xv = &S.u.g.zs[cl][0][c]; // xv[18 v], v = vx + 2 vy + 4 vz
      // the state at the 8 points: the same tensor interpolation, values only
      {
        const float *sv = &S.u.g.xs[cl][0][c];
        float aq[2][4];
#pragma unroll
        for (int t = 0; t < 4; ++t) gauss2f(sv[18 * t], sv[18 * (t + 4)], aq[0][t], aq[1][t]);
        // along y, in place: aq[qz][2 qy + vx]
#pragma unroll
        for (int qz = 0; qz < 2; ++qz)
#pragma unroll
          for (int vx = 0; vx < 2; ++vx)
            {
              float y0, y1;
              gauss2f(aq[qz][vx], aq[qz][2 + vx], y0, y1);
              aq[qz][vx] = y0;
              aq[qz][2 + vx] = y1;
            }
#pragma unroll
        for (int qz = 0; qz < 2; ++qz)
#pragma unroll
          for (int qy = 0; qy < 2; ++qy)
            {
              float v0, v1;
              gauss2f(aq[qz][2 * qy], aq[qz][2 * qy + 1], v0, v1);
              const int p0 = cl * 8 + 2 * qy + 4 * qz;
              S.X[p0][c] = v0;
              S.X[p0 + 1][c] = v1;
            }
      }
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
  // w = H_q Z_q in three partial sums, thread (point, group of bulk terms), from the state
  // and the direction at the point (hvp_part)
  {
    const int pq = tid & (kMPts - 1), g = tid / kMPts, cl = pq >> 3;
    float zq[18], aq[18], acc[18];
#pragma unroll
    for (int i = 0; i < 18; ++i)
      {
        zq[i] = S.Z[pq][i];
        aq[i] = S.X[pq][i];
      }
    float cf[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) cf[k] = S.bulk[cl][k];
    __syncthreads(); // zs / xs (aliased by the partial sums) are no longer read
    if (cl < ncb)
      {
        if (g == 0)
          hvp_part<0>(aq, zq, cf, acc);
        else if (g == 1)
          hvp_part<1>(aq, zq, cf, acc);
        else
          hvp_part<2>(aq, zq, cf, acc);
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
}

// Node gather: thread (node, component), 16 nodes per CTA.  s = sum of the row's cell
// contributions (the identity on constrained rows and components), then by mode
//   0: y = s,  1: y = b - s,  2: y = z + omega D^-1 (b - s)  (D^-1 [Nn][324], one sweep).
// The 18 threads of a node read the same contribution entries (one transaction each) and
// 18 consecutive floats of every cell result; the contribution lists are loaded for all
// (up to 8 at a time) before the cell values, so the value loads are in flight together.
constexpr int kMgNodes = 16;
constexpr int kMgThreads = kMgNodes * 18;

__global__ void __launch_bounds__(kMgThreads, 5) k_mf_gather(DevMesh m, const float *__restrict__ ycell,
                                                          const float *__restrict__ z, const float *__restrict__ b,
                                                          const float *__restrict__ dinv, float *__restrict__ y,
                                                          float omega, int mode, const uint8_t *__restrict__ act)
{
  __shared__ float t_s[kMgNodes][18];
  const int ln = threadIdx.x / 18, c = threadIdx.x - 18 * (threadIdx.x / 18);
  const int64_t n = static_cast<int64_t>(blockIdx.x) * kMgNodes + ln;
  const bool on = n < m.nn && !(act && !act[m.node_inst[n]]);
  float s = 0.f;
  if (on)
    {
      const int k0 = m.rc_ptr[n], k1 = m.rc_ptr[n + 1];
      for (int base = k0; base < k1; base += 8)
        {
          const int nk = (k1 - base) < 8 ? (k1 - base) : 8;
          int cell[8], vtx[8];
          float w[8];
#pragma unroll
          for (int k = 0; k < 8; ++k)
            {
              cell[k] = 0;
              vtx[k] = 0;
              w[k] = 0.f;
              if (k < nk)
                {
                  cell[k] = m.rc_cell[base + k];
                  vtx[k] = m.rc_a[base + k];
                  w[k] = m.rc_wf[base + k];
                }
            }
          float v[8];
#pragma unroll
          for (int k = 0; k < 8; ++k)
            v[k] = (k < nk) ? __ldg(ycell + static_cast<int64_t>(cell[k]) * 144 + vtx[k] * 18 + c) : 0.f;
#pragma unroll
          for (int k = 0; k < 8; ++k) s = fmaf(w[k], v[k], s);
        }
      if (m.hptr[n + 1] > m.hptr[n] || ((m.mask[n] >> c) & 1u)) s = z[n * 18 + c];
    }
  if (mode == 0)
    {
      if (on) y[n * 18 + c] = s;
      return;
    }
  const float t = on ? b[n * 18 + c] - s : 0.f;
  if (mode == 1)
    {
      if (on) y[n * 18 + c] = t;
      return;
    }
  // u = D^-1 t: row c of the node's 18 x 18 block against the node's t
  t_s[ln][c] = t;
  __syncthreads();
  if (!on) return;
  const float *row = dinv + n * 324 + c * 18;
  float u = 0.f;
#pragma unroll
  for (int d = 0; d < 18; ++d) u = fmaf(__ldg(row + d), t_s[ln][d], u);
  y[n * 18 + c] = z[n * 18 + c] + omega * u;
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
static cudaError_t launch_mf_cell(const DevMesh &m, const float *xs, const float *z, float *ycell, const uint8_t *act,
                                  cudaStream_t s)
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
  k_mf_cell<NC><<<static_cast<unsigned>(gc), 24 * NC, sizeof(MfSmem<NC>), s>>>(m, xs, z, ycell, act);
  return cudaGetLastError();
}

cudaError_t launch_mf(const DevMesh &m, const float *xs, const float *z, float *ycell, float *y, const float *b,
                      const float *dinv, float omega, int mode, const uint8_t *act, cudaStream_t s,
                      int cells_per_cta)
{
  if (m.dim != 3 || m.B != 18 || m.nv != 8) return cudaErrorInvalidValue;
  if (mode == 2 && !dinv) return cudaErrorInvalidValue;
  if (mode >= 1 && !b) return cudaErrorInvalidValue;
  cudaError_t e = cells_per_cta == 4    ? launch_mf_cell<4>(m, xs, z, ycell, act, s)
                  : cells_per_cta == 16 ? launch_mf_cell<16>(m, xs, z, ycell, act, s)
                                        : launch_mf_cell<8>(m, xs, z, ycell, act, s);
  if (e != cudaSuccess) return e;
  if ((e = launch_robin_mf(m, z, ycell, act, s)) != cudaSuccess) return e;
  const int64_t gn = (m.nn + kMgNodes - 1) / kMgNodes;
  k_mf_gather<<<static_cast<unsigned>(gn), kMgThreads, 0, s>>>(m, ycell, z, b, dinv, y, omega, mode, act);
  return cudaGetLastError();
}

} // namespace glgpu
