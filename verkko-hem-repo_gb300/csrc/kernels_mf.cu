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
// cells per CTA (NC = 4, 8 or 16, a run-time choice); 16 NC threads: two per Gauss point in
// the Hessian-vector product, one per (cell, component pair) in the interpolation and the
// contraction.  A component pair is (c, c + 9) = (u_c, v_c), the real and imaginary part of
// one entry of A: the pair is one float2 and its arithmetic runs as packed FP32x2
// (fma.rn.f32x2), two lanes per instruction.
constexpr float kGaF = 0.21132486540518711775f; // Gauss point 1/2 - sqrt(3)/6 on [0, 1]
constexpr float kGbF = 0.78867513459481288225f;

// Shared layouts: per point the 9 complex entries in pair order [2 k + part] (k = 3 mu + j),
// padded to 20 floats (80 bytes, so a point's row loads as 16-byte vectors).
// per-cell constants: 1/hx, 1/hy, 1/hz, JxW, K1, K2+K3, alpha, beta1..beta5
constexpr int kParIh = 0, kParJxw = 3, kParK1 = 4, kParK23 = 5, kParBulk = 6, kPar = 12;

template <int NC> struct MfSmem
{
  union
  {
    struct
    {
      float zs[NC][8][18]; // nodal values of the direction (gather -> interpolation)
      float xs[NC][8][18]; // nodal values of the state
    } g;
    float part[2][NC * 8][20]; // H Z per point, two partial sums (product -> contraction)
  } u;
  float X[NC * 8][20]; // the state A at the points
  float Z[NC * 8][20]; // the direction Z at the points
  float gZ[NC * 8][3][18]; // dZ / dx_k at the points, pair order
  float par[NC][kPar];
};

// the shared arrays the compute phases read and write (NC cells, 8 NC points); part rows
// are PLD floats apart
template <int NC, int PLD> struct MfView
{
  const float (*zs)[8][18];
  const float (*xs)[8][18];
  float (*X)[20];
  float (*Z)[20];
  float (*gZ)[3][18];
  float (*part)[NC * 8][PLD];
  const float (*par)[kPar];
};

using C2 = float2; // complex (re, im), or a component pair (u_c, v_c)

__device__ __forceinline__ C2 c2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ C2 add2(C2 a, C2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ C2 sub2(C2 a, C2 b) { return __fadd2_rn(a, c2(-b.x, -b.y)); }
__device__ __forceinline__ C2 scl2(C2 a, float s) { return __fmul2_rn(a, c2(s, s)); }
// c + a s, s real (both lanes)
__device__ __forceinline__ C2 macr(C2 a, float s, C2 c) { return __ffma2_rn(a, c2(s, s), c); }
// Gauss values of a linear function with end values f0, f1
__device__ __forceinline__ void gauss2(C2 f0, C2 f1, C2 &q0, C2 &q1)
{
  q0 = __ffma2_rn(f0, c2(kGbF, kGbF), __fmul2_rn(f1, c2(kGaF, kGaF)));
  q1 = __ffma2_rn(f0, c2(kGaF, kGaF), __fmul2_rn(f1, c2(kGbF, kGbF)));
}

__device__ __forceinline__ void load_c9(const float *row, C2 (&a)[9])
{
  const float4 *v = reinterpret_cast<const float4 *>(row);
#pragma unroll
  for (int k = 0; k < 4; ++k)
    {
      const float4 t = v[k];
      a[2 * k] = c2(t.x, t.y);
      a[2 * k + 1] = c2(t.z, t.w);
    }
  const float2 t = reinterpret_cast<const float2 *>(row)[8];
  a[8] = t;
}

__device__ __forceinline__ void store_c9(float *row, const C2 (&a)[9])
{
  float4 *v = reinterpret_cast<float4 *>(row);
#pragma unroll
  for (int k = 0; k < 4; ++k) v[k] = make_float4(a[2 * k].x, a[2 * k].y, a[2 * k + 1].x, a[2 * k + 1].y);
  reinterpret_cast<float2 *>(row)[8] = a[8];
}

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
// Grouped by the right factor (w_t = 2 beta_t):
//   H F = Y1 A + Y2 A^* + M F + N F^*
//   Y1 = w4 (S4 + S4^+) + w5 (S4^* + S4^T) + w2 dq 1,  S4 = F A^+
//   Y2 = w3 (S3 + S3^T) + w1 dp 1,                     S3 = A F^T
//   M  = (alpha + w2 q) 1 + w4 Q + w5 Q^*,   N = w3 P + w1 p 1,
// and with A = Ar + i Ai, F = Fr + i Fi (real 3x3 matrices)
//   Y1 A + Y2 A^* = (Y1 + Y2) Ar + i (Y1 - Y2) Ai,   M F + N F^* = (M + N) Fr + i (M - N) Fi:
// four complex-by-real 3x3 products, 27 packed FMAs each.  Role 0 forms the direction-
// dependent Y1, Y2 and their products with A; role 1 the state-only M, N and their products
// with F.  Both write their share of H F; the contraction adds the two.
// ---------------------------------------------------------------------------------
template <int ROLE>
__device__ __forceinline__ void hvp_role(const C2 (&A)[9], const C2 (&F)[9], const float *cf, C2 (&out)[9])
{
  const float w1 = 2.f * cf[1], w2 = 2.f * cf[2], w3 = 2.f * cf[3], w4 = 2.f * cf[4], w5 = 2.f * cf[5];
  const float wp = w4 + w5, wm = w4 - w5;
  // left factors of the real and imaginary parts of the right factor (A for role 0, F for
  // role 1), as separate real and imaginary arrays: the complex-by-complex products below
  // run as scalar FMAs
  float Lr[9], Li[9], Rr[9], Ri[9];
  if constexpr (ROLE == 0)
    {
      float dpr = 0.f, dpi = 0.f, dq = 0.f;
#pragma unroll
      for (int k = 0; k < 9; ++k)
        {
          dpr = fmaf(A[k].x, F[k].x, fmaf(-A[k].y, F[k].y, dpr));
          dpi = fmaf(A[k].x, F[k].y, fmaf(A[k].y, F[k].x, dpi));
          dq = fmaf(A[k].x, F[k].x, fmaf(A[k].y, F[k].y, dq));
        }
      // Y2 in L: S3 = A F^T, symmetrised
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          {
            float sr = 0.f, si = 0.f;
#pragma unroll
            for (int k = 0; k < 3; ++k)
              {
                const C2 a = A[3 * i + k], f = F[3 * j + k];
                sr = fmaf(a.x, f.x, fmaf(-a.y, f.y, sr));
                si = fmaf(a.x, f.y, fmaf(a.y, f.x, si));
              }
            Lr[3 * i + j] = sr;
            Li[3 * i + j] = si;
          }
#pragma unroll
      for (int i = 0; i < 3; ++i)
        {
#pragma unroll
          for (int j = i + 1; j < 3; ++j)
            {
              const float sr = w3 * (Lr[3 * i + j] + Lr[3 * j + i]), si = w3 * (Li[3 * i + j] + Li[3 * j + i]);
              Lr[3 * i + j] = Lr[3 * j + i] = sr;
              Li[3 * i + j] = Li[3 * j + i] = si;
            }
          Lr[4 * i] = fmaf(2.f * w3, Lr[4 * i], 2.f * w1 * dpr);
          Li[4 * i] = fmaf(2.f * w3, Li[4 * i], 2.f * w1 * dpi);
        }
      // Y1 in R: S4 = F A^+; Re part (w4 + w5)(Sr + Sr^T), Im part (w4 - w5)(Si - Si^T)
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          {
            float sr = 0.f, si = 0.f;
#pragma unroll
            for (int k = 0; k < 3; ++k)
              {
                const C2 f = F[3 * i + k], a = A[3 * j + k];
                sr = fmaf(f.x, a.x, fmaf(f.y, a.y, sr));
                si = fmaf(f.y, a.x, fmaf(-f.x, a.y, si));
              }
            Rr[3 * i + j] = sr;
            Ri[3 * i + j] = si;
          }
#pragma unroll
      for (int i = 0; i < 3; ++i)
        {
#pragma unroll
          for (int j = i + 1; j < 3; ++j)
            {
              const float sr = wp * (Rr[3 * i + j] + Rr[3 * j + i]);
              const float si = wm * (Ri[3 * i + j] - Ri[3 * j + i]);
              Rr[3 * i + j] = Rr[3 * j + i] = sr;
              Ri[3 * i + j] = si;
              Ri[3 * j + i] = -si;
            }
          Rr[4 * i] = fmaf(2.f * wp, Rr[4 * i], 2.f * w2 * dq);
          Ri[4 * i] = 0.f;
        }
      // (Y1 + Y2) in L and i (Y1 - Y2) in R
#pragma unroll
      for (int k = 0; k < 9; ++k)
        {
          const float y1r = Rr[k], y1i = Ri[k], y2r = Lr[k], y2i = Li[k];
          Lr[k] = y1r + y2r;
          Li[k] = y1i + y2i;
          Rr[k] = y2i - y1i;
          Ri[k] = y1r - y2r;
        }
    }
  else
    {
      float pr = 0.f, pi = 0.f, q = 0.f;
#pragma unroll
      for (int k = 0; k < 9; ++k)
        {
          pr = fmaf(A[k].x, A[k].x, fmaf(-A[k].y, A[k].y, pr));
          pi = fmaf(2.f * A[k].x, A[k].y, pi);
          q = fmaf(A[k].x, A[k].x, fmaf(A[k].y, A[k].y, q));
        }
      // M in L, N in R
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = i; j < 3; ++j)
          {
            float Pr = 0.f, Pi = 0.f, Qr = 0.f, Qi = 0.f;
#pragma unroll
            for (int k = 0; k < 3; ++k)
              {
                const C2 a = A[3 * i + k], b = A[3 * j + k];
                Pr = fmaf(a.x, b.x, fmaf(-a.y, b.y, Pr));
                Pi = fmaf(a.x, b.y, fmaf(a.y, b.x, Pi));
                Qr = fmaf(a.x, b.x, fmaf(a.y, b.y, Qr));
                Qi = fmaf(a.y, b.x, fmaf(-a.x, b.y, Qi));
              }
            if (i == j)
              {
                Lr[4 * i] = cf[0] + w2 * q + wp * Qr;
                Li[4 * i] = 0.f;
                Rr[4 * i] = fmaf(w3, Pr, w1 * pr);
                Ri[4 * i] = fmaf(w3, Pi, w1 * pi);
              }
            else
              {
                Lr[3 * i + j] = Lr[3 * j + i] = wp * Qr;
                Li[3 * i + j] = wm * Qi;
                Li[3 * j + i] = -wm * Qi;
                Rr[3 * i + j] = Rr[3 * j + i] = w3 * Pr;
                Ri[3 * i + j] = Ri[3 * j + i] = w3 * Pi;
              }
          }
#pragma unroll
      for (int k = 0; k < 9; ++k)
        {
          const float mr = Lr[k], mi = Li[k], nr = Rr[k], ni = Ri[k];
          Lr[k] = mr + nr;
          Li[k] = mi + ni;
          Rr[k] = ni - mi;
          Ri[k] = mr - nr;
        }
    }
  // out = L Re(B) + R Im(B): complex-by-real products, each real entry of B broadcast to a
  // pair once and used for the three rows
  const C2(&B)[9] = ROLE == 0 ? A : F;
#pragma unroll
  for (int k = 0; k < 9; ++k) out[k] = c2(0.f, 0.f);
#pragma unroll
  for (int k = 0; k < 3; ++k)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      {
        const C2 br = c2(B[3 * k + j].x, B[3 * k + j].x), bi = c2(B[3 * k + j].y, B[3 * k + j].y);
#pragma unroll
        for (int i = 0; i < 3; ++i)
          {
            out[3 * i + j] = __ffma2_rn(c2(Lr[3 * i + k], Li[3 * i + k]), br, out[3 * i + j]);
            out[3 * i + j] = __ffma2_rn(c2(Rr[3 * i + k], Ri[3 * i + k]), bi, out[3 * i + j]);
          }
      }
}

// r[a] = sum_q val_q(a) w[q] + sum_k sum_q dval_q(a)/dxi_k F_k[q] (reference cube), a = ax + 2 ay + 4 az:
// the transposed interpolation, sum-factorised axis by axis, on component pairs
__device__ __forceinline__ void mf_contract(const C2 (&w)[8], const C2 (&F)[3][8], C2 (&r)[8])
{
  {
    C2 tx[2][4];
#pragma unroll
    for (int t = 0; t < 4; ++t) gauss2(w[2 * t], w[2 * t + 1], tx[0][t], tx[1][t]);
    C2 ty[2][2][2];
#pragma unroll
    for (int ax = 0; ax < 2; ++ax)
#pragma unroll
      for (int qz = 0; qz < 2; ++qz) gauss2(tx[ax][2 * qz], tx[ax][2 * qz + 1], ty[ax][0][qz], ty[ax][1][qz]);
#pragma unroll
    for (int ax = 0; ax < 2; ++ax)
#pragma unroll
      for (int ay = 0; ay < 2; ++ay) gauss2(ty[ax][ay][0], ty[ax][ay][1], r[ax + 2 * ay], r[ax + 2 * ay + 4]);
  }
  {
    C2 sx[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) sx[t] = add2(F[0][2 * t], F[0][2 * t + 1]);
    C2 uy[2][2];
#pragma unroll
    for (int qz = 0; qz < 2; ++qz) gauss2(sx[2 * qz], sx[2 * qz + 1], uy[0][qz], uy[1][qz]);
#pragma unroll
    for (int ay = 0; ay < 2; ++ay)
      {
        C2 v0, v1;
        gauss2(uy[ay][0], uy[ay][1], v0, v1);
        r[1 + 2 * ay] = add2(r[1 + 2 * ay], v0);
        r[2 * ay] = sub2(r[2 * ay], v0);
        r[5 + 2 * ay] = add2(r[5 + 2 * ay], v1);
        r[4 + 2 * ay] = sub2(r[4 + 2 * ay], v1);
      }
  }
  {
    C2 sy[4];
#pragma unroll
    for (int qz = 0; qz < 2; ++qz)
#pragma unroll
      for (int qx = 0; qx < 2; ++qx) sy[qx + 2 * qz] = add2(F[1][qx + 4 * qz], F[1][qx + 2 + 4 * qz]);
    C2 ux[2][2];
#pragma unroll
    for (int qz = 0; qz < 2; ++qz) gauss2(sy[2 * qz], sy[2 * qz + 1], ux[0][qz], ux[1][qz]);
#pragma unroll
    for (int ax = 0; ax < 2; ++ax)
      {
        C2 v0, v1;
        gauss2(ux[ax][0], ux[ax][1], v0, v1);
        r[ax + 2] = add2(r[ax + 2], v0);
        r[ax] = sub2(r[ax], v0);
        r[ax + 6] = add2(r[ax + 6], v1);
        r[ax + 4] = sub2(r[ax + 4], v1);
      }
  }
  {
    C2 sz[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) sz[t] = add2(F[2][t], F[2][t + 4]);
    C2 ux[2][2];
#pragma unroll
    for (int qy = 0; qy < 2; ++qy) gauss2(sz[2 * qy], sz[2 * qy + 1], ux[0][qy], ux[1][qy]);
#pragma unroll
    for (int ax = 0; ax < 2; ++ax)
      {
        C2 v0, v1;
        gauss2(ux[ax][0], ux[ax][1], v0, v1);
        r[ax + 4] = add2(r[ax + 4], v0);
        r[ax] = sub2(r[ax], v0);
        r[ax + 6] = add2(r[ax + 6], v1);
        r[ax + 2] = sub2(r[ax + 2], v1);
      }
  }
}

// A, Z and dZ/dx at the points from the nodal values: thread (cell, component pair)
template <int NC, int PLD>
__device__ __forceinline__ void mf_points(const MfView<NC, PLD> &v, int tid)
{
  if (tid >= NC * 9) return;
  const int cl = tid / 9, cp = tid - 9 * cl;
  auto zval = [&](int t, int c) -> float { return v.zs[cl][t][c]; };
  {
    C2 aq[2][4];
#pragma unroll
    for (int t = 0; t < 4; ++t)
      gauss2(c2(v.xs[cl][t][cp], v.xs[cl][t][cp + 9]), c2(v.xs[cl][t + 4][cp], v.xs[cl][t + 4][cp + 9]), aq[0][t],
             aq[1][t]);
#pragma unroll
    for (int qz = 0; qz < 2; ++qz)
#pragma unroll
      for (int vx = 0; vx < 2; ++vx)
        {
          C2 y0, y1;
          gauss2(aq[qz][vx], aq[qz][2 + vx], y0, y1);
          aq[qz][vx] = y0;
          aq[qz][2 + vx] = y1;
        }
#pragma unroll
    for (int qz = 0; qz < 2; ++qz)
#pragma unroll
      for (int qy = 0; qy < 2; ++qy)
        {
          C2 v0, v1;
          gauss2(aq[qz][2 * qy], aq[qz][2 * qy + 1], v0, v1);
          const int p0 = cl * 8 + 2 * qy + 4 * qz;
          reinterpret_cast<float2 *>(v.X[p0])[cp] = v0;
          reinterpret_cast<float2 *>(v.X[p0 + 1])[cp] = v1;
        }
  }
  C2 zq[2][4], zd[4];
#pragma unroll
  for (int t = 0; t < 4; ++t)
    {
      const C2 f0 = c2(zval(t, cp), zval(t, cp + 9));
      const C2 f1 = c2(zval(t + 4, cp), zval(t + 4, cp + 9));
      gauss2(f0, f1, zq[0][t], zq[1][t]);
      zd[t] = sub2(f1, f0);
    }
  C2 yq[2][2][2], ydy[2][2], zdq[2][2];
#pragma unroll
  for (int vx = 0; vx < 2; ++vx)
    {
#pragma unroll
      for (int qz = 0; qz < 2; ++qz)
        {
          gauss2(zq[qz][vx], zq[qz][2 + vx], yq[qz][0][vx], yq[qz][1][vx]);
          ydy[qz][vx] = sub2(zq[qz][2 + vx], zq[qz][vx]);
        }
      gauss2(zd[vx], zd[2 + vx], zdq[0][vx], zdq[1][vx]);
    }
  const float i0 = v.par[cl][kParIh], i1 = v.par[cl][kParIh + 1], i2 = v.par[cl][kParIh + 2];
#pragma unroll
  for (int qz = 0; qz < 2; ++qz)
#pragma unroll
    for (int qy = 0; qy < 2; ++qy)
      {
        C2 v0, v1;
        gauss2(yq[qz][qy][0], yq[qz][qy][1], v0, v1);
        const C2 dx = scl2(sub2(yq[qz][qy][1], yq[qz][qy][0]), i0);
        const int p0 = cl * 8 + 2 * qy + 4 * qz;
        reinterpret_cast<float2 *>(v.Z[p0])[cp] = v0;
        reinterpret_cast<float2 *>(v.Z[p0 + 1])[cp] = v1;
        reinterpret_cast<float2 *>(v.gZ[p0][0])[cp] = dx;
        reinterpret_cast<float2 *>(v.gZ[p0 + 1][0])[cp] = dx;
      }
#pragma unroll
  for (int qz = 0; qz < 2; ++qz)
    {
      C2 d0, d1;
      gauss2(ydy[qz][0], ydy[qz][1], d0, d1);
#pragma unroll
      for (int qy = 0; qy < 2; ++qy)
        {
          const int p0 = cl * 8 + 2 * qy + 4 * qz;
          reinterpret_cast<float2 *>(v.gZ[p0][1])[cp] = scl2(d0, i1);
          reinterpret_cast<float2 *>(v.gZ[p0 + 1][1])[cp] = scl2(d1, i1);
        }
    }
#pragma unroll
  for (int qy = 0; qy < 2; ++qy)
    {
      C2 d0, d1;
      gauss2(zdq[qy][0], zdq[qy][1], d0, d1);
#pragma unroll
      for (int qz = 0; qz < 2; ++qz)
        {
          const int p0 = cl * 8 + 2 * qy + 4 * qz;
          reinterpret_cast<float2 *>(v.gZ[p0][2])[cp] = scl2(d0, i2);
          reinterpret_cast<float2 *>(v.gZ[p0 + 1][2])[cp] = scl2(d1, i2);
        }
    }
}

// H Z at each point in two shares: thread (role, point), role uniform over a warp for NC >= 4
template <int NC, int PLD>
__device__ __forceinline__ void mf_products(const MfView<NC, PLD> &v, int tid, int ncb)
{
  constexpr int kMPts = 8 * NC;
  const int role = tid / kMPts, pq = tid - role * kMPts, cl = pq >> 3;
  if (cl >= ncb) return;
  C2 A[9], F[9], out[9];
  load_c9(v.X[pq], A);
  load_c9(v.Z[pq], F);
  float cf[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) cf[k] = v.par[cl][kParBulk + k];
  if (role == 0)
    hvp_role<0>(A, F, cf, out);
  else
    hvp_role<1>(A, F, cf, out);
  float2 *row = reinterpret_cast<float2 *>(v.part[role][pq]);
#pragma unroll
  for (int k = 0; k < 9; ++k) row[k] = out[k];
}

// contraction with the test functions and the cell results: thread (cell, component pair)
template <int NC, int PLD>
__device__ __forceinline__ void mf_contract_store(const MfView<NC, PLD> &v, int tid, int ncb, float *__restrict__ yc)
{
  if (tid >= NC * 9) return;
  const int cl = tid / 9, cp = tid - 9 * cl;
  const int mu = cp / 3, jc = cp % 3;
  const float K1 = v.par[cl][kParK1], K23 = v.par[cl][kParK23];
  const float ih[3] = {v.par[cl][kParIh], v.par[cl][kParIh + 1], v.par[cl][kParIh + 2]};
  C2 w[8], F[3][8];
#pragma unroll
  for (int q = 0; q < 8; ++q)
    {
      const int pq = cl * 8 + q;
      w[q] = add2(reinterpret_cast<const float2 *>(v.part[0][pq])[cp], reinterpret_cast<const float2 *>(v.part[1][pq])[cp]);
      const C2 dv = scl2(add2(add2(reinterpret_cast<const float2 *>(v.gZ[pq][0])[3 * mu],
                                   reinterpret_cast<const float2 *>(v.gZ[pq][1])[3 * mu + 1]),
                              reinterpret_cast<const float2 *>(v.gZ[pq][2])[3 * mu + 2]),
                         K23);
#pragma unroll
      for (int k = 0; k < 3; ++k)
        {
          C2 g = scl2(reinterpret_cast<const float2 *>(v.gZ[pq][k])[cp], K1);
          if (k == jc) g = add2(g, dv);
          F[k][q] = scl2(g, ih[k]);
        }
    }
  C2 r[8];
  mf_contract(w, F, r);
  if (cl < ncb)
    {
      const float jxw = v.par[cl][kParJxw];
      float *out = yc + cl * 144 + cp;
#pragma unroll
      for (int a = 0; a < 8; ++a)
        {
          out[18 * a] = r[a].x * jxw;
          out[18 * a + 9] = r[a].y * jxw;
        }
    }
}

// per-cell constants of cell e into p (zeros past the mesh)
__device__ __forceinline__ void mf_cell_par(const DevMesh &m, int64_t e, float (&p)[kPar])
{
#pragma unroll
  for (int k = 0; k < kPar; ++k) p[k] = 0.f;
  if (e >= m.nc) return;
  const int inst = m.cell_inst[e];
  const float4 g = m.geo_f[e];
  p[kParIh] = g.x;
  p[kParIh + 1] = g.y;
  p[kParIh + 2] = g.z;
  p[kParJxw] = 0.125f * g.w;
  p[kParK1] = m.coef_f[inst * kCoef + 0];
  p[kParK23] = m.coef_f[inst * kCoef + 1];
#pragma unroll
  for (int k = 0; k < 6; ++k) p[kParBulk + k] = m.coef_f[inst * kCoef + 2 + k];
}

// One CTA per NC cells.
template <int NC>
__global__ void __launch_bounds__(16 * NC, 40 / NC) k_mf_cell(DevMesh m, const float *__restrict__ xs,
                                                        const float *__restrict__ z, float *__restrict__ ycell,
                                                        const uint8_t *__restrict__ act)
{
  pdl_wait();
  pdl_trigger();
  constexpr int kMCells = NC, kMThreads = 16 * NC;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  MfSmem<NC> &S = *reinterpret_cast<MfSmem<NC> *>(smem_raw);
  const int tid = threadIdx.x;
  const int64_t e0 = static_cast<int64_t>(blockIdx.x) * kMCells;
  const int ncb = static_cast<int>((m.nc - e0) < kMCells ? (m.nc - e0) : kMCells);
  if (act)
    {
      // a CTA whose cells all belong to inactive instances (converged, or waiting in a
      // batched solve) has nothing to contribute: the gather skips their nodes
      if (!__syncthreads_or(tid < ncb && act[m.cell_inst[e0 + tid]])) return;
    }
  if (tid < kMCells)
    {
      float p[kPar];
      mf_cell_par(m, e0 + tid, p);
#pragma unroll
      for (int k = 0; k < kPar; ++k) S.par[tid][k] = p[k];
    }
  // nodal values: the 16 threads of cell cl = tid / 16 take its vertices two per vertex;
  // half h of vertex a loads the float2 pairs j0 = 5 h .. 4 + 4 h of the vertex's 18 values
  // (a row is 72 bytes, 8-byte aligned) and the vertex's component mask once.  Constraint
  // rows (hanging nodes, periodic images) are expanded from their parents.
  {
    static_assert(kMThreads == 16 * kMCells, "16 threads per cell");
    const int cl = tid >> 4, a = (tid & 15) >> 1, h = tid & 1;
    const int j0 = 5 * h, nj = 5 - h;
    const int node = (cl < ncb) ? m.cells[(e0 + cl) * 8 + a] : -1;
    float2 zv[5], xv[5];
    uint32_t mk = ~0u;
    if (node >= 0)
      {
        const float2 *zr = reinterpret_cast<const float2 *>(z + static_cast<int64_t>(node) * 18) + j0;
        const float2 *xr = reinterpret_cast<const float2 *>(xs + static_cast<int64_t>(node) * 18) + j0;
#pragma unroll
        for (int q = 0; q < 5; ++q)
          if (q < nj)
            {
              zv[q] = zr[q];
              xv[q] = xr[q];
            }
        mk = m.mask[node];
      }
    else
#pragma unroll
      for (int q = 0; q < 5; ++q) zv[q] = xv[q] = make_float2(0.f, 0.f);
    const bool hang = m.has_constraints && node >= 0 && m.hptr[node + 1] > m.hptr[node];
    float2 *zs2 = reinterpret_cast<float2 *>(&S.u.g.zs[cl][a][0]) + j0;
    float2 *xs2 = reinterpret_cast<float2 *>(&S.u.g.xs[cl][a][0]) + j0;
#pragma unroll
    for (int q = 0; q < 5; ++q)
      if (q < nj)
        {
          const int c = 2 * (j0 + q);
          float2 val = make_float2(((mk >> c) & 1u) ? 0.f : zv[q].x, ((mk >> (c + 1)) & 1u) ? 0.f : zv[q].y);
          if (hang)
            {
              val = make_float2(0.f, 0.f);
              for (int k = m.hptr[node]; k < m.hptr[node + 1]; ++k)
                {
                  // a parent's zero-Dirichlet components do not enter
                  const int par = m.hpar[k];
                  const uint32_t pm = m.mask[par];
                  const float w = static_cast<float>(m.hw[k]);
                  const float2 pv = reinterpret_cast<const float2 *>(z + static_cast<int64_t>(par) * 18)[j0 + q];
                  if (!((pm >> c) & 1u)) val.x += w * pv.x;
                  if (!((pm >> (c + 1)) & 1u)) val.y += w * pv.y;
                }
            }
          zs2[q] = val;
          xs2[q] = xv[q]; // the state is stored distributed: vertex values as they are
        }
  }
  __syncthreads();
  const MfView<NC, 20> v = {S.u.g.zs, S.u.g.xs, S.X, S.Z, S.gZ, S.u.part, S.par};
  mf_points<NC, 20>(v, tid);
  __syncthreads(); // X, Z, gZ complete; the gathered nodal values are no longer read
  mf_products<NC, 20>(v, tid, ncb);
  __syncthreads();
  mf_contract_store<NC, 20>(v, tid, ncb, ycell + e0 * 144);
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
                                                          const __half *__restrict__ dinv, float *__restrict__ y,
                                                          float omega, int mode, const uint8_t *__restrict__ act)
{
  pdl_wait();
  pdl_trigger();
  __shared__ float t_s[kMgNodes][18];
  const int ln = threadIdx.x / 18, c = threadIdx.x - 18 * (threadIdx.x / 18);
  const int64_t n = static_cast<int64_t>(blockIdx.x) * kMgNodes + ln;
  const bool on = n < m.nn && !(act && !act[m.node_inst[n]]);
  float s = 0.f;
  if (on && m.rc_off8)
    {
      // meshes without constraint rows: the node's (at most 8) contribution offsets in one
      // 32-byte load, then the values; the same additions in the same order as the list path
      // (weight 1, padded slots add 0)
      const int4 *op = reinterpret_cast<const int4 *>(m.rc_off8 + n * 8);
      const int4 o0 = __ldg(op), o1 = __ldg(op + 1);
      const int off[8] = {o0.x, o0.y, o0.z, o0.w, o1.x, o1.y, o1.z, o1.w};
      float v[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) v[k] = (off[k] >= 0) ? __ldg(ycell + off[k] + c) : 0.f;
#pragma unroll
      for (int k = 0; k < 8; ++k) s = fmaf(off[k] >= 0 ? 1.f : 0.f, v[k], s);
      if ((m.mask[n] >> c) & 1u) s = z[n * 18 + c];
    }
  else if (on)
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
  // the row's 18 FP16 entries: 36 bytes at a 4-byte boundary, nine half2 loads
  const __half2 *row = reinterpret_cast<const __half2 *>(dinv + n * 324 + c * 18);
  float u = 0.f;
#pragma unroll
  for (int d = 0; d < 9; ++d)
    {
      const float2 w = __half22float2(__ldg(row + d));
      u = fmaf(w.x, t_s[ln][2 * d], u);
      u = fmaf(w.y, t_s[ln][2 * d + 1], u);
    }
  y[n * 18 + c] = z[n * 18 + c] + omega * u;
}

// Robin faces in the matrix-free operator: ycell[e] += W z_e for the Robin cells, z_e the
// cell's vertex values expanded through the constraints and column masks exactly as
// k_mf_cell reads them (one CTA per Robin cell, thread = (vertex, component)).
constexpr int kRobinMfThreads = 160;

__global__ void __launch_bounds__(kRobinMfThreads) k_robin_mf(DevMesh m, const float *__restrict__ z,
                                                              float *__restrict__ ycell, const uint8_t *__restrict__ act)
{
  pdl_wait();
  pdl_trigger();
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
  pdl_launch(k_robin_mf, static_cast<unsigned>(m.n_robin), kRobinMfThreads, 0, s, m, z, ycell, act);
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
  pdl_launch(k_mf_cell<NC>, static_cast<unsigned>(gc), 16 * NC, sizeof(MfSmem<NC>), s, m, xs, z, ycell, act);
  return cudaGetLastError();
}

cudaError_t launch_mf(const DevMesh &m, const float *xs, const float *z, float *ycell, float *y, const float *b,
                      const __half *dinv, float omega, int mode, const uint8_t *act, cudaStream_t s,
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
  pdl_launch(k_mf_gather, static_cast<unsigned>(gn), kMgThreads, 0, s, m, ycell, z, b, dinv, y, omega, mode, act);
  return cudaGetLastError();
}

} // namespace glgpu
