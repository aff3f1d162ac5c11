// Assembly kernels (sm_103a).
//
// The reference assembles the Jacobian by evaluating nine FullMatrix kernels for
// every (test dof i, trial dof j, quadrature point q) of every cell, 165,888 tuples
// per Q1 hexahedron (femgl/src/assemble.cc:188-280).  Here the same matrix comes in
// two passes that touch HBM once each:
//
//  1. k_cell3d: one CTA per 4 cells.  Nodal 18-vectors are gathered into shared
//     memory, A and grad A are interpolated at the 8 Gauss points, and for every
//     point the 171 unique entries of the symmetric bulk Hessian
//     H_q = alpha I + 2 sum_t beta_t d^2(I_t/4) are written out ([cell][171][q]),
//     together with the cell residual and free energy when asked.
//  2. k_rows3d_reg / k_rows3d: one CTA per block row.  Every cell touching the row
//     contributes block(a,b) = vol sum_q S_abq H_q + K1 G_ab + (K2+K3) D_ab; full
//     interior rows accumulate their 27 blocks in registers at compile-time slots,
//     the other rows (boundary, constrained) in shared memory at slots precomputed on
//     the host.  Each row is written once, contiguously.  No atomics, no colouring.
//
// The per-q formulas are the closed forms of the reference's kernels: the
// quarter-gradient of invariant I_t is Re<G_t, Phi> with G1 = tr(AA^T) A^*,
// G2 = tr(AA^+) A, G3 = AA^T A^*, G4 = AA^+ A, G5 = (AA^+)^* A, and the Hessian
// entries are the directional derivatives of G_t along unit directions.
#include <cstdint>
#include <cuda_runtime.h>

#include "device.h"
#include "dfloat.h"
#include "glgpu_internal.h"

namespace glgpu
{
// ---------------------------------------------------------------------------------
// reference-element tables (unit cube, QGauss(2), q = qx + 2 qy + 4 qz)
// ---------------------------------------------------------------------------------
__constant__ double c_val3[8][8];    // [q][v]
__constant__ double c_grd3[8][8][3]; // [q][v][k] derivative on the unit cube
__constant__ double c_S3[8][8][8];   // [a][b][q] = val[q][a] val[q][b] / 8
__constant__ double c_D3[8][8][9];   // [a][b][3j+k] = (1/8) sum_q grd[q][a][j] grd[q][b][k]
__constant__ float c_val3f[8][8];
__constant__ float c_grd3f[8][8][3];
__constant__ float c_S3f[8][8][8];
__constant__ float c_D3f[8][8][9];
__constant__ unsigned char c_symc[kNS3], c_symd[kNS3];
__constant__ double c_val2[4][4];
__constant__ double c_grd2[4][4][2];
__constant__ double c_S2[4][4][4];
__constant__ double c_D2[4][4][4];

cudaError_t init_constants()
{
  const double g = 0.5 - 0.28867513459481288225; // 1/2 - sqrt(3)/6
  const double gp[2] = {g, 1.0 - g};
  double val3[8][8], grd3[8][8][3], S3[8][8][8], D3[8][8][9];
  for (int q = 0; q < 8; ++q)
    {
      const double xi[3] = {gp[q & 1], gp[(q >> 1) & 1], gp[(q >> 2) & 1]};
      for (int v = 0; v < 8; ++v)
        {
          double s[3], ds[3];
          for (int d = 0; d < 3; ++d)
            {
              const int bit = (v >> d) & 1;
              s[d] = bit ? xi[d] : 1.0 - xi[d];
              ds[d] = bit ? 1.0 : -1.0;
            }
          val3[q][v] = s[0] * s[1] * s[2];
          grd3[q][v][0] = ds[0] * s[1] * s[2];
          grd3[q][v][1] = s[0] * ds[1] * s[2];
          grd3[q][v][2] = s[0] * s[1] * ds[2];
        }
    }
  for (int a = 0; a < 8; ++a)
    for (int b = 0; b < 8; ++b)
      {
        for (int q = 0; q < 8; ++q) S3[a][b][q] = val3[q][a] * val3[q][b] * 0.125;
        for (int j = 0; j < 3; ++j)
          for (int k = 0; k < 3; ++k)
            {
              double s = 0;
              for (int q = 0; q < 8; ++q) s += grd3[q][a][j] * grd3[q][b][k];
              D3[a][b][3 * j + k] = 0.125 * s;
            }
      }
  unsigned char sc[kNS3], sd[kNS3];
  int t = 0;
  for (int c = 0; c < 18; ++c)
    for (int d = c; d < 18; ++d)
      {
        sc[t] = static_cast<unsigned char>(c);
        sd[t] = static_cast<unsigned char>(d);
        ++t;
      }
  double val2[4][4], grd2[4][4][2], S2[4][4][4], D2[4][4][4];
  for (int q = 0; q < 4; ++q)
    {
      const double xi[2] = {gp[q & 1], gp[(q >> 1) & 1]};
      for (int v = 0; v < 4; ++v)
        {
          double s[2], ds[2];
          for (int d = 0; d < 2; ++d)
            {
              const int bit = (v >> d) & 1;
              s[d] = bit ? xi[d] : 1.0 - xi[d];
              ds[d] = bit ? 1.0 : -1.0;
            }
          val2[q][v] = s[0] * s[1];
          grd2[q][v][0] = ds[0] * s[1];
          grd2[q][v][1] = s[0] * ds[1];
        }
    }
  for (int a = 0; a < 4; ++a)
    for (int b = 0; b < 4; ++b)
      {
        for (int q = 0; q < 4; ++q) S2[a][b][q] = val2[q][a] * val2[q][b] * 0.25;
        for (int j = 0; j < 2; ++j)
          for (int k = 0; k < 2; ++k)
            {
              double s = 0;
              for (int q = 0; q < 4; ++q) s += grd2[q][a][j] * grd2[q][b][k];
              D2[a][b][2 * j + k] = 0.25 * s;
            }
      }
  float val3f[8][8], grd3f[8][8][3], S3f[8][8][8], D3f[8][8][9];
  for (int i = 0; i < 64; ++i) (&val3f[0][0])[i] = static_cast<float>((&val3[0][0])[i]);
  for (int i = 0; i < 192; ++i) (&grd3f[0][0][0])[i] = static_cast<float>((&grd3[0][0][0])[i]);
  for (int i = 0; i < 512; ++i) (&S3f[0][0][0])[i] = static_cast<float>((&S3[0][0][0])[i]);
  for (int i = 0; i < 576; ++i) (&D3f[0][0][0])[i] = static_cast<float>((&D3[0][0][0])[i]);
  cudaError_t e;
  if ((e = cudaMemcpyToSymbol(c_val3f, val3f, sizeof val3f)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(c_grd3f, grd3f, sizeof grd3f)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(c_S3f, S3f, sizeof S3f)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(c_D3f, D3f, sizeof D3f)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(c_val3, val3, sizeof val3)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(c_grd3, grd3, sizeof grd3)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(c_S3, S3, sizeof S3)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(c_D3, D3, sizeof D3)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(c_symc, sc, sizeof sc)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(c_symd, sd, sizeof sd)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(c_val2, val2, sizeof val2)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(c_grd2, grd2, sizeof grd2)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(c_S2, S2, sizeof S2)) != cudaSuccess) return e;
  return cudaMemcpyToSymbol(c_D2, D2, sizeof D2);
}

void regular_row_stiffness(double K1, double K23, const double *h, double *out)
{
  const double g = 0.5 - 0.28867513459481288225;
  const double gp[2] = {g, 1.0 - g};
  double grd[8][8][3];
  for (int q = 0; q < 8; ++q)
    {
      const double xi[3] = {gp[q & 1], gp[(q >> 1) & 1], gp[(q >> 2) & 1]};
      for (int v = 0; v < 8; ++v)
        {
          double s3[3], ds[3];
          for (int d = 0; d < 3; ++d)
            {
              const int bit = (v >> d) & 1;
              s3[d] = bit ? xi[d] : 1.0 - xi[d];
              ds[d] = bit ? 1.0 : -1.0;
            }
          grd[q][v][0] = ds[0] * s3[1] * s3[2];
          grd[q][v][1] = s3[0] * ds[1] * s3[2];
          grd[q][v][2] = s3[0] * s3[1] * ds[2];
        }
    }
  const double vol = h[0] * h[1] * h[2];
  const double ih[3] = {1.0 / h[0], 1.0 / h[1], 1.0 / h[2]};
  for (int i = 0; i < 27 * 324; ++i) out[i] = 0.0;
  for (int a = 0; a < 8; ++a)
    for (int b = 0; b < 8; ++b)
      {
        double D[9];
        for (int j = 0; j < 3; ++j)
          for (int k = 0; k < 3; ++k)
            {
              double sum = 0;
              for (int q = 0; q < 8; ++q) sum += grd[q][a][j] * grd[q][b][k];
              D[3 * j + k] = 0.125 * sum;
            }
        const int sl = 13 + ((b & 1) - (a & 1)) + 3 * (((b >> 1) & 1) - ((a >> 1) & 1)) + 9 * (((b >> 2) & 1) - ((a >> 2) & 1));
        const double kd = K1 * vol * (D[0] * ih[0] * ih[0] + D[4] * ih[1] * ih[1] + D[8] * ih[2] * ih[2]);
        for (int c = 0; c < 18; ++c)
          for (int d = 0; d < 18; ++d)
            {
              double v = (c == d) ? kd : 0.0;
              const int pmc = 3 * (c / 9) + (c % 9) / 3, jc = c % 3, pmd = 3 * (d / 9) + (d % 9) / 3, jd = d % 3;
              if (pmc == pmd) v += K23 * vol * ih[jc] * ih[jd] * D[3 * jc + jd];
              out[sl * 324 + c * 18 + d] += v;
            }
      }
}

// typed access to the tables, geometry and weights: FP32 kernels read FP32 copies
template <typename T> struct Tab;
template <> struct Tab<float>
{
  static __device__ __forceinline__ float val(int q, int v) { return c_val3f[q][v]; }
  static __device__ __forceinline__ float grd(int q, int v, int k) { return c_grd3f[q][v][k]; }
  static __device__ __forceinline__ float S(int a, int b, int q) { return c_S3f[a][b][q]; }
  static __device__ __forceinline__ const float *D() { return &c_D3f[0][0][0]; }
  static __device__ __forceinline__ float4 geo(const DevMesh &m, int64_t e) { return m.geo_f[e]; }
  static __device__ __forceinline__ float coef(const DevMesh &m, int inst, int k) { return m.coef_f[inst * kCoef + k]; }
  static __device__ __forceinline__ float w(const DevMesh &m, int64_t k) { return m.rc_wf[k]; }
  static __device__ __forceinline__ const float *tmpl(const DevMesh &m) { return m.reg_tmpl_f; }
};
template <> struct Tab<double>
{
  static __device__ __forceinline__ double val(int q, int v) { return c_val3[q][v]; }
  static __device__ __forceinline__ double grd(int q, int v, int k) { return c_grd3[q][v][k]; }
  static __device__ __forceinline__ double S(int a, int b, int q) { return c_S3[a][b][q]; }
  static __device__ __forceinline__ const double *D() { return &c_D3[0][0][0]; }
  static __device__ __forceinline__ GeoD geo(const DevMesh &m, int64_t e) { return m.geo_d[e]; }
  static __device__ __forceinline__ double coef(const DevMesh &m, int inst, int k) { return m.coef[inst * kCoef + k]; }
  static __device__ __forceinline__ double w(const DevMesh &m, int64_t k) { return m.rc_w[k]; }
  static __device__ __forceinline__ const double *tmpl(const DevMesh &m) { return m.reg_tmpl_d; }
};

// ---------------------------------------------------------------------------------
// small complex helpers
// ---------------------------------------------------------------------------------
template <typename T> struct cx
{
  T r, i;
};
template <typename T> __device__ __forceinline__ cx<T> cmul(cx<T> a, cx<T> b)
{
  return {a.r * b.r - a.i * b.i, a.r * b.i + a.i * b.r};
}
template <typename T> __device__ __forceinline__ cx<T> cconj(cx<T> a) { return {a.r, -a.i}; }
template <typename T> __device__ __forceinline__ cx<T> cadd(cx<T> a, cx<T> b) { return {a.r + b.r, a.i + b.i}; }
template <typename T> __device__ __forceinline__ cx<T> cscale(cx<T> a, T s) { return {a.r * s, a.i * s}; }
// multiply by s = 1 (v == 0) or s = i (v == 1)
template <typename T> __device__ __forceinline__ cx<T> mul_s(cx<T> a, int v)
{
  return v ? cx<T>{-a.i, a.r} : a;
}
// multiply by conj(s)
template <typename T> __device__ __forceinline__ cx<T> mul_cs(cx<T> a, int v)
{
  return v ? cx<T>{a.i, -a.r} : a;
}

// per-(cell, q) state in shared memory: complex 3x3 matrices stored as re[9], im[9]
template <typename T> struct QS
{
  T *A;   // [18]: re 0..8, im 9..17 (the 18-vector packing)
  T *P;   // A A^T
  T *Q;   // A A^+
  T *M2;  // A^+ A
  T *M3;  // A^T A
  T *pq;  // p.r, p.i, q
};
template <typename T> __device__ __forceinline__ cx<T> at(const T *M, int i, int j)
{
  return {M[3 * i + j], M[9 + 3 * i + j]};
}

// Hessian entry H[c][d] (without the alpha term) / 2 of the quartic part:
// Hb = 2 sum_t beta_t dG_t[s E_{mu j}], output Re (c < 9) or Im (c >= 9) at (i, l).
template <typename T>
__device__ __forceinline__ T hess_entry(const QS<T> &s, const T *beta, int c, int d)
{
  const int pc = c / 9, i = (c % 9) / 3, l = c % 3;
  const int pd = d / 9, mu = (d % 9) / 3, j = d % 3;
  const cx<T> p = {s.pq[0], s.pq[1]};
  const T q = s.pq[2];
  const bool dim_ = (i == mu), djl = (j == l);
  const cx<T> A_mj = at(s.A, mu, j), A_il = at(s.A, i, l), A_ij = at(s.A, i, j), A_ml = at(s.A, mu, l);
  // T1 = 2 s A_mj conj(A_il) + p conj(s) d_im d_lj
  cx<T> t1 = cscale(mul_s(cmul(A_mj, cconj(A_il)), pd), T(2));
  if (dim_ && djl) t1 = cadd(t1, mul_cs(p, pd));
  // T2 = 2 Re(s conj(A_mj)) A_il + q s d_im d_lj
  const T re_s_cA = mul_s(cconj(A_mj), pd).r;
  cx<T> t2 = cscale(A_il, T(2) * re_s_cA);
  if (dim_ && djl) t2 = cadd(t2, mul_s(cx<T>{q, T(0)}, pd));
  // T3 = s A_ij conj(A_ml) + s d_im conj(M2_jl) + conj(s) P_im d_jl
  cx<T> t3 = mul_s(cmul(A_ij, cconj(A_ml)), pd);
  if (dim_) t3 = cadd(t3, mul_s(cconj(at(s.M2, j, l)), pd));
  if (djl) t3 = cadd(t3, mul_cs(at(s.P, i, mu), pd));
  // T4 = s d_im M2_jl + conj(s) A_ij A_ml + s Q_im d_jl
  cx<T> t4 = mul_cs(cmul(A_ij, A_ml), pd);
  if (dim_) t4 = cadd(t4, mul_s(at(s.M2, j, l), pd));
  if (djl) t4 = cadd(t4, mul_s(at(s.Q, i, mu), pd));
  // T5 = conj(s) d_im M3_jl + s conj(A_ij) A_ml + s conj(Q_im) d_jl
  cx<T> t5 = mul_s(cmul(cconj(A_ij), A_ml), pd);
  if (dim_) t5 = cadd(t5, mul_cs(at(s.M3, j, l), pd));
  if (djl) t5 = cadd(t5, mul_s(cconj(at(s.Q, i, mu)), pd));
  const cx<T> hb = cadd(cadd(cadd(cscale(t1, beta[0]), cscale(t2, beta[1])), cadd(cscale(t3, beta[2]), cscale(t4, beta[3]))),
                        cscale(t5, beta[4]));
  return T(2) * (pc ? hb.i : hb.r);
}

// ---------------------------------------------------------------------------------
// k_cell3d: per-cell quadrature data
// ---------------------------------------------------------------------------------
constexpr int kCPB = 4;             // cells per CTA
constexpr int kNPQ = kCPB * 8;      // (cell, q) pairs per CTA
constexpr int kCellThreads = 128;

template <typename T> struct CellSmem
{
  T xs[kCPB][8][18];
  // per-point rows padded to 19 scalars: lane = point reads hit distinct banks
  T A[kNPQ][19];
  T gA[kNPQ][3][18];
  T P[kNPQ][19], Q[kNPQ][19], M2[kNPQ][19], M3[kNPQ][19];
  T pq[kNPQ][3];
  T rb[kNPQ][18];
  T dv[kNPQ][6];
  T en[kNPQ];
  T ec[kNPQ][18];
  T coef[kCPB][kCoef];
  T ih[kCPB][3];
  T jxw[kCPB];
};

template <typename T, bool WH, bool WR>
__global__ void __launch_bounds__(kCellThreads) k_cell3d(DevMesh m, const double *__restrict__ x, T *__restrict__ Hout,
                                                          double *__restrict__ r_cell, double *__restrict__ e_cell,
                                                          const uint8_t *__restrict__ inst_active)
{
  pdl_wait();
  pdl_trigger();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  CellSmem<T> &S = *reinterpret_cast<CellSmem<T> *>(smem_raw);
  const int tid = threadIdx.x;
  const int64_t e0 = static_cast<int64_t>(blockIdx.x) * kCPB;
  const int ncb = static_cast<int>((m.nc - e0) < kCPB ? (m.nc - e0) : kCPB);
  __shared__ int s_skip[kCPB];
  if (tid < kCPB)
    {
      int skip = 1;
      if (tid < ncb)
        {
          const int64_t e = e0 + tid;
          const int inst = m.cell_inst[e];
          skip = (inst_active && !inst_active[inst]) ? 1 : 0;
          for (int k = 0; k < kCoef; ++k) S.coef[tid][k] = Tab<T>::coef(m, inst, k);
          const auto g = Tab<T>::geo(m, e);
          S.ih[tid][0] = g.x;
          S.ih[tid][1] = g.y;
          S.ih[tid][2] = g.z;
          S.jxw[tid] = T(0.125) * g.w;
        }
      s_skip[tid] = skip;
    }
  // gather nodal values
  for (int idx = tid; idx < kCPB * 144; idx += kCellThreads)
    {
      const int cl = idx / 144, rem = idx % 144, v = rem / 18, c = rem % 18;
      T val = T(0);
      if (cl < ncb)
        {
          const int node = m.cells[(e0 + cl) * 8 + v];
          val = static_cast<T>(x[static_cast<int64_t>(node) * 18 + c]);
        }
      S.xs[cl][v][c] = val;
    }
  __syncthreads();
  // A and grad A at the Gauss points
  for (int idx = tid; idx < kNPQ * 18; idx += kCellThreads)
    {
      const int pq = idx / 18, c = idx % 18, cl = pq >> 3, q = pq & 7;
      T a = 0, g0 = 0, g1 = 0, g2 = 0;
#pragma unroll
      for (int v = 0; v < 8; ++v)
        {
          const T xv = S.xs[cl][v][c];
          a += Tab<T>::val(q, v) * xv;
          g0 += Tab<T>::grd(q, v, 0) * xv;
          g1 += Tab<T>::grd(q, v, 1) * xv;
          g2 += Tab<T>::grd(q, v, 2) * xv;
        }
      S.A[pq][c] = a;
      S.gA[pq][0][c] = g0 * S.ih[cl][0];
      S.gA[pq][1][c] = g1 * S.ih[cl][1];
      S.gA[pq][2][c] = g2 * S.ih[cl][2];
    }
  __syncthreads();
  // P = A A^T, Q = A A^+ (residual and Hessian), M2 = A^+ A, M3 = A^T A (Hessian only)
  for (int idx = tid; idx < kNPQ * (WH ? 36 : 18); idx += kCellThreads)
    {
      constexpr int per = WH ? 36 : 18;
      const int pq = idx / per, r = idx % per, which = r / 9, ent = r % 9, i = ent / 3, l = ent % 3;
      const T *A = S.A[pq];
      cx<T> s = {T(0), T(0)};
#pragma unroll
      for (int k = 0; k < 3; ++k)
        {
          cx<T> x1, x2;
          switch (which)
            {
            case 0: x1 = at(A, i, k); x2 = at(A, l, k); break;                  // P_il = sum_k A_ik A_lk
            case 1: x1 = at(A, i, k); x2 = cconj(at(A, l, k)); break;           // Q_il = sum_k A_ik conj(A_lk)
            case 2: x1 = cconj(at(A, k, i)); x2 = at(A, k, l); break;           // M2_il = sum_k conj(A_ki) A_kl
            default: x1 = at(A, k, i); x2 = at(A, k, l); break;                 // M3_il = sum_k A_ki A_kl
            }
          s = cadd(s, cmul(x1, x2));
        }
      T *dst = (which == 0) ? S.P[pq] : (which == 1) ? S.Q[pq] : (which == 2) ? S.M2[pq] : S.M3[pq];
      dst[ent] = s.r;
      dst[9 + ent] = s.i;
    }
  __syncthreads();
  if (tid < kNPQ)
    {
      S.pq[tid][0] = S.P[tid][0] + S.P[tid][4] + S.P[tid][8];
      S.pq[tid][1] = S.P[tid][9] + S.P[tid][13] + S.P[tid][17];
      S.pq[tid][2] = S.Q[tid][0] + S.Q[tid][4] + S.Q[tid][8];
    }
  __syncthreads();
  if (WH)
    {
      // lane = (cell, point) pair, warps stride over the 171 entries: all lanes of a warp
      // evaluate the same entry (no divergence), and a cell's 8 points fill 32 contiguous
      // bytes of H[cell][entry][point]
      static_assert(kNPQ == 32, "one warp covers the CTA's (cell, point) pairs");
      const int pq = tid & 31, cl = pq >> 3;
      const bool live = cl < ncb && !s_skip[cl];
      const QS<T> qs = {S.A[pq], S.P[pq], S.Q[pq], S.M2[pq], S.M3[pq], S.pq[pq]};
      const T *beta = &S.coef[cl][3];
      const T alpha = S.coef[cl][2];
      T *hdst = Hout + (e0 + cl) * static_cast<int64_t>(kNS3) * 8 + (pq & 7);
      for (int sidx = tid >> 5; sidx < kNS3; sidx += kCellThreads / 32)
        {
          const int c = c_symc[sidx], d = c_symd[sidx];
          T h = hess_entry(qs, beta, c, d);
          if (c == d) h += alpha;
          if (live) hdst[sidx * 8] = h;
        }
    }
  if (WR)
    {
      // bulk residual Rb = alpha A + 2 sum_t beta_t G_t and the free-energy density
      for (int idx = tid; idx < kNPQ * 18; idx += kCellThreads)
        {
          const int pq = idx / 18, c = idx % 18, cl = pq >> 3;
          const int part = c / 9, i = (c % 9) / 3, l = c % 3;
          const T *A = S.A[pq];
          const cx<T> p = {S.pq[pq][0], S.pq[pq][1]};
          const T qq = S.pq[pq][2];
          const cx<T> Ail = at(A, i, l);
          cx<T> G[5];
          G[0] = cmul(p, cconj(Ail));
          G[1] = cscale(Ail, qq);
          G[2] = G[3] = G[4] = cx<T>{T(0), T(0)};
#pragma unroll
          for (int k = 0; k < 3; ++k)
            {
              G[2] = cadd(G[2], cmul(at(S.P[pq], i, k), cconj(at(A, k, l))));
              G[3] = cadd(G[3], cmul(at(S.Q[pq], i, k), at(A, k, l)));
              G[4] = cadd(G[4], cmul(cconj(at(S.Q[pq], i, k)), at(A, k, l)));
            }
          const T *cf = S.coef[cl];
          const T ac = A[c];
          T rb = cf[2] * ac, eb = cf[2] * ac * ac;
#pragma unroll
          for (int t = 0; t < 5; ++t)
            {
              const T g = part ? G[t].i : G[t].r;
              rb += T(2) * cf[3 + t] * g;
              eb += cf[3 + t] * g * ac;
            }
          T eg = 0;
#pragma unroll
          for (int k = 0; k < 3; ++k) eg += S.gA[pq][k][c] * S.gA[pq][k][c];
          S.rb[pq][c] = rb;
          S.ec[pq][c] = eb + cf[0] * eg; // energy density of this component (bulk + K1 part)
        }
      __syncthreads();
      if (tid < kNPQ)
        {
          const int pq = tid, cl = pq >> 3;
          T div[6];
#pragma unroll
          for (int pm = 0; pm < 6; ++pm)
            {
              const int base = 9 * (pm / 3) + 3 * (pm % 3);
              div[pm] = S.gA[pq][0][base + 0] + S.gA[pq][1][base + 1] + S.gA[pq][2][base + 2];
              S.dv[pq][pm] = div[pm];
            }
          T e = 0;
          for (int c = 0; c < 18; ++c) e += S.ec[pq][c];
          for (int pm = 0; pm < 6; ++pm) e += S.coef[cl][1] * div[pm] * div[pm];
          S.en[pq] = e;
        }
      __syncthreads();
      for (int idx = tid; idx < kCPB * 144; idx += kCellThreads)
        {
          const int cl = idx / 144, a = (idx % 144) / 18, c = idx % 18;
          if (cl >= ncb || s_skip[cl]) continue;
          const int pm = 3 * (c / 9) + (c % 9) / 3, jc = c % 3;
          const T K1 = S.coef[cl][0], K23 = S.coef[cl][1];
          T r = 0;
#pragma unroll
          for (int q = 0; q < 8; ++q)
            {
              const int pq = cl * 8 + q;
              T s = Tab<T>::val(q, a) * S.rb[pq][c];
              s += K1 * (Tab<T>::grd(q, a, 0) * S.ih[cl][0] * S.gA[pq][0][c] +
                         Tab<T>::grd(q, a, 1) * S.ih[cl][1] * S.gA[pq][1][c] +
                         Tab<T>::grd(q, a, 2) * S.ih[cl][2] * S.gA[pq][2][c]);
              s += K23 * Tab<T>::grd(q, a, jc) * S.ih[cl][jc] * S.dv[pq][pm];
              r += s;
            }
          r_cell[(e0 + cl) * 144 + a * 18 + c] = static_cast<double>(r * S.jxw[cl]);
        }
      if (e_cell && tid < kCPB && tid < ncb && !s_skip[tid])
        {
          T e = 0;
          for (int q = 0; q < 8; ++q) e += S.en[tid * 8 + q];
          e_cell[e0 + tid] = static_cast<double>(e * S.jxw[tid]);
        }
    }
}

// ---------------------------------------------------------------------------------
// k_res3d: the FP64 residual (and, when asked, the cell free energies), 8 cells per CTA.
// The FP64 pipe bounds it, so the arithmetic is organised to do little of it:
//  * interpolation of the 8 nodal values of a component to the 2x2x2 Gauss points and
//    the transposed contraction with the test functions are sum-factorised along the
//    axes (the Q1 gradient along an axis does not depend on that axis' point);
//  * the quartic terms fold into two complex 3x3 products per point:
//    rho = (alpha + 2 b2 q) A + (2 b1 p 1 + 2 b3 P) A^* + (2 b4 Q + 2 b5 Q^*) A,
//    with P = A A^T, Q = A A^+, p = tr P, q = tr Q (the same quarter-gradients G_t as the
//    Hessian kernel: G1 = p A^*, G2 = q A, G3 = P A^*, G4 = Q A, G5 = Q^* A);
//  * the energy density alpha q + sum_t beta_t I_t + K1 |grad A|^2 + (K2+K3) sum div^2,
//    with I1 = |p|^2, I2 = q^2, I3 = sum |P_ik|^2, I4 = sum |Q_ik|^2, I5 = Re sum Q_ik^2,
//    only when the caller wants it.
// ---------------------------------------------------------------------------------
constexpr int kRCells = 8;               // cells per CTA
constexpr int kRPts = kRCells * 8;       // (cell, point) pairs per CTA
constexpr int kRThreads = 192;           // = 3 * kRPts (one thread per (point, row i))
constexpr double kGa = 0.21132486540518711775; // 1/2 - sqrt(3)/6: Gauss point on [0, 1]
constexpr double kGb = 0.78867513459481288225; // 1/2 + sqrt(3)/6

// R = double (FP64 mode) or DF (double-float on the FP32 pipe, mixed mode)
template <typename R> struct ResSmemT
{
  R xs[kRCells][8][18];
  R A[kRPts][19];
  R gA[kRPts][3][18];
  R P[kRPts][19], Q[kRPts][19];
  R rb[kRPts][18];
  R en[kRPts];
  R coef[kRCells][kCoef];
  R ih[kRCells][3];
  R jxw[kRCells];
  int skip[kRCells];
};
using ResSmem = ResSmemT<double>;

// linear interpolation of (f0, f1) to the two Gauss points of [0, 1]
__device__ __forceinline__ void gauss2(double f0, double f1, double &q0, double &q1)
{
  q0 = kGb * f0 + kGa * f1;
  q1 = kGa * f0 + kGb * f1;
}
template <typename R> __device__ __forceinline__ void gauss2r(R ga, R gb, R f0, R f1, R &q0, R &q1)
{
  q0 = gb * f0 + ga * f1;
  q1 = ga * f0 + gb * f1;
}

template <typename R>
__global__ void __launch_bounds__(kRThreads) k_res3d(DevMesh m, const double *__restrict__ x, double *__restrict__ r_cell,
                                                     double *__restrict__ e_cell, const uint8_t *__restrict__ inst_active)
{
  pdl_wait();
  pdl_trigger();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ResSmemT<R> &S = *reinterpret_cast<ResSmemT<R> *>(smem_raw);
  const R ga = from_d<R>(kGa), gb = from_d<R>(kGb);
  const int tid = threadIdx.x;
  const int64_t e0 = static_cast<int64_t>(blockIdx.x) * kRCells;
  const int ncb = static_cast<int>((m.nc - e0) < kRCells ? (m.nc - e0) : kRCells);
  if (tid < kRCells)
    {
      int skip = 1;
      if (tid < ncb)
        {
          const int64_t e = e0 + tid;
          const int inst = m.cell_inst[e];
          skip = (inst_active && !inst_active[inst]) ? 1 : 0;
          for (int k = 0; k < kCoef; ++k) S.coef[tid][k] = from_d<R>(m.coef[inst * kCoef + k]);
          const GeoD g = m.geo_d[e];
          S.ih[tid][0] = from_d<R>(g.x);
          S.ih[tid][1] = from_d<R>(g.y);
          S.ih[tid][2] = from_d<R>(g.z);
          S.jxw[tid] = from_d<R>(0.125 * g.w);
        }
      S.skip[tid] = skip;
    }
  for (int idx = tid; idx < kRCells * 144; idx += kRThreads)
    {
      const int cl = idx / 144, rem = idx - 144 * cl, v = rem / 18, c = rem - 18 * v;
      R val = R(0.f);
      if (cl < ncb)
        {
          const int node = m.cells[(e0 + cl) * 8 + v];
          val = from_d<R>(x[static_cast<int64_t>(node) * 18 + c]);
        }
      S.xs[cl][v][c] = val;
    }
  __syncthreads();
  // values and gradients at the points: thread (cell, component)
  if (tid < kRCells * 18)
    {
      const int cl = tid / 18, c = tid - 18 * cl;
      const R *xv = &S.xs[cl][0][c]; // xv[18 * v], v = vx + 2 vy + 4 vz
      R zq[2][4], zd[4];             // [qz][vy vx], z-difference [vy vx]
#pragma unroll
      for (int t = 0; t < 4; ++t)
        {
          const R f0 = xv[18 * t], f1 = xv[18 * (t + 4)];
          gauss2r(ga, gb, f0, f1, zq[0][t], zq[1][t]);
          zd[t] = f1 - f0;
        }
      R yq[2][2][2], ydy[2][2], zdq[2][2]; // [qz][qy][vx], [qz][vx], [qy][vx]
#pragma unroll
      for (int vx = 0; vx < 2; ++vx)
        {
#pragma unroll
          for (int qz = 0; qz < 2; ++qz)
            {
              gauss2r(ga, gb, zq[qz][vx], zq[qz][2 + vx], yq[qz][0][vx], yq[qz][1][vx]);
              ydy[qz][vx] = zq[qz][2 + vx] - zq[qz][vx];
            }
          gauss2r(ga, gb, zd[vx], zd[2 + vx], zdq[0][vx], zdq[1][vx]);
        }
      const R i0 = S.ih[cl][0], i1 = S.ih[cl][1], i2 = S.ih[cl][2];
#pragma unroll
      for (int qz = 0; qz < 2; ++qz)
#pragma unroll
        for (int qy = 0; qy < 2; ++qy)
          {
            R v0, v1;
            gauss2r(ga, gb, yq[qz][qy][0], yq[qz][qy][1], v0, v1);
            const R dx = (yq[qz][qy][1] - yq[qz][qy][0]) * i0;
            const int p0 = cl * 8 + 2 * qy + 4 * qz;
            S.A[p0][c] = v0;
            S.A[p0 + 1][c] = v1;
            S.gA[p0][0][c] = dx;
            S.gA[p0 + 1][0][c] = dx;
          }
#pragma unroll
      for (int qz = 0; qz < 2; ++qz)
        {
          R d0, d1;
          gauss2r(ga, gb, ydy[qz][0], ydy[qz][1], d0, d1);
#pragma unroll
          for (int qy = 0; qy < 2; ++qy)
            {
              const int p0 = cl * 8 + 2 * qy + 4 * qz;
              S.gA[p0][1][c] = d0 * i1;
              S.gA[p0 + 1][1][c] = d1 * i1;
            }
        }
#pragma unroll
      for (int qy = 0; qy < 2; ++qy)
        {
          R d0, d1;
          gauss2r(ga, gb, zdq[qy][0], zdq[qy][1], d0, d1);
#pragma unroll
          for (int qz = 0; qz < 2; ++qz)
            {
              const int p0 = cl * 8 + 2 * qy + 4 * qz;
              S.gA[p0][2][c] = d0 * i2;
              S.gA[p0 + 1][2][c] = d1 * i2;
            }
        }
    }
  __syncthreads();
  // P = A A^T and Q = A A^+: thread (point, row i)
  {
    const int pq = tid / 3, i = tid - 3 * pq;
    const R *A = S.A[pq];
    // j and l (below) index shared memory only: the loops stay rolled, which keeps the
    // double-float kernel's code within the instruction cache
#pragma unroll 1
    for (int j = 0; j < 3; ++j)
      {
        cx<R> pp = {R(0.f), R(0.f)}, qq = {R(0.f), R(0.f)};
#pragma unroll
        for (int k = 0; k < 3; ++k)
          {
            const cx<R> aik = at(A, i, k), ajk = at(A, j, k);
            pp = cadd(pp, cmul(aik, ajk));
            qq = cadd(qq, cmul(aik, cconj(ajk)));
          }
        S.P[pq][3 * i + j] = pp.r;
        S.P[pq][9 + 3 * i + j] = pp.i;
        S.Q[pq][3 * i + j] = qq.r;
        S.Q[pq][9 + 3 * i + j] = qq.i;
      }
  }
  __syncthreads();
  // rho, row i: thread (point, row i)
  {
    const int pq = tid / 3, i = tid - 3 * pq, cl = pq >> 3;
    const R *A = S.A[pq], *P = S.P[pq], *Q = S.Q[pq], *cf = S.coef[cl];
    const cx<R> p = {P[0] + P[4] + P[8], P[9] + P[13] + P[17]};
    const R q = Q[0] + Q[4] + Q[8];
    const R s0 = cf[2] + R(2.f) * cf[4] * q;
    cx<R> N[3], M[3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
      {
        const cx<R> pik = at(P, i, k), qik = at(Q, i, k);
        N[k] = cscale(pik, R(2.f) * cf[5]);
        if (k == i) N[k] = cadd(N[k], cscale(p, R(2.f) * cf[3]));
        M[k] = {R(2.f) * (cf[6] + cf[7]) * qik.r, R(2.f) * (cf[6] - cf[7]) * qik.i};
      }
#pragma unroll 1
    for (int l = 0; l < 3; ++l)
      {
        cx<R> r = cscale(at(A, i, l), s0);
#pragma unroll
        for (int k = 0; k < 3; ++k)
          {
            const cx<R> akl = at(A, k, l);
            r = cadd(r, cmul(N[k], cconj(akl)));
            r = cadd(r, cmul(M[k], akl));
          }
        S.rb[pq][3 * i + l] = r.r;
        S.rb[pq][9 + 3 * i + l] = r.i;
      }
  }
  __syncthreads();
  // contraction with the test functions: thread (cell, component)
  if (tid < kRCells * 18)
    {
      const int cl = tid / 18, c = tid - 18 * cl;
      const int part = c / 9, mu = (c % 9) / 3, jc = c % 3;
      const R K1 = S.coef[cl][0], K23 = S.coef[cl][1];
      const R ih[3] = {S.ih[cl][0], S.ih[cl][1], S.ih[cl][2]};
      // w = rho, F_k = K1 ih_k dA/dx_k + [k == jc] K23 ih_jc div, at the 8 points
      R w[8], F[3][8];
#pragma unroll
      for (int q = 0; q < 8; ++q)
        {
          const int pq = cl * 8 + q;
          w[q] = S.rb[pq][c];
          const int base = 9 * part + 3 * mu;
          const R dterm = K23 * (S.gA[pq][0][base] + S.gA[pq][1][base + 1] + S.gA[pq][2][base + 2]);
#pragma unroll
          for (int k = 0; k < 3; ++k) F[k][q] = ih[k] * (K1 * S.gA[pq][k][c] + (k == jc ? dterm : R(0.f)));
        }
      // r[a] = sum_q val_q(a) w[q] + sum_k sum_q dval_q(a)/dxi_k F_k[q], a = ax + 2 ay + 4 az
      R r[8];
      {
        // value part: transpose of the interpolation, axis by axis (x, then y, then z)
        R tx[2][4]; // [ax][qy + 2 qz]
#pragma unroll
        for (int t = 0; t < 4; ++t)
          {
            tx[0][t] = gb * w[2 * t] + ga * w[2 * t + 1];
            tx[1][t] = ga * w[2 * t] + gb * w[2 * t + 1];
          }
        R ty[2][2][2]; // [ax][ay][qz]
#pragma unroll
        for (int ax = 0; ax < 2; ++ax)
#pragma unroll
          for (int qz = 0; qz < 2; ++qz)
            {
              ty[ax][0][qz] = gb * tx[ax][2 * qz] + ga * tx[ax][2 * qz + 1];
              ty[ax][1][qz] = ga * tx[ax][2 * qz] + gb * tx[ax][2 * qz + 1];
            }
#pragma unroll
        for (int ax = 0; ax < 2; ++ax)
#pragma unroll
          for (int ay = 0; ay < 2; ++ay)
            {
              r[ax + 2 * ay] = gb * ty[ax][ay][0] + ga * ty[ax][ay][1];
              r[ax + 2 * ay + 4] = ga * ty[ax][ay][0] + gb * ty[ax][ay][1];
            }
      }
      {
        // x gradient: dval/dxi_x = (2 ax - 1) L(qy, ay) L(qz, az): sum over qx first
        R sx[4]; // [qy + 2 qz]
#pragma unroll
        for (int t = 0; t < 4; ++t) sx[t] = F[0][2 * t] + F[0][2 * t + 1];
        R uy[2][2]; // [ay][qz]
#pragma unroll
        for (int qz = 0; qz < 2; ++qz)
          {
            uy[0][qz] = gb * sx[2 * qz] + ga * sx[2 * qz + 1];
            uy[1][qz] = ga * sx[2 * qz] + gb * sx[2 * qz + 1];
          }
#pragma unroll
        for (int ay = 0; ay < 2; ++ay)
#pragma unroll
          for (int az = 0; az < 2; ++az)
            {
              const R v = az ? ga * uy[ay][0] + gb * uy[ay][1] : gb * uy[ay][0] + ga * uy[ay][1];
              r[1 + 2 * ay + 4 * az] += v;
              r[2 * ay + 4 * az] -= v;
            }
      }
      {
        // y gradient: sum over qy first
        R sy[4]; // [qx + 2 qz]
#pragma unroll
        for (int qz = 0; qz < 2; ++qz)
#pragma unroll
          for (int qx = 0; qx < 2; ++qx) sy[qx + 2 * qz] = F[1][qx + 4 * qz] + F[1][qx + 2 + 4 * qz];
        R ux[2][2]; // [ax][qz]
#pragma unroll
        for (int qz = 0; qz < 2; ++qz)
          {
            ux[0][qz] = gb * sy[2 * qz] + ga * sy[2 * qz + 1];
            ux[1][qz] = ga * sy[2 * qz] + gb * sy[2 * qz + 1];
          }
#pragma unroll
        for (int ax = 0; ax < 2; ++ax)
#pragma unroll
          for (int az = 0; az < 2; ++az)
            {
              const R v = az ? ga * ux[ax][0] + gb * ux[ax][1] : gb * ux[ax][0] + ga * ux[ax][1];
              r[ax + 2 + 4 * az] += v;
              r[ax + 4 * az] -= v;
            }
      }
      {
        // z gradient: sum over qz first
        R sz[4]; // [qx + 2 qy]
#pragma unroll
        for (int t = 0; t < 4; ++t) sz[t] = F[2][t] + F[2][t + 4];
        R ux[2][2]; // [ax][qy]
#pragma unroll
        for (int qy = 0; qy < 2; ++qy)
          {
            ux[0][qy] = gb * sz[2 * qy] + ga * sz[2 * qy + 1];
            ux[1][qy] = ga * sz[2 * qy] + gb * sz[2 * qy + 1];
          }
#pragma unroll
        for (int ax = 0; ax < 2; ++ax)
#pragma unroll
          for (int ay = 0; ay < 2; ++ay)
            {
              const R v = ay ? ga * ux[ax][0] + gb * ux[ax][1] : gb * ux[ax][0] + ga * ux[ax][1];
              r[ax + 2 * ay + 4] += v;
              r[ax + 2 * ay] -= v;
            }
      }
      if (cl < ncb && !S.skip[cl])
        {
          const R jxw = S.jxw[cl];
          double *out = r_cell + (e0 + cl) * 144 + c;
#pragma unroll
          for (int a = 0; a < 8; ++a) out[18 * a] = to_d(r[a] * jxw);
        }
    }
  if (!e_cell) return;
  // energy density per point, then per cell
  if (tid < kRPts)
    {
      const int pq = tid, cl = pq >> 3;
      const R *P = S.P[pq], *Q = S.Q[pq], *cf = S.coef[cl];
      const R pr = P[0] + P[4] + P[8], pi = P[9] + P[13] + P[17], q = Q[0] + Q[4] + Q[8];
      R i3 = R(0.f), i4 = R(0.f), i5 = R(0.f);
#pragma unroll
      for (int t = 0; t < 9; ++t)
        {
          i3 += P[t] * P[t] + P[9 + t] * P[9 + t];
          i4 += Q[t] * Q[t] + Q[9 + t] * Q[9 + t];
          i5 += Q[t] * Q[t] - Q[9 + t] * Q[9 + t];
        }
      R e = cf[2] * q + cf[3] * (pr * pr + pi * pi) + cf[4] * q * q + cf[5] * i3 + cf[6] * i4 + cf[7] * i5;
      R eg = R(0.f);
#pragma unroll
      for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int c = 0; c < 18; ++c) eg += S.gA[pq][k][c] * S.gA[pq][k][c];
      R ed = R(0.f);
#pragma unroll
      for (int pm = 0; pm < 6; ++pm)
        {
          const int base = 9 * (pm / 3) + 3 * (pm % 3);
          const R dv = S.gA[pq][0][base] + S.gA[pq][1][base + 1] + S.gA[pq][2][base + 2];
          ed += dv * dv;
        }
      S.en[pq] = e + cf[0] * eg + cf[1] * ed;
    }
  __syncthreads();
  if (tid < ncb && !S.skip[tid])
    {
      R e = R(0.f);
#pragma unroll
      for (int q = 0; q < 8; ++q) e += S.en[tid * 8 + q];
      e_cell[e0 + tid] = to_d(e * S.jxw[tid]);
    }
}

// ---------------------------------------------------------------------------------
// k_rows3d: one CTA per block row, accumulation in shared memory
// ---------------------------------------------------------------------------------
constexpr int kRowThreads = 192;

// the 8 point values of Hessian entry `ent` of cell e: 32 (FP32) or 64 (FP64) contiguous bytes
__device__ __forceinline__ void load_hq(const float *H, int64_t e, int ent, bool act, float (&hq)[8])
{
  float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
  if (act)
    {
      const float4 *p = reinterpret_cast<const float4 *>(H + (e * kNS3 + ent) * 8);
      a = __ldg(p);
      b = __ldg(p + 1);
    }
  hq[0] = a.x; hq[1] = a.y; hq[2] = a.z; hq[3] = a.w;
  hq[4] = b.x; hq[5] = b.y; hq[6] = b.z; hq[7] = b.w;
}
__device__ __forceinline__ void load_hq(const double *H, int64_t e, int ent, bool act, double (&hq)[8])
{
#pragma unroll
  for (int k = 0; k < 4; ++k)
    {
      double2 v = make_double2(0.0, 0.0);
      if (act) v = __ldg(reinterpret_cast<const double2 *>(H + (e * kNS3 + ent) * 8) + k);
      hq[2 * k] = v.x;
      hq[2 * k + 1] = v.y;
    }
}

// k_rows3d_reg: full interior rows (27 blocks, eight unit-weight cell contributions stored
// in local-vertex order, no constraint on the row, cells of one size; classified on the
// host).  Only the bulk term depends on the state: block (a, b) of the cell whose vertex a
// is the row node adds vol sum_q S_abq H_q to slot 13 + dx + 3 dy + 9 dz, (dx, dy, dz) =
// bits(b) - bits(a).  Thread t owns entry t = 18 c + d of all 27 blocks (the symmetric
// Hessian entry is read for both halves), so loads of the template and stores of the row
// are contiguous across a warp; the loops are fully unrolled, so every slot is a
// compile-time register.  The gradient part of the row is the same for every interior row
// of an instance and comes from the instance's template; columns' Dirichlet masks apply
// at the store.
constexpr int kRegThreads = 324;

template <typename T>
__global__ void __launch_bounds__(kRegThreads) k_rows3d_reg(DevMesh m, const T *__restrict__ H, T *__restrict__ vals)
{
  pdl_wait();
  pdl_trigger();
  __shared__ uint32_t s_cmask[27];
  const int64_t n = m.reg_rows[blockIdx.x];
  const int tid = threadIdx.x;
  const int r0 = m.rowptr[n];
  if (tid < 27) s_cmask[tid] = m.mask[m.cols[r0 + tid]];
  const int c = tid / 18, d = tid - 18 * (tid / 18);
  const int lo = c < d ? c : d, hi = c < d ? d : c;
  const int ent = 18 * lo - (lo * (lo - 1)) / 2 + (hi - lo); // index of (lo, hi) in the upper triangle
  T acc[27];
#pragma unroll
  for (int s = 0; s < 27; ++s) acc[s] = T(0);
  const int k0 = m.rc_ptr[n];
#pragma unroll
  for (int a = 0; a < 8; ++a)
    {
      const int64_t e = m.rc_cell[k0 + a];
      T hq[8];
      load_hq(H, e, ent, true, hq);
      const T vol = Tab<T>::geo(m, e).w;
#pragma unroll
      for (int q = 0; q < 8; ++q) hq[q] *= vol;
#pragma unroll
      for (int b = 0; b < 8; ++b)
        {
          const int sl = 13 + ((b & 1) - (a & 1)) + 3 * (((b >> 1) & 1) - ((a >> 1) & 1)) + 9 * (((b >> 2) & 1) - ((a >> 2) & 1));
          T bulk = 0;
#pragma unroll
          for (int q = 0; q < 8; ++q) bulk += Tab<T>::S(a, b, q) * hq[q];
          acc[sl] += bulk;
        }
    }
  __syncthreads();
  const T *tp = Tab<T>::tmpl(m) + static_cast<int64_t>(m.node_inst[n]) * 27 * 324 + tid;
  T *out = vals + static_cast<int64_t>(r0) * 324 + tid;
#pragma unroll
  for (int s = 0; s < 27; ++s) out[s * 324] = ((s_cmask[s] >> d) & 1u) ? T(0) : acc[s] + __ldg(tp + s * 324);
}

// The FP64 variant: the FP64 pipe, not the store pattern, bounds it, so thread t owns the
// symmetric pair (c, d) / (d, c) of Hessian entry t and evaluates each bulk sum once.
template <typename T>
__global__ void __launch_bounds__(kRowThreads) k_rows3d_reg_sym(DevMesh m, const T *__restrict__ H,
                                                               T *__restrict__ vals)
{
  pdl_wait();
  pdl_trigger();
  __shared__ uint32_t s_cmask[27];
  const int64_t n = m.reg_rows[blockIdx.x];
  const int tid = threadIdx.x;
  const int r0 = m.rowptr[n];
  if (tid < 27) s_cmask[tid] = m.mask[m.cols[r0 + tid]];
  const bool act = tid < kNS3;
  const int c = act ? c_symc[tid] : 0, d = act ? c_symd[tid] : 0;
  T acc[27];
#pragma unroll
  for (int s = 0; s < 27; ++s) acc[s] = T(0);
  const int k0 = m.rc_ptr[n];
#pragma unroll
  for (int a = 0; a < 8; ++a)
    {
      const int64_t e = m.rc_cell[k0 + a];
      T hq[8];
      load_hq(H, e, tid, act, hq);
      const T vol = Tab<T>::geo(m, e).w;
#pragma unroll
      for (int q = 0; q < 8; ++q) hq[q] *= vol;
#pragma unroll
      for (int b = 0; b < 8; ++b)
        {
          const int sl = 13 + ((b & 1) - (a & 1)) + 3 * (((b >> 1) & 1) - ((a >> 1) & 1)) + 9 * (((b >> 2) & 1) - ((a >> 2) & 1));
          T bulk = 0;
#pragma unroll
          for (int q = 0; q < 8; ++q) bulk += Tab<T>::S(a, b, q) * hq[q];
          acc[sl] += bulk;
        }
    }
  __syncthreads();
  if (!act) return;
  const T *tp = Tab<T>::tmpl(m) + static_cast<int64_t>(m.node_inst[n]) * 27 * 324;
  T *out = vals + static_cast<int64_t>(r0) * 324;
  const int cd = c * 18 + d, dc = d * 18 + c;
#pragma unroll
  for (int s = 0; s < 27; ++s)
    {
      const uint32_t cm = s_cmask[s];
      out[s * 324 + cd] = ((cm >> d) & 1u) ? T(0) : acc[s] + __ldg(tp + s * 324 + cd);
      if (c != d) out[s * 324 + dc] = ((cm >> c) & 1u) ? T(0) : acc[s] + __ldg(tp + s * 324 + dc);
    }
}

constexpr int kRowMaxContrib = 96; // contributions staged in shared memory per pass

template <typename T>
__global__ void __launch_bounds__(kRowThreads) k_rows3d(DevMesh m, const T *__restrict__ H, T *__restrict__ vals)
{
  pdl_wait();
  pdl_trigger();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *acc = reinterpret_cast<T *>(smem_raw);
  __shared__ T sD[8 * 8 * 9];
  __shared__ int s_cell[kRowMaxContrib], s_a[kRowMaxContrib];
  __shared__ T s_w[kRowMaxContrib];
  __shared__ int16_t s_slot[kRowMaxContrib * 8];
  const int64_t n = m.gen_rows ? m.gen_rows[blockIdx.x] : static_cast<int64_t>(blockIdx.x);
  const int tid = threadIdx.x;
  const int r0 = m.rowptr[n];
  const int nb = m.rowptr[n + 1] - r0;
  // row metadata (column ids and their Dirichlet masks) follow the accumulator
  int *s_col = reinterpret_cast<int *>(acc + static_cast<size_t>(m.max_row_blocks) * 324);
  uint32_t *s_cmask = reinterpret_cast<uint32_t *>(s_col + m.max_row_blocks);
  for (int i = tid; i < nb * 324; i += kRowThreads) acc[i] = T(0);
  for (int i = tid; i < 576; i += kRowThreads) sD[i] = Tab<T>::D()[i];
  for (int i = tid; i < nb; i += kRowThreads)
    {
      const int col = m.cols[r0 + i];
      s_col[i] = col;
      s_cmask[i] = m.mask[col];
    }
  const bool act = tid < kNS3;
  const int c = act ? c_symc[tid] : 0, d = act ? c_symd[tid] : 0;
  const int pmc = 3 * (c / 9) + (c % 9) / 3, jc = c % 3, pmd = 3 * (d / 9) + (d % 9) / 3, jd = d % 3;
  const bool kpair = (pmc == pmd);
  const struct HangTarget *tg = reinterpret_cast<const HangTarget *>(m.hang_tg);
  const int k0 = m.rc_ptr[n], k1 = m.rc_ptr[n + 1];
  for (int kb = k0; kb < k1; kb += kRowMaxContrib)
    {
      const int nk = min(kRowMaxContrib, k1 - kb);
      __syncthreads();
      for (int i = tid; i < nk; i += kRowThreads)
        {
          s_cell[i] = m.rc_cell[kb + i];
          s_a[i] = m.rc_a[kb + i];
          s_w[i] = Tab<T>::w(m, kb + i);
        }
      for (int i = tid; i < nk * 8; i += kRowThreads) s_slot[i] = m.rc_slot[static_cast<int64_t>(kb) * 8 + i];
      __syncthreads();
      for (int kk = 0; kk < nk; ++kk)
        {
          const int64_t e = s_cell[kk];
          const int a = s_a[kk];
          const T wa = s_w[kk];
          T hq[8];
          load_hq(H, e, tid, act, hq);
          const int inst = m.cell_inst[e];
          const T K1 = Tab<T>::coef(m, inst, 0), K23 = Tab<T>::coef(m, inst, 1);
          const int rbits = (m.robin && c == d) ? m.robin[e] : 0;
          const T wR = rbits ? Tab<T>::coef(m, inst, 8) : T(0);
          const auto g = Tab<T>::geo(m, e);
          const T vol = g.w;
          const T i0 = g.x, i1 = g.y, i2 = g.z;
          const T ihc = jc == 0 ? i0 : (jc == 1 ? i1 : i2);
          const T ihd = jd == 0 ? i0 : (jd == 1 ? i1 : i2);
          const T kd = K1 * vol;
          const T kc = K23 * vol * ihc * ihd;
          const T g0 = i0 * i0, g1 = i1 * i1, g2 = i2 * i2;
#pragma unroll 2
          for (int b = 0; b < 8; ++b)
            {
              T bulk = 0;
#pragma unroll
              for (int q = 0; q < 8; ++q) bulk += Tab<T>::S(a, b, q) * hq[q];
              bulk *= vol;
              const T *D = sD + (a * 8 + b) * 9;
              T gcd = 0, gdc = 0;
              if (c == d) gcd = gdc = kd * (D[0] * g0 + D[4] * g1 + D[8] * g2);
              if (rbits) gcd += robin_weight<T>(rbits, a, b, c % 3, wR, vol, i0, i1, i2); // diagonal entries only
              if (kpair)
                {
                  gcd += kc * D[3 * jc + jd];
                  gdc += kc * D[3 * jd + jc];
                }
              const int sl = s_slot[kk * 8 + b];
              if (sl >= 0)
                {
                  if (act)
                    {
                      acc[sl * 324 + c * 18 + d] += wa * (bulk + gcd);
                      if (c != d) acc[sl * 324 + d * 18 + c] += wa * (bulk + gdc);
                    }
                }
              else
                {
                  const HangTarget &t = tg[m.ht_off[n] + (-1 - sl)];
                  const int cnt = t.count;
                  for (int j = 0; j < cnt; ++j)
                    if (act)
                      {
                        const T w = wa * static_cast<T>(t.w[j]); // hanging rows only: rare
                        acc[t.slot[j] * 324 + c * 18 + d] += w * (bulk + gcd);
                        if (c != d) acc[t.slot[j] * 324 + d * 18 + c] += w * (bulk + gdc);
                      }
                }
            }
        }
    }
  __syncthreads();
  const uint32_t rmask = m.mask[n];
  const bool hang_row = m.hptr[n + 1] > m.hptr[n];
  T *out = vals + static_cast<int64_t>(r0) * 324;
  for (int i = tid; i < nb * 324; i += kRowThreads)
    {
      const int sl = i / 324, e2 = i - sl * 324, cc = e2 / 18, dd = e2 - cc * 18;
      const int col = s_col[sl];
      T v = acc[i];
      if (hang_row)
        v = (cc == dd) ? T(1) : T(0);
      else if ((rmask >> cc) & 1u)
        v = (col == n && cc == dd) ? (v != T(0) ? fabs(v) : T(1)) : T(0);
      else if ((s_cmask[sl] >> dd) & 1u)
        v = T(0);
      out[i] = v;
    }
}

// ---------------------------------------------------------------------------------
// 2D complex GL (2 components): thread per cell / thread per row
// ---------------------------------------------------------------------------------
template <typename T, bool WH, bool WR>
__global__ void k_cell2d(DevMesh m, const double *__restrict__ x, T *__restrict__ Hout, double *__restrict__ r_cell,
                         double *__restrict__ e_cell, const uint8_t *__restrict__ inst_active)
{
  pdl_wait();
  pdl_trigger();
  const int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= m.nc) return;
  const int inst = m.cell_inst[e];
  if (inst_active && !inst_active[inst]) return;
  const T gw = static_cast<T>(0.5 * m.coef[inst * kCoef + 0]);
  const T alpha = static_cast<T>(m.coef[inst * kCoef + 2]);
  const T beta = static_cast<T>(m.coef[inst * kCoef + 3]);
  const T ih[2] = {static_cast<T>(1.0 / m.cell_h[3 * e]), static_cast<T>(1.0 / m.cell_h[3 * e + 1])};
  const T jxw = static_cast<T>(0.25 * m.cell_h[3 * e] * m.cell_h[3 * e + 1]);
  T xv[4][2];
  for (int v = 0; v < 4; ++v)
    {
      const int node = m.cells[e * 4 + v];
      xv[v][0] = static_cast<T>(x[2 * static_cast<int64_t>(node)]);
      xv[v][1] = static_cast<T>(x[2 * static_cast<int64_t>(node) + 1]);
    }
  T r[4][2] = {};
  T en = 0;
  for (int q = 0; q < 4; ++q)
    {
      T u = 0, w = 0, gu[2] = {0, 0}, gv[2] = {0, 0};
      for (int v = 0; v < 4; ++v)
        {
          const T s = static_cast<T>(c_val2[q][v]);
          u += s * xv[v][0];
          w += s * xv[v][1];
          for (int k = 0; k < 2; ++k)
            {
              const T g = static_cast<T>(c_grd2[q][v][k]) * ih[k];
              gu[k] += g * xv[v][0];
              gv[k] += g * xv[v][1];
            }
        }
      const T s2 = u * u + w * w;
      if (WH)
        {
          T *h = Hout + (e * 4 + q) * 3;
          h[0] = alpha + beta * (T(3) * u * u + w * w);
          h[1] = T(2) * beta * u * w;
          h[2] = alpha + beta * (T(3) * w * w + u * u);
        }
      if (WR)
        {
          const T bulk = alpha + beta * s2;
          en += gw * (gu[0] * gu[0] + gu[1] * gu[1] + gv[0] * gv[0] + gv[1] * gv[1]) + alpha * s2 + T(0.5) * beta * s2 * s2;
          for (int a = 0; a < 4; ++a)
            {
              const T va = static_cast<T>(c_val2[q][a]);
              const T g0 = static_cast<T>(c_grd2[q][a][0]) * ih[0], g1 = static_cast<T>(c_grd2[q][a][1]) * ih[1];
              r[a][0] += gw * (g0 * gu[0] + g1 * gu[1]) + bulk * u * va;
              r[a][1] += gw * (g0 * gv[0] + g1 * gv[1]) + bulk * w * va;
            }
        }
    }
  if (WR)
    {
      for (int a = 0; a < 4; ++a)
        for (int c = 0; c < 2; ++c) r_cell[e * 8 + a * 2 + c] = static_cast<double>(r[a][c] * jxw);
      if (e_cell) e_cell[e] = static_cast<double>(en * jxw);
    }
}

template <typename T>
__global__ void k_rows2d(DevMesh m, const T *__restrict__ H, T *__restrict__ vals)
{
  pdl_wait();
  pdl_trigger();
  const int64_t n = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (n >= m.nn) return;
  const int r0 = m.rowptr[n], nb = m.rowptr[n + 1] - r0;
  T *out = vals + static_cast<int64_t>(r0) * 4;
  for (int i = 0; i < nb * 4; ++i) out[i] = T(0);
  const struct HangTarget *tg = reinterpret_cast<const HangTarget *>(m.hang_tg);
  for (int k = m.rc_ptr[n]; k < m.rc_ptr[n + 1]; ++k)
    {
      const int64_t e = m.rc_cell[k];
      const int a = m.rc_a[k];
      const T wa = static_cast<T>(m.rc_w[k]);
      const int inst = m.cell_inst[e];
      const T gw = static_cast<T>(0.5 * m.coef[inst * kCoef + 0]);
      const double hx = m.cell_h[3 * e], hy = m.cell_h[3 * e + 1];
      const T area = static_cast<T>(hx * hy);
      const T ih2[2] = {static_cast<T>(1.0 / (hx * hx)), static_cast<T>(1.0 / (hy * hy))};
      for (int b = 0; b < 4; ++b)
        {
          T blk[4] = {0, 0, 0, 0};
          for (int q = 0; q < 4; ++q)
            {
              const T s = static_cast<T>(c_S2[a][b][q]) * area;
              const T *h = H + (e * 4 + q) * 3;
              blk[0] += s * h[0];
              blk[1] += s * h[1];
              blk[2] += s * h[1];
              blk[3] += s * h[2];
            }
          const T g = gw * area * (static_cast<T>(c_D2[a][b][0]) * ih2[0] + static_cast<T>(c_D2[a][b][3]) * ih2[1]);
          blk[0] += g;
          blk[3] += g;
          const int sl = m.rc_slot[static_cast<int64_t>(k) * 4 + b];
          if (sl >= 0)
            for (int i = 0; i < 4; ++i) out[sl * 4 + i] += wa * blk[i];
          else
            {
              const HangTarget &t = tg[m.ht_off[n] + (-1 - sl)];
              for (int j = 0; j < t.count; ++j)
                for (int i = 0; i < 4; ++i) out[t.slot[j] * 4 + i] += wa * static_cast<T>(t.w[j]) * blk[i];
            }
        }
    }
  const uint32_t rmask = m.mask[n];
  const bool hang_row = m.hptr[n + 1] > m.hptr[n];
  for (int sl = 0; sl < nb; ++sl)
    {
      const int col = m.cols[r0 + sl];
      for (int cc = 0; cc < 2; ++cc)
        for (int dd = 0; dd < 2; ++dd)
          {
            T &v = out[sl * 4 + cc * 2 + dd];
            if (hang_row)
              v = (cc == dd) ? T(1) : T(0);
            else if ((rmask >> cc) & 1u)
              v = (col == n && cc == dd) ? (v != T(0) ? fabs(v) : T(1)) : T(0);
            else if ((m.mask[col] >> dd) & 1u)
              v = T(0);
          }
    }
}

// ---------------------------------------------------------------------------------
// residual gather
// ---------------------------------------------------------------------------------
__global__ void k_res_gather(DevMesh m, const double *__restrict__ r_cell, double *__restrict__ R,
                             const uint8_t *__restrict__ inst_active)
{
  pdl_wait();
  pdl_trigger();
  const int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= m.nn * m.B) return;
  const int64_t n = idx / m.B;
  const int c = static_cast<int>(idx % m.B);
  if (inst_active && !inst_active[m.node_inst[n]]) return;
  double s = 0.0;
  const bool hanging = m.hptr[n + 1] > m.hptr[n];
  if (!hanging && !((m.mask[n] >> c) & 1u))
    {
      const int stride = m.nv * m.B;
      for (int k = m.rc_ptr[n]; k < m.rc_ptr[n + 1]; ++k)
        s += m.rc_w[k] * r_cell[static_cast<int64_t>(m.rc_cell[k]) * stride + m.rc_a[k] * m.B + c];
    }
  R[idx] = s;
}

// ---------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------
template <typename T, bool WH, bool WR>
static cudaError_t launch_cell_t(const DevMesh &m, const double *x, T *H, double *r_cell, double *e_cell,
                                 const uint8_t *act, cudaStream_t s)
{
  if (m.dim == 3)
    {
      const size_t sm = sizeof(CellSmem<T>);
      static bool attr_set = false;
      if (!attr_set)
        {
          cudaError_t e = cudaFuncSetAttribute(k_cell3d<T, WH, WR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               static_cast<int>(sm));
          if (e != cudaSuccess) return e;
          attr_set = true;
        }
      const int64_t grid = (m.nc + kCPB - 1) / kCPB;
      pdl_launch(k_cell3d<T, WH, WR>, static_cast<unsigned>(grid), kCellThreads, sm, s, m, x, H, r_cell, e_cell, act);
    }
  else
    {
      const int64_t grid = (m.nc + 127) / 128;
      pdl_launch(k_cell2d<T, WH, WR>, static_cast<unsigned>(grid), 128, 0, s, m, x, H, r_cell, e_cell, act);
    }
  return cudaGetLastError();
}

template <typename R>
static cudaError_t launch_res3d(const DevMesh &m, const double *x, double *r_cell, double *e_cell, const uint8_t *act,
                                cudaStream_t s)
{
  static bool attr = false;
  if (!attr)
    {
      cudaError_t e = cudaFuncSetAttribute(k_res3d<R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           static_cast<int>(sizeof(ResSmemT<R>)));
      if (e != cudaSuccess) return e;
      attr = true;
    }
  const int64_t grid = (m.nc + kRCells - 1) / kRCells;
  pdl_launch(k_res3d<R>, static_cast<unsigned>(grid), kRThreads, sizeof(ResSmemT<R>), s, m, x, r_cell, e_cell, act);
  return cudaGetLastError();
}

cudaError_t launch_cell(const DevMesh &m, bool fp32, const double *x, void *H, double *r_cell, double *e_cell,
                        const uint8_t *act, cudaStream_t s)
{
  const bool wh = H != nullptr, wr = r_cell != nullptr;
  if (fp32)
    {
      // the mixed mode's residual (and energy): double-float arithmetic on the FP32 pipe
      if (wr && !wh && m.dim == 3 && m.B == 18) return launch_res3d<DF>(m, x, r_cell, e_cell, act, s);
      if (wr) return cudaErrorInvalidValue;
      return launch_cell_t<float, true, false>(m, x, static_cast<float *>(H), nullptr, nullptr, act, s);
    }
  if (wh && wr) return launch_cell_t<double, true, true>(m, x, static_cast<double *>(H), r_cell, e_cell, act, s);
  if (wh) return launch_cell_t<double, true, false>(m, x, static_cast<double *>(H), nullptr, nullptr, act, s);
  if (m.dim == 3) return launch_res3d<double>(m, x, r_cell, e_cell, act, s);
  return launch_cell_t<double, false, true>(m, x, nullptr, r_cell, e_cell, act, s);
}

template <typename T> static cudaError_t launch_rows_t(const DevMesh &m, const T *H, T *vals, cudaStream_t s)
{
  if (m.dim == 3)
    {
      const size_t sm = static_cast<size_t>(m.max_row_blocks) * (324 * sizeof(T) + 2 * sizeof(int));
      static size_t attr = 0;
      if (sm > attr)
        {
          cudaError_t e =
            cudaFuncSetAttribute(k_rows3d<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sm));
          if (e != cudaSuccess) return e;
          attr = sm;
        }
      if (m.n_gen > 0) pdl_launch(k_rows3d<T>, static_cast<unsigned>(m.n_gen), kRowThreads, sm, s, m, H, vals);
      if (m.n_reg > 0)
        {
          if (sizeof(T) == 4)
            pdl_launch(k_rows3d_reg<T>, static_cast<unsigned>(m.n_reg), kRegThreads, 0, s, m, H, vals);
          else
            pdl_launch(k_rows3d_reg_sym<T>, static_cast<unsigned>(m.n_reg), kRowThreads, 0, s, m, H, vals);
        }
    }
  else
    pdl_launch(k_rows2d<T>, static_cast<unsigned>((m.nn + 127) / 128), 128, 0, s, m, H, vals);
  return cudaGetLastError();
}

cudaError_t launch_rows(const DevMesh &m, bool fp32, const void *H, void *vals, cudaStream_t s)
{
  if (fp32) return launch_rows_t<float>(m, static_cast<const float *>(H), static_cast<float *>(vals), s);
  return launch_rows_t<double>(m, static_cast<const double *>(H), static_cast<double *>(vals), s);
}

// ---------------------------------------------------------------------------------
// Robin (AdGR) faces of the pair-breaking boundary (assemble.cc:286-348, residual.cc:235-278):
// on face f the surface energy wR int |A_t|^2 dS, wR = K1/bt, A_t = A with the orbital column
// of the face normal zeroed.  The face mass of Q1 is exact in closed form (robin_weight), so
// the term is sum_b W_ab(c) x_b[c] for the tangential components c of the faces holding a.
// One CTA per Robin cell, thread = (vertex a, component c): every output element is written
// by one thread after the cell kernel, so the sums stay deterministic.
// ---------------------------------------------------------------------------------
constexpr int kRobinThreads = 160; // 144 (vertex, component) threads, padded to whole warps

__global__ void __launch_bounds__(kRobinThreads) k_robin_res(DevMesh m, const double *__restrict__ x,
                                                             double *__restrict__ r_cell, double *__restrict__ e_cell,
                                                             const uint8_t *__restrict__ act)
{
  pdl_wait();
  pdl_trigger();
  __shared__ double xs[144];
  __shared__ double red[kRobinThreads / 32];
  const int64_t e = m.robin_cells[blockIdx.x];
  const int inst = m.cell_inst[e];
  if (act && !act[inst]) return; // uniform over the CTA
  const int tid = threadIdx.x;
  if (tid < 144) xs[tid] = x[static_cast<int64_t>(m.cells[e * 8 + tid / 18]) * 18 + tid % 18];
  __syncthreads();
  double en = 0.0;
  if (tid < 144)
    {
      const int a = tid / 18, c = tid % 18;
      const GeoD g = m.geo_d[e];
      const double wR = m.coef[inst * kCoef + 8];
      const int bits = m.robin[e];
      double y = 0.0;
      for (int b = 0; b < 8; ++b) y += robin_weight<double>(bits, a, b, c % 3, wR, g.w, g.x, g.y, g.z) * xs[18 * b + c];
      r_cell[e * 144 + tid] += y;
      en = xs[tid] * y;
    }
  if (!e_cell) return;
  for (int o = 16; o > 0; o >>= 1) en += __shfl_xor_sync(0xffffffffu, en, o);
  if ((tid & 31) == 0) red[tid >> 5] = en;
  __syncthreads();
  if (tid == 0)
    {
      double t = 0.0;
      for (int w = 0; w < kRobinThreads / 32; ++w) t += red[w];
      e_cell[e] += t;
    }
}

cudaError_t launch_robin_res(const DevMesh &m, const double *x, double *r_cell, double *e_cell, const uint8_t *act,
                             cudaStream_t s)
{
  if (m.n_robin == 0) return cudaSuccess;
  if (m.dim != 3 || m.B != 18 || !m.robin || !m.robin_cells) return cudaErrorInvalidValue;
  pdl_launch(k_robin_res, static_cast<unsigned>(m.n_robin), kRobinThreads, 0, s, m, x, r_cell, e_cell, act);
  return cudaGetLastError();
}

cudaError_t launch_res_gather(const DevMesh &m, const double *r_cell, double *R, const uint8_t *act, cudaStream_t s)
{
  const int64_t n = m.nn * m.B;
  pdl_launch(k_res_gather, static_cast<unsigned>((n + 255) / 256), 256, 0, s, m, r_cell, R, act);
  return cudaGetLastError();
}

} // namespace glgpu
