/*
 * C entry points around the reference's own, unmodified cell kernels
 * (femgl/src/cell_mat_vec/*.cc) and material parameters (matep/src/matep.cc),
 * compiled by oracle/refshim/build_ref.sh into oracle/_ref/libglref.so.
 *
 * TEST INFRASTRUCTURE ONLY.  Used by tests/golden/make_golden.py to generate the
 * golden fixtures, by the CPU tests to pin the oracle restatement, and by the
 * CPU-baseline leg of bench.py to time the reference's per-(i,j,q) assembly.
 *
 * Packing of an 18-vector (reference femgl/src/s_vector2matrix.cc:154-161):
 *   c in [0,9)  -> u(c/3, c%3);   c in [9,18) -> v((c-9)/3, (c-9)%3).
 * A gradient is stored [k][c], k = spatial derivative 0..2.
 */
#include <cmath>
#include <vector>

#include "femgl.h"
#include "matep.h"

using dealii::FullMatrix;
using FemGL_mpi::FemGL;

namespace
{
  void unpack(const double *a, FullMatrix<double> &u, FullMatrix<double> &v)
  {
    for (int c = 0; c < 9; ++c)
      {
        u(c / 3, c % 3) = a[c];
        v(c / 3, c % 3) = a[9 + c];
      }
  }

  void unpack_grad(const double *g, std::vector<FullMatrix<double>> &gu, std::vector<FullMatrix<double>> &gv)
  {
    for (int k = 0; k < 3; ++k) unpack(g + 18 * k, gu[k], gv[k]);
  }

  FemGL<3> &obj()
  {
    static FemGL<3> f;
    return f;
  }
} // namespace

extern "C" {

/* term: 0 alpha, 1..5 beta_t.  Returns the reference's mat_lhs_<term>(A; Phi_i, Phi_j). */
double ref_bulk_mat(int term, const double *A, const double *Pi, const double *Pj)
{
  FullMatrix<double> u0(3, 3), v0(3, 3), pui(3, 3), pvi(3, 3), puj(3, 3), pvj(3, 3);
  unpack(A, u0, v0);
  unpack(Pi, pui, pvi);
  unpack(Pj, puj, pvj);
  FemGL<3> &f = obj();
  switch (term)
    {
    case 0: return f.mat_lhs_alpha(pui, puj, pvi, pvj);
    case 1: return f.mat_lhs_beta1(u0, v0, pui, puj, pvi, pvj);
    case 2: return f.mat_lhs_beta2(u0, v0, pui, puj, pvi, pvj);
    case 3: return f.mat_lhs_beta3(u0, v0, pui, puj, pvi, pvj);
    case 4: return f.mat_lhs_beta4(u0, v0, pui, puj, pvi, pvj);
    case 5: return f.mat_lhs_beta5(u0, v0, pui, puj, pvi, pvj);
    default: return NAN;
    }
}

/* term: 0 alpha, 1..5 beta_t.  Returns the reference's vec_rhs_<term>(A; Phi_i). */
double ref_bulk_vec(int term, const double *A, const double *Pi)
{
  FullMatrix<double> u0(3, 3), v0(3, 3), pui(3, 3), pvi(3, 3);
  unpack(A, u0, v0);
  unpack(Pi, pui, pvi);
  FemGL<3> &f = obj();
  switch (term)
    {
    case 0: return f.vec_rhs_alpha(pui, pvi, u0, v0);
    case 1: return f.vec_rhs_beta1(u0, v0, pui, pvi);
    case 2: return f.vec_rhs_beta2(u0, v0, pui, pvi);
    case 3: return f.vec_rhs_beta3(u0, v0, pui, pvi);
    case 4: return f.vec_rhs_beta4(u0, v0, pui, pvi);
    case 5: return f.vec_rhs_beta5(u0, v0, pui, pvi);
    default: return NAN;
    }
}

/* term: 0 K1, 1 K2K3.  gPi, gPj are [3][18] gradients of the test/trial tensors. */
double ref_grad_mat(int term, const double *gPi, const double *gPj)
{
  std::vector<FullMatrix<double>> gui(3, FullMatrix<double>(3, 3)), gvi(3, FullMatrix<double>(3, 3)),
    guj(3, FullMatrix<double>(3, 3)), gvj(3, FullMatrix<double>(3, 3));
  unpack_grad(gPi, gui, gvi);
  unpack_grad(gPj, guj, gvj);
  FemGL<3> &f = obj();
  if (term == 0) return f.mat_lhs_K1(gui, gvi, guj, gvj);
  if (term == 1) return f.mat_lhs_K2K3(gui, gvi, guj, gvj);
  return NAN;
}

/* term: 0 K1, 1 K2K3.  gA is the [3][18] gradient of the iterate, gPi of the test tensor. */
double ref_grad_vec(int term, const double *gA, const double *gPi)
{
  std::vector<FullMatrix<double>> gu(3, FullMatrix<double>(3, 3)), gv(3, FullMatrix<double>(3, 3)),
    gui(3, FullMatrix<double>(3, 3)), gvi(3, FullMatrix<double>(3, 3));
  unpack_grad(gA, gu, gv);
  unpack_grad(gPi, gui, gvi);
  FemGL<3> &f = obj();
  if (term == 0) return f.vec_rhs_K1(gu, gv, gui, gvi);
  if (term == 1) return f.vec_rhs_K2K3(gui, gvi, gu, gv);
  return NAN;
}

/* Robin face terms (active only when the AdGR length bt < 1e10). */
double ref_face_mat(const double *Pi, const double *Pj)
{
  FullMatrix<double> pui(3, 3), pvi(3, 3), puj(3, 3), pvj(3, 3);
  unpack(Pi, pui, pvi);
  unpack(Pj, puj, pvj);
  return obj().mat_face_lhs_K1(pui, puj, pvi, pvj);
}

double ref_face_vec(const double *A, const double *Pi)
{
  FullMatrix<double> u0(3, 3), v0(3, 3), pui(3, 3), pvi(3, 3);
  unpack(A, u0, v0);
  unpack(Pi, pui, pvi);
  return obj().vec_face_rhs_K1(pui, pvi, u0, v0);
}

/* Material parameters from the reference's Matep at (p [bar], t = T/Tc).
 * out = {alpha, beta1..beta5, gap_A, gap_B, Tc_mK, f_A, f_B, beta_A, beta_B}. */
void ref_matep(double p, double t, int scc, double *out)
{
  FemGL_mpi::Matep m;
  m.with_SCC(scc != 0);
  out[0] = m.alpha_td(t);
  out[1] = m.beta1_td(p, t);
  out[2] = m.beta2_td(p, t);
  out[3] = m.beta3_td(p, t);
  out[4] = m.beta4_td(p, t);
  out[5] = m.beta5_td(p, t);
  out[6] = m.gap_A_td(p, t);
  out[7] = m.gap_B_td(p, t);
  out[8] = m.Tcp_mK(p);
  out[9] = m.f_A_td(p, t);
  out[10] = m.f_B_td(p, t);
  out[11] = m.beta_A_td(p, t);
  out[12] = m.beta_B_td(p, t);
}

/*
 * One Q1 hexahedral cell, axis-aligned with edge lengths h[3], evaluated the way
 * the reference's assemble_system does it (femgl/src/assemble.cc:188-280):
 * for every quadrature point q of QGauss(2), for every test dof i and trial dof j
 * of the 144 cell dofs, the full tensors Phi_i, Phi_j, grad Phi_i, grad Phi_j are
 * built (FESystem(FE_Q(1),18): dof i -> vertex i/18, component i%18) and the
 * nine reference kernels are called with the coefficients of assemble.cc:229-276.
 *
 * x: nodal values [8][18] in deal.II vertex order (vertex v = ix + 2 iy + 4 iz).
 * coef = {K1, K2, K3, alpha, beta1..beta5}.
 * cell_matrix: [144][144] (may be NULL to skip the Jacobian), cell_rhs: [144].
 * The sign convention is the reference's: cell_rhs = -R.
 */
void ref_cell_assemble(const double *h, const double *x, const double *coef, double *cell_matrix,
                       double *cell_rhs)
{
  const double K1 = coef[0], K2 = coef[1], K3 = coef[2], alpha = coef[3];
  const double b1 = coef[4], b2 = coef[5], b3 = coef[6], b4 = coef[7], b5 = coef[8];
  const double g = 0.5 - std::sqrt(3.0) / 6.0;
  const double gp[2] = {g, 1.0 - g};
  const double JxW = 0.125 * h[0] * h[1] * h[2];
  FemGL<3> &f = obj();

  if (cell_matrix)
    for (int k = 0; k < 144 * 144; ++k) cell_matrix[k] = 0.0;
  for (int k = 0; k < 144; ++k) cell_rhs[k] = 0.0;

  double val[8][8], grd[8][8][3];
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
              ds[d] = (bit ? 1.0 : -1.0) / h[d];
            }
          val[q][v] = s[0] * s[1] * s[2];
          grd[q][v][0] = ds[0] * s[1] * s[2];
          grd[q][v][1] = s[0] * ds[1] * s[2];
          grd[q][v][2] = s[0] * s[1] * ds[2];
        }
    }

  const FullMatrix<double> zero33(3, 3);
  FullMatrix<double> u0(3, 3), v0(3, 3);
  std::vector<FullMatrix<double>> gu0(3, zero33), gv0(3, zero33);
  FullMatrix<double> pui(3, 3), pvi(3, 3), puj(3, 3), pvj(3, 3);
  std::vector<FullMatrix<double>> gpui(3, zero33), gpvi(3, zero33), gpuj(3, zero33), gpvj(3, zero33);

  auto shape = [&](int i, int q, FullMatrix<double> &pu, FullMatrix<double> &pv, std::vector<FullMatrix<double>> &gpu,
                   std::vector<FullMatrix<double>> &gpv) {
    pu = 0.0;
    pv = 0.0;
    for (int k = 0; k < 3; ++k)
      {
        gpu[k] = 0.0;
        gpv[k] = 0.0;
      }
    const int v = i / 18, c = i % 18;
    FullMatrix<double> &P = (c < 9) ? pu : pv;
    std::vector<FullMatrix<double>> &G = (c < 9) ? gpu : gpv;
    const int cc = c % 9;
    P(cc / 3, cc % 3) = val[q][v];
    for (int k = 0; k < 3; ++k) G[k](cc / 3, cc % 3) = grd[q][v][k];
  };

  for (int q = 0; q < 8; ++q)
    {
      u0 = 0.0;
      v0 = 0.0;
      for (int k = 0; k < 3; ++k)
        {
          gu0[k] = 0.0;
          gv0[k] = 0.0;
        }
      for (int v = 0; v < 8; ++v)
        for (int c = 0; c < 18; ++c)
          {
            const double xv = x[18 * v + c];
            FullMatrix<double> &M = (c < 9) ? u0 : v0;
            std::vector<FullMatrix<double>> &G = (c < 9) ? gu0 : gv0;
            const int cc = c % 9;
            M(cc / 3, cc % 3) += xv * val[q][v];
            for (int k = 0; k < 3; ++k) G[k](cc / 3, cc % 3) += xv * grd[q][v][k];
          }

      for (int i = 0; i < 144; ++i)
        {
          shape(i, q, pui, pvi, gpui, gpvi);
          if (cell_matrix)
            for (int j = 0; j < 144; ++j)
              {
                shape(j, q, puj, pvj, gpuj, gpvj);
                cell_matrix[144 * i + j] +=
                  ((K1 * f.mat_lhs_K1(gpui, gpvi, gpuj, gpvj)) + ((K2 + K3) * f.mat_lhs_K2K3(gpui, gpvi, gpuj, gpvj)) +
                   (alpha * f.mat_lhs_alpha(pui, puj, pvi, pvj)) +
                   2.0 * ((b1 * f.mat_lhs_beta1(u0, v0, pui, puj, pvi, pvj)) +
                          (b2 * f.mat_lhs_beta2(u0, v0, pui, puj, pvi, pvj)) +
                          (b3 * f.mat_lhs_beta3(u0, v0, pui, puj, pvi, pvj)) +
                          (b4 * f.mat_lhs_beta4(u0, v0, pui, puj, pvi, pvj)) +
                          (b5 * f.mat_lhs_beta5(u0, v0, pui, puj, pvi, pvj)))) *
                  JxW;
              }
          cell_rhs[i] -= ((K1 * f.vec_rhs_K1(gu0, gv0, gpui, gpvi)) + ((K2 + K3) * f.vec_rhs_K2K3(gpui, gpvi, gu0, gv0)) +
                          (alpha * f.vec_rhs_alpha(pui, pvi, u0, v0)) +
                          2.0 * ((b1 * f.vec_rhs_beta1(u0, v0, pui, pvi)) + (b2 * f.vec_rhs_beta2(u0, v0, pui, pvi)) +
                                 (b3 * f.vec_rhs_beta3(u0, v0, pui, pvi)) + (b4 * f.vec_rhs_beta4(u0, v0, pui, pvi)) +
                                 (b5 * f.vec_rhs_beta5(u0, v0, pui, pvi)))) *
                         JxW;
        }
    }
}

/*
 * The Robin (AdGR) face term of one face of the same axis-aligned Q1 cell, evaluated the
 * way the reference's assemble_system does it (femgl/src/assemble.cc:286-348): for every
 * point of the face rule QGauss<2>(2), the iterate and every test / trial tensor are built
 * with the face's normal column zeroed (femgl/src/s_vector2matrix.cc:220-292,
 * femgl/src/phi_vector2matrix.cc:153-190) and the reference's face kernels are called with
 * the weights and signs of assemble.cc:322-336.
 *
 * face = 2 * axis + side: the face whose vertices have bit `axis` of v equal to `side`;
 * it plays the boundary id 2 + axis.  Adds into cell_matrix [144][144] (may be NULL) and
 * cell_rhs [144].
 */
void ref_face_assemble(const double *h, const double *x, double K1, double bt, int face, double *cell_matrix,
                       double *cell_rhs)
{
  const int axis = face / 2, side = face % 2;
  const int t1 = (axis == 0) ? 1 : 0, t2 = (axis == 2) ? 1 : 2;
  const double g = 0.5 - std::sqrt(3.0) / 6.0;
  const double gp[2] = {g, 1.0 - g};
  const double JxW = 0.25 * h[t1] * h[t2];
  FemGL<3> &f = obj();
  FullMatrix<double> u0(3, 3), v0(3, 3), pui(3, 3), pvi(3, 3), puj(3, 3), pvj(3, 3);

  for (int q = 0; q < 4; ++q)
    {
      double val[8];
      for (int v = 0; v < 8; ++v)
        {
          const int b1 = (v >> t1) & 1, b2 = (v >> t2) & 1;
          const double s1 = b1 ? gp[q & 1] : 1.0 - gp[q & 1], s2 = b2 ? gp[q >> 1] : 1.0 - gp[q >> 1];
          val[v] = (((v >> axis) & 1) == side) ? s1 * s2 : 0.0;
        }
      auto shape = [&](int i, FullMatrix<double> &pu, FullMatrix<double> &pv) {
        pu = 0.0;
        pv = 0.0;
        const int v = i / 18, c = i % 18, cc = c % 9;
        if (cc % 3 == axis) return; /* the normal column stays zero */
        ((c < 9) ? pu : pv)(cc / 3, cc % 3) = val[v];
      };
      u0 = 0.0;
      v0 = 0.0;
      for (int v = 0; v < 8; ++v)
        for (int c = 0; c < 18; ++c)
          {
            const int cc = c % 9;
            if (cc % 3 == axis) continue;
            ((c < 9) ? u0 : v0)(cc / 3, cc % 3) += x[18 * v + c] * val[v];
          }
      for (int i = 0; i < 144; ++i)
        {
          shape(i, pui, pvi);
          if (cell_matrix)
            for (int j = 0; j < 144; ++j)
              {
                shape(j, puj, pvj);
                cell_matrix[144 * i + j] -= K1 * (-1.0 / bt) * f.mat_face_lhs_K1(pui, puj, pvi, pvj) * JxW;
              }
          cell_rhs[i] -= (-K1) * (-1.0 / bt) * f.vec_face_rhs_K1(pui, pvi, u0, v0) * JxW;
        }
    }
}

} // extern "C"
