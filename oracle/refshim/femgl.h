/*
 * Stand-in for the reference's femgl/inc/femgl.h, used ONLY by the oracle build
 * (oracle/refshim/build_ref.sh) to compile femgl/src/cell_mat_vec/*.cc unmodified.
 * It declares just the 18 cell-function members those sources define
 * (reference femgl/inc/femgl.h:147-222), with identical signatures, on a class
 * that carries no other state.  TEST INFRASTRUCTURE: not part of the product.
 */
#ifndef GLORACLE_FEMGL_STUB_H
#define GLORACLE_FEMGL_STUB_H

#include <vector>
#include "dealii_shim.h"

namespace FemGL_mpi
{
  using namespace dealii;

  template <int dim>
  class FemGL
  {
  public:
    double mat_lhs_alpha(FullMatrix<double> &phi_u_i_q, FullMatrix<double> &phi_u_j_q,
                         FullMatrix<double> &phi_v_i_q, FullMatrix<double> &phi_v_j_q);
    double mat_lhs_beta1(FullMatrix<double> &u0, FullMatrix<double> &v0,
                         FullMatrix<double> &pui, FullMatrix<double> &puj,
                         FullMatrix<double> &pvi, FullMatrix<double> &pvj);
    double mat_lhs_beta2(FullMatrix<double> &u0, FullMatrix<double> &v0,
                         FullMatrix<double> &pui, FullMatrix<double> &puj,
                         FullMatrix<double> &pvi, FullMatrix<double> &pvj);
    double mat_lhs_beta3(FullMatrix<double> &u0, FullMatrix<double> &v0,
                         FullMatrix<double> &pui, FullMatrix<double> &puj,
                         FullMatrix<double> &pvi, FullMatrix<double> &pvj);
    double mat_lhs_beta4(FullMatrix<double> &u0, FullMatrix<double> &v0,
                         FullMatrix<double> &pui, FullMatrix<double> &puj,
                         FullMatrix<double> &pvi, FullMatrix<double> &pvj);
    double mat_lhs_beta5(FullMatrix<double> &u0, FullMatrix<double> &v0,
                         FullMatrix<double> &pui, FullMatrix<double> &puj,
                         FullMatrix<double> &pvi, FullMatrix<double> &pvj);
    double mat_lhs_K1(std::vector<FullMatrix<double>> &gpui, std::vector<FullMatrix<double>> &gpvi,
                      std::vector<FullMatrix<double>> &gpuj, std::vector<FullMatrix<double>> &gpvj);
    double mat_face_lhs_K1(FullMatrix<double> &pufi, FullMatrix<double> &pufj,
                           FullMatrix<double> &pvfi, FullMatrix<double> &pvfj);
    double mat_lhs_K2K3(std::vector<FullMatrix<double>> gpui, std::vector<FullMatrix<double>> gpvi,
                        std::vector<FullMatrix<double>> gpuj, std::vector<FullMatrix<double>> gpvj);

    double vec_rhs_alpha(FullMatrix<double> &pui, FullMatrix<double> &pvi,
                         FullMatrix<double> &u0, FullMatrix<double> &v0);
    double vec_rhs_beta1(FullMatrix<double> &u0, FullMatrix<double> &v0,
                         FullMatrix<double> &pui, FullMatrix<double> &pvi);
    double vec_rhs_beta2(FullMatrix<double> &u0, FullMatrix<double> &v0,
                         FullMatrix<double> &pui, FullMatrix<double> &pvi);
    double vec_rhs_beta3(FullMatrix<double> &u0, FullMatrix<double> &v0,
                         FullMatrix<double> &pui, FullMatrix<double> &pvi);
    double vec_rhs_beta4(FullMatrix<double> &u0, FullMatrix<double> &v0,
                         FullMatrix<double> &pui, FullMatrix<double> &pvi);
    double vec_rhs_beta5(FullMatrix<double> &u0, FullMatrix<double> &v0,
                         FullMatrix<double> &pui, FullMatrix<double> &pvi);
    double vec_rhs_K1(std::vector<FullMatrix<double>> &gu0, std::vector<FullMatrix<double>> &gv0,
                      std::vector<FullMatrix<double>> &gpui, std::vector<FullMatrix<double>> &gpvi);
    double vec_face_rhs_K1(FullMatrix<double> &pufi, FullMatrix<double> &pvfi,
                           FullMatrix<double> &ufo, FullMatrix<double> &vfo);
    double vec_rhs_K2K3(std::vector<FullMatrix<double>> gpui, std::vector<FullMatrix<double>> gpvi,
                        std::vector<FullMatrix<double>> gu0, std::vector<FullMatrix<double>> gv0);
  };
} // namespace FemGL_mpi

#endif
