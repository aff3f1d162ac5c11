/*
 * C entry point around the reference's own PDW initial-state function
 * (femgl/inc/pdw_config.h, class PDWconfig<3>), compiled unmodified by
 * oracle/refshim/build_ref.sh into oracle/_ref/libglref.so.  TEST INFRASTRUCTURE ONLY:
 * used to pin the product's restatement (glgpu_pdw_guess).
 */
#include "dealii_shim.h"

#include "pdw_config.h"

extern "C" void ref_pdw_value(double u, double q, double half_D, double gap, double x, double y, double z, double *out)
{
  FemGL_mpi::PDWconfig<3> f(u, q, half_D, gap);
  dealii::Vector<double> v(18);
  f.vector_value(dealii::Point<3>(x, y, z), v);
  for (int c = 0; c < 18; ++c) out[c] = v(c);
}
