// Instantiation of the patch assembly kernels (forward and backward) for
// TM_TET4 (one translation unit per element type so the build compiles them
// in parallel).
#include "backward_impl.cuh"
#include "p1tet_elast.cuh"

namespace tmg {
int assemble_tet4(const tm_patch_plan& plan, const tm_assemble_args& a, cudaStream_t s) {
  // the specialised kernels report TM_ERR_INDEX when their shared-memory
  // layout does not fit this plan (e.g. a few rows of very high degree); the
  // generic kernel then takes the launch
  int st = TM_ERR_INDEX;
  if (p1tet_fast_ok(plan) && a.form == TM_FORM_LAPLACE && a.dtype == TM_F64 && a.precision == TM_PREC_EMULATED)
    st = launch_p1tet_laplace_fast<double, L2>(plan, a, s);
  else if (p1tet_fast_ok(plan) && a.form == TM_FORM_LAPLACE && a.dtype == TM_F32)
    st = launch_p1tet_laplace_fast<float, float>(plan, a, s);
  const bool elast_coef = a.coef_kind == TM_COEF_SCALAR || a.coef_kind == TM_COEF_ELEMENT;
  if (p1tet_elast_ok(plan) && a.form == TM_FORM_ELASTICITY && elast_coef && a.dtype == TM_F64 &&
      a.precision == TM_PREC_EMULATED)
    st = launch_p1tet_elast<double, L2>(plan, a, s);
  else if (p1tet_elast_ok(plan) && a.form == TM_FORM_ELASTICITY && elast_coef && a.dtype == TM_F32)
    st = launch_p1tet_elast<float, float>(plan, a, s);
  if (st != TM_ERR_INDEX) return st;
  return assemble_element<TM_TET4>(plan, a, s);
}
int backward_tet4(const tm_patch_plan& plan, const tm_assemble_args& a, const tm_backward_args& bw, cudaStream_t s) {
  return backward_element<TM_TET4>(plan, a, bw, s);
}
}  // namespace tmg
