// TM_TET10 patch assembly kernels for one arithmetic (<double, double>); dispatched from
// assemble_tet10.cu.
#include "assemble_impl.cuh"

namespace tmg {
int assemble_tet10_f64(const tm_patch_plan& plan, const tm_assemble_args& a, cudaStream_t s) {
  return assemble_element_as<TM_TET10, double, double>(plan, a, s);
}
}  // namespace tmg
