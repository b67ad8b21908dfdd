// TM_TET10 patch assembly kernels for one arithmetic (<float, float>); dispatched from
// assemble_tet10.cu.
#include "assemble_impl.cuh"

namespace tmg {
int assemble_tet10_f32(const tm_patch_plan& plan, const tm_assemble_args& a, cudaStream_t s) {
  return assemble_element_as<TM_TET10, float, float>(plan, a, s);
}
}  // namespace tmg
