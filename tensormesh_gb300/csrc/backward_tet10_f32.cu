// TM_TET10 patch backward kernels for one value type (float); dispatched from
// assemble_tet10.cu.
#include "backward_impl.cuh"

namespace tmg {
int backward_tet10_f32(const tm_patch_plan& plan, const tm_assemble_args& a, const tm_backward_args& bw,
                       cudaStream_t s) {
  return backward_element_as<TM_TET10, float>(plan, a, bw, s);
}
}  // namespace tmg
