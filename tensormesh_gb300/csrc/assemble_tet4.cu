// Instantiation of the patch assembly kernels (forward and backward) for
// TM_TET4 (one translation unit per element type so the build compiles them
// in parallel).
#include "backward_impl.cuh"

namespace tmg {
int assemble_tet4(const tm_patch_plan& plan, const tm_assemble_args& a, cudaStream_t s) {
  return assemble_element<TM_TET4>(plan, a, s);
}
int backward_tet4(const tm_patch_plan& plan, const tm_assemble_args& a, const tm_backward_args& bw, cudaStream_t s) {
  return backward_element<TM_TET4>(plan, a, bw, s);
}
}  // namespace tmg
