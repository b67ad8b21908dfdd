// Instantiation of the patch assembly kernels (forward and backward) for
// TM_TRI6 (one translation unit per element type so the build compiles them
// in parallel).
#include "backward_impl.cuh"

namespace tmg {
int assemble_tri6(const tm_patch_plan& plan, const tm_assemble_args& a, cudaStream_t s) {
  return assemble_element<TM_TRI6>(plan, a, s);
}
int backward_tri6(const tm_patch_plan& plan, const tm_assemble_args& a, const tm_backward_args& bw, cudaStream_t s) {
  return backward_element<TM_TRI6>(plan, a, bw, s);
}
}  // namespace tmg
