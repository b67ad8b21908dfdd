// Instantiation of the patch assembly kernels (forward and backward) for
// TM_TRI3 (one translation unit per element type so the build compiles them
// in parallel).
#include "backward_impl.cuh"

namespace tmg {
int assemble_tri3(const tm_patch_plan& plan, const tm_assemble_args& a, cudaStream_t s) {
  return assemble_element<TM_TRI3>(plan, a, s);
}
int backward_tri3(const tm_patch_plan& plan, const tm_assemble_args& a, const tm_backward_args& bw, cudaStream_t s) {
  return backward_element<TM_TRI3>(plan, a, bw, s);
}
}  // namespace tmg
