// Patch assembly (forward and backward) for TM_TET10.  Its kernels are the
// heaviest to compile, so each arithmetic is instantiated in its own
// translation unit (assemble_tet10_{f32,f64,df64}.cu, backward_tet10_{f32,f64}.cu)
// and this file only dispatches, in the order assemble_element and
// backward_element use.
#include "../../include/tensormesh_gb300.h"
#include <cuda_runtime.h>

namespace tmg {
int assemble_tet10_f32(const tm_patch_plan&, const tm_assemble_args&, cudaStream_t);
int assemble_tet10_f64(const tm_patch_plan&, const tm_assemble_args&, cudaStream_t);
int assemble_tet10_df64(const tm_patch_plan&, const tm_assemble_args&, cudaStream_t);
int backward_tet10_f32(const tm_patch_plan&, const tm_assemble_args&, const tm_backward_args&, cudaStream_t);
int backward_tet10_f64(const tm_patch_plan&, const tm_assemble_args&, const tm_backward_args&, cudaStream_t);

int assemble_tet10(const tm_patch_plan& plan, const tm_assemble_args& a, cudaStream_t s) {
  if (a.dtype == TM_F32) return assemble_tet10_f32(plan, a, s);
  if (a.precision == TM_PREC_NATIVE) return assemble_tet10_f64(plan, a, s);
  return assemble_tet10_df64(plan, a, s);
}
int backward_tet10(const tm_patch_plan& plan, const tm_assemble_args& a, const tm_backward_args& bw, cudaStream_t s) {
  if (a.dtype == TM_F32) return backward_tet10_f32(plan, a, bw, s);
  return backward_tet10_f64(plan, a, bw, s);
}
}  // namespace tmg
