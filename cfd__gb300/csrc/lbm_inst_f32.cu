// lbm_inst_f32.cu — kernel instantiation for the f32 population storage form.
#include "lbm_kernels.cuh"

namespace lbm {
Ops ops_f32() {
  Ops o = OpsImpl<StF32>::make();
  o.step_closure = closure_f32();
  return o;
}
}  // namespace lbm
