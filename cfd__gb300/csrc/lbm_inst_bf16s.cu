// lbm_inst_bf16s.cu — kernel instantiation for the bf16s population storage form.
#include "lbm_kernels.cuh"

namespace lbm {
Ops ops_bf16s() {
  Ops o = OpsImpl<StBF16S>::make();
  o.step_closure = closure_bf16s();
  return o;
}
}  // namespace lbm
