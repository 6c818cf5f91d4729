// lbm_inst_f16s.cu — kernel instantiation for the f16s population storage form.
#include "lbm_kernels.cuh"

namespace lbm {
Ops ops_f16s() {
  Ops o = OpsImpl<StF16S>::make();
  o.step_closure = closure_f16s();
  return o;
}
}  // namespace lbm
