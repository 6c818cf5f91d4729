// lbm_inst_f16sr.cu — kernel instantiation for the f16sr population storage form
// (16-bit stores rounded stochastically).
#include "lbm_kernels.cuh"

namespace lbm {
Ops ops_f16sr() {
  Ops o = OpsImpl<StF16SR>::make();
  o.step_closure = closure_f16sr();
  return o;
}
}  // namespace lbm
