// lbm_inst_bf16sr.cu — kernel instantiation for the bf16sr population storage form
// (16-bit stores rounded stochastically).
#include "lbm_kernels.cuh"

namespace lbm {
Ops ops_bf16sr() {
  Ops o = OpsImpl<StBF16SR>::make();
  o.step_closure = closure_bf16sr();
  return o;
}
}  // namespace lbm
