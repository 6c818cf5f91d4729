// lbm_inst_bf16sr.cu — kernel instantiation for the bf16sr population storage form
// (16-bit stores rounded stochastically).
#include "lbm_kernels.cuh"

namespace lbm {
Ops ops_bf16sr() { return OpsImpl<StBF16SR>::make(); }
}  // namespace lbm
