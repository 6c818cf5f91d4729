// lbm_inst_bf16sr_clo.cu — the learned-closure step kernels for the bf16sr population
// storage form (16-bit stores rounded stochastically; a unit of their own).
#include "lbm_kernels.cuh"

namespace lbm {
StepClosureFn closure_bf16sr() { return OpsImpl<StBF16SR>::closure_entry(); }
}  // namespace lbm
