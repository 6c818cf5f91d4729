// lbm_inst_f16sr_clo.cu — the learned-closure step kernels for the f16sr population
// storage form (16-bit stores rounded stochastically; a unit of their own).
#include "lbm_kernels.cuh"

namespace lbm {
StepClosureFn closure_f16sr() { return OpsImpl<StF16SR>::closure_entry(); }
}  // namespace lbm
