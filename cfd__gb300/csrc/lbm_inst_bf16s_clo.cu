// lbm_inst_bf16s_clo.cu — the learned-closure step kernels for the bf16s population
// storage form (a unit of their own: they are the longest to compile).
#include "lbm_kernels.cuh"

namespace lbm {
StepClosureFn closure_bf16s() { return OpsImpl<StBF16S>::closure_entry(); }
}  // namespace lbm
