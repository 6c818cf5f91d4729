// lbm_inst_f16s_clo.cu — the learned-closure step kernels for the f16s population
// storage form (a unit of their own: they are the longest to compile).
#include "lbm_kernels.cuh"

namespace lbm {
StepClosureFn closure_f16s() { return OpsImpl<StF16S>::closure_entry(); }
}  // namespace lbm
