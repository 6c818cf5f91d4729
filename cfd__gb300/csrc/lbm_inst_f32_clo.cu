// lbm_inst_f32_clo.cu — the learned-closure step kernels for the f32 population
// storage form (a unit of their own: they are the longest to compile).
#include "lbm_kernels.cuh"

namespace lbm {
StepClosureFn closure_f32() { return OpsImpl<StF32>::closure_entry(); }
}  // namespace lbm
