// lbm_inst_f64.cu — kernel instantiation for the f64 population storage form.
#include "lbm_kernels.cuh"

namespace lbm {
Ops ops_f64() { return OpsImpl<StF64>::make(); }
}  // namespace lbm
