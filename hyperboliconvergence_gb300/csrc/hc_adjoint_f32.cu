// hc_adjoint_f32.cu -- the discrete adjoint driver for FP32 contexts (a
// translation unit of its own so it compiles in parallel with the FP64 one).
#include "hc_adjoint_driver.cuh"

namespace hc {
namespace adj {
template int objective_forward<float>(hc_ctx*, int, const hc_objective*, const double*, double*, double*);
template int wall_force<float>(hc_ctx*, const double*, double*);
template int adjoint_record<float>(hc_ctx*, int, int, const hc_objective*, const double*, double*, double*);
template int adjoint_reverse<float>(hc_ctx*, double*, double*, bool, hc_adjoint_stats*);
template int adjoint_gradient<float>(hc_ctx*, int, int, const hc_objective*, const double*, double*, double*,
                                     double*, hc_adjoint_stats*);
}  // namespace adj
}  // namespace hc
