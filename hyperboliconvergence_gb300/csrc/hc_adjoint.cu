// hc_adjoint.cu -- C ABI of the discrete adjoint (include/hc.h): FP64 and
// double-float contexts run the R = double driver instantiated here, FP32
// contexts the R = float one instantiated in hc_adjoint_f32.cu.
#include "hc_adjoint_driver.cuh"

namespace hc {
namespace adj {
extern template int objective_forward<float>(hc_ctx*, int, const hc_objective*, const double*, double*, double*);
extern template int adjoint_gradient<float>(hc_ctx*, int, int, const hc_objective*, const double*, double*, double*,
                                            double*, hc_adjoint_stats*);
}  // namespace adj
}  // namespace hc

extern "C" {

int hc_objective_forward(hc_ctx* c, int nsteps, const hc_objective* obj, const double* rates_in, double* rates_out,
                         double* J) {
  if (!c) return hc::fail(HC_ERR_ARG, "null context");
  if (c->fp32) return hc::adj::objective_forward<float>(c, nsteps, obj, rates_in, rates_out, J);
  return hc::adj::objective_forward<double>(c, nsteps, obj, rates_in, rates_out, J);
}

int hc_adjoint_gradient(hc_ctx* c, int nsteps, int snapshots, const hc_objective* obj, const double* rates_in,
                        double* q0_bar, double* ref_bar, double* rates_out, hc_adjoint_stats* stats) {
  if (!c) return hc::fail(HC_ERR_ARG, "null context");
  if (c->fp32)
    return hc::adj::adjoint_gradient<float>(c, nsteps, snapshots, obj, rates_in, q0_bar, ref_bar, rates_out, stats);
  return hc::adj::adjoint_gradient<double>(c, nsteps, snapshots, obj, rates_in, q0_bar, ref_bar, rates_out, stats);
}

}  // extern "C"
