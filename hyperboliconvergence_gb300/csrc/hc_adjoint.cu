// hc_adjoint.cu -- C ABI of the discrete adjoint (include/hc.h): FP64 and
// double-float contexts run the R = double driver instantiated here, FP32
// contexts the R = float one instantiated in hc_adjoint_f32.cu.
#include "hc_adjoint_driver.cuh"

namespace hc {
namespace adj {
extern template int objective_forward<float>(hc_ctx*, int, const hc_objective*, const double*, double*, double*);
extern template int wall_force<float>(hc_ctx*, const double*, double*);
extern template int adjoint_record<float>(hc_ctx*, int, int, const hc_objective*, const double*, double*, double*);
extern template int adjoint_reverse<float>(hc_ctx*, double*, double*, bool, hc_adjoint_stats*);
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

int hc_adjoint_record(hc_ctx* c, int nsteps, int snapshots, const hc_objective* obj, const double* rates_in,
                      double* rates_out, double* J) {
  if (!c) return hc::fail(HC_ERR_ARG, "null context");
  if (c->fp32) return hc::adj::adjoint_record<float>(c, nsteps, snapshots, obj, rates_in, rates_out, J);
  return hc::adj::adjoint_record<double>(c, nsteps, snapshots, obj, rates_in, rates_out, J);
}

int hc_adjoint_reverse(hc_ctx* c, double* q0_bar, double* ref_bar, int on_device, hc_adjoint_stats* stats) {
  if (!c) return hc::fail(HC_ERR_ARG, "null context");
  if (c->fp32) return hc::adj::adjoint_reverse<float>(c, q0_bar, ref_bar, on_device != 0, stats);
  return hc::adj::adjoint_reverse<double>(c, q0_bar, ref_bar, on_device != 0, stats);
}

int hc_wall_force(hc_ctx* c, const double dir[2], double* force) {
  if (!c) return hc::fail(HC_ERR_ARG, "null context");
  if (c->fp32) return hc::adj::wall_force<float>(c, dir, force);
  return hc::adj::wall_force<double>(c, dir, force);
}

int hc_adjoint_gradient(hc_ctx* c, int nsteps, int snapshots, const hc_objective* obj, const double* rates_in,
                        double* q0_bar, double* ref_bar, double* rates_out, hc_adjoint_stats* stats) {
  if (!c) return hc::fail(HC_ERR_ARG, "null context");
  if (c->fp32)
    return hc::adj::adjoint_gradient<float>(c, nsteps, snapshots, obj, rates_in, q0_bar, ref_bar, rates_out, stats);
  return hc::adj::adjoint_gradient<double>(c, nsteps, snapshots, obj, rates_in, q0_bar, ref_bar, rates_out, stats);
}

}  // extern "C"
