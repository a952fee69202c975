// FP64 parity form of the fused narrow-band curvature flow (-fmad=false).
#include "bandflow.cuh"

extern "C" int lsmgpu_band_flow_weno5_tvdrk3_f64(double *phi, const int *gb, const int *fb, double dx, double a_n,
                                                 double b_n, double cfl, double gamma, double beta, int n_steps,
                                                 int rebuild_every, double *dt_log, long long *band_log) {
  using namespace lsmgpu;
  if (!phi || !gb || !fb) {
    set_error(LSMGPU_ERR_ARGUMENT, "band flow: null argument");
    return LSMGPU_ERR_ARGUMENT;
  }
  const Box g = mkbox(gb, gb + 1, gb + 2, gb + 3, gb + 4, gb + 5), f = mkbox(fb, fb + 1, fb + 2, fb + 3, fb + 4, fb + 5);
  return bandflow::run<double, true>("lsmgpu_band_flow_weno5_tvdrk3_f64", phi, g, f, dx, a_n, b_n, cfl, gamma, beta,
                                     n_steps, rebuild_every, dt_log, band_log);
}
