// FP32 form of the fused narrow-band curvature flow (fast WENO weights on
// packed cell pairs); the band's distance test gives the FP64 decisions.
#include "bandflow.cuh"

extern "C" int lsmgpu_band_flow_weno5_tvdrk3_f32(float *phi, const int *gb, const int *fb, float dx, float a_n,
                                                 float b_n, float cfl, float gamma, float beta, int n_steps,
                                                 int rebuild_every, double *dt_log, long long *band_log) {
  using namespace lsmgpu;
  if (!phi || !gb || !fb) {
    set_error(LSMGPU_ERR_ARGUMENT, "band flow: null argument");
    return LSMGPU_ERR_ARGUMENT;
  }
  const Box g = mkbox(gb, gb + 1, gb + 2, gb + 3, gb + 4, gb + 5), f = mkbox(fb, fb + 1, fb + 2, fb + 3, fb + 4, fb + 5);
  return bandflow::run<float, false>("lsmgpu_band_flow_weno5_tvdrk3_f32", phi, g, f, dx, a_n, b_n, cfl, gamma, beta,
                                     n_steps, rebuild_every, dt_log, band_log);
}
