// LSMLIB's scalar smoothed Heaviside and delta functions
// (src/toolbox/lsm_calculus_toolbox.f:25, :68) with their symbol names and
// argument lists.  They evaluate one value for one x: the calling thread
// computes it (a kernel launch would cost thousands of times the arithmetic).
// The array kernels that integrate with these functions (geometry.cu,
// adjoint.cuh) evaluate the same formulas on the device.
//
// Host arithmetic in the reference's operation order, compiled without FP
// contraction, with the reference's constants: pi to 21 digits and 1/pi
// truncated to 0.31830988618379.
#include <math.h>

#include "../../include/lsmgpu_toolbox3d.h"

extern "C" {

void lsmheaviside_(double *H, const double *x, const double *epsilon) {
  const double xv = *x, e = *epsilon;
  const double pi = 3.14159265358979323846, one_over_pi = 0.31830988618379;
  if (xv < -e) {
    *H = 0.0;
  } else if (xv > e) {
    *H = 1.0;
  } else {
    const double ooe = 1.0 / e;
    *H = 0.5 * (1.0 + xv * ooe + one_over_pi * sin(pi * xv * ooe));
  }
}

void lsmdeltafunction_(double *delta, const double *x, const double *epsilon) {
  const double xv = *x, e = *epsilon;
  const double pi = 3.14159265358979323846;
  if (fabs(xv) > e) {
    *delta = 0.0;
  } else {
    const double ooe = 1.0 / e;
    *delta = 0.5 * ooe * (1.0 + cos(pi * xv * ooe));
  }
}

}  // extern "C"
