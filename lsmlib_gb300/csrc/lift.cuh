// Running LSMLIB's 2D and 1D drop-in routines on the 3D kernels.
//
// A 2D array phi(ilo:ihi, jlo:jhi) has the memory of the 3D array
// phi(ilo:ihi, jlo:jhi, 0:0).  A 2D entry point (lifted.cu) passes its arrays
// to the 3D routine with k bounds 0:0, dx for the missing dz (1 where the 3D
// routine multiplies dx dy dz into a cell volume), a zeroed device buffer for
// each missing input component (phi_z, vel_z, phi_xz ...) and a scratch
// device buffer for each missing output component, while a Lift object holds
// g_lift_dims at 2 (1 for 1D entries).  In that state every view has stride
// 0 along the missing axes, so a stencil reaching along them reads the centre
// cell and its differences are exactly 0, and boxes need no reach along them.
// With those zeros the 3D formulas reduce term for term to the 2D and 1D
// routines of the reference: each lifted entry point is checked bit for bit
// against them.
#pragma once

#include "lsmgpu_common.cuh"

namespace lsmgpu {

class Lift {
 public:
  Lift(int dims, const char *name);
  ~Lift();
  Lift(const Lift &) = delete;
  Lift &operator=(const Lift &) = delete;
  // Records the size of one of the call's index boxes (2D: four bounds,
  // 1D: two) or the bounds of an index list (all lists of a call together:
  // their entries are numbered from the lowest nlo to the highest nhi), so
  // the stand-in buffers cover them.
  void box(const int *ilo, const int *ihi, const int *jlo = nullptr, const int *jhi = nullptr);
  void list(const int *nlo, const int *nhi);
  // Sets up the stand-in buffers; false (status recorded) when it cannot.
  bool ready();
  double *junk() const { return junk_; }
  const double *zero() const { return zero_; }
  int *zero_int() const { return (int *)zero_; }
  const int k0 = 0;        // the k (and, in 1D, j) bounds of every lifted box
  const double one = 1.0;  // dz (dy) where the 3D routine multiplies a cell volume
  const int x_axis = 1;    // the direction argument of a 1D routine

 private:
  int saved_;
  const char *name_;
  long long need_ = 1, list_lo_ = 0, list_hi_ = -1;
  bool bad_ = false;
  double *junk_ = nullptr, *zero_ = nullptr;
};

}  // namespace lsmgpu
