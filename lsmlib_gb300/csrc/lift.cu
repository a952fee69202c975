// Lift: the state and stand-in buffers of a 2D / 1D entry point running on
// the 3D routines (lift.cuh).  The buffers are per device, grow by doubling
// and are kept for the life of the process (a buffer in use by queued work
// is never released); the zero buffer is cleared once when allocated and
// only ever read.
#include <mutex>

#include "lift.cuh"

namespace lsmgpu {
namespace {

struct Standins {
  double *zero = nullptr, *junk = nullptr;
  long long cap = 0;
};
std::mutex g_standin_lock;
Standins g_standins[64];

}  // namespace

Lift::Lift(int dims, const char *name) : saved_(g_lift_dims), name_(name) { g_lift_dims = dims; }

Lift::~Lift() { g_lift_dims = saved_; }

void Lift::box(const int *ilo, const int *ihi, const int *jlo, const int *jhi) {
  if (!ilo || !ihi || (jlo && !jhi)) {
    bad_ = true;
    return;
  }
  long long n = (long long)*ihi - *ilo + 1;
  if (jlo) n *= (long long)*jhi - *jlo + 1;
  if (n > need_) need_ = n;
}

void Lift::list(const int *nlo, const int *nhi) {
  if (!nlo || !nhi) {
    bad_ = true;
    return;
  }
  if (list_hi_ < list_lo_) {
    list_lo_ = *nlo;
    list_hi_ = *nhi;
  } else {
    if (*nlo < list_lo_) list_lo_ = *nlo;
    if (*nhi > list_hi_) list_hi_ = *nhi;
  }
  const long long n = list_hi_ - list_lo_ + 1;
  if (n > need_) need_ = n;
}

bool Lift::ready() {
  if (bad_) {
    set_error(LSMGPU_ERR_ARGUMENT, "%s: null bound argument", name_);
    return false;
  }
  int dev = 0;
  if (!cuda_ok(cudaGetDevice(&dev), name_)) return false;
  if (dev < 0 || dev >= 64) {
    set_error(LSMGPU_ERR_ARGUMENT, "%s: device index %d out of range", name_, dev);
    return false;
  }
  std::lock_guard<std::mutex> lock(g_standin_lock);
  Standins &S = g_standins[dev];
  if (S.cap < need_) {
    long long cap = S.cap > 0 ? S.cap : 4096;
    while (cap < need_) cap *= 2;
    double *z = nullptr, *j = nullptr;
    if (!cuda_ok(cudaMalloc((void **)&z, (size_t)cap * sizeof(double)), name_)) return false;
    if (!cuda_ok(cudaMalloc((void **)&j, (size_t)cap * sizeof(double)), name_)) return false;
    if (!cuda_ok(cudaMemset(z, 0, (size_t)cap * sizeof(double)), name_)) return false;
    if (!cuda_ok(cudaDeviceSynchronize(), name_)) return false;  // cleared before any stream reads it
    S.zero = z;
    S.junk = j;
    S.cap = cap;
  }
  zero_ = S.zero;
  junk_ = S.junk;
  return true;
}

}  // namespace lsmgpu
