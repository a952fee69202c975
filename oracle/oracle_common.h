/*
 * Shared helpers for the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY: this directory is the checker the GPU library is
 * measured against.  Nothing in lsmlib_gb300/ includes or links it.
 *
 * The oracle restates LSMLIB's Fortran-77 kernels in C, routine by routine,
 * keeping every floating-point operation in the reference's order so that
 * results are bit-identical to a gfortran -fdefault-real-8 build on a machine
 * without fused multiply-add (compile with -ffp-contract=off).  Arrays are
 * column-major with arbitrary lower bounds, exactly as the reference declares
 * them: a(ilo:ihi, jlo:jhi, klo:khi).
 */
#ifndef LSM_ORACLE_COMMON_H
#define LSM_ORACLE_COMMON_H

#include <math.h>
#include <stdlib.h>

#ifndef ORACLE_REAL
#define ORACLE_REAL double
#endif
typedef ORACLE_REAL real_t;

/* template constants of the FP64 build (src/CMakeLists.txt:10-20) */
#define ORACLE_ZERO_TOL 1.e-11
#define ORACLE_TINY 1.e-36

/* A ghost box: lower/upper bounds per axis plus column-major strides. */
typedef struct {
  int lo[3], hi[3];
  long s[3];
} gbox;

static inline gbox mk_box(const int *ilo, const int *ihi, const int *jlo,
                          const int *jhi, const int *klo, const int *khi) {
  gbox b;
  b.lo[0] = *ilo; b.hi[0] = *ihi;
  b.lo[1] = *jlo; b.hi[1] = *jhi;
  b.lo[2] = *klo; b.hi[2] = *khi;
  b.s[0] = 1;
  b.s[1] = (long)(b.hi[0] - b.lo[0] + 1);
  b.s[2] = b.s[1] * (long)(b.hi[1] - b.lo[1] + 1);
  return b;
}

static inline long at(const gbox *b, int i, int j, int k) {
  return (long)(i - b->lo[0]) + b->s[1] * (long)(j - b->lo[1]) +
         b->s[2] * (long)(k - b->lo[2]);
}

/* Fortran MAX/MIN of two values as gfortran selects them. */
static inline real_t fmax2(real_t a, real_t b) { return a > b ? a : b; }
static inline real_t fmin2(real_t a, real_t b) { return a < b ? a : b; }

/* loop over an inclusive index box, k outermost like the Fortran loops */
#define FOR_BOX(lo0, hi0, lo1, hi1, lo2, hi2)                 \
  for (int k = (lo2); k <= (hi2); k++)                         \
    for (int j = (lo1); j <= (hi1); j++)                       \
      for (int i = (lo0); i <= (hi0); i++)

#define BOX6(p) p##_ilo, p##_ihi, p##_jlo, p##_jhi, p##_klo, p##_khi

#endif
