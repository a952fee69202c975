// Geometry: LSMLIB's volume, surface-area and integral reductions, voxel
// counts and mean absolute difference (lsm_math_utils3d.f.in:81-250, :573-850,
// :1420-2008; lsm_geometry3d_fort.f.in:395-1330), and the pointwise unit
// normals and mean curvature (lsm_geometry3d_fort.f.in:27-394), with LSMLIB's
// symbol names and argument lists.
//
// Sums.  The reference adds its terms serially in (k, j, i) order.  Here one
// warp owns one (j, k) row of the index box: lane l takes the row's cells at
// i = ilo + l, ilo + l + 32, ... in increasing i, a fixed shuffle tree adds
// the lanes, a block adds its 16 rows in order, and one block adds the block
// partials in a fixed order (two-sum for the last tree).  The result depends
// only on the data and the box, not on the launch or the run, and its
// rounding error is far below the serial sum's.  Each term keeps the
// reference's operation order (this unit is compiled without FMA
// contraction), so terms made of +, -, *, / and sqrt are bit-identical; sin
// and cos are CUDA's (within 2 ulp), so terms inside the smoothing band
// |phi| < epsilon can differ in the last bits.  Voxel counts are integers.
//
// Arithmetic: GB300's FP64 rate is a small fraction of its FP32 rate, so a
// cell's class (outside, full, smoothing band) is decided on integers, full
// cells are counted (or, for the integrals, their F summed) and scaled by dV
// once, and only band cells evaluate their FP64 term; partial sums that are
// zero skip their FP64 additions.  Memory: each row is read once, coalesced
// along x, with four 32-cell segments per lane in flight; F and the gradient
// are read only for cells whose term needs them, as the reference does.
#include <cstring>

#include "lsmgpu_common.cuh"
#include "stencil_math.cuh"
#include "../../include/lsmgpu_toolbox3d.h"

namespace lsmgpu {
namespace {

typedef double R;

#define BOXARG(b) const int *b##_ilo, const int *b##_ihi, const int *b##_jlo, const int *b##_jhi, const int *b##_klo, const int *b##_khi
#define BOXOF(b) mkbox(b##_ilo, b##_ihi, b##_jlo, b##_jhi, b##_klo, b##_khi)
#define IBARGS const int *ilo_ib, const int *ihi_ib, const int *jlo_ib, const int *jhi_ib, const int *klo_ib, const int *khi_ib
#define IBOX mkbox(ilo_ib, ihi_ib, jlo_ib, jhi_ib, klo_ib, khi_ib)
#define FBARGS const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const int *klo_fb, const int *khi_fb
#define FBOX mkbox(ilo_fb, ihi_fb, jlo_fb, jhi_fb, klo_fb, khi_fb)
#define DXP const R *dx, const R *dy, const R *dz
#define CVARGS const R *control_vol, BOXARG(c), const int *control_vol_sgn

// parameters of the reference routines (math_utils3d.f.in:616-619)
constexpr R kPi = 3.14159265358979323846;
constexpr R kOneOverPi = 0.31830988618379;

enum SumKind {
  VOL_LT,      // geometry3d_fort.f.in:395  sum (1 - H) dV
  VOL_GT,      // :484                     sum H dV
  AREA,        // :574                     sum delta |grad phi| dV
  AREA_DELTA,  // :669                     sum delta_phi |grad phi| dV over delta_phi > 0
  INT_LT,      // math_utils3d.f.in:573    sum (1 - H) F dV
  INT_GT,      // :659                     sum H F dV
  SURF_INT,    // :745                     sum delta |grad phi| F dV
  ABS_DIFF,    // :81                      sum |f1 - f2| / count
  COUNT_GT,    // :154                     #{phi > 0}
  COUNT_LT     // :203                     #{phi < 0}
};

struct SumArgs {
  View<const R> phi;         // phi | delta_phi | field1
  View<const R> f;           // F | field2
  View<const R> px, py, pz;  // gradient
  View<const R> cv;          // control volume
  int cv_sgn;                // 0: every cell; > 0: control_vol > 0; < 0: control_vol < 0
  int eps_bits_ok;           // epsilon is positive and finite: classify on bit patterns
  unsigned long long eps_bits;
  R eps, inv_eps, dv;
};

__device__ __forceinline__ R grad_norm(const SumArgs &A, int i, int j, int k) {
  const R x = A.px(i, j, k), y = A.py(i, j, k), z = A.pz(i, j, k);
  return sqrt(x * x + y * y + z * z);
}

// GB300 runs FP64 arithmetic at a small fraction of its FP32 rate, so the
// comparisons that decide a cell's class are made on the IEEE bit pattern
// (sign and magnitude as integers), which orders finite doubles exactly as
// the reference's FP64 comparisons do (-0 equals +0, NaN compares false).
constexpr unsigned long long kMag = 0x7fffffffffffffffULL, kInf = 0x7ff0000000000000ULL;

enum CellClass { C_NONE = 0, C_FULL = 1, C_BAND = 2 };

// b: the bit pattern of phi; EB: epsilon is positive and finite
template <int K, bool EB>
__device__ __forceinline__ int classify(const SumArgs &A, unsigned long long b) {
  if (K == ABS_DIFF) return C_BAND;  // every cell (a NaN propagates, as in the reference)
  const unsigned long long m = b & kMag;
  const bool neg = (b >> 63) != 0;
  if (m > kInf) return C_NONE;  // NaN: every comparison of the reference is false
  if (K == COUNT_GT) return (!neg && m != 0) ? C_FULL : C_NONE;
  if (K == COUNT_LT) return (neg && m != 0) ? C_FULL : C_NONE;
  if (K == AREA_DELTA) return (!neg && m != 0) ? C_BAND : C_NONE;
  if (EB) {
    const unsigned long long e = A.eps_bits;
    if (K == VOL_LT || K == INT_LT) {  // p < -eps; -eps <= p < eps
      if (neg && m > e) return C_FULL;
      return ((neg && m <= e) || (!neg && m < e)) ? C_BAND : C_NONE;
    }
    if (K == VOL_GT || K == INT_GT) {  // p > eps; -eps < p <= eps
      if (!neg && m > e) return C_FULL;
      return ((!neg && m <= e) || (neg && m < e)) ? C_BAND : C_NONE;
    }
    return m < e ? C_BAND : C_NONE;  // AREA, SURF_INT: |p| < eps
  }
  // epsilon zero, negative or not finite: the reference's comparisons as written
  const R p = __longlong_as_double((long long)b);
  if (K == VOL_LT || K == INT_LT) return p < -A.eps ? C_FULL : (p < A.eps ? C_BAND : C_NONE);
  if (K == VOL_GT || K == INT_GT) return p > A.eps ? C_FULL : (p > -A.eps ? C_BAND : C_NONE);
  return fabs(p) < A.eps ? C_BAND : C_NONE;
}

__device__ __forceinline__ bool cv_takes(int sgn, unsigned long long b) {
  const unsigned long long m = b & kMag;
  if (m == 0 || m > kInf) return false;  // zero or NaN
  return sgn > 0 ? (b >> 63) == 0 : (b >> 63) != 0;
}

__device__ __forceinline__ bool nonzero(R v) { return (__double_as_longlong(v) & (long long)kMag) != 0; }

// the term of a smoothing-band cell, given its phi value p (reference line
// numbers in the kind list above; factor order as written there).  A full
// cell adds dV (volumes), F dV (integrals) or 1 (counts): those are counted
// (or their F summed) and scaled once, further up.
template <int K>
__device__ __forceinline__ R band_term(const SumArgs &A, R p, int i, int j, int k) {
  if (K == VOL_LT || K == INT_LT) {
    const R q = p / A.eps;
    const R omh = R(0.5) * (R(1) - q - kOneOverPi * sin(kPi * q));
    return K == VOL_LT ? omh * A.dv : omh * A.f(i, j, k) * A.dv;
  }
  if (K == VOL_GT || K == INT_GT) {
    const R q = p / A.eps;
    const R h = R(0.5) * (R(1) + q + kOneOverPi * sin(kPi * q));
    return K == VOL_GT ? h * A.dv : h * A.f(i, j, k) * A.dv;
  }
  if (K == AREA || K == SURF_INT) {
    const R delta = R(0.5) * A.inv_eps * (R(1) + cos(kPi * p * A.inv_eps));
    const R ng = grad_norm(A, i, j, k);
    return K == AREA ? delta * ng * A.dv : delta * ng * A.f(i, j, k) * A.dv;
  }
  if (K == AREA_DELTA) return p * grad_norm(A, i, j, k) * A.dv;
  return fabs(p - A.f(i, j, k));  // ABS_DIFF
}

// fixed-order sum over the 32 lanes (lane 0 holds it); skipped, and zero,
// when every lane holds zero, which costs no FP64 work
__device__ __forceinline__ R warp_sum(R v) {
  if (!__any_sync(0xffffffffu, nonzero(v))) return R(0);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

constexpr int kRowWarps = 16;  // rows per block, one warp each
constexpr int kSeg = 4;        // 32-cell segments per lane in flight

// One warp per (j, k) row of the index box, one partial per block of 16
// rows: the number of full cells (an integer) and the FP64 rest, which is
// (sum of F over full cells) * dV for the integrals plus the band terms.
// Band cells are scattered (a few per 32-cell segment), so a warp queues
// them in shared memory (value and i) and evaluates their FP64 terms 32 at a
// time with every lane busy; the order of the queue is fixed by the data.
template <int K, bool EB>
__global__ void __launch_bounds__(32 * kRowWarps) k_row_sums(SumArgs A, Box ib, long long nrows,
                                                              unsigned long long *part_n, R *part_v) {
  __shared__ unsigned sn[kRowWarps];
  __shared__ R sv[kRowWarps];
  __shared__ unsigned long long qp[kRowWarps][64];
  __shared__ int qx[kRowWarps][64];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long r = (long long)blockIdx.x * kRowWarps + w;
  constexpr bool kFullF = (K == INT_LT || K == INT_GT);
  constexpr bool kQueue = (K != ABS_DIFF);  // every cell of ABS_DIFF is a term: no divergence
  unsigned nfull = 0;
  R band = R(0), ffull = R(0);
  if (r < nrows) {
    const long long ny = ib.n(1);
    const int j = ib.lo[1] + (int)(r % ny), k = ib.lo[2] + (int)(r / ny);
    const int nx = (int)ib.n(0), i0 = ib.lo[0];
    // rows are read as bit patterns: the hot loop does no FP64 arithmetic
    const unsigned long long *prow = (const unsigned long long *)&A.phi(i0, j, k);
    const unsigned long long *crow = A.cv_sgn ? (const unsigned long long *)&A.cv(i0, j, k) : nullptr;
    int qn = 0;  // queued band cells (the same in every lane)
    for (int x0 = 0; x0 < nx; x0 += 32 * kSeg) {
      unsigned long long p[kSeg], c[kSeg];
#pragma unroll
      for (int u = 0; u < kSeg; u++) {
        const int x = x0 + 32 * u + lane;
        p[u] = x < nx ? __ldg(prow + x) : 0ull;
        c[u] = (crow && x < nx) ? __ldg(crow + x) : 0ull;
      }
#pragma unroll
      for (int u = 0; u < kSeg; u++) {
        const int x = x0 + 32 * u + lane;
        const bool ok = x < nx && (!A.cv_sgn || cv_takes(A.cv_sgn, c[u]));
        const int cls = ok ? classify<K, EB>(A, p[u]) : C_NONE;
        if (cls == C_FULL) {
          if (kFullF)
            ffull += A.f(i0 + x, j, k);
          else
            nfull++;
        }
        if (!kQueue) {
          if (cls == C_BAND) band += band_term<K>(A, __longlong_as_double((long long)p[u]), i0 + x, j, k);
          continue;
        }
        const unsigned m = __ballot_sync(0xffffffffu, cls == C_BAND);
        if (m == 0u) continue;
        if (cls == C_BAND) {
          const int slot = qn + __popc(m & ((1u << lane) - 1u));
          qp[w][slot] = p[u];
          qx[w][slot] = x;
        }
        qn += __popc(m);
        if (qn >= 32) {
          __syncwarp();
          band += band_term<K>(A, __longlong_as_double((long long)qp[w][lane]), i0 + qx[w][lane], j, k);
          __syncwarp();
          if (lane < qn - 32) {
            qp[w][lane] = qp[w][32 + lane];
            qx[w][lane] = qx[w][32 + lane];
          }
          __syncwarp();
          qn -= 32;
        }
      }
    }
    if (kQueue && qn > 0) {
      __syncwarp();
      if (lane < qn) band += band_term<K>(A, __longlong_as_double((long long)qp[w][lane]), i0 + qx[w][lane], j, k);
    }
  }
  const unsigned n_w = __reduce_add_sync(0xffffffffu, nfull);
  R v_w = warp_sum(band);
  if (kFullF) {
    const R f_w = warp_sum(ffull);
    if (lane == 0 && nonzero(f_w)) v_w = f_w * A.dv + v_w;
  }
  if (lane == 0) {
    sn[w] = n_w;
    sv[w] = v_w;
  }
  __syncthreads();
  if (w == 0) {
    const unsigned n = lane < kRowWarps ? sn[lane] : 0u;
    const R v = warp_sum(lane < kRowWarps ? sv[lane] : R(0));
    const unsigned nb = __reduce_add_sync(0xffffffffu, n);
    if (lane == 0) {
      part_n[blockIdx.x] = nb;
      part_v[blockIdx.x] = v;
    }
  }
}

// s + e = a + b exactly (Knuth's two-sum)
__device__ __forceinline__ void two_sum(R a, R b, R &s, R &e) {
  s = a + b;
  const R bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

constexpr int kFinal = 1024;

// Adds the block partials in a fixed order: thread t takes partials t,
// t + 1024, ... (integers exactly, FP64 values in order, zeros skipped), a
// fixed tree combines the threads (FP64 with two-sum).  Writes the routine's
// scalar: count * unit + rest, the mean (ABS_DIFF) or the count.
__global__ void __launch_bounds__(kFinal) k_sum_parts(const unsigned long long *part_n, const R *part_v,
                                                      long long nparts, int kind, R unit, R npts, R *out,
                                                      int *count) {
  __shared__ unsigned long long hn[kFinal];
  __shared__ R hs[kFinal], he[kFinal];
  unsigned long long n = 0;
  R s = R(0);
  for (long long b = threadIdx.x; b < nparts; b += kFinal) {
    n += part_n[b];
    const R v = part_v[b];
    if (nonzero(v)) s += v;
  }
  hn[threadIdx.x] = n;
  hs[threadIdx.x] = s;
  he[threadIdx.x] = R(0);
  __syncthreads();
  for (int h = kFinal / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) {
      hn[threadIdx.x] += hn[threadIdx.x + h];
      const R a = hs[threadIdx.x], b = hs[threadIdx.x + h], eb = he[threadIdx.x + h];
      if (nonzero(b)) {
        R t, d;
        two_sum(a, b, t, d);
        hs[threadIdx.x] = t;
        he[threadIdx.x] += d;
      }
      if (nonzero(eb)) he[threadIdx.x] += eb;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const R rest = hs[0] + he[0];
    if (kind == COUNT_GT || kind == COUNT_LT)
      *count = (int)hn[0];
    else if (kind == ABS_DIFF)
      *out = npts > R(0) ? rest / npts : R(0);
    else
      *out = (R)hn[0] * unit + rest;
  }
}

template <int K>
void launch_rows(const SumArgs &A, const Box &ib, long long nrows, long long nparts, unsigned long long *pn,
                 R *pv) {
  if (A.eps_bits_ok)
    LSMGPU_LAUNCH((k_row_sums<K, true>), (unsigned)nparts, 32 * kRowWarps, 0, A, ib, nrows, pn, pv);
  else
    LSMGPU_LAUNCH((k_row_sums<K, false>), (unsigned)nparts, 32 * kRowWarps, 0, A, ib, nrows, pn, pv);
}

// Runs one reduction.  Arrays in `need` must cover the index box.
struct SumCall {
  Call call;
  SumArgs A{};
  Box ib;
  explicit SumCall(const char *name, const Box &b) : call(name), ib(b) {}
  View<const R> in(const R *p, const Box &b) {
    if (!b.contains(ib, 0, 0, 0)) call.fail("ghost box does not cover the index box");
    if (!call.ok()) return View<const R>{};
    return view((const R *)call.in(p, b.size()), b);
  }
  void control_volume(const R *cv, const Box &cb, int sgn) {
    A.cv = in(cv, cb);
    A.cv_sgn = sgn > 0 ? 1 : -1;
  }
  void cell_volume(R dx, R dy, R dz) { A.dv = dx * dy * dz; }
  void epsilon(R eps) {
    A.eps = eps;
    A.inv_eps = R(1.0) / eps;
    A.eps_bits_ok = eps > R(0) && eps <= 1.7976931348623157e308;
    memcpy(&A.eps_bits, &eps, sizeof(eps));
  }
  void run(int kind, R *out, int *count) {
    if (!call.ok()) return;
    R *dout = nullptr;
    int *dcount = nullptr;
    if (count)
      dcount = call.scalar_out(count);
    else
      dout = call.scalar_out(out);
    const long long nrows = ib.empty() ? 0 : ib.n(1) * ib.n(2);
    const long long nparts = (nrows + kRowWarps - 1) / kRowWarps;
    unsigned long long *pn = call.temp<unsigned long long>(nparts > 0 ? nparts : 1);
    R *pv = call.temp<R>(nparts > 0 ? nparts : 1);
    if (!call.ok()) return;
    if (nparts > 0) {
      switch (kind) {
        case VOL_LT: launch_rows<VOL_LT>(A, ib, nrows, nparts, pn, pv); break;
        case VOL_GT: launch_rows<VOL_GT>(A, ib, nrows, nparts, pn, pv); break;
        case AREA: launch_rows<AREA>(A, ib, nrows, nparts, pn, pv); break;
        case AREA_DELTA: launch_rows<AREA_DELTA>(A, ib, nrows, nparts, pn, pv); break;
        case INT_LT: launch_rows<INT_LT>(A, ib, nrows, nparts, pn, pv); break;
        case INT_GT: launch_rows<INT_GT>(A, ib, nrows, nparts, pn, pv); break;
        case SURF_INT: launch_rows<SURF_INT>(A, ib, nrows, nparts, pn, pv); break;
        case ABS_DIFF: launch_rows<ABS_DIFF>(A, ib, nrows, nparts, pn, pv); break;
        case COUNT_GT: launch_rows<COUNT_GT>(A, ib, nrows, nparts, pn, pv); break;
        default: launch_rows<COUNT_LT>(A, ib, nrows, nparts, pn, pv); break;
      }
    }
    LSMGPU_LAUNCH(k_sum_parts, 1, kFinal, 0, pn, pv, nparts, kind, A.dv, (R)ib.size(), dout, dcount);
    call.finish();
  }
};

// ---- pointwise geometry (geometry3d_fort.f.in:27-394) ------------------------------
__global__ void k_unit_normal(View<R> nx, View<R> ny, View<R> nz, View<const R> px, View<const R> py,
                              View<const R> pz, Box fb) {
  LSMGPU_CELL_INDEX(fb, i, j, k);
  const R x = px(i, j, k), y = py(i, j, k), z = pz(i, j, k);
  const R ng = sqrt(x * x + y * y + z * z);
  if (ng >= Consts<R>::zero_tol) {
    const R inv = R(1.0) / ng;
    nx(i, j, k) = x * inv;
    ny(i, j, k) = y * inv;
    nz(i, j, k) = z * inv;
  } else {
    nx(i, j, k) = R(1);
    ny(i, j, k) = R(0);
    nz(i, j, k) = R(0);
  }
}

__global__ void k_signed_unit_normal(View<R> nx, View<R> ny, View<R> nz, View<const R> px, View<const R> py,
                                     View<const R> pz, View<const R> phi, Box fb, R dx_sq) {
  LSMGPU_CELL_INDEX(fb, i, j, k);
  const R p = phi(i, j, k);
  R a = R(0), b = R(0), c = R(0);
  if (fabs(p) > Consts<R>::zero_tol) {
    const R x = px(i, j, k), y = py(i, j, k), z = pz(i, j, k);
    const R ngs = x * x + y * y + z * z;
    if (ngs >= Consts<R>::zero_tol) {
      const R sgn = p / sqrt(p * p + ngs * dx_sq);
      const R inv = R(1.0) / sqrt(ngs);
      a = sgn * x * inv;
      b = sgn * y * inv;
      c = sgn * z * inv;
    } else {
      a = R(1);
    }
  }
  nx(i, j, k) = a;
  ny(i, j, k) = b;
  nz(i, j, k) = c;
}

// kappa = numerator / |grad phi|^3; the reference writes the denominator as
// norm_grad_phi_sq ** 1.5 (:366), evaluated here as s * sqrt(s) (within 2 ulp
// of the exact power)
__global__ void k_mean_curvature(View<R> kap, View<const R> px, View<const R> py, View<const R> pz,
                                 View<const R> xx, View<const R> xy, View<const R> xz, View<const R> yy,
                                 View<const R> yz, View<const R> zz, Box fb) {
  LSMGPU_CELL_INDEX(fb, i, j, k);
  const R x = px(i, j, k), y = py(i, j, k), z = pz(i, j, k);
  const R s = x * x + y * y + z * z;
  if (s < Consts<R>::zero_tol) {
    kap(i, j, k) = R(0);
    return;
  }
  const R hxx = xx(i, j, k), hxy = xy(i, j, k), hxz = xz(i, j, k);
  const R hyy = yy(i, j, k), hyz = yz(i, j, k), hzz = zz(i, j, k);
  const R num = hxx * y * y - R(2) * hxy * x * y + hyy * x * x + hxx * z * z - R(2) * hxz * x * z +
                hzz * x * x + hyy * z * z - R(2) * hyz * y * z + hzz * y * y;
  kap(i, j, k) = num / (s * sqrt(s));
}

}  // namespace
}  // namespace lsmgpu

using namespace lsmgpu;

extern "C" {

// ---- math_utils3d.f.in -----------------------------------------------------------

void lsm3daveabsdiff_(R *ave_abs_diff, const R *field1, BOXARG(a), const R *field2, BOXARG(b), IBARGS) {
  SumCall s("lsm3daveabsdiff_", IBOX);
  s.A.phi = s.in(field1, BOXOF(a));
  s.A.f = s.in(field2, BOXOF(b));
  s.run(ABS_DIFF, ave_abs_diff, nullptr);
}

void lsm3dvoxelcountgreaterthanzero_(int *count, const R *phi, BOXARG(g), IBARGS) {
  SumCall s("lsm3dvoxelcountgreaterthanzero_", IBOX);
  s.A.phi = s.in(phi, BOXOF(g));
  s.run(COUNT_GT, nullptr, count);
}

void lsm3dvoxelcountlessthanzero_(int *count, const R *phi, BOXARG(g), IBARGS) {
  SumCall s("lsm3dvoxelcountlessthanzero_", IBOX);
  s.A.phi = s.in(phi, BOXOF(g));
  s.run(COUNT_LT, nullptr, count);
}

static void volume_integral(const char *name, int kind, R *int_F, const R *F, const Box &fb, const R *phi,
                            const Box &pb, const R *cv, const Box &cb, int sgn, const Box &ib, R dx, R dy, R dz,
                            R eps) {
  SumCall s(name, ib);
  s.A.f = s.in(F, fb);
  s.A.phi = s.in(phi, pb);
  if (cv) s.control_volume(cv, cb, sgn);
  s.cell_volume(dx, dy, dz);
  s.epsilon(eps);
  s.run(kind, int_F, nullptr);
}

void lsm3dvolumeintegralphilessthanzero_(R *int_F, const R *F, BOXARG(F), const R *phi, BOXARG(p), IBARGS, DXP,
                                         const R *epsilon) {
  volume_integral("lsm3dvolumeintegralphilessthanzero_", INT_LT, int_F, F, BOXOF(F), phi, BOXOF(p), nullptr,
                  Box{}, 0, IBOX, *dx, *dy, *dz, *epsilon);
}

void lsm3dvolumeintegralphigreaterthanzero_(R *int_F, const R *F, BOXARG(F), const R *phi, BOXARG(p), IBARGS,
                                            DXP, const R *epsilon) {
  volume_integral("lsm3dvolumeintegralphigreaterthanzero_", INT_GT, int_F, F, BOXOF(F), phi, BOXOF(p), nullptr,
                  Box{}, 0, IBOX, *dx, *dy, *dz, *epsilon);
}

static void surface_integral(const char *name, R *int_F, const R *F, const Box &fb, const R *phi, const Box &pb,
                             const R *phi_x, const R *phi_y, const R *phi_z, const Box &gb, const R *cv,
                             const Box &cb, int sgn, const Box &ib, R dx, R dy, R dz, R eps) {
  SumCall s(name, ib);
  s.A.f = s.in(F, fb);
  s.A.phi = s.in(phi, pb);
  s.A.px = s.in(phi_x, gb);
  s.A.py = s.in(phi_y, gb);
  s.A.pz = s.in(phi_z, gb);
  if (cv) s.control_volume(cv, cb, sgn);
  s.cell_volume(dx, dy, dz);
  s.epsilon(eps);
  s.run(SURF_INT, int_F, nullptr);
}

void lsm3dsurfaceintegral_(R *int_F, const R *F, BOXARG(F), const R *phi, BOXARG(p), const R *phi_x,
                           const R *phi_y, const R *phi_z, BOXARG(g), IBARGS, DXP, const R *epsilon) {
  surface_integral("lsm3dsurfaceintegral_", int_F, F, BOXOF(F), phi, BOXOF(p), phi_x, phi_y, phi_z, BOXOF(g),
                   nullptr, Box{}, 0, IBOX, *dx, *dy, *dz, *epsilon);
}

void lsm3dvolumeintegralphilessthanzerocontrolvolume_(R *int_F, const R *F, BOXARG(F), const R *phi, BOXARG(p),
                                                      CVARGS, IBARGS, DXP, const R *epsilon) {
  volume_integral("lsm3dvolumeintegralphilessthanzerocontrolvolume_", INT_LT, int_F, F, BOXOF(F), phi, BOXOF(p),
                  control_vol, BOXOF(c), *control_vol_sgn, IBOX, *dx, *dy, *dz, *epsilon);
}

void lsm3dvolumeintegralphigreaterthanzerocontrolvolume_(R *int_F, const R *F, BOXARG(F), const R *phi,
                                                         BOXARG(p), CVARGS, IBARGS, DXP, const R *epsilon) {
  volume_integral("lsm3dvolumeintegralphigreaterthanzerocontrolvolume_", INT_GT, int_F, F, BOXOF(F), phi,
                  BOXOF(p), control_vol, BOXOF(c), *control_vol_sgn, IBOX, *dx, *dy, *dz, *epsilon);
}

void lsm3dsurfaceintegralcontrolvolume_(R *int_F, const R *F, BOXARG(F), const R *phi, BOXARG(p), const R *phi_x,
                                        const R *phi_y, const R *phi_z, BOXARG(g), CVARGS, IBARGS, DXP,
                                        const R *epsilon) {
  surface_integral("lsm3dsurfaceintegralcontrolvolume_", int_F, F, BOXOF(F), phi, BOXOF(p), phi_x, phi_y, phi_z,
                   BOXOF(g), control_vol, BOXOF(c), *control_vol_sgn, IBOX, *dx, *dy, *dz, *epsilon);
}

void lsm3dvoxelcountgreaterthanzerocontrolvolume_(int *count, const R *phi, BOXARG(g), CVARGS, IBARGS) {
  SumCall s("lsm3dvoxelcountgreaterthanzerocontrolvolume_", IBOX);
  s.A.phi = s.in(phi, BOXOF(g));
  s.control_volume(control_vol, BOXOF(c), *control_vol_sgn);
  s.run(COUNT_GT, nullptr, count);
}

void lsm3dvoxelcountlessthanzerocontrolvolume_(int *count, const R *phi, BOXARG(g), CVARGS, IBARGS) {
  SumCall s("lsm3dvoxelcountlessthanzerocontrolvolume_", IBOX);
  s.A.phi = s.in(phi, BOXOF(g));
  s.control_volume(control_vol, BOXOF(c), *control_vol_sgn);
  s.run(COUNT_LT, nullptr, count);
}

// ---- geometry3d_fort.f.in --------------------------------------------------------

void lsm3dcomputeunitnormal_(R *normal_x, R *normal_y, R *normal_z, BOXARG(n), const R *phi_x, const R *phi_y,
                             const R *phi_z, BOXARG(g), FBARGS) {
  Call call("lsm3dcomputeunitnormal_");
  Box nb = BOXOF(n), gb = BOXOF(g), fb = FBOX;
  if (!nb.contains(fb, 0, 0, 0) || !gb.contains(fb, 0, 0, 0)) call.fail("ghost box does not cover the fill box");
  if (!call.ok() || fb.empty()) return;
  const long long nn = nb.size(), ng = gb.size();
  View<R> X = view(call.inout(normal_x, nn), nb), Y = view(call.inout(normal_y, nn), nb),
          Z = view(call.inout(normal_z, nn), nb);
  View<const R> PX = view((const R *)call.in(phi_x, ng), gb), PY = view((const R *)call.in(phi_y, ng), gb),
                PZ = view((const R *)call.in(phi_z, ng), gb);
  if (!call.ok()) return;
  Grid3 g3 = cover(fb);
  LSMGPU_LAUNCH(k_unit_normal, g3.grid, g3.block, 0, X, Y, Z, PX, PY, PZ, fb);
  call.finish();
}

void lsm3dcomputesignedunitnormal_(R *normal_x, R *normal_y, R *normal_z, BOXARG(n), const R *phi_x,
                                   const R *phi_y, const R *phi_z, BOXARG(g), const R *phi, BOXARG(f), FBARGS,
                                   DXP) {
  Call call("lsm3dcomputesignedunitnormal_");
  Box nb = BOXOF(n), gb = BOXOF(g), pb = BOXOF(f), fb = FBOX;
  if (!nb.contains(fb, 0, 0, 0) || !gb.contains(fb, 0, 0, 0) || !pb.contains(fb, 0, 0, 0))
    call.fail("ghost box does not cover the fill box");
  if (!call.ok() || fb.empty()) return;
  const long long nn = nb.size(), ng = gb.size();
  View<R> X = view(call.inout(normal_x, nn), nb), Y = view(call.inout(normal_y, nn), nb),
          Z = view(call.inout(normal_z, nn), nb);
  View<const R> PX = view((const R *)call.in(phi_x, ng), gb), PY = view((const R *)call.in(phi_y, ng), gb),
                PZ = view((const R *)call.in(phi_z, ng), gb), P = view((const R *)call.in(phi, pb.size()), pb);
  if (!call.ok()) return;
  R dx_sq = rmax(rmax(*dx, *dy), *dz);
  dx_sq = dx_sq * dx_sq;
  Grid3 g3 = cover(fb);
  LSMGPU_LAUNCH(k_signed_unit_normal, g3.grid, g3.block, 0, X, Y, Z, PX, PY, PZ, P, fb, dx_sq);
  call.finish();
}

void lsm3dcomputemeancurvature_(R *kappa, BOXARG(k), const R *phi_x, const R *phi_y, const R *phi_z, BOXARG(g),
                                const R *phi_xx, const R *phi_xy, const R *phi_xz, const R *phi_yy,
                                const R *phi_yz, const R *phi_zz, BOXARG(h), FBARGS) {
  Call call("lsm3dcomputemeancurvature_");
  Box kb = BOXOF(k), gb = BOXOF(g), hb = BOXOF(h), fb = FBOX;
  if (!kb.contains(fb, 0, 0, 0) || !gb.contains(fb, 0, 0, 0) || !hb.contains(fb, 0, 0, 0))
    call.fail("ghost box does not cover the fill box");
  if (!call.ok() || fb.empty()) return;
  const long long ng = gb.size(), nh = hb.size();
  View<R> K = view(call.inout(kappa, kb.size()), kb);
  View<const R> X = view((const R *)call.in(phi_x, ng), gb), Y = view((const R *)call.in(phi_y, ng), gb),
                Z = view((const R *)call.in(phi_z, ng), gb);
  View<const R> XX = view((const R *)call.in(phi_xx, nh), hb), XY = view((const R *)call.in(phi_xy, nh), hb),
                XZ = view((const R *)call.in(phi_xz, nh), hb), YY = view((const R *)call.in(phi_yy, nh), hb),
                YZ = view((const R *)call.in(phi_yz, nh), hb), ZZ = view((const R *)call.in(phi_zz, nh), hb);
  if (!call.ok()) return;
  Grid3 g3 = cover(fb);
  LSMGPU_LAUNCH(k_mean_curvature, g3.grid, g3.block, 0, K, X, Y, Z, XX, XY, XZ, YY, YZ, ZZ, fb);
  call.finish();
}

static void volume_region(const char *name, int kind, R *volume, const R *phi, const Box &pb, const R *cv,
                          const Box &cb, int sgn, const Box &ib, R dx, R dy, R dz, R eps) {
  SumCall s(name, ib);
  s.A.phi = s.in(phi, pb);
  if (cv) s.control_volume(cv, cb, sgn);
  s.cell_volume(dx, dy, dz);
  s.epsilon(eps);
  s.run(kind, volume, nullptr);
}

void lsm3dvolumeregionphilessthanzero_(R *volume, const R *phi, BOXARG(p), IBARGS, DXP, const R *epsilon) {
  volume_region("lsm3dvolumeregionphilessthanzero_", VOL_LT, volume, phi, BOXOF(p), nullptr, Box{}, 0, IBOX, *dx,
                *dy, *dz, *epsilon);
}

void lsm3dvolumeregionphigreaterthanzero_(R *volume, const R *phi, BOXARG(p), IBARGS, DXP, const R *epsilon) {
  volume_region("lsm3dvolumeregionphigreaterthanzero_", VOL_GT, volume, phi, BOXOF(p), nullptr, Box{}, 0, IBOX,
                *dx, *dy, *dz, *epsilon);
}

void lsm3dvolumeregionphilessthanzerocontrolvolume_(R *volume, const R *phi, BOXARG(p), CVARGS, IBARGS, DXP,
                                                    const R *epsilon) {
  volume_region("lsm3dvolumeregionphilessthanzerocontrolvolume_", VOL_LT, volume, phi, BOXOF(p), control_vol,
                BOXOF(c), *control_vol_sgn, IBOX, *dx, *dy, *dz, *epsilon);
}

void lsm3dvolumeregionphigreaterthanzerocontrolvolume_(R *volume, const R *phi, BOXARG(p), CVARGS, IBARGS, DXP,
                                                       const R *epsilon) {
  volume_region("lsm3dvolumeregionphigreaterthanzerocontrolvolume_", VOL_GT, volume, phi, BOXOF(p), control_vol,
                BOXOF(c), *control_vol_sgn, IBOX, *dx, *dy, *dz, *epsilon);
}

static void surface_area(const char *name, bool delta_form, R *area, const R *phi, const Box &pb, const R *phi_x,
                         const R *phi_y, const R *phi_z, const Box &gb, const R *cv, const Box &cb, int sgn,
                         const Box &ib, R dx, R dy, R dz, R eps) {
  SumCall s(name, ib);
  s.A.phi = s.in(phi, pb);
  s.A.px = s.in(phi_x, gb);
  s.A.py = s.in(phi_y, gb);
  s.A.pz = s.in(phi_z, gb);
  if (cv) s.control_volume(cv, cb, sgn);
  s.cell_volume(dx, dy, dz);
  if (!delta_form) s.epsilon(eps);
  s.run(delta_form ? AREA_DELTA : AREA, area, nullptr);
}

void lsm3dsurfaceareazerolevelset_(R *surface_area_out, const R *phi, BOXARG(p), const R *phi_x, const R *phi_y,
                                   const R *phi_z, BOXARG(g), IBARGS, DXP, const R *epsilon) {
  surface_area("lsm3dsurfaceareazerolevelset_", false, surface_area_out, phi, BOXOF(p), phi_x, phi_y, phi_z,
               BOXOF(g), nullptr, Box{}, 0, IBOX, *dx, *dy, *dz, *epsilon);
}

void lsm3dsurfaceareazerolevelsetdelta_(R *surface_area_out, const R *delta_phi, BOXARG(p), const R *phi_x,
                                        const R *phi_y, const R *phi_z, BOXARG(g), IBARGS, DXP) {
  surface_area("lsm3dsurfaceareazerolevelsetdelta_", true, surface_area_out, delta_phi, BOXOF(p), phi_x, phi_y,
               phi_z, BOXOF(g), nullptr, Box{}, 0, IBOX, *dx, *dy, *dz, R(0));
}

void lsm3dsurfaceareazerolevelsetcontrolvolume_(R *surface_area_out, const R *phi, BOXARG(p), const R *phi_x,
                                                const R *phi_y, const R *phi_z, BOXARG(g), CVARGS, IBARGS, DXP,
                                                const R *epsilon) {
  surface_area("lsm3dsurfaceareazerolevelsetcontrolvolume_", false, surface_area_out, phi, BOXOF(p), phi_x, phi_y,
               phi_z, BOXOF(g), control_vol, BOXOF(c), *control_vol_sgn, IBOX, *dx, *dy, *dz, *epsilon);
}

void lsm3dsurfaceareazerolevelsetdeltacontrolvolume_(R *surface_area_out, const R *delta_phi, BOXARG(p),
                                                     const R *phi_x, const R *phi_y, const R *phi_z, BOXARG(g),
                                                     CVARGS, IBARGS, DXP) {
  surface_area("lsm3dsurfaceareazerolevelsetdeltacontrolvolume_", true, surface_area_out, delta_phi, BOXOF(p),
               phi_x, phi_y, phi_z, BOXOF(g), control_vol, BOXOF(c), *control_vol_sgn, IBOX, *dx, *dy, *dz, R(0));
}

}  // extern "C"
