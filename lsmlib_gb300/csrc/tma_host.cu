// Host-side tensor-map encoding through the driver entry point (the library
// does not link libcuda directly; cudart resolves the symbol at run time).
#include <cudaTypedefs.h>

#include <mutex>

#include "lsmgpu_common.cuh"
#include "tma.cuh"

namespace lsmgpu {

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  });
  return fn;
}

bool encode_tmap_3d(CUtensorMap *out, const void *base, int esize, long long nx, long long ny,
                    long long nz, long long pitch_y, long long pitch_z, int bx, int by, int bz) {
  PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
  if (!fn) {
    set_error(LSMGPU_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    return false;
  }
  cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
  cuuint64_t strides[2] = {(cuuint64_t)(pitch_y * esize), (cuuint64_t)(pitch_z * esize)};
  cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, (cuuint32_t)bz};
  cuuint32_t estr[3] = {1, 1, 1};
  CUtensorMapDataType dt = esize == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
  CUresult r = fn(out, dt, 3, const_cast<void *>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error(LSMGPU_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return false;
  }
  return true;
}

}  // namespace lsmgpu
