// FP32 advection adjoint (FP32 state and adjoint fields, FP64 objective).
#define LSMGPU_ADJ_R float
#define LSMGPU_ADJ_EXACT false
#define LSMGPU_ADJ_SUFFIX f32
#include "adjoint_entry.cuh"
