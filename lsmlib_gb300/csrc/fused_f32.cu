// FP32 form of the fused steppers (FMA contraction, fast reciprocals).
#define LSMGPU_FUSED_R float
#define LSMGPU_FUSED_EXACT false
#define LSMGPU_FUSED_SUFFIX f32
#include "fused_entry.cuh"
