// FP64 parity form of the fused steppers (compiled with -fmad=false).
#define LSMGPU_FUSED_R double
#define LSMGPU_FUSED_EXACT true
#define LSMGPU_FUSED_SUFFIX f64
#include "fused_entry.cuh"
