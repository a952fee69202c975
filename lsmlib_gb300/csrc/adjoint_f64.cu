// FP64 advection adjoint (no FMA contraction; forward states bit-identical
// to the FP64 fused stepper).
#define LSMGPU_ADJ_R double
#define LSMGPU_ADJ_EXACT true
#define LSMGPU_ADJ_SUFFIX f64
#include "adjoint_entry.cuh"
