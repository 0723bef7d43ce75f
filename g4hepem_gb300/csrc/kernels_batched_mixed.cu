// kernels_batched_mixed.cu -- the precision form's FP32 stage kernels: the
// batched unit compiled a second time with HEPEM_MIXED_UNIT, so that these
// kernels are built with FMA contraction while the FP64 unit is not (see
// kernels_batched.cu).
#define HEPEM_MIXED_UNIT
#include "kernels_batched.cu"
