// Float64 instantiation of the world step (compiled with -fmad=false: no
// fused multiply-add, so every rounding matches the CPU restatement).
#define GB_REAL double
#include "gb_kernels.cuh"
