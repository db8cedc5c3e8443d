// Float32-bulk instantiation of the world step (positions, angles, sleep
// timers, GJK and time of impact stay float64).
#define GB_REAL float
#include "gb_kernels.cuh"
