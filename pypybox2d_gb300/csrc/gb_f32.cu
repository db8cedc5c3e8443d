// Float32-bulk instantiation of the world step (positions, angles, sleep
// timers, GJK and time of impact stay float64; the rotations of the float64
// poses and the shape extents of the fat boxes are float32-accurate).
#define GB_REAL float
#define GB_POSE_ROT_F32 1
#include "gb_kernels.cuh"
