// Instantiation of the collide kernels for double, n = 32.
#include "collide_kernels.cuh"
PII_INSTANTIATE(double, 32)
