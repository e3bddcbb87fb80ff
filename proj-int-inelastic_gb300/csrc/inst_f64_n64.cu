// Instantiation of the collide kernels for double, n = 64.
#include "collide_kernels.cuh"
PII_INSTANTIATE(double, 64)
