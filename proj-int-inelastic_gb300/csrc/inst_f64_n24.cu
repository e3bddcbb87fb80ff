// Instantiation of the collide kernels for double, n = 24.
#include "collide_kernels.cuh"
PII_INSTANTIATE(double, 24)
