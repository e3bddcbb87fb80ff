// Instantiation of the collide kernels for double, n = 8.
#include "collide_kernels.cuh"
PII_INSTANTIATE(double, 8)
