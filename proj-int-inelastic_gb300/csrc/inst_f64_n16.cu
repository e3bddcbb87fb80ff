// Instantiation of the collide kernels for double, n = 16.
#include "collide_kernels.cuh"
PII_INSTANTIATE(double, 16)
