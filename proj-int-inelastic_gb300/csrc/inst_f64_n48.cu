// Instantiation of the collide kernels for double, n = 48.
#include "collide_kernels.cuh"
PII_INSTANTIATE(double, 48)
