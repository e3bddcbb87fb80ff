// Instantiation of the collide kernels for float, n = 64.
#include "collide_kernels.cuh"
PII_INSTANTIATE(float, 64)
