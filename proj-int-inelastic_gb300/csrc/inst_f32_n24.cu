// Instantiation of the collide kernels for float, n = 24.
#include "collide_kernels.cuh"
PII_INSTANTIATE(float, 24)
