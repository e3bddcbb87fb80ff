// Instantiation of the collide kernels for float, n = 8.
#include "collide_kernels.cuh"
PII_INSTANTIATE(float, 8)
