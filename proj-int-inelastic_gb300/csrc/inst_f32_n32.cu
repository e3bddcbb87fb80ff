// Instantiation of the collide kernels for float, n = 32.
#include "collide_kernels.cuh"
PII_INSTANTIATE(float, 32)
