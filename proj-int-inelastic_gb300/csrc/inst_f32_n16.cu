// Instantiation of the collide kernels for float, n = 16.
#include "collide_kernels.cuh"
PII_INSTANTIATE(float, 16)
