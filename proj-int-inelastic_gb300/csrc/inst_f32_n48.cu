// Instantiation of the collide kernels for float, n = 48.
#include "collide_kernels.cuh"
PII_INSTANTIATE(float, 48)
