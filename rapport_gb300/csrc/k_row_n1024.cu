// Row kernels of the split forms instantiated for N_t = 1024 (one
// translation unit per size group, compiled in parallel).
#include "k_rowfused.cuh"

template struct RowKernels<1024>;
