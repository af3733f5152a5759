// Row kernels of the split forms instantiated for N_t = 16, 32, 64 (one
// translation unit per size group, compiled in parallel).
#include "k_rowfused.cuh"

template struct RowKernels<16>;
template struct RowKernels<32>;
template struct RowKernels<64>;
