// Launch counting and optional per-launch timing of the trailing-update
// GEMM (the dominant kernel), for the benchmark's roofline figures.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace mgt {
void count_launch(int n = 1);
// brackets one dominant-kernel launch on `s`; `flops` algorithmic flops,
// `bytes` algorithmic DRAM bytes of that launch
void dom_begin(cudaStream_t s);
void dom_end(cudaStream_t s, double flops, double bytes);
}  // namespace mgt
