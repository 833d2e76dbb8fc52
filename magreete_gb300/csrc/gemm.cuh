// Complex GEMM update C -= A * B used by the LU trailing update and the
// blocked triangular solves.
#pragma once
#include "common.cuh"

namespace mgt {
// C (M x N) -= A (M x K) * B (K x N); complex, row-major, leading dims in elements.
template <typename T>
int gemm_sub(int M, int N, int K, const cplx<T>* A, int64_t lda, const cplx<T>* B, int64_t ldb,
             cplx<T>* C, int64_t ldc, cudaStream_t s);
}  // namespace mgt
