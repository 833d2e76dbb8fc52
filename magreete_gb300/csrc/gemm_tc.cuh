// tcgen05 (TF32x3) complex trailing update for the complex64 LU.
#pragma once
#include <cuda.h>

#include "common.cuh"

namespace mgt {

// Split operand buffers and their TMA descriptors, built once per
// factorisation for matrices of order <= nmax.
struct TcPlan {
  float* Ahi = nullptr;
  float* Alo = nullptr;
  float* Bhi = nullptr;
  float* Blo = nullptr;
  int64_t nmax = 0;
  CUtensorMap mAhi, mAlo, mBhi, mBlo;
  int init(void* scratch, int64_t nmax);
};

size_t tc_scratch_bytes(int64_t n);
bool tc_available();

// C (M x N complex64, ldc even) -= A (M x K) * B (K x N), K <= 64
int gemm_sub_tc(const TcPlan& plan, int M, int N, int K, const float2* A, int64_t lda, const float2* B,
                int64_t ldb, float2* C, int64_t ldc, int* status, cudaStream_t s);

}  // namespace mgt
