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

// TMA map of a complex64 matrix C (rows x cols, leading dimension ldc even,
// 16-byte aligned base) viewed as fp32 (rows x 2 cols), 128 x 32 boxes.
int tc_make_cmap(CUtensorMap* map, float2* C, int64_t rows, int64_t cols, int64_t ldc);

// C -= A (M x K) * B (K x N), K <= 128, where C is the M x N block of the
// matrix described by cmap starting at fp32 column cx0 (= 2 * complex
// column) and row cy0; the block must extend to the matrix's last row and
// column (TMA stores are clipped there).  max_ctas <= 0: one CTA per SM.
int gemm_sub_tc(const TcPlan& plan, const CUtensorMap& cmap, int M, int N, int K, const float2* A, int64_t lda,
                const float2* B, int64_t ldb, int cx0, int cy0, int* status, cudaStream_t s, int max_ctas = 0);

}  // namespace mgt
