// tcgen05 (TF32x3) complex trailing update for the complex64 LU.
#pragma once
#include <cuda.h>

#include "common.cuh"

namespace mgt {

// Split operand buffers and their TMA descriptors, built once per
// factorisation for matrices of order <= nmax.
struct TcPlan {
  void* Ahi = nullptr;     // fp32 (TF32x3) or fp16 (F16x2) split operands
  void* Alo = nullptr;
  void* Bhi = nullptr;
  void* Blo = nullptr;
  float* invA = nullptr;   // F16x2: inverse row scales of A, inverse column scales of B
  float* invB = nullptr;
  int mode = 0;            // MGT_TC_TF32X3 or MGT_TC_F16X2, fixed when the plan is built
  int64_t nmax = 0;
  CUtensorMap mAhi, mAlo, mBhi, mBlo;
  int init(void* scratch, int64_t nmax);
};

size_t tc_scratch_bytes(int64_t n);
// split-product scheme of the tensor-core update (MGT_TC_TF32X3 / MGT_TC_F16X2)
int tc_set_mode(int mode);
int tc_get_mode();
bool tc_available();

// TMA map of a complex64 matrix C (rows x cols, leading dimension ldc even,
// 16-byte aligned base) viewed as fp32 (rows x 2 cols), 128 x 32 boxes.
int tc_make_cmap(CUtensorMap* map, float2* C, int64_t rows, int64_t cols, int64_t ldc);

// C -= A (M x K) * B (K x N), K <= 256, where C is the M x N block of the
// matrix described by cmap starting at fp32 column cx0 (= 2 * complex
// column) and row cy0; the block must extend to the matrix's last row and
// column (TMA stores are clipped there).  max_ctas <= 0: one CTA per SM.
int gemm_sub_tc(const TcPlan& plan, const CUtensorMap& cmap, int M, int N, int K, const float2* A, int64_t lda,
                const float2* B, int64_t ldb, int cx0, int cy0, int* status, cudaStream_t s, int max_ctas = 0);

// The same in its three steps: operand splits into the plan's buffers, then
// the tcgen05 kernel, which reads only the split buffers and the C block.
int tc_split_a(const TcPlan& plan, int M, int K, const float2* A, int64_t lda, cudaStream_t s);
int tc_split_b(const TcPlan& plan, int N, int K, const float2* B, int64_t ldb, cudaStream_t s);
// bcol: the first column of B (within the split) this launch uses.
int tc_gemm(const TcPlan& plan, const CUtensorMap& cmap, int M, int N, int K, int cx0, int cy0, int* status,
            cudaStream_t s, int max_ctas = 0, int bcol = 0);

}  // namespace mgt
