// Tensor-core residual R = B - M X (M double-float, X, B, R complex128): the
// digit-split (Ozaki-scheme) kernels of residual_tc.cu.  M's digits are made
// once (residual_tc_prepare) and applied to any number of X (residual_tc_apply).
#pragma once
#include "common.cuh"

namespace mgt {

// the tcgen05 residual handles these shapes on this device
bool residual_tc_supported(int64_t rows, int64_t kdim, int64_t ncols);
// bytes of M's digits (rows x kdim), and of one application's workspace
size_t residual_tc_digits_bytes(int64_t rows, int64_t kdim);
size_t residual_tc_apply_bytes(int64_t rows, int64_t kdim, int64_t ncols);
// row exponents (rows ints) and digits (16-byte aligned) of M
int residual_tc_prepare(const float4* M, int64_t ldm, int rows, int kdim, int* rowexp, unsigned char* digits,
                        cudaStream_t s);
// R (rows x ncols) = B - M X from M's row exponents and digits; B may be null
// (zero).  The status word (MGT_OK or MGT_ERR_TIMEOUT) is the first int of work.
int residual_tc_apply(const unsigned char* digits, const int* rowexp, int rows, int kdim, const double2* X,
                      int64_t ldx, int ncols, const double2* B, int64_t ldb, double2* R, int64_t ldr, void* work,
                      size_t work_bytes, cudaStream_t s);
// both steps in one call: workspace = row exponents + digits + one application
size_t residual_tc_workspace_bytes(int64_t rows, int64_t kdim, int64_t ncols);
// that workspace's parts (any pointer may be null); returns the application part's offset
size_t residual_tc_split(void* work, int64_t rows, int64_t kdim, int** rowexp, unsigned char** digits, char** aw);
int residual_tc(const float4* M, int64_t ldm, int rows, int kdim, const double2* X, int64_t ldx, int ncols,
                const double2* B, int64_t ldb, double2* R, int64_t ldr, void* work, size_t work_bytes,
                cudaStream_t s);

}  // namespace mgt
