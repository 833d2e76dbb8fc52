// Tensor-core residual R = B - M X (M double-float, X, B, R complex128): the
// digit-split (Ozaki-scheme) kernel of residual_tc.cu.
#pragma once
#include "common.cuh"

namespace mgt {

// the tcgen05 residual handles these shapes on this device
bool residual_tc_supported(int64_t rows, int64_t kdim, int64_t ncols);
// workspace of residual_tc for M (rows x kdim) and ncols right-hand sides
size_t residual_tc_workspace_bytes(int64_t rows, int64_t kdim, int64_t ncols);
// row exponents of M (what residual_tc computes when it is given none)
int residual_tc_rowexp(const float4* M, int64_t ldm, int rows, int kdim, int* out, cudaStream_t s);
// R (rows x ncols) = B - M X; B may be null (zero).  rowexp: the row
// exponents from residual_tc_rowexp, or null to compute them here.
int residual_tc(const float4* M, int64_t ldm, int rows, int kdim, const double2* X, int64_t ldx, int ncols,
                const double2* B, int64_t ldb, double2* R, int64_t ldr, const int* rowexp, void* work,
                size_t work_bytes, cudaStream_t s);

}  // namespace mgt
