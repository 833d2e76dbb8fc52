// SIMT complex GEMM update (FP64 pipe for complex128, FP32 pipe for
// complex64).  64 x 64 output tile per CTA, K staged through shared memory
// 16 at a time, 4 x 4 complex outputs per thread.
#include "gemm.cuh"
#include "diag.cuh"

namespace mgt {

constexpr int kGT = 64, kGK = 16;

template <typename T>
__global__ void __launch_bounds__(256)
cgemm_sub_kernel(int M, int N, int K, const cplx<T>* __restrict__ A, int64_t lda,
                 const cplx<T>* __restrict__ B, int64_t ldb, cplx<T>* __restrict__ C, int64_t ldc) {
  using V = cplx<T>;
  __shared__ V As[kGK][kGT + 1];
  __shared__ V Bs[kGK][kGT];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int row0 = blockIdx.y * kGT, col0 = blockIdx.x * kGT;
  V acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = czero<V>();
  for (int k0 = 0; k0 < K; k0 += kGK) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int idx = tid + 256 * q;
      int r = idx >> 4, kk = idx & 15;
      V v = czero<V>();
      if (row0 + r < M && k0 + kk < K) v = A[(int64_t)(row0 + r) * lda + k0 + kk];
      As[kk][r] = v;
      int kb = idx >> 6, cc = idx & 63;
      V u = czero<V>();
      if (k0 + kb < K && col0 + cc < N) u = B[(int64_t)(k0 + kb) * ldb + col0 + cc];
      Bs[kb][cc] = u;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kGK; ++kk) {
      V a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) cfma(acc[i][j], a[i], b[j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    int r = row0 + ty + 16 * i;
    if (r >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int c = col0 + tx + 16 * j;
      if (c < N) {
        V* p = C + (int64_t)r * ldc + c;
        *p = csub(*p, acc[i][j]);
      }
    }
  }
}

template <typename T>
int gemm_sub(int M, int N, int K, const cplx<T>* A, int64_t lda, const cplx<T>* B, int64_t ldb,
             cplx<T>* C, int64_t ldc, cudaStream_t s) {
  if (M <= 0 || N <= 0 || K <= 0) return MGT_OK;
  dim3 grid((N + kGT - 1) / kGT, (M + kGT - 1) / kGT);
  if (grid.y > 65535) return MGT_ERR_UNSUPPORTED;
  count_launch();
  cgemm_sub_kernel<T><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc);
  return cudaGetLastError() == cudaSuccess ? MGT_OK : MGT_ERR_CUDA;
}

template int gemm_sub<double>(int, int, int, const double2*, int64_t, const double2*, int64_t, double2*, int64_t, cudaStream_t);
template int gemm_sub<float>(int, int, int, const float2*, int64_t, const float2*, int64_t, float2*, int64_t, cudaStream_t);

}  // namespace mgt
