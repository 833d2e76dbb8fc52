// K3: multi-RHS triangular solves with the LU factors, one persistent launch
// per triangle (the ?getrs half of torch.linalg.solve in solve(),
// Transmission2D.py:230 / Transmission3D.py:205).
//
// Block rows of 64.  CTAs claim block rows in dependency order from an
// atomic counter (first row first for L, last row first for U).  A CTA
// accumulates B_i - sum_j T_ij X_j over the blocks j its row depends on,
// waiting (bounded) on each X_j's ready flag as it goes, then solves the
// 64 x 64 diagonal block in shared memory, writes X_i and releases its flag.
// Rows that depend on many blocks do their updates while earlier rows are
// still being solved, so the solve costs about one block step per block row
// instead of four kernel launches per block row.  No CTA waits on a row that
// was not claimed earlier by a running CTA, so progress is guaranteed.
#include <algorithm>
#include <atomic>
#include <mutex>

#include "common.cuh"
#include "diag.cuh"

namespace mgt {

constexpr int kTB = 64;      // block rows
constexpr int kTC = 64;      // right-hand-side columns per pass

__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

template <typename T, bool UPPER>
__global__ void __launch_bounds__(256)
tri_solve_kernel(const cplx<T>* __restrict__ F, int64_t ldf, cplx<T>* __restrict__ X, int64_t ldx, int n,
                 int ncols, unsigned* counter, unsigned* flags, unsigned epoch, int* status) {
  using V = cplx<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* Ts = reinterpret_cast<V*>(smem_raw);          // [kTB][kTB + 1]
  V* Xs = Ts + kTB * (kTB + 1);                      // [kTB][kTC]
  __shared__ unsigned s_blk;
  __shared__ int s_fail;
  __shared__ V dinv[kTB];
  const int tid = threadIdx.x, tr = tid >> 4, tc = tid & 15;
  const int nb = (n + kTB - 1) / kTB;
  while (true) {
    if (tid == 0) { s_blk = atomicAdd(counter, 1u); s_fail = 0; }
    __syncthreads();
    const unsigned k = s_blk;
    if (k >= (unsigned)nb) break;
    const int i = UPPER ? nb - 1 - (int)k : (int)k;
    const int r0 = i * kTB, rb = min(kTB, n - r0);
    V acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        const int r = tr + 16 * a, c = tc + 16 * b;
        acc[a][b] = (r < rb && c < ncols) ? X[(int64_t)(r0 + r) * ldx + c] : czero<V>();
      }
    // ---- accumulate the dependencies: acc -= T[i, j] X_j, in the order the
    // X_j complete (ascending j for L, descending j for U)
    const int ndep = UPPER ? nb - 1 - i : i;
    for (int d = 0; d < ndep; ++d) {
      const int j = UPPER ? nb - 1 - d : d;
      const int c0 = j * kTB, cb = min(kTB, n - c0);
      if (tid == 0) {
        unsigned it = 0;
        while (ld_acquire_u32(flags + j) != epoch) {
          if (++it > kSpinLimit) { s_fail = 1; atomicExch(status, MGT_ERR_TIMEOUT); break; }
          if (it > 16) __nanosleep(64);
        }
      }
      __syncthreads();
      if (s_fail) return;
      for (int idx = tid; idx < kTB * kTB; idx += 256) {
        int r = idx >> 6, c = idx & 63;
        Ts[r * (kTB + 1) + c] = (r < rb && c < cb) ? F[(int64_t)(r0 + r) * ldf + c0 + c] : czero<V>();
      }
      for (int idx = tid; idx < kTB * kTC; idx += 256) {
        int r = idx >> 6, c = idx & 63;
        Xs[r * kTC + c] = (r < cb && c < ncols) ? ldcg(X + (int64_t)(c0 + r) * ldx + c) : czero<V>();
      }
      __syncthreads();
#pragma unroll 4
      for (int kk = 0; kk < kTB; ++kk) {
        V a[4], x[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) a[q] = Ts[(tr + 16 * q) * (kTB + 1) + kk];
#pragma unroll
        for (int q = 0; q < 4; ++q) x[q] = Xs[kk * kTC + tc + 16 * q];
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
          for (int b = 0; b < 4; ++b) cfms(acc[q][b], a[q], x[b]);
      }
      __syncthreads();
    }
    // ---- diagonal block
    for (int idx = tid; idx < kTB * kTB; idx += 256) {
      int r = idx >> 6, c = idx & 63;
      Ts[r * (kTB + 1) + c] = (r < rb && c < rb) ? F[(int64_t)(r0 + r) * ldf + r0 + c] : czero<V>();
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) Xs[(tr + 16 * a) * kTC + tc + 16 * b] = acc[a][b];
    __syncthreads();
    if (UPPER)
      for (int r = tid; r < rb; r += 256) dinv[r] = crecip(Ts[r * (kTB + 1) + r]);
    __syncthreads();
    {
      // 4 lanes per column, 8 columns per warp
      const int warp = tid >> 5, lane = tid & 31;
      const int col = warp * 8 + (lane >> 2), t4 = lane & 3;
      if (!UPPER) {
        for (int kk = 0; kk < rb - 1; ++kk) {
          __syncwarp();
          const V xk = Xs[kk * kTC + col];
          for (int r = kk + 1 + t4; r < rb; r += 4) cfms(Xs[r * kTC + col], Ts[r * (kTB + 1) + kk], xk);
        }
      } else {
        for (int kk = rb - 1; kk >= 0; --kk) {
          __syncwarp();
          if (t4 == 0) Xs[kk * kTC + col] = cmul(Xs[kk * kTC + col], dinv[kk]);
          __syncwarp();
          const V xk = Xs[kk * kTC + col];
          for (int r = t4; r < kk; r += 4) cfms(Xs[r * kTC + col], Ts[r * (kTB + 1) + kk], xk);
        }
      }
    }
    __syncthreads();
    for (int idx = tid; idx < kTB * kTC; idx += 256) {
      int r = idx >> 6, c = idx & 63;
      if (r < rb && c < ncols) X[(int64_t)(r0 + r) * ldx + c] = Xs[r * kTC + c];
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) st_release_u32(flags + i, epoch);
  }
}

static std::atomic<unsigned> g_solve_epoch{0};

size_t tri_solve_workspace_bytes(int64_t n) { return (size_t)(((n + kTB - 1) / kTB) + 64) * sizeof(unsigned) + 256; }

static int resident_ctas(const void* kern, size_t smem) {
  int dev = 0, sms = 1, per = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, 256, smem);
  return std::max(1, sms * std::max(1, per));
}

// In-place X = T^-1 X for all nrhs columns (T = unit lower or upper part of F).
template <typename T, bool UPPER>
int tri_solve(const cplx<T>* F, int64_t ldf, cplx<T>* X, int64_t ldx, int n, int nrhs, void* work, int* status,
              cudaStream_t s) {
  using V = cplx<T>;
  const size_t smem = (size_t)(kTB * (kTB + 1) + kTB * kTC) * sizeof(V);
  static int max_ctas = 0;
  static std::once_flag once;
  std::call_once(once, [smem] {
    cudaFuncSetAttribute(tri_solve_kernel<T, UPPER>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    max_ctas = resident_ctas((const void*)tri_solve_kernel<T, UPPER>, smem);
  });
  const int nb = (n + kTB - 1) / kTB;
  unsigned* counter = (unsigned*)work;
  unsigned* flags = counter + 64;
  for (int c0 = 0; c0 < nrhs; c0 += kTC) {
    const int nc = std::min(kTC, nrhs - c0);
    const unsigned epoch = g_solve_epoch.fetch_add(1) + 1;
    if (cudaMemsetAsync(counter, 0, sizeof(unsigned), s) != cudaSuccess) return MGT_ERR_CUDA;
    count_launch();
    tri_solve_kernel<T, UPPER><<<std::min(nb, max_ctas), 256, smem, s>>>(F, ldf, X + c0, ldx, n, nc, counter, flags,
                                                                       epoch, status);
  }
  return cudaGetLastError() == cudaSuccess ? MGT_OK : MGT_ERR_CUDA;
}

template int tri_solve<double, false>(const double2*, int64_t, double2*, int64_t, int, int, void*, int*, cudaStream_t);
template int tri_solve<double, true>(const double2*, int64_t, double2*, int64_t, int, int, void*, int*, cudaStream_t);
template int tri_solve<float, false>(const float2*, int64_t, float2*, int64_t, int, int, void*, int*, cudaStream_t);
template int tri_solve<float, true>(const float2*, int64_t, float2*, int64_t, int, int, void*, int*, cudaStream_t);

}  // namespace mgt
