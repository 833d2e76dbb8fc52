// Tensor-core (tcgen05, kind::tf32) complex trailing update for the
// complex64 LU:  C (M x N, complex64) -= A (M x K) * B (K x N),  K <= 64.
//
// Complex -> real: with A stored interleaved (re, im) the row of A is a real
// row of length 2K, and
//   Re C[i,j] -= sum_k A'[i,2k] Br[k,j] + A'[i,2k+1] (-Bi[k,j])
//   Im C[i,j] -= sum_k A'[i,2k] Bi[k,j] + A'[i,2k+1] ( Br[k,j])
// so C' (M x 2N real, interleaved) -= A' (M x 2K) * B' (2K x 2N), where the
// prep kernel writes B'^T (2N rows, 2K contiguous) -- a K-major operand.
//
// Precision: FP32 inputs are split x = hi + lo with hi = tf32(x) (round to
// nearest, low 13 bits zero) and lo = x - hi; the product is accumulated in
// FP32 in TMEM as hi*hi + hi*lo + lo*hi ("TF32x3", the split-product scheme of
// Markidis et al. 2018 / Ootomo & Yokota 2022), which keeps ~FP32 accuracy.
//
// Kernel: one CTA per 128 x 256 tile of C' (128 rows, 128 complex columns).
//   warp 0 lane 0 : TMA producer (cp.async.bulk.tensor, 128B swizzle) of the
//                   A_hi/A_lo (128 x 32 fp32) and B_hi/B_lo (256 x 32 fp32)
//                   tiles of each 32-wide K block, 2-stage mbarrier ring
//   warp 1 lane 0 : tcgen05.mma issuer (M=128, N=256, K=8 per instruction,
//                   12 instructions per K block), tcgen05.commit to free a
//                   stage and, at the end, to publish the accumulator
//   warp 2        : TMEM allocation / deallocation (256 columns)
//   warps 4-7     : epilogue: tcgen05.ld 32 columns at a time, C -= acc
// Every wait is bounded; on expiry the CTA records MGT_ERR_TIMEOUT, drains
// the MMAs it issued, frees its TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>

#include "common.cuh"
#include "diag.cuh"
#include "gemm.cuh"
#include "gemm_tc.cuh"

namespace mgt {

namespace tc {

constexpr int BM = 128;            // tile rows (M)
constexpr int BN = 256;            // tile real columns (N')
constexpr int BK = 32;             // fp32 elements per 128-byte swizzle row
constexpr int KR = 128;            // real K of the split buffers (2 * 64)
constexpr int KBLOCKS = KR / BK;   // 4
constexpr int STAGES = 2;
constexpr uint32_t A_TILE = BM * BK * 4;   // 16 KB
constexpr uint32_t B_TILE = BN * BK * 4;   // 32 KB
constexpr uint32_t STAGE_BYTES = 2 * A_TILE + 2 * B_TILE;   // 96 KB
constexpr uint32_t TMEM_COLS = 256;
constexpr int THREADS = 256;
constexpr size_t SMEM_BYTES = STAGES * STAGE_BYTES + 1024 /* alignment slack */ + 256 /* barriers */;
constexpr uint32_t kWaitLimit = 1u << 22;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: false if the CTA aborted or the limit ran out (then abort is set).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort) {
  for (uint32_t it = 0; it < kWaitLimit; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*abort) return false;
  }
  *abort = 1;
  return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];"
      ::"r"(smem_u32(dst)), "l"((uint64_t)map), "r"(smem_u32(bar)), "r"(c0), "r"(c1)
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// K-major operand, 128-byte swizzle: rows of 128 B, 8-row groups 1024 B apart.
__device__ __forceinline__ uint64_t kmajor_sw128_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);   // start address
  d |= (uint64_t)1 << 16;                     // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;           // stride byte offset: next 8-row group
  d |= (uint64_t)1 << 46;                     // descriptor version
  d |= (uint64_t)2 << 61;                     // SWIZZLE_128B
  return d;
}

// kind::tf32, D = F32, A = B = TF32, both K-major, M = 128, N = 256
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n"
      ::"r"(d_tmem), "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__global__ void __launch_bounds__(THREADS, 1)
cgemm_tf32x3_kernel(const __grid_constant__ CUtensorMap mapAhi, const __grid_constant__ CUtensorMap mapAlo,
                    const __grid_constant__ CUtensorMap mapBhi, const __grid_constant__ CUtensorMap mapBlo,
                    float* __restrict__ C, int64_t ldc_real, int M, int Nreal, int* status) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // 1024-byte aligned stage area (128B-swizzle atoms must start on 1024 B)
  unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = reinterpret_cast<uint64_t*>(base + STAGES * STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* accum = empty + STAGES;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(accum + 1);
  volatile int* abort = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
    mbar_init(accum, 1);
    *abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 2) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // ---------------- TMA producer
    for (int kb = 0; kb < KBLOCKS; ++kb) {
      const int s = kb % STAGES;
      if (kb >= STAGES && !mbar_wait(&empty[s], ((kb / STAGES) - 1) & 1, abort)) break;
      unsigned char* st = base + s * STAGE_BYTES;
      mbar_expect_tx(&full[s], STAGE_BYTES);
      tma_load_2d(st, &mapAhi, &full[s], kb * BK, m0);
      tma_load_2d(st + A_TILE, &mapAlo, &full[s], kb * BK, m0);
      tma_load_2d(st + 2 * A_TILE, &mapBhi, &full[s], kb * BK, n0);
      tma_load_2d(st + 2 * A_TILE + B_TILE, &mapBlo, &full[s], kb * BK, n0);
    }
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer
    int issued = 0;
    for (int kb = 0; kb < KBLOCKS; ++kb) {
      const int s = kb % STAGES;
      if (!mbar_wait(&full[s], (kb / STAGES) & 1, abort)) break;
      tc_fence_after();
      const uint32_t st = smem_u32(base + s * STAGE_BYTES);
      const uint64_t ahi = kmajor_sw128_desc(st), alo = kmajor_sw128_desc(st + A_TILE);
      const uint64_t bhi = kmajor_sw128_desc(st + 2 * A_TILE), blo = kmajor_sw128_desc(st + 2 * A_TILE + B_TILE);
#pragma unroll
      for (int k = 0; k < BK / 8; ++k) {
        const uint64_t off = (uint64_t)((k * 32) >> 4);   // 8 tf32 = 32 bytes along K
        mma_tf32(tmem, alo + off, bhi + off, issued > 0);
        mma_tf32(tmem, ahi + off, blo + off, 1);
        mma_tf32(tmem, ahi + off, bhi + off, 1);
        ++issued;
      }
      mma_commit(&empty[s]);
    }
    mma_commit(accum);   // arrives once every MMA issued above has completed
  } else if (warp >= 4) {
    // ---------------- epilogue
    const int q = warp - 4;              // TMEM lanes 32q .. 32q+31
    const int row = m0 + q * 32 + lane;
    if (mbar_wait(accum, 0, abort)) {
      tc_fence_after();
      float* crow = C + (int64_t)row * ldc_real;
#pragma unroll 1
      for (int cc = 0; cc < BN; cc += 32) {
        float v[32];
        tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)cc, v);
        const int col = n0 + cc;
        if (row < M) {
          if (col + 32 <= Nreal) {
            float4* p = reinterpret_cast<float4*>(crow + col);
#pragma unroll
            for (int i = 0; i < 8; ++i) {
              float4 c = p[i];
              c.x -= v[4 * i];
              c.y -= v[4 * i + 1];
              c.z -= v[4 * i + 2];
              c.w -= v[4 * i + 3];
              p[i] = c;
            }
          } else {
#pragma unroll
            for (int i = 0; i < 32; ++i)
              if (col + i < Nreal) crow[col + i] -= v[i];
          }
        }
      }
    }
  }
  // drain: the accumulator barrier completes once all issued MMAs are done
  if (threadIdx.x == 0 && *abort) {
    mbar_wait(accum, 0, abort);
    atomicExch(status, MGT_ERR_TIMEOUT);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 2) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

__device__ __forceinline__ float tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// A (M x K complex) -> Ahi, Alo (M x 128 fp32), zero beyond 2K.
__global__ void split_a_kernel(const float2* __restrict__ A, int64_t lda, int M, int K, float* __restrict__ Ahi,
                               float* __restrict__ Alo) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)M * KR) return;
  int i = (int)(idx / KR), k = (int)(idx - (int64_t)i * KR);
  float v = 0.f;
  if (k < 2 * K) {
    float2 a = A[(int64_t)i * lda + (k >> 1)];
    v = (k & 1) ? a.y : a.x;
  }
  float h = tf32_rna(v);
  Ahi[idx] = h;
  Alo[idx] = v - h;
}

// B (K x N complex) -> B'^T hi/lo (2N x 128 fp32):
//   row 2j   : (Br[k,j], -Bi[k,j]) for k = 0..K-1, then zeros
//   row 2j+1 : (Bi[k,j],  Br[k,j])
__global__ void split_b_kernel(const float2* __restrict__ B, int64_t ldb, int K, int N, float* __restrict__ Bhi,
                               float* __restrict__ Blo) {
  __shared__ float2 t[64][33];
  const int j0 = blockIdx.x * 32;
  for (int idx = threadIdx.x; idx < 64 * 32; idx += blockDim.x) {
    int k = idx / 32, jj = idx - k * 32;
    t[k][jj] = (k < K && j0 + jj < N) ? B[(int64_t)k * ldb + j0 + jj] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  // 64 output rows (2 per column j) x 128 reals
  for (int idx = threadIdx.x; idx < 64 * KR; idx += blockDim.x) {
    int r = idx / KR, kr = idx - r * KR;
    int jj = r >> 1, j = j0 + jj;
    if (j >= N) continue;
    int k = kr >> 1;
    float2 b = t[k][jj];
    float v;
    if ((r & 1) == 0) v = (kr & 1) ? -b.y : b.x;
    else v = (kr & 1) ? b.x : b.y;
    float h = tf32_rna(v);
    int64_t o = (int64_t)(2 * j + (r & 1)) * KR + kr;
    Bhi[o] = h;
    Blo[o] = v - h;
  }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  });
  return fn;
}

// 2D fp32 tensor (rows x 128), box (32 x box_rows), 128-byte swizzle
static bool make_map(CUtensorMap* map, float* base, int64_t rows, int box_rows) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[2] = {(cuuint64_t)KR, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)KR * 4};
  cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace tc

size_t tc_scratch_bytes(int64_t n) {
  // Ahi, Alo: n x 128; Bhi, Blo: 2n x 128 (fp32)
  return (size_t)(2 * n + 4 * n) * tc::KR * sizeof(float) + 4096;
}

bool tc_available() { return tc::encode_fn() != nullptr; }

int TcPlan::init(void* scratch, int64_t nmax) {
  char* b = (char*)(((uintptr_t)scratch + 1023) & ~(uintptr_t)1023);
  Ahi = (float*)b;
  Alo = Ahi + nmax * tc::KR;
  Bhi = Alo + nmax * tc::KR;
  Blo = Bhi + 2 * nmax * tc::KR;
  this->nmax = nmax;
  bool ok = tc::make_map(&mAhi, Ahi, nmax, tc::BM) && tc::make_map(&mAlo, Alo, nmax, tc::BM) &&
            tc::make_map(&mBhi, Bhi, 2 * nmax, tc::BN) && tc::make_map(&mBlo, Blo, 2 * nmax, tc::BN);
  return ok ? MGT_OK : MGT_ERR_CUDA;
}

int gemm_sub_tc(const TcPlan& plan, int M, int N, int K, const float2* A, int64_t lda, const float2* B, int64_t ldb,
                float2* C, int64_t ldc, int* status, cudaStream_t s) {
  if (M <= 0 || N <= 0 || K <= 0) return MGT_OK;
  if (K > 64 || M > plan.nmax || N > plan.nmax) return MGT_ERR_UNSUPPORTED;
  if ((ldc & 1) != 0) return MGT_ERR_ARG;   // float4 epilogue needs 16-byte aligned rows
  static std::once_flag once;
  std::call_once(once, [] {
    cudaFuncSetAttribute(tc::cgemm_tf32x3_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc::SMEM_BYTES);
  });
  int64_t na = (int64_t)M * tc::KR;
  count_launch();
  tc::split_a_kernel<<<(unsigned)((na + 255) / 256), 256, 0, s>>>(A, lda, M, K, plan.Ahi, plan.Alo);
  count_launch();
  tc::split_b_kernel<<<(N + 31) / 32, 256, 0, s>>>(B, ldb, K, N, plan.Bhi, plan.Blo);
  const int Nreal = 2 * N;
  dim3 grid((Nreal + tc::BN - 1) / tc::BN, (M + tc::BM - 1) / tc::BM);
  if (grid.y > 65535) return MGT_ERR_UNSUPPORTED;
  count_launch();
  tc::cgemm_tf32x3_kernel<<<grid, tc::THREADS, tc::SMEM_BYTES, s>>>(plan.mAhi, plan.mAlo, plan.mBhi, plan.mBlo,
                                                                    reinterpret_cast<float*>(C), 2 * ldc, M, Nreal,
                                                                    status);
  return cudaGetLastError() == cudaSuccess ? MGT_OK : MGT_ERR_CUDA;
}

}  // namespace mgt

// ---------------------------------------------------------------- C ABI: standalone update

extern "C" int mgt_cgemm_workspace_bytes(int64_t nmax, size_t* bytes) {
  if (!bytes || nmax <= 0) return MGT_ERR_ARG;
  *bytes = mgt::tc_scratch_bytes(nmax) + 256;
  return MGT_OK;
}

extern "C" int mgt_cgemm_sub(int dtype, int use_tensor_cores, int64_t M, int64_t N, int64_t K, const void* A,
                             int64_t lda, const void* B, int64_t ldb, void* C, int64_t ldc, void* work,
                             size_t work_bytes, void* stream) {
  using namespace mgt;
  if (!A || !B || !C || M <= 0 || N <= 0 || K <= 0 || lda < K || ldb < N || ldc < N) return MGT_ERR_ARG;
  if (M > (1 << 30) || N > (1 << 30)) return MGT_ERR_UNSUPPORTED;
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == MGT_C128)
    return gemm_sub<double>((int)M, (int)N, (int)K, (const double2*)A, lda, (const double2*)B, ldb, (double2*)C, ldc, s);
  if (dtype != MGT_C64) return MGT_ERR_ARG;
  if (!use_tensor_cores)
    return gemm_sub<float>((int)M, (int)N, (int)K, (const float2*)A, lda, (const float2*)B, ldb, (float2*)C, ldc, s);
  if (K > 64) return MGT_ERR_UNSUPPORTED;
  int64_t nmax = std::max(M, N);
  if (!work || work_bytes < tc_scratch_bytes(nmax) + 256) return MGT_ERR_WORKSPACE;
  if (!tc_available()) return MGT_ERR_UNSUPPORTED;
  int* status = (int*)work;
  TcPlan plan;
  int e = plan.init((char*)work + 256, nmax);
  if (e != MGT_OK) return e;
  return gemm_sub_tc(plan, (int)M, (int)N, (int)K, (const float2*)A, lda, (const float2*)B, ldb, (float2*)C, ldc,
                     status, s);
}
