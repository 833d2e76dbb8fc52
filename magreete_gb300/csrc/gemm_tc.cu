// Tensor-core (tcgen05) complex trailing update for the complex64 LU:
//   C (M x N, complex64) -= A (M x K) * B (K x N),  K <= 256.
// Two split-product schemes: F16x2 with kind::f16 MMAs (the default) and
// TF32x3 with kind::tf32 MMAs (MGT_TUNE_TC_PRECISION).
//
// Complex -> real: with A stored interleaved (re, im) the row of A is a real
// row of length 2K, and
//   Re C[i,j] -= sum_k A'[i,2k] Br[k,j] + A'[i,2k+1] (-Bi[k,j])
//   Im C[i,j] -= sum_k A'[i,2k] Bi[k,j] + A'[i,2k+1] ( Br[k,j])
// so C' (M x 2N real, interleaved) -= A' (M x 2K) * B' (2K x 2N), where the
// prep kernel writes B'^T (2N rows, 2K contiguous) -- a K-major operand.
//
// TF32x3: FP32 inputs are split x = hi + lo with hi = tf32(x) (round to
// nearest, low 13 bits zero) and lo = x - hi; the product is accumulated in
// FP32 in TMEM as hi*hi + hi*lo + lo*hi (the split-product scheme of
// Markidis et al. 2018 / Ootomo & Yokota 2022), which keeps ~FP32 accuracy.
//
// F16x2 variant (default): both operands are first scaled by a power of two
// -- A per row, B per complex output column -- so that the largest magnitude
// lies in [0.5, 1), then split x = hi + lo with hi = fp16(x), lo = fp16(x - hi)
// (22 significant bits, the same as the TF32 split) and multiplied with
// kind::f16 MMAs, which issue at twice the TF32 rate; the epilogue multiplies
// the accumulator by the inverse scales.  Values below 2^-24 of their row's
// (column's) largest flush to zero, an absolute error below that of FP32
// rounding of the row's largest entry.
//
// Kernel: persistent, one CTA per SM walking 128 x 256 tiles of C' (128 rows,
// 128 complex columns; N = 256 keeps the MMA's shared-memory operand reads
// and the operand bytes per flop below those of a square 128 x 128 tile):
//   warp 0 lane 0 : TMA producer (cp.async.bulk.tensor, 128B swizzle) of the
//                   A_hi/A_lo (128 rows) and B_hi/B_lo (256 rows of B'^T)
//                   tiles of each K block (one 128-byte row: 64 fp16 or 32
//                   fp32), 2-stage mbarrier ring of 96 KB stages
//   warp 1 lane 0 : tcgen05.mma issuer (M = 128, N = 256, 32 bytes of K per
//                   instruction, 12 instructions per K block), tcgen05.commit
//                   to free a stage and, at the end, to publish the accumulator
//   warp 2        : TMEM allocation / deallocation (2 accumulators x 256
//                   columns: all of TMEM)
//   warp 3 lane 0 : C mover: TMA reduce-adds of 128 x 32 chunks into C
//   warps 4-7     : epilogue: tcgen05.ld 32 columns at a time, -acc staged
// Every wait is bounded; on expiry the CTA records MGT_ERR_TIMEOUT, drains
// the MMAs it issued, frees its TMEM and returns.
#include <cuda.h>
#include <cuda_fp16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <atomic>
#include <mutex>

#include "common.cuh"
#include "diag.cuh"
#include "gemm.cuh"
#include "gemm_tc.cuh"
#include "tcgen05.cuh"

namespace mgt {

namespace tc {

constexpr int BM = 128;            // tile rows (M)
constexpr int BN = 256;            // tile real columns (N') = 128 complex columns
constexpr int KMAX = 256;          // largest complex K of one update
constexpr int KR = 2 * KMAX;       // real K stride of the split buffers
constexpr uint32_t A_TILE = BM * 128;      // 16 KB: 128 rows of one 128-byte swizzle row
constexpr uint32_t B_TILE = BN * 128;      // 32 KB
constexpr uint32_t STAGE_BYTES = 2 * A_TILE + 2 * B_TILE;   // 96 KB
constexpr int CHUNKS = BN / 32;            // epilogue chunks per tile (32 fp32 columns each)
constexpr uint32_t CHUNK_BYTES = BM * 128; // 16 KB
constexpr uint32_t TMEM_COLS = 2 * BN;     // two accumulators
constexpr int THREADS = 256;
// pipeline shape: operand stages x C ring slots (2 x 2: 192 + 32 KB)
template <int STAGES, int CSLOTS>
constexpr size_t smem_bytes() {
  return STAGES * STAGE_BYTES + CSLOTS * CHUNK_BYTES + 1024 /* alignment slack */ + 256;
}
// Operand element per mode: K elements per 128-byte swizzle row (one stage)
// and the instruction descriptor (D = F32, both operands K-major, M = 128,
// N = 128): kind::tf32 with A = B = TF32 (code 2), kind::f16 with A = B = F16
// (code 0).  Either way one MMA covers 32 bytes of K.
template <bool F16>
struct Mode {
  static constexpr int ELEM = F16 ? 2 : 4;
  static constexpr int BK = 128 / ELEM;
  static constexpr uint32_t kAB = F16 ? 0u : 2u;
  static constexpr uint32_t kIdesc =
      (1u << 4) | (kAB << 7) | (kAB << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
};

template <bool F16>
__device__ __forceinline__ void mma_split(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
  if constexpr (F16) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
        ::"r"(d_tmem), "l"(a), "l"(b), "r"(Mode<true>::kIdesc), "r"(accumulate)
        : "memory");
  } else {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n"
        ::"r"(d_tmem), "l"(a), "l"(b), "r"(Mode<false>::kIdesc), "r"(accumulate)
        : "memory");
  }
}
// Persistent kernel: each CTA walks tiles blockIdx.x, +gridDim.x, ...; TMEM
// holds two accumulators so the epilogue of tile t overlaps the MMAs of
// tile t+1.  C is never loaded into the SM: the epilogue stages -acc in a
// ring of 128 x 32 fp32 chunks and one C-mover thread adds each chunk into C
// with a TMA reduce (f32 add at L2), handing a slot back once its reduce has
// read it.
// invA / invB (F16 mode): inverse row scales of A and inverse complex-column
// scales of B.  The update reads the B split from row boff (twice its first
// complex column) on, so that one split serves several launches.
template <bool F16, int STAGES, int CSLOTS>
__global__ void __launch_bounds__(THREADS, 1)
cgemm_split3_kernel(const __grid_constant__ CUtensorMap mapAhi, const __grid_constant__ CUtensorMap mapAlo,
                    const __grid_constant__ CUtensorMap mapBhi, const __grid_constant__ CUtensorMap mapBlo,
                    const __grid_constant__ CUtensorMap mapC, int cx0, int cy0, int boff, int tiles_n,
                    int total_tiles, int kblocks, const float* __restrict__ invA, const float* __restrict__ invB,
                    int* status) {
  constexpr int BK = Mode<F16>::BK;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  unsigned char* cring = base + STAGES * STAGE_BYTES;
  uint64_t* full = reinterpret_cast<uint64_t*>(cring + CSLOTS * CHUNK_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* tfull = empty + STAGES;
  uint64_t* tempty = tfull + 2;
  uint64_t* cfree = tempty + 2;
  uint64_t* cdone = cfree + CSLOTS;
  uint64_t* done = cdone + CSLOTS;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  volatile int* abort = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
    for (int a = 0; a < 2; ++a) { mbar_init(&tfull[a], 1); mbar_init(&tempty[a], 128); }
    for (int c = 0; c < CSLOTS; ++c) { mbar_init(&cfree[c], 1); mbar_init(&cdone[c], 128); }
    mbar_init(done, 1);
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
  const int first = blockIdx.x, stride = gridDim.x;

  if (warp == 0 && lane == 0) {
    // ---------------- TMA producer: A/B K blocks into the stage ring
    int it = 0;
    for (int t = first; t < total_tiles && !*abort; t += stride) {
      const int m0 = (t / tiles_n) * BM, n0 = (t % tiles_n) * BN;
      for (int kb = 0; kb < kblocks; ++kb, ++it) {
        const int s = it % STAGES;
        if (it >= STAGES && !mbar_wait(&empty[s], ((it / STAGES) - 1) & 1, abort)) break;
        unsigned char* st = base + s * STAGE_BYTES;
        mbar_expect_tx(&full[s], STAGE_BYTES);
        tma_load_2d(st, &mapAhi, &full[s], kb * BK, m0);
        tma_load_2d(st + A_TILE, &mapAlo, &full[s], kb * BK, m0);
        tma_load_2d(st + 2 * A_TILE, &mapBhi, &full[s], kb * BK, boff + n0);
        tma_load_2d(st + 2 * A_TILE + B_TILE, &mapBlo, &full[s], kb * BK, boff + n0);
      }
    }
    // (abort path) the last stages' loads land before the CTA may exit
    for (int j = (it > STAGES ? it - STAGES : 0); j < it; ++j) mbar_wait_plain(&full[j % STAGES], (j / STAGES) & 1);
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer
    int it = 0, lt = 0;
    for (int t = first; t < total_tiles && !*abort; t += stride, ++lt) {
      const int acc = lt & 1;
      if (lt >= 2 && !mbar_wait(&tempty[acc], ((lt >> 1) - 1) & 1, abort)) break;
      tc_fence_after();
      const uint32_t d = tmem + (uint32_t)(acc * BN);
      bool ok = true;
      for (int kb = 0; kb < kblocks; ++kb, ++it) {
        const int s = it % STAGES;
        if (!mbar_wait(&full[s], (it / STAGES) & 1, abort)) { ok = false; break; }
        tc_fence_after();
        const uint32_t st = smem_u32(base + s * STAGE_BYTES);
        const uint64_t ahi = kmajor_sw128_desc(st), alo = kmajor_sw128_desc(st + A_TILE);
        const uint64_t bhi = kmajor_sw128_desc(st + 2 * A_TILE), blo = kmajor_sw128_desc(st + 2 * A_TILE + B_TILE);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const uint64_t off = (uint64_t)((k * 32) >> 4);   // 32 bytes along K per MMA
          mma_split<F16>(d, alo + off, bhi + off, (kb | k) != 0);
          mma_split<F16>(d, ahi + off, blo + off, 1);
          mma_split<F16>(d, ahi + off, bhi + off, 1);
        }
        mma_commit(&empty[s]);
      }
      mma_commit(&tfull[acc]);
      if (!ok) break;
    }
    mma_commit(done);   // arrives once every MMA this thread issued has completed
  } else if (warp == 3 && lane == 0) {
    // ---------------- C mover: each updated chunk (-acc, staged by the
    // epilogue) is added into C by a TMA reduce (f32 add at L2), so C is never
    // loaded into the SM; a slot is handed back once its reduce has read it
    const int ntiles = total_tiles > first ? (total_tiles - first + stride - 1) / stride : 0;
    const int G = ntiles * CHUNKS;
    for (int g = 0; g < G; ++g) {
      const int slot = g % CSLOTS;
      if (!mbar_wait(&cdone[slot], (g / CSLOTS) & 1, abort)) break;
      const int t = first + (g / CHUNKS) * stride;
      tma_reduce_add_2d(&mapC, cring + slot * CHUNK_BYTES, cx0 + (t % tiles_n) * BN + (g % CHUNKS) * 32,
                        cy0 + (t / tiles_n) * BM);
      bulk_commit();
      // every reduce but the newest has read its slot
      if (g >= 1) {
        bulk_wait_read1();
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&cfree[(g - 1) % CSLOTS])) : "memory");
      }
    }
    bulk_wait0();
  } else if (warp >= 4) {
    // ---------------- epilogue: 128 threads, thread = accumulator row; each
    // chunk: TMEM -> registers, -acc (scaled) into a free slot, handed to the
    // C mover for its reduce into C
    const int q = warp - 4, r = q * 32 + lane;
    const int ntiles = total_tiles > first ? (total_tiles - first + stride - 1) / stride : 0;
    for (int lt = 0; lt < ntiles; ++lt) {
      const int acc = lt & 1;
      if (!mbar_wait(&tfull[acc], (lt >> 1) & 1, abort)) break;
      tc_fence_after();
      bool ok = true;
      const int tile = first + lt * stride;
      const int tm0 = (tile / tiles_n) * BM, tn0 = (tile % tiles_n) * BN;
      const float rs = F16 ? -__ldg(invA + tm0 + r) : -1.f;
      for (int c = 0; c < CHUNKS; ++c) {
        const int g = lt * CHUNKS + c, slot = g % CSLOTS;
        float v[32];
        tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(acc * BN + c * 32), v);
        if (c == CHUNKS - 1) {
          // every TMEM read of this accumulator is done
          tc_fence_before();
          asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&tempty[acc])) : "memory");
        }
        if constexpr (F16) {
          const float* cs = invB + ((boff + tn0 + c * 32) >> 1);
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const float f = rs * __ldg(cs + j);
            v[2 * j] *= f;
            v[2 * j + 1] *= f;
          }
        } else {
#pragma unroll
          for (int j = 0; j < 32; ++j) v[j] = -v[j];
        }
        if (g >= CSLOTS && !mbar_wait(&cfree[slot], ((g / CSLOTS) - 1) & 1, abort)) { ok = false; break; }
        unsigned char* rowp = cring + slot * CHUNK_BYTES + r * 128;
#pragma unroll
        for (int j = 0; j < 8; ++j)
          *reinterpret_cast<float4*>(rowp + ((j ^ (r & 7)) << 4)) =
              make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
        fence_async_smem();
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&cdone[slot])) : "memory");
      }
      if (!ok) break;
    }
  }
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x == 0 && *abort) atomicExch(status, MGT_ERR_TIMEOUT);
  if (warp == 2) {
    // every issued MMA has completed before the accumulator columns are freed
    bool drained = (lane == 0) ? mbar_wait_plain(done, 0) : true;
    __syncwarp();
    (void)drained;
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

__device__ __forceinline__ float tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// A (M x K complex) -> Ahi, Alo (M rows, stride KR fp32): the first kcols
// reals of each row (2K rounded up to the 32-wide K blocks), zero beyond 2K.
__global__ void split_a_kernel(const float2* __restrict__ A, int64_t lda, int M, int K, int kcols,
                               float* __restrict__ Ahi, float* __restrict__ Alo) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)M * kcols) return;
  int i = (int)(idx / kcols), k = (int)(idx - (int64_t)i * kcols);
  float v = 0.f;
  if (k < 2 * K) {
    float2 a = A[(int64_t)i * lda + (k >> 1)];
    v = (k & 1) ? a.y : a.x;
  }
  float h = tf32_rna(v);
  const int64_t o = (int64_t)i * KR + k;
  Ahi[o] = h;
  Alo[o] = v - h;
}

// B splits: one CTA per SB_COLS complex columns of B, all K rows staged in
// shared memory.  Columns N .. (grid end) are written as zeros so that the
// tile columns past the matrix edge accumulate exactly zero (TMA stores clip
// the inner dimension only at 16-byte granularity; a zero update leaves those
// bytes as they were loaded).
constexpr int SB_COLS = 16;

__global__ void split_b_kernel(const float2* __restrict__ B, int64_t ldb, int K, int N, int kcols,
                               float* __restrict__ Bhi, float* __restrict__ Blo) {
  __shared__ float2 t[KMAX][SB_COLS + 1];
  const int j0 = blockIdx.x * SB_COLS, krows = kcols >> 1;
  for (int idx = threadIdx.x; idx < krows * SB_COLS; idx += blockDim.x) {
    int k = idx / SB_COLS, jj = idx - k * SB_COLS;
    t[k][jj] = (k < K && j0 + jj < N) ? B[(int64_t)k * ldb + j0 + jj] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  // 2 SB_COLS output rows (2 per column j) x kcols reals
  for (int idx = threadIdx.x; idx < 2 * SB_COLS * kcols; idx += blockDim.x) {
    int r = idx / kcols, kr = idx - r * kcols;
    int jj = r >> 1, j = j0 + jj;
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

// F16 mode.  A (M x K complex) -> Ahi, Alo (fp16, M rows of stride KR): row i
// scaled by 2^-e_i, e_i the exponent of its largest |re|, |im|
// (max * 2^-e_i in [0.5, 1)); invA[i] = 2^e_i.  One warp per row.
__global__ void split_a_f16_kernel(const float2* __restrict__ A, int64_t lda, int M, int K, int kcols,
                                   __half* __restrict__ Ahi, __half* __restrict__ Alo, float* __restrict__ invA) {
  const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (i >= M) return;
  float v[KR / 32];
  unsigned mx = 0;
#pragma unroll
  for (int j = 0; j < KR / 32; ++j) {
    const int k = lane + 32 * j;
    float x = 0.f;
    if (k < 2 * K) {
      const float2 a = A[(int64_t)i * lda + (k >> 1)];
      x = (k & 1) ? a.y : a.x;
    }
    v[j] = x;
    mx = max(mx, __float_as_uint(fabsf(x)));
  }
  mx = __reduce_max_sync(0xffffffffu, mx);
  int e = 0;
  if (mx != 0u && mx < 0x7F800000u) {
    frexpf(__uint_as_float(mx), &e);
    e = max(-120, min(120, e));
  }
  const float sc = ldexpf(1.f, -e);
#pragma unroll
  for (int j = 0; j < KR / 32; ++j) {
    const int k = lane + 32 * j;
    if (k < kcols) {
      const float x = v[j] * sc;
      const __half h = __float2half_rn(x);
      const int64_t o = (int64_t)i * KR + k;
      Ahi[o] = h;
      Alo[o] = __float2half_rn(x - __half2float(h));
    }
  }
  if (lane == 0) invA[i] = ldexpf(1.f, e);
}

// F16 mode.  B (K x N complex) -> B'^T rows 2j, 2j+1 (fp16), both scaled by
// 2^-e_j, e_j the exponent of the largest |re|, |im| of column j; invB[j] = 2^e_j.
// Columns N .. (grid end) are zero (see split_b_kernel).
__global__ void split_b_f16_kernel(const float2* __restrict__ B, int64_t ldb, int K, int N, int kcols,
                                   __half* __restrict__ Bhi, __half* __restrict__ Blo, float* __restrict__ invB) {
  __shared__ float2 t[KMAX][SB_COLS + 1];
  __shared__ float sc[SB_COLS];
  const int j0 = blockIdx.x * SB_COLS, krows = kcols >> 1;
  for (int idx = threadIdx.x; idx < krows * SB_COLS; idx += blockDim.x) {
    int k = idx / SB_COLS, jj = idx - k * SB_COLS;
    t[k][jj] = (k < K && j0 + jj < N) ? B[(int64_t)k * ldb + j0 + jj] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  // column scales: warp w handles columns w, w + 8, ...
  for (int jj = threadIdx.x >> 5; jj < SB_COLS; jj += blockDim.x >> 5) {
    const int lane = threadIdx.x & 31;
    unsigned mx = 0;
    for (int k = lane; k < krows; k += 32)
      mx = max(mx, max(__float_as_uint(fabsf(t[k][jj].x)), __float_as_uint(fabsf(t[k][jj].y))));
    mx = __reduce_max_sync(0xffffffffu, mx);
    int e = 0;
    if (mx != 0u && mx < 0x7F800000u) {
      frexpf(__uint_as_float(mx), &e);
      e = max(-120, min(120, e));
    }
    if (lane == 0) {
      sc[jj] = ldexpf(1.f, -e);
      invB[j0 + jj] = ldexpf(1.f, e);
    }
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < 2 * SB_COLS * kcols; idx += blockDim.x) {
    int r = idx / kcols, kr = idx - r * kcols;
    int jj = r >> 1, j = j0 + jj;
    int k = kr >> 1;
    float2 b = t[k][jj];
    float v;
    if ((r & 1) == 0) v = (kr & 1) ? -b.y : b.x;
    else v = (kr & 1) ? b.x : b.y;
    v *= sc[jj];
    const __half h = __float2half_rn(v);
    int64_t o = (int64_t)(2 * j + (r & 1)) * KR + kr;
    Bhi[o] = h;
    Blo[o] = __float2half_rn(v - __half2float(h));
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

// 2D tensor (rows x KR) of fp32 or fp16, box (one 128-byte row x box_rows), 128-byte swizzle
static bool make_map(CUtensorMap* map, void* base, int64_t rows, int box_rows, bool f16) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  const int elem = f16 ? 2 : 4;
  cuuint64_t dims[2] = {(cuuint64_t)KR, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)KR * elem};
  cuuint32_t box[2] = {(cuuint32_t)(128 / elem), (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  return fn(map, f16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims, strides, box,
            estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace tc

// rows of the B split buffers for order n: 2n plus one tile of zero padding
static int64_t b_rows(int64_t n) { return 2 * n + tc::BN; }

size_t tc_scratch_bytes(int64_t n) {
  // Ahi, Alo: n x KR; Bhi, Blo: (2n + BN) x KR (fp32 -- the larger mode), inverse scales, alignment
  return (size_t)(2 * n + 2 * b_rows(n)) * tc::KR * sizeof(float) + (size_t)(n + b_rows(n)) * sizeof(float) + 4096;
}

bool tc_available() { return tc::encode_fn() != nullptr; }

static std::atomic<int> g_tc_mode{MGT_TC_F16X2};

int tc_set_mode(int mode) {
  if (mode != MGT_TC_TF32X3 && mode != MGT_TC_F16X2) return MGT_ERR_ARG;
  g_tc_mode.store(mode);
  return MGT_OK;
}
int tc_get_mode() { return g_tc_mode.load(); }

// Scratch: Ahi, Alo (nmax rows), Bhi, Blo (b_rows rows), KR elements a row
// (fp32, or fp16 in F16 mode), then (F16) invA[nmax], invB[b_rows / 2].
int TcPlan::init(void* scratch, int64_t nmax) {
  mode = g_tc_mode.load();
  const bool f16 = mode == MGT_TC_F16X2;
  const size_t elem = f16 ? 2 : 4;
  char* b = (char*)(((uintptr_t)scratch + 1023) & ~(uintptr_t)1023);
  Ahi = b;
  Alo = b + (size_t)nmax * tc::KR * elem;
  Bhi = (char*)Alo + (size_t)nmax * tc::KR * elem;
  Blo = (char*)Bhi + (size_t)b_rows(nmax) * tc::KR * elem;
  invA = (float*)((char*)Blo + (size_t)b_rows(nmax) * tc::KR * elem);
  invB = invA + nmax;
  this->nmax = nmax;
  bool ok = tc::make_map(&mAhi, Ahi, nmax, tc::BM, f16) && tc::make_map(&mAlo, Alo, nmax, tc::BM, f16) &&
            tc::make_map(&mBhi, Bhi, b_rows(nmax), tc::BN, f16) && tc::make_map(&mBlo, Blo, b_rows(nmax), tc::BN, f16);
  return ok ? MGT_OK : MGT_ERR_CUDA;
}

int tc_make_cmap(CUtensorMap* map, float2* C, int64_t rows, int64_t cols, int64_t ldc) {
  tc::EncodeTiledFn fn = tc::encode_fn();
  if (!fn) return MGT_ERR_UNSUPPORTED;
  if (((uintptr_t)C & 15) != 0 || (ldc & 1) != 0) return MGT_ERR_ARG;
  cuuint64_t dims[2] = {(cuuint64_t)(2 * cols), (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)ldc * 8};
  cuuint32_t box[2] = {32, (cuuint32_t)tc::BM};
  cuuint32_t estr[2] = {1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)C, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS
             ? MGT_OK
             : MGT_ERR_CUDA;
}

static int tc_num_sms() { return device_sm_count(); }

static void tc_init_attrs() {
  static OncePerDevice once;
  once([] {
    cudaFuncSetAttribute(tc::cgemm_split3_kernel<false, 2, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)tc::smem_bytes<2, 2>());
    cudaFuncSetAttribute(tc::cgemm_split3_kernel<true, 2, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)tc::smem_bytes<2, 2>());
  });
}

static int tc_kcols(const TcPlan& plan, int K) {
  const int bk = plan.mode == MGT_TC_F16X2 ? tc::Mode<true>::BK : tc::Mode<false>::BK;
  return ((2 * K + bk - 1) / bk) * bk;
}

int tc_split_a(const TcPlan& plan, int M, int K, const float2* A, int64_t lda, cudaStream_t s) {
  if (M <= 0 || K <= 0) return MGT_OK;
  if (K > tc::KMAX || M > plan.nmax) return MGT_ERR_UNSUPPORTED;
  const int kcols = tc_kcols(plan, K);
  count_launch();
  if (plan.mode == MGT_TC_F16X2) {
    tc::split_a_f16_kernel<<<(M + 7) / 8, 256, 0, s>>>(A, lda, M, K, kcols, (__half*)plan.Ahi, (__half*)plan.Alo,
                                                       plan.invA);
  } else {
    int64_t na = (int64_t)M * kcols;
    tc::split_a_kernel<<<(unsigned)((na + 255) / 256), 256, 0, s>>>(A, lda, M, K, kcols, (float*)plan.Ahi,
                                                                   (float*)plan.Alo);
  }
  return cudaGetLastError() == cudaSuccess ? MGT_OK : MGT_ERR_CUDA;
}

int tc_split_b(const TcPlan& plan, int N, int K, const float2* B, int64_t ldb, cudaStream_t s) {
  if (N <= 0 || K <= 0) return MGT_OK;
  if (K > tc::KMAX || N > plan.nmax) return MGT_ERR_UNSUPPORTED;
  const int kcols = tc_kcols(plan, K);
  // cover every column of the last tile (2N rounded up to BN reals)
  const int bgrid = (int)((((2 * (int64_t)N + tc::BN - 1) / tc::BN) * tc::BN / 2 + tc::SB_COLS - 1) / tc::SB_COLS);
  count_launch();
  if (plan.mode == MGT_TC_F16X2)
    tc::split_b_f16_kernel<<<bgrid, 256, 0, s>>>(B, ldb, K, N, kcols, (__half*)plan.Bhi, (__half*)plan.Blo,
                                                 plan.invB);
  else
    tc::split_b_kernel<<<bgrid, 256, 0, s>>>(B, ldb, K, N, kcols, (float*)plan.Bhi, (float*)plan.Blo);
  return cudaGetLastError() == cudaSuccess ? MGT_OK : MGT_ERR_CUDA;
}

int tc_gemm(const TcPlan& plan, const CUtensorMap& cmap, int M, int N, int K, int cx0, int cy0, int* status,
            cudaStream_t s, int max_ctas, int bcol) {
  if (M <= 0 || N <= 0 || K <= 0) return MGT_OK;
  if (K > tc::KMAX || M > plan.nmax || bcol < 0 || (int64_t)bcol + N > plan.nmax) return MGT_ERR_UNSUPPORTED;
  tc_init_attrs();
  const int kblocks = tc_kcols(plan, K) / (plan.mode == MGT_TC_F16X2 ? tc::Mode<true>::BK : tc::Mode<false>::BK);
  const int tiles_n = (2 * N + tc::BN - 1) / tc::BN, tiles_m = (M + tc::BM - 1) / tc::BM;
  const int total = tiles_n * tiles_m;
  int ctas = std::min(total, max_ctas > 0 ? max_ctas : tc_num_sms());
  count_launch();
#define MGT_TC_LAUNCH(F16, ST, CS)                                                                              \
  tc::cgemm_split3_kernel<F16, ST, CS><<<ctas, tc::THREADS, tc::smem_bytes<ST, CS>(), s>>>(                    \
      plan.mAhi, plan.mAlo, plan.mBhi, plan.mBlo, cmap, cx0, cy0, 2 * bcol, tiles_n, total, kblocks, plan.invA,    \
      plan.invB, status)
  if (plan.mode == MGT_TC_F16X2)
    MGT_TC_LAUNCH(true, 2, 2);
  else
    MGT_TC_LAUNCH(false, 2, 2);
#undef MGT_TC_LAUNCH
  return cudaGetLastError() == cudaSuccess ? MGT_OK : MGT_ERR_CUDA;
}

int gemm_sub_tc(const TcPlan& plan, const CUtensorMap& cmap, int M, int N, int K, const float2* A, int64_t lda,
                const float2* B, int64_t ldb, int cx0, int cy0, int* status, cudaStream_t s, int max_ctas) {
  if (M <= 0 || N <= 0 || K <= 0) return MGT_OK;
  if (K > tc::KMAX || M > plan.nmax || N > plan.nmax) return MGT_ERR_UNSUPPORTED;
  int e = tc_split_a(plan, M, K, A, lda, s);
  if (e == MGT_OK) e = tc_split_b(plan, N, K, B, ldb, s);
  if (e == MGT_OK) e = tc_gemm(plan, cmap, M, N, K, cx0, cy0, status, s, max_ctas);
  return e;
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
  if (K > tc::KMAX) return MGT_ERR_UNSUPPORTED;
  int64_t nmax = std::max(M, N);
  if (!work || work_bytes < tc_scratch_bytes(nmax) + 256) return MGT_ERR_WORKSPACE;
  if (!tc_available()) return MGT_ERR_UNSUPPORTED;
  int* status = (int*)work;
  TcPlan plan;
  int e = plan.init((char*)work + 256, nmax);
  if (e != MGT_OK) return e;
  CUtensorMap cmap;
  e = tc_make_cmap(&cmap, (float2*)C, M, N, ldc);
  if (e != MGT_OK) return e;
  return gemm_sub_tc(plan, cmap, (int)M, (int)N, (int)K, (const float2*)A, lda, (const float2*)B, ldb, 0, 0, status, s,
                     0);
}
