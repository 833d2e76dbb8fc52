// Tensor-core residual R = B - M X for iterative refinement: M in
// double-float form (MGT_CDF), X, B, R complex128.
//
// Method: an error-free splitting of both operands into small integers
// ("digits") that FP16 holds exactly, multiplied on the tensor cores with
// FP32 accumulation kept exact -- the Ozaki scheme (Ozaki, Ogita, Oishi and
// Rump, "Error-free transformations of matrix multiplication by using fast
// routines of matrix multiplication and its applications", Numer.
// Algorithms 2012), in its FP16 tensor-core form (Mukunoki, Ozaki, Ogita and
// Imamura, "DGEMM using Tensor Cores, and Its Accurate and Reproducible
// Versions", ISC 2020).
//  * The complex product is the real product A' B' of A' (rows x 2 kdim,
//    row i = Mr_i0, Mi_i0, Mr_i1, Mi_i1, ...) and B'^T (2 nrhs x 2 kdim: row
//    2j = Xr_0j, -Xi_0j, ...; row 2j+1 = Xi_0j, Xr_0j, ...).
//  * Row i of A' is scaled by 2^-e_i, 2^e_i bounding the row's largest
//    |re|, |im|, and every entry becomes the integer
//    X = round((hi + lo) 2^(54 - e_i)), |X| < 2^54, written with seven
//    balanced base-256 digits X = sum_{p=0..6} d_p 256^p: the bytes of
//    X + 128 (256^0 + ... + 256^6) minus 128, so d_0 .. d_5 lie in
//    [-128, 127] and the top digit d_6 in [-64, 64].  The columns of B' are
//    scaled by their own power of two the same way.
//  * A digit needs at most 8 bits and is exact in FP16; a product of two is
//    at most 2^14.  Counting digits from the top (s = 6 - p), the pairs
//    (s, t) with s + t = l share the weight 256^-l and accumulate in one
//    TMEM accumulator per level l = 0 .. 6; pairs with s + t > 6 lie below
//    2^-55 of the row and column scales and are not formed.  A level
//    receives at most 7 pairs x 128 products (6 * 2^21 < 2^24 with the
//    smaller top digits) before it is read out, so its FP32 sum is an exact
//    integer.
//  * Every 128 real K the level sums are read out of TMEM and folded into
//    one 64-bit integer per output in units of 2^-48 of the row and column
//    scales: levels 0 .. 4 exactly, 5 and 6 rounded to the nearest unit.  A
//    64-bit accumulator per output in shared memory sums them exactly (at
//    most 2^15 real K per CTA keeps it below 2^63); the result is scaled back
//    once at the end.
// Accuracy (a numpy emulation of exactly this scheme on 2D / 3D systems of
// order 1400 / 2100): residual errors of 3e-14 / 1e-14 of ||B||, where six
// digits give 8e-12 / 2e-12.
//
// Kernel: one CTA per (128 rows) x (32 complex right-hand sides) x (a range
// of K in 32-column chunks), 512 threads:
//   warp 0     : bulk copies of the right-hand sides' digit blocks (made by
//                bdigits_kernel in the layout shared memory needs), 2 stages
//   warp 1     : MMA issuer.  Per chunk and digit s of A', one MMA per
//                16-wide K step covers the levels s .. 6 at once: the seven
//                digit slices of B' are stacked along N, so the levels s + t,
//                t = 0 .. 6 - s, are adjacent TMEM columns (N <= 256 per MMA:
//                10 MMAs per K step instead of 28, A read once per MMA)
//   warp 2     : TMEM allocation (7 levels x 64 columns)
//   warps 4-7  : epilogue, thread = row: level sums -> 64-bit accumulators
//   warps 8-23 : converters, eight rows each: the double-float entries of M
//                are loaded for a whole chunk at once, turned into 54-bit
//                integers, and their digits (one byte permute, one logic op
//                and one fp16 subtract per re / im pair) written straight
//                into the 128-byte-swizzled K-major layout of the MMA's A
//                operand, one digit slice at a time through a ring
// Every wait is bounded; a CTA whose wait runs out writes NaN outputs, sets
// MGT_ERR_TIMEOUT in the status word, drains what it issued and returns.
#include <cuda_fp16.h>

#include <algorithm>

#include "common.cuh"
#include "diag.cuh"
#include "gemm_tc.cuh"
#include "residual_tc.cuh"
#include "tcgen05.cuh"

namespace mgt {
namespace rtc {

constexpr int BM = 128;                 // rows of M per tile
constexpr int BNC = 32;                 // complex right-hand sides per tile
constexpr int BN = 2 * BNC;             // real columns per tile (TMEM columns per level)
constexpr int KCC = 32;                 // complex K per chunk (64 real: one 128-byte fp16 row)
constexpr int DIG = 7;                  // digits per operand
constexpr int ASLOTS = 3;               // A digit-slice ring
constexpr uint32_t A_SLICE = BM * 128;              // 16 KB
constexpr uint32_t B_SLICE = BN * 128;              // 8 KB
constexpr uint32_t B_BLOCK = DIG * B_SLICE;         // 56 KB: one chunk of B', all digit slices
constexpr uint32_t W_BYTES = BM * BN * 8;           // 64-bit accumulators
constexpr uint32_t TMEM_COLS = 512;
constexpr int NCONV = 16, NEPI = 4;
constexpr int THREADS = (4 + NEPI + NCONV) * 32;
constexpr int ROWS_PER_CONV = BM / NCONV;           // 8
// at most 512 chunks (32768 real K) per CTA: |sum| <= 2^15 * 2^48 = 2^63
// units of 2^-48, less the rounding of levels 5 and 6
constexpr int MAX_SPLIT_CHUNKS = 512;
constexpr long long BIAS = 0x0080808080808080LL;    // 128 in each of the seven digit positions
constexpr int FIX = 54;                             // |X| < 2^FIX

constexpr size_t smem_bytes() { return 1024 + ASLOTS * A_SLICE + 2 * B_BLOCK + W_BYTES + BM * sizeof(int) + 256; }

// round(f * 2^sh) as a 64-bit integer (|f| * 2^sh < 2^54 by the row scale);
// zero and subnormal f (below 2^-126) give 0
__device__ __forceinline__ long long fixed_point(float f, int sh) {
  const uint32_t u = __float_as_uint(f);
  const int ex = (int)((u >> 23) & 0xFFu);
  if (ex == 0) return 0;
  const uint32_t m = (u & 0x7FFFFFu) | 0x800000u;   // |f| = m * 2^(ex - 150)
  const int s = ex - 150 + sh;
  long long r;
  if (s >= 0) r = (long long)m << min(s, 39);
  else if (s > -32) r = (long long)((m + (1u << (-s - 1))) >> (-s));
  else r = 0;
  return (u >> 31) ? -r : r;
}

// round(f * 2^sh) for the low part of a double-float entry (|f| * 2^sh < 2^30):
// one exact power-of-two multiply and one conversion
__device__ __forceinline__ long long fixed_low(float f, int sh) {
  if (sh > 127 || sh < -126) return fixed_point(f, sh);
  return (long long)__float2int_rn(f * __int_as_float((127 + sh) << 23));
}

// Digit at position p (0 = lowest) of y = X + BIAS, as an exact float.
__device__ __forceinline__ float digit_f(long long y, int p) {
  const uint32_t lo = (uint32_t)y, hi = (uint32_t)((unsigned long long)y >> 32);
  const uint32_t w = p < 4 ? lo : hi;
  const uint32_t byte = (w >> (8 * (p & 3))) & 255u;
  return __int_as_float(0x4B400000 | (int)byte) - 12583040.0f;   // byte - 128
}

// fp16 pair (digit P of yr, digit P of yi) as one 32-bit word: the two bytes
// are picked by one byte permute, turned into the fp16 encodings of
// 1024 + byte, and 1152 is subtracted (byte - 128, exact)
template <int P>
__device__ __forceinline__ uint32_t digit_pair(long long yr, long long yi) {
  const uint32_t wr = P < 4 ? (uint32_t)yr : (uint32_t)((unsigned long long)yr >> 32);
  const uint32_t wi = P < 4 ? (uint32_t)yi : (uint32_t)((unsigned long long)yi >> 32);
  constexpr uint32_t b = P & 3;
  const uint32_t x = __byte_perm(wr, wi, b | (b << 4) | ((4 + b) << 8) | ((4 + b) << 12));
  const uint32_t h = (x & 0x00FF00FFu) | 0x64006400u;
  const __half2 c = __halves2half2(__ushort_as_half((unsigned short)0x6480), __ushort_as_half((unsigned short)0x6480));
  const __half2 d = __hsub2(*reinterpret_cast<const __half2*>(&h), c);
  return *reinterpret_cast<const uint32_t*>(&d);
}

// one digit slice of a converter warp's rows: row cw + NCONV t, lane = complex column
template <int P>
__device__ __forceinline__ void conv_pass(unsigned char* tile, const long long (&yr)[ROWS_PER_CONV],
                                          const long long (&yi)[ROWS_PER_CONV], int cw, int lane);

// row exponent of a row holding a NaN or an infinity: its outputs are NaN
constexpr int kRowNonFinite = 0x40000000;

__device__ __forceinline__ int clamp_exp(int e) { return (e < -300 || e > 300) ? 0 : e; }

// Byte offset of real K index kr (even) of row rho in a 128-row tile whose rows
// are 128-byte lines (64 fp16), 8-row groups 1024 B apart, 16-byte chunks
// XOR-swizzled by the row within its group: the K-major 128B-swizzle layout.
__device__ __forceinline__ uint32_t swz(int rho, int kr) {
  return (uint32_t)rho * 128u + ((uint32_t)(((kr >> 3) ^ (rho & 7)) << 4)) + (uint32_t)((kr & 7) * 2);
}

template <int P>
__device__ __forceinline__ void conv_pass(unsigned char* tile, const long long (&yr)[ROWS_PER_CONV],
                                          const long long (&yi)[ROWS_PER_CONV], int cw, int lane) {
#pragma unroll
  for (int t = 0; t < ROWS_PER_CONV; ++t)
    *reinterpret_cast<uint32_t*>(tile + swz(cw + NCONV * t, 2 * lane)) = digit_pair<P>(yr[t], yi[t]);
}

__global__ void __launch_bounds__(THREADS, 1)
residual_tc_kernel(const float4* __restrict__ M, int64_t ldm, int rows, int kdim, const int* __restrict__ row_exp,
                   const int* __restrict__ col_exp, const unsigned char* __restrict__ bdig, int nch_total, int ncols,
                   int chunks_per_split, const double2* __restrict__ B, int64_t ldb, double2* __restrict__ R,
                   int64_t ldr, double2* __restrict__ partial, int* status) {
  using namespace tc;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  unsigned char* aring = base;
  unsigned char* bring = aring + ASLOTS * A_SLICE;
  long long* wacc = reinterpret_cast<long long*>(bring + 2 * B_BLOCK);   // [BN][BM]
  int* rexp = reinterpret_cast<int*>(reinterpret_cast<unsigned char*>(wacc) + W_BYTES);
  uint64_t* full_a = reinterpret_cast<uint64_t*>(rexp + BM);
  uint64_t* empty_a = full_a + ASLOTS;
  uint64_t* full_b = empty_a + ASLOTS;
  uint64_t* empty_b = full_b + 2;
  uint64_t* tfull = empty_b + 2;
  uint64_t* tempty = tfull + 1;
  uint64_t* done = tempty + 1;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  volatile int* abort = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row0 = blockIdx.x * BM, ct = blockIdx.y, sp = blockIdx.z;
  const int c_begin = sp * chunks_per_split;
  const int nchunk = max(0, min(nch_total, c_begin + chunks_per_split) - c_begin);
  const int nread = (nchunk + 1) >> 1;

  if (threadIdx.x < BM) rexp[threadIdx.x] = (row0 + (int)threadIdx.x < rows) ? clamp_exp(row_exp[row0 + threadIdx.x]) : 0;
  if (threadIdx.x == 0) {
    for (int s = 0; s < ASLOTS; ++s) { mbar_init(&full_a[s], NCONV); mbar_init(&empty_a[s], 1); }
    for (int s = 0; s < 2; ++s) { mbar_init(&full_b[s], 1); mbar_init(&empty_b[s], 1); }
    mbar_init(tfull, 1);
    mbar_init(tempty, NEPI);
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

  if (warp == 0 && lane == 0) {
    // ---------------- producer: digit blocks of B' for each chunk
    int i = 0;
    for (; i < nchunk && !*abort; ++i) {
      const int st = i & 1;
      if (i >= 2 && !mbar_wait(&empty_b[st], ((i >> 1) - 1) & 1, abort)) break;
      mbar_expect_tx(&full_b[st], B_BLOCK);
      bulk_load(bring + st * B_BLOCK, bdig + ((size_t)ct * nch_total + c_begin + i) * B_BLOCK, B_BLOCK, &full_b[st]);
    }
    // copies in flight land before the CTA may exit
    for (int j = max(0, i - 2); j < i; ++j) mbar_wait_plain(&full_b[j & 1], (j >> 1) & 1);
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer
    int q = 0;
    bool ok = true;
    for (int i = 0; i < nchunk && ok; ++i) {
      const bool first = (i & 1) == 0;
      if (first && i >= 2) {
        if (!mbar_wait(tempty, ((i >> 1) - 1) & 1, abort)) { ok = false; break; }
        tc_fence_after();
      }
      const int st = i & 1;
      if (!mbar_wait(&full_b[st], (i >> 1) & 1, abort)) { ok = false; break; }
      tc_fence_after();
      const uint32_t bb = smem_u32(bring + st * B_BLOCK);
      for (int s = 0; s < DIG; ++s, ++q) {
        const int slot = q % ASLOTS;
        if (!mbar_wait(&full_a[slot], (q / ASLOTS) & 1, abort)) { ok = false; break; }
        tc_fence_after();
        const uint64_t ad = kmajor_sw128_desc(smem_u32(aring + slot * A_SLICE));
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {
          const uint32_t acc = (first && s == 0 && ks == 0) ? 0u : 1u;
          for (int t0 = 0; t0 < DIG - s; t0 += 4) {
            const int nt = min(4, DIG - s - t0);
            const uint64_t bd = kmajor_sw128_desc(bb + (uint32_t)t0 * B_SLICE);
            mma_f16(tmem + (uint32_t)((s + t0) * BN), ad + (uint64_t)(2 * ks), bd + (uint64_t)(2 * ks),
                    idesc_f16_m128(nt * BN), acc);
          }
        }
        mma_commit(&empty_a[slot]);
      }
      if (!ok) break;
      mma_commit(&empty_b[st]);
      if (!first || i == nchunk - 1) mma_commit(tfull);
    }
    mma_commit(done);   // arrives once every MMA issued above has completed
  } else if (warp >= 4 && warp < 4 + NEPI) {
    // ---------------- epilogue: thread = row of the tile
    const int qd = warp - 4, r = qd * 32 + lane;
    for (int j = 0; j < BN; ++j) wacc[j * BM + r] = 0;
    const uint32_t tbase = tmem + ((uint32_t)(qd * 32) << 16);
    bool ok = true;
    for (int ro = 0; ro < nread; ++ro) {
      if (!mbar_wait(tfull, ro & 1, abort)) { ok = false; break; }
      tc_fence_after();
#pragma unroll 1
      for (int p = 0; p < BN / 8; ++p) {
        uint32_t v[DIG][8];
#pragma unroll
        for (int l = 0; l < DIG; ++l) tmem_ld8(tbase + (uint32_t)(l * BN + p * 8), v[l]);
        tmem_wait_ld();
        if (p == BN / 8 - 1) {
          tc_fence_before();
          __syncwarp();
          if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(tempty)) : "memory");
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          // level l weighs 2^(36 - 8 l) units of 2^-48
          const long long low = ((long long)__float2int_rz(__uint_as_float(v[5][j])) << 8) +
                                (long long)__float2int_rz(__uint_as_float(v[6][j]));
          const long long w = ((long long)__float2int_rz(__uint_as_float(v[0][j])) << 36) +
                              ((long long)__float2int_rz(__uint_as_float(v[1][j])) << 28) +
                              ((long long)__float2int_rz(__uint_as_float(v[2][j])) << 20) +
                              ((long long)__float2int_rz(__uint_as_float(v[3][j])) << 12) +
                              ((long long)__float2int_rz(__uint_as_float(v[4][j])) << 4) + ((low + 2048) >> 12);
          wacc[(p * 8 + j) * BM + r] += w;
        }
      }
    }
    const int row = row0 + r;
    if (row < rows) {
      const bool good = ok && !*abort && row_exp[row] != kRowNonFinite;
      const int ea = rexp[r];
      for (int jc = 0; jc < BNC; ++jc) {
        const int col = ct * BNC + jc;
        if (col >= ncols) break;
        double2 val;
        if (good) {
          const int sc = ea + clamp_exp(col_exp[col]) - 48;
          val = make_double2(ldexp((double)wacc[(2 * jc) * BM + r], sc), ldexp((double)wacc[(2 * jc + 1) * BM + r], sc));
        } else {
          val = make_double2(__longlong_as_double(0x7FF8000000000000LL), __longlong_as_double(0x7FF8000000000000LL));
        }
        if (partial) {
          partial[((int64_t)sp * rows + row) * ncols + col] = val;
        } else {
          const double2 b = B ? B[(int64_t)row * ldb + col] : make_double2(0.0, 0.0);
          R[(int64_t)row * ldr + col] = make_double2(b.x - val.x, b.y - val.y);
        }
      }
    }
  } else if (warp >= 4 + NEPI) {
    // ---------------- converters: rows cw, cw + NCONV, ...; lane = complex column of the chunk
    const int cw = warp - 4 - NEPI;
    int q = 0;
    float4 v[ROWS_PER_CONV];
    auto load_chunk = [&](int i) {
      const int kc = (c_begin + i) * KCC + lane;
#pragma unroll
      for (int t = 0; t < ROWS_PER_CONV; ++t) {
        const int row = row0 + cw + NCONV * t;
        v[t] = (i < nchunk && row < rows && kc < kdim) ? __ldg(&M[(int64_t)row * ldm + kc])
                                                       : make_float4(0.f, 0.f, 0.f, 0.f);
      }
    };
    load_chunk(0);
    for (int i = 0; i < nchunk && !*abort; ++i) {
      long long yr[ROWS_PER_CONV], yi[ROWS_PER_CONV];
#pragma unroll
      for (int t = 0; t < ROWS_PER_CONV; ++t) {
        const int sh = FIX - rexp[cw + NCONV * t];
        yr[t] = fixed_point(v[t].x, sh) + fixed_low(v[t].y, sh) + BIAS;
        yi[t] = fixed_point(v[t].z, sh) + fixed_low(v[t].w, sh) + BIAS;
      }
      bool ok = true;
#pragma unroll
      for (int s = 0; s < DIG; ++s) {
        const int slot = (q + s) % ASLOTS;
        if (ok && q + s >= ASLOTS && !mbar_wait(&empty_a[slot], (((q + s) / ASLOTS) - 1) & 1, abort)) ok = false;
        if (ok) {
          unsigned char* tile = aring + slot * A_SLICE;
          switch (DIG - 1 - s) {
            case 0: conv_pass<0>(tile, yr, yi, cw, lane); break;
            case 1: conv_pass<1>(tile, yr, yi, cw, lane); break;
            case 2: conv_pass<2>(tile, yr, yi, cw, lane); break;
            case 3: conv_pass<3>(tile, yr, yi, cw, lane); break;
            case 4: conv_pass<4>(tile, yr, yi, cw, lane); break;
            case 5: conv_pass<5>(tile, yr, yi, cw, lane); break;
            default: conv_pass<6>(tile, yr, yi, cw, lane); break;
          }
          fence_async_smem();
          __syncwarp();
          if (lane == 0)
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&full_a[slot])) : "memory");
        }
        // the top three digits come from the high words, which are dead now:
        // the next chunk's entries load during the other four passes
        if (s == 2) load_chunk(i + 1);
      }
      q += DIG;
      if (!ok) break;
    }
  }
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x == 0 && *abort) atomicExch(status, MGT_ERR_TIMEOUT);
  if (warp == 2) {
    // every issued MMA has completed before the accumulator columns are freed
    if (lane == 0) mbar_wait_plain(done, 0);
    __syncwarp();
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

// e_i of each row: 2^e_i bounds the row's largest |re|, |im| (hi parts); one
// warp per row.  Rows with a NaN or an infinity get kRowNonFinite.
__global__ void rowexp_kernel(const float4* __restrict__ M, int64_t ldm, int rows, int kdim, int* __restrict__ out) {
  const int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (row >= rows) return;
  uint32_t m = 0;
  for (int k = lane; k < kdim; k += 32) {
    const float4 v = __ldg(&M[(int64_t)row * ldm + k]);
    m = max(m, max(__float_as_uint(fabsf(v.x)), __float_as_uint(fabsf(v.z))));
  }
  m = __reduce_max_sync(0xffffffffu, m);
  int e = 0;
  if (m >= 0x7F800000u) e = kRowNonFinite;
  else if (m != 0u) frexpf(__uint_as_float(m), &e);
  if (lane == 0) out[row] = e;
}

// f_j of each right-hand side: 2^f_j bounds the column's largest |re|, |im|.
// Block (32 columns x 8 row lanes) over a range of rows; atomicMax per column
// (the output starts at a large negative value).
__global__ void colexp_kernel(const double2* __restrict__ X, int64_t ldx, int kdim, int ncols, int* __restrict__ out) {
  const int j = blockIdx.x * 32 + (threadIdx.x & 31), ty = threadIdx.x >> 5;
  __shared__ double red[8][32];
  double m = 0.0;
  if (j < ncols)
    for (int k = blockIdx.y * 8 + ty; k < kdim; k += gridDim.y * 8) {
      const double2 x = X[(int64_t)k * ldx + j];
      m = fmax(m, fmax(fabs(x.x), fabs(x.y)));
    }
  red[ty][threadIdx.x & 31] = m;
  __syncthreads();
  if (ty == 0 && j < ncols) {
    for (int t = 1; t < 8; ++t) m = fmax(m, red[t][threadIdx.x & 31]);
    if (m > 0.0) {
      int e = 0;
      frexp(m, &e);
      atomicMax(&out[j], e);
    }
  }
}

// Digit blocks of B'^T: block (column tile ct, chunk c) holds the seven digit
// slices (top digit first) of its 64 rows x 64 real K, each slice in the
// swizzled layout the MMA reads; zeros beyond kdim and ncols.  One thread per
// (complex K index, complex column).
__global__ void bdigits_kernel(const double2* __restrict__ X, int64_t ldx, int kdim, int ncols,
                               const int* __restrict__ col_exp, unsigned char* __restrict__ out, int nch, int ctiles) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int cols = ctiles * BNC;
  if (idx >= (int64_t)nch * KCC * cols) return;
  const int j = (int)(idx % cols), k = (int)(idx / cols);
  double2 x = make_double2(0.0, 0.0);
  int e = 0;
  if (j < ncols) {
    e = clamp_exp(col_exp[j]);
    if (k < kdim) x = X[(int64_t)k * ldx + j];
  }
  const long long xr = __double2ll_rn(ldexp(x.x, FIX - e)), xi = __double2ll_rn(ldexp(x.y, FIX - e));
  const long long yr = xr + BIAS, yi = xi + BIAS, yn = BIAS - xi;
  const int ctile = j / BNC, jj = j % BNC, c = k / KCC, kk = k % KCC;
  unsigned char* blk = out + ((size_t)ctile * nch + c) * B_BLOCK;
#pragma unroll
  for (int s = 0; s < DIG; ++s) {
    const int p = DIG - 1 - s;
    const int rho = s * BN + 2 * jj;
    // row 2jj (real part): Xr, -Xi; row 2jj + 1 (imaginary part): Xi, Xr
    *reinterpret_cast<__half2*>(blk + swz(rho, 2 * kk)) = __floats2half2_rn(digit_f(yr, p), digit_f(yn, p));
    *reinterpret_cast<__half2*>(blk + swz(rho + 1, 2 * kk)) = __floats2half2_rn(digit_f(yi, p), digit_f(yr, p));
  }
}

// R = B - sum of the split-K partials (FP64); partial is [split][row][col]
__global__ void tc_reduce_kernel(const double2* __restrict__ partial, int splits, int rows, int ncols,
                                 const double2* __restrict__ B, int64_t ldb, double2* __restrict__ R, int64_t ldr) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)rows * ncols) return;
  const int r = (int)(idx / ncols), c = (int)(idx - (int64_t)r * ncols);
  double2 acc = B ? B[(int64_t)r * ldb + c] : make_double2(0.0, 0.0);
  for (int q = 0; q < splits; ++q) {
    const double2 v = partial[(int64_t)q * rows * ncols + idx];
    acc.x -= v.x;
    acc.y -= v.y;
  }
  R[(int64_t)r * ldr + c] = acc;
}

// Split of the K range: about four waves of CTAs, at least 8 chunks (4
// readouts) per split, at most 16 splits and MAX_SPLIT_CHUNKS chunks each,
// an even number of chunks per split (whole readouts).
static void plan_splits(int rows, int kdim, int ncols, int* splits, int* cps) {
  const int nch = (kdim + KCC - 1) / KCC;
  const int tiles = ((rows + BM - 1) / BM) * ((ncols + BNC - 1) / BNC);
  const int sms = device_sm_count();
  const int want = (4 * sms + tiles - 1) / tiles;
  int sp = std::max(1, std::min(want, std::min(16, nch / 8)));
  sp = std::max(sp, (nch + MAX_SPLIT_CHUNKS - 1) / MAX_SPLIT_CHUNKS);
  int c = (nch + sp - 1) / sp;
  if ((c & 1) && c < nch) ++c;
  *cps = c;
  *splits = (nch + c - 1) / c;
}

struct TcResWs {
  int* status;
  int* rowexp;
  int* colexp;
  unsigned char* bdig;
  double2* partial;
  int splits, cps, nch, ctiles;
  size_t total;
  TcResWs(void* base, int rows, int kdim, int ncols) {
    char* b = (char*)base;
    size_t off = 0;
    auto take = [&](size_t bytes, size_t align) {
      off = (off + align - 1) / align * align;
      char* p = b ? b + off : nullptr;
      off += bytes;
      return p;
    };
    plan_splits(rows, kdim, ncols, &splits, &cps);
    nch = (kdim + KCC - 1) / KCC;
    ctiles = (ncols + BNC - 1) / BNC;
    status = (int*)take(256, 256);
    rowexp = (int*)take((size_t)rows * sizeof(int), 256);
    colexp = (int*)take((size_t)ncols * sizeof(int), 256);
    bdig = (unsigned char*)take((size_t)ctiles * nch * B_BLOCK, 1024);
    partial = splits > 1 ? (double2*)take((size_t)splits * rows * ncols * sizeof(double2), 256) : nullptr;
    total = off + 256;
  }
};

}  // namespace rtc

bool residual_tc_supported(int64_t rows, int64_t kdim, int64_t ncols) {
  return tc_available() && rows > 0 && kdim > 0 && ncols > 0 && rows <= (1 << 24) && kdim <= (1 << 22) &&
         ncols <= (1 << 16);
}

size_t residual_tc_workspace_bytes(int64_t rows, int64_t kdim, int64_t ncols) {
  if (!residual_tc_supported(rows, kdim, ncols)) return 0;
  return rtc::TcResWs(nullptr, (int)rows, (int)kdim, (int)ncols).total;
}

int residual_tc_rowexp(const float4* M, int64_t ldm, int rows, int kdim, int* out, cudaStream_t s) {
  count_launch();
  rtc::rowexp_kernel<<<(rows + 7) / 8, 256, 0, s>>>(M, ldm, rows, kdim, out);
  return cudaGetLastError() == cudaSuccess ? MGT_OK : MGT_ERR_CUDA;
}

int residual_tc(const float4* M, int64_t ldm, int rows, int kdim, const double2* X, int64_t ldx, int ncols,
                const double2* B, int64_t ldb, double2* R, int64_t ldr, const int* rowexp, void* work,
                size_t work_bytes, cudaStream_t s) {
  using namespace rtc;
  if (!residual_tc_supported(rows, kdim, ncols)) return MGT_ERR_UNSUPPORTED;
  TcResWs w(work, rows, kdim, ncols);
  if (!work || work_bytes < w.total) return MGT_ERR_WORKSPACE;
  static OncePerDevice once;
  once([] {
    cudaFuncSetAttribute(residual_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes());
  });
  if (cudaMemsetAsync(w.status, 0, sizeof(int), s) != cudaSuccess) return MGT_ERR_CUDA;
  if (!rowexp) {
    int e = residual_tc_rowexp(M, ldm, rows, kdim, w.rowexp, s);
    if (e != MGT_OK) return e;
    rowexp = w.rowexp;
  }
  // column exponents start far below any real one (0x80808080)
  if (cudaMemsetAsync(w.colexp, 0x80, (size_t)ncols * sizeof(int), s) != cudaSuccess) return MGT_ERR_CUDA;
  count_launch(2);
  colexp_kernel<<<dim3((ncols + 31) / 32, std::min(64, (kdim + 7) / 8)), 256, 0, s>>>(X, ldx, kdim, ncols, w.colexp);
  const int64_t nb = (int64_t)w.nch * KCC * w.ctiles * BNC;
  bdigits_kernel<<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(X, ldx, kdim, ncols, w.colexp, w.bdig, w.nch, w.ctiles);
  count_launch();
  dim3 grid((rows + BM - 1) / BM, w.ctiles, w.splits);
  residual_tc_kernel<<<grid, THREADS, smem_bytes(), s>>>(M, ldm, rows, kdim, rowexp, w.colexp, w.bdig, w.nch, ncols,
                                                           w.cps, B, ldb, R, ldr, w.partial, w.status);
  if (w.splits > 1) {
    const int64_t tot = (int64_t)rows * ncols;
    count_launch();
    tc_reduce_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(w.partial, w.splits, rows, ncols, B, ldb, R, ldr);
  }
  return cudaGetLastError() == cudaSuccess ? MGT_OK : MGT_ERR_CUDA;
}

}  // namespace mgt
