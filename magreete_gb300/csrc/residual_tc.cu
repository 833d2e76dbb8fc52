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
//    scales: levels 0 .. 4 exactly, 5 and 6 rounded to within 0.53 unit.  A
//    64-bit accumulator per output sums them exactly (at most 2^15 real K per
//    CTA keeps it below 2^63); the result is scaled back once at the end.
// Accuracy (a numpy emulation of exactly this scheme on 2D / 3D systems of
// order 1400 / 2100): residual errors of 3e-14 / 1e-14 of ||B||, where six
// digits give 8e-12 / 2e-12.
//
// Two passes.  digitize_kernel turns M into its digits once per matrix
// (refinement reuses them for every residual): one byte per digit (the
// biased digit d + 128), seven digit slices of 128 rows x 64 real K per
// (row tile, 32-column chunk), 56 KB contiguous, each slice laid out as the
// MMA operand's 128-byte-swizzled K-major rows at half width, so that
// widening byte k of a slice to fp16 lands at byte 2k of the operand.
// residual_tc_kernel: one CTA per (32 complex right-hand sides) x (128 rows)
// x (a range of K in chunks), 512 threads:
//   warp 0      : TMEM allocation (7 levels x 64 columns); bulk copies: per chunk the right-hand sides' digit block
//                 (bdigits_kernel, 56 KB, 2 stages) and the seven 8 KB digit
//                 slices of M (6-slice ring), whichever has a free slot
//   warp 1      : MMA issuer.  Per chunk and digit s of A', one MMA per
//                 16-wide K step covers the levels s .. 6 at once: the seven
//                 digit slices of B' are stacked along N, so the levels
//                 s + t, t = 0 .. 6 - s, are adjacent TMEM columns (N <= 256
//                 per MMA: 10 MMAs per K step instead of 28)
//   warps 2-9   : epilogue: thread = (row, half of the 64 real columns);
//                 level sums -> 64-bit accumulators in registers
//   warps 10-15 : converters: a staged byte slice -> the fp16 operand slice
//                 (one byte permute and one fp16 subtract per digit pair)
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
constexpr int ASLOTS = 4;               // fp16 operand-slice ring
constexpr int DSLOTS = 6;               // byte-slice staging ring
constexpr uint32_t A_SLICE = BM * 128;              // 16 KB: one fp16 digit slice of A'
constexpr uint32_t D_SLICE = BM * 64;               // 8 KB: the same slice, one byte per digit
constexpr uint32_t B_SLICE = BN * 128;              // 8 KB
constexpr uint32_t B_BLOCK = DIG * B_SLICE;         // 56 KB: one chunk of B', all digit slices
constexpr uint32_t TMEM_COLS = 512;
constexpr int NEPI = 8, NCONV = 6;
constexpr int EPI0 = 2;                             // first epilogue warp
// 16 warps: four per SM sub-partition leave 128 registers per thread
constexpr int THREADS = (EPI0 + NEPI + NCONV) * 32;
constexpr int EPI_COLS = BN / (NEPI / 4);           // real columns per epilogue thread
// at most 512 chunks (32768 real K) per CTA: |sum| <= 2^15 * 2^48 = 2^63
// units of 2^-48, less the rounding of levels 5 and 6
constexpr int MAX_SPLIT_CHUNKS = 512;
constexpr long long BIAS = 0x0080808080808080LL;    // 128 in each of the seven digit positions
constexpr int FIX = 54;                             // |X| < 2^FIX

constexpr size_t smem_bytes() {
  return 1024 + ASLOTS * A_SLICE + DSLOTS * D_SLICE + 2 * B_BLOCK + BM * sizeof(int) + 256;
}

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

// Four biased digit bytes b0..b3 -> two fp16 pairs (b0 - 128, b1 - 128),
// (b2 - 128, b3 - 128): a byte permute places each byte under 0x64 (the fp16
// encoding of 1024 + byte), and 1152 is subtracted (exact).
__device__ __forceinline__ uint2 widen4(uint32_t x) {
  const uint32_t h0 = __byte_perm(x, 0x64646464u, 0x4140), h1 = __byte_perm(x, 0x64646464u, 0x4342);
  const __half2 c = __halves2half2(__ushort_as_half((unsigned short)0x6480), __ushort_as_half((unsigned short)0x6480));
  const __half2 d0 = __hsub2(*reinterpret_cast<const __half2*>(&h0), c);
  const __half2 d1 = __hsub2(*reinterpret_cast<const __half2*>(&h1), c);
  return make_uint2(*reinterpret_cast<const uint32_t*>(&d0), *reinterpret_cast<const uint32_t*>(&d1));
}

// row exponent of a row holding a NaN or an infinity: its outputs are NaN
constexpr int kRowNonFinite = 0x40000000;

__device__ __forceinline__ int clamp_exp(int e) { return (e < -300 || e > 300) ? 0 : e; }

// Byte offset of real K index kr (even) of row rho in a 128-row tile whose rows
// are 128-byte lines (64 fp16), 8-row groups 1024 B apart, 16-byte chunks
// XOR-swizzled by the row within its group: the K-major 128B-swizzle layout.
__device__ __forceinline__ uint32_t swz(int rho, int kr) {
  return (uint32_t)rho * 128u + ((uint32_t)(((kr >> 3) ^ (rho & 7)) << 4)) + (uint32_t)((kr & 7) * 2);
}

__global__ void __launch_bounds__(THREADS, 1)
residual_tc_kernel(const unsigned char* __restrict__ D, int rows, const int* __restrict__ row_exp,
                   const int* __restrict__ col_exp, const unsigned char* __restrict__ bdig, int nch_total, int ncols,
                   int chunks_per_split, const double2* __restrict__ B, int64_t ldb, double2* __restrict__ R,
                   int64_t ldr, double2* __restrict__ partial, int* status) {
  using namespace tc;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  unsigned char* aring = base;
  unsigned char* bring = aring + ASLOTS * A_SLICE;
  unsigned char* dring = bring + 2 * B_BLOCK;
  int* rexp = reinterpret_cast<int*>(dring + DSLOTS * D_SLICE);
  uint64_t* full_a = reinterpret_cast<uint64_t*>(rexp + BM);
  uint64_t* empty_a = full_a + ASLOTS;
  uint64_t* full_d = empty_a + ASLOTS;
  uint64_t* empty_d = full_d + DSLOTS;
  uint64_t* full_b = empty_d + DSLOTS;
  uint64_t* empty_b = full_b + 2;
  uint64_t* tfull = empty_b + 2;
  uint64_t* tempty = tfull + 1;
  uint64_t* done = tempty + 1;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  volatile int* abort = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ct = blockIdx.x, rt = blockIdx.y, sp = blockIdx.z, row0 = rt * BM;
  const int c_begin = sp * chunks_per_split;
  const int nchunk = max(0, min(nch_total, c_begin + chunks_per_split) - c_begin);
  const int nread = (nchunk + 1) >> 1;

  if (threadIdx.x < BM) rexp[threadIdx.x] = (row0 + (int)threadIdx.x < rows) ? clamp_exp(row_exp[row0 + threadIdx.x]) : 0;
  if (threadIdx.x == 0) {
    for (int s = 0; s < ASLOTS; ++s) { mbar_init(&full_a[s], NCONV); mbar_init(&empty_a[s], 1); }
    for (int s = 0; s < DSLOTS; ++s) { mbar_init(&full_d[s], 1); mbar_init(&empty_d[s], NCONV); }
    for (int s = 0; s < 2; ++s) { mbar_init(&full_b[s], 1); mbar_init(&empty_b[s], 1); }
    mbar_init(tfull, 1);
    mbar_init(tempty, NEPI);
    mbar_init(done, 1);
    *abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
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
    // ---------------- producer: digit blocks of B', digit slices of A'.
    // Whichever copy has a free slot is issued (B blocks first), so a B
    // block goes out as soon as the MMAs of the block two back have completed
    // rather than behind the slices of the current chunk.
    const unsigned char* dsrc = D + ((size_t)rt * nch_total + c_begin) * DIG * D_SLICE;
    const int nq = nchunk * DIG;
    int ib = 0, q = 0;
    uint32_t idle = 0;
    while ((ib < nchunk || q < nq) && !*abort) {
      bool progress = false;
      if (ib < nchunk && (ib < 2 || mbar_try_wait(&empty_b[ib & 1], ((ib >> 1) - 1) & 1))) {
        mbar_expect_tx(&full_b[ib & 1], B_BLOCK);
        bulk_load(bring + (ib & 1) * B_BLOCK, bdig + ((size_t)ct * nch_total + c_begin + ib) * B_BLOCK, B_BLOCK,
                  &full_b[ib & 1]);
        ++ib;
        progress = true;
      }
      if (q < nq && (q < DSLOTS || mbar_try_wait(&empty_d[q % DSLOTS], ((q / DSLOTS) - 1) & 1))) {
        mbar_expect_tx(&full_d[q % DSLOTS], D_SLICE);
        bulk_load(dring + (q % DSLOTS) * D_SLICE, dsrc + (size_t)q * D_SLICE, D_SLICE, &full_d[q % DSLOTS]);
        ++q;
        progress = true;
      }
      if (progress) idle = 0;
      else if (++idle >= kWaitLimit) { *abort = 1; break; }
    }
    // copies in flight land before the CTA may exit
    for (int j = max(0, ib - 2); j < ib; ++j) mbar_wait_plain(&full_b[j & 1], (j >> 1) & 1);
    for (int j = max(0, q - DSLOTS); j < q; ++j) mbar_wait_plain(&full_d[j % DSLOTS], (j / DSLOTS) & 1);
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
  } else if (warp >= EPI0 && warp < EPI0 + NEPI) {
    // ---------------- epilogue: thread = (row, half of the real columns)
    // a warp reads the TMEM lanes of its rank modulo 4
    const int qd = warp & 3, part = (warp - EPI0) >> 2, r = qd * 32 + lane;
    long long acc[EPI_COLS];
#pragma unroll
    for (int j = 0; j < EPI_COLS; ++j) acc[j] = 0;
    const uint32_t tbase = tmem + ((uint32_t)(qd * 32) << 16) + (uint32_t)(part * EPI_COLS);
    bool ok = true;
    for (int ro = 0; ro < nread; ++ro) {
      if (!mbar_wait(tfull, ro & 1, abort)) { ok = false; break; }
      tc_fence_after();
      // a fresh copy per readout keeps the 28 TMEM addresses from being
      // hoisted out of the loop into registers
      uint32_t tb;
      asm volatile("mov.b32 %0, %1;" : "=r"(tb) : "r"(tbase));
#pragma unroll
      for (int p = 0; p < EPI_COLS / 4; ++p) {
        uint32_t v[DIG][4];
#pragma unroll
        for (int l = 0; l < DIG; ++l) tmem_ld4(tb + (uint32_t)(l * BN + p * 4), v[l]);
        tmem_wait_ld();
        if (p == EPI_COLS / 4 - 1) {
          tc_fence_before();
          __syncwarp();
          if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(tempty)) : "memory");
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          // level l weighs 2^(36 - 8 l) units of 2^-48.  With |L_0| <= 2^19,
          // |L_1| <= 2^21, |L_2| <= 2^22, |L_3| < 2^22.6, |L_4| <= 2^23 (top
          // digits at most 64): hi = L_0 2^8 + L_1 and mid = L_2 2^8 + L_3 are
          // exact in 32 bits; levels 5 and 6 round to the nearest unit through
          // one FMA ((L_5 + L_6 / 256) / 16, its own rounding below 1/32 unit)
          const int hi = (__float2int_rz(__uint_as_float(v[0][j])) << 8) + __float2int_rz(__uint_as_float(v[1][j]));
          const int mid = (__float2int_rz(__uint_as_float(v[2][j])) << 8) + __float2int_rz(__uint_as_float(v[3][j]));
          const int l4 = __float2int_rz(__uint_as_float(v[4][j]));
          const int l56 = __float2int_rn(
              0.0625f * fmaf(__uint_as_float(v[6][j]), 0.00390625f, __uint_as_float(v[5][j])));
          acc[p * 4 + j] += ((long long)hi << 28) + ((long long)mid << 12) + (long long)((l4 << 4) + l56);
        }
      }
    }
    const int row = row0 + r;
    if (row < rows) {
      const bool good = ok && !*abort && row_exp[row] != kRowNonFinite;
      const int ea = rexp[r];
#pragma unroll
      for (int jc = 0; jc < EPI_COLS / 2; ++jc) {
        const int col = ct * BNC + part * (EPI_COLS / 2) + jc;
        if (col < ncols) {
          double2 val;
          if (good) {
            // 2^sc, sc in [-648, 552]: a normal double
            const double sc = __longlong_as_double((long long)(ea + clamp_exp(col_exp[col]) - 48 + 1023) << 52);
            val = make_double2((double)acc[2 * jc] * sc, (double)acc[2 * jc + 1] * sc);
          } else {
            val = make_double2(__longlong_as_double(0x7FF8000000000000LL),
                               __longlong_as_double(0x7FF8000000000000LL));
          }
          if (partial) {
            partial[((int64_t)sp * rows + row) * ncols + col] = val;
          } else {
            const double2 b = B ? B[(int64_t)row * ldb + col] : make_double2(0.0, 0.0);
            R[(int64_t)row * ldr + col] = make_double2(b.x - val.x, b.y - val.y);
          }
        }
      }
    }
  } else if (warp >= EPI0 + NEPI) {
    // ---------------- converters: staged byte slice -> fp16 operand slice
    const int ctid = threadIdx.x - (EPI0 + NEPI) * 32;
    const int nq = nchunk * DIG;
    for (int q = 0; q < nq; ++q) {
      const int ds = q % DSLOTS, as = q % ASLOTS;
      if (!mbar_wait(&full_d[ds], (q / DSLOTS) & 1, abort)) break;
      if (q >= ASLOTS && !mbar_wait(&empty_a[as], ((q / ASLOTS) - 1) & 1, abort)) break;
      const unsigned char* src = dring + ds * D_SLICE;
      unsigned char* dst = aring + as * A_SLICE;
      // thread: 8 digit bytes -> 16 contiguous operand bytes (both accesses
      // contiguous across the warp)
      for (int u = ctid; u < (int)(D_SLICE / 8); u += NCONV * 32) {
        const uint32_t off = (uint32_t)u * 8u;
        const uint2 v = *reinterpret_cast<const uint2*>(src + off);
        const uint2 w0 = widen4(v.x), w1 = widen4(v.y);
        *reinterpret_cast<uint4*>(dst + 2 * off) = make_uint4(w0.x, w0.y, w1.x, w1.y);
      }
      fence_async_smem();
      __syncwarp();
      if (lane == 0) {
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&full_a[as])) : "memory");
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&empty_d[ds])) : "memory");
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x == 0 && *abort) atomicExch(status, MGT_ERR_TIMEOUT);
  if (warp == 0) {
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

// Byte p (0 = lowest) of each of four 64-bit words, packed low to high.
__device__ __forceinline__ uint32_t pick_bytes(const long long* y, int p) {
  const int b = p & 3;
  uint32_t w[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) w[k] = p < 4 ? (uint32_t)y[k] : (uint32_t)((unsigned long long)y[k] >> 32);
  const uint32_t sel = (uint32_t)(b | ((4 + b) << 4));
  return __byte_perm(__byte_perm(w[0], w[1], sel), __byte_perm(w[2], w[3], sel), 0x5410);
}

// Digits of M (the A' operand) for every (row tile, chunk): block
// (rt, c) holds slices s = 0 .. 6 (digit p = 6 - s), 8 KB each, byte
// (rho, kr) of a slice at rho * 64 + (((kr >> 3) ^ (rho & 7)) << 3) + (kr & 7):
// the swizzled fp16 operand layout at half width.  Zeros beyond rows and kdim.
// Thread = (row, 8 real K = 4 complex entries), four per thread.
__global__ void __launch_bounds__(256)
digitize_kernel(const float4* __restrict__ M, int64_t ldm, int rows, int kdim, const int* __restrict__ row_exp,
                unsigned char* __restrict__ D, int nch) {
  const int c = blockIdx.x, rt = blockIdx.y;
  unsigned char* blk = D + ((size_t)rt * nch + c) * DIG * D_SLICE;
#pragma unroll 1
  for (int t = threadIdx.x; t < BM * 8; t += 256) {
    const int rho = t >> 3, grp = t & 7, row = rt * BM + rho;
    const bool rin = row < rows;
    const int sh = FIX - (rin ? clamp_exp(row_exp[row]) : 0);
    long long y[8];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int kc = c * KCC + grp * 4 + e;
      const float4 v = (rin && kc < kdim) ? __ldg(&M[(int64_t)row * ldm + kc]) : make_float4(0.f, 0.f, 0.f, 0.f);
      y[2 * e] = fixed_point(v.x, sh) + fixed_low(v.y, sh) + BIAS;
      y[2 * e + 1] = fixed_point(v.z, sh) + fixed_low(v.w, sh) + BIAS;
    }
    const uint32_t off = (uint32_t)rho * 64u + ((uint32_t)(grp ^ (rho & 7)) << 3);
#pragma unroll
    for (int s = 0; s < DIG; ++s) {
      const int p = DIG - 1 - s;
      *reinterpret_cast<uint2*>(blk + s * D_SLICE + off) = make_uint2(pick_bytes(y, p), pick_bytes(y + 4, p));
    }
  }
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

// workspace of one application (the digits of M are the caller's)
struct TcResWs {
  int* status;
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
    colexp = (int*)take((size_t)ncols * sizeof(int), 256);
    bdig = (unsigned char*)take((size_t)ctiles * nch * B_BLOCK, 1024);
    partial = splits > 1 ? (double2*)take((size_t)splits * rows * ncols * sizeof(double2), 256) : nullptr;
    total = off + 256;
  }
};

static size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

}  // namespace rtc

bool residual_tc_supported(int64_t rows, int64_t kdim, int64_t ncols) {
  return tc_available() && rows > 0 && kdim > 0 && ncols > 0 && rows <= (1 << 24) && kdim <= (1 << 22) &&
         ncols <= (1 << 16);
}

size_t residual_tc_digits_bytes(int64_t rows, int64_t kdim) {
  using namespace rtc;
  return (size_t)((rows + BM - 1) / BM) * (size_t)((kdim + KCC - 1) / KCC) * DIG * D_SLICE;
}

size_t residual_tc_apply_bytes(int64_t rows, int64_t kdim, int64_t ncols) {
  if (!residual_tc_supported(rows, kdim, ncols)) return 0;
  return rtc::TcResWs(nullptr, (int)rows, (int)kdim, (int)ncols).total;
}

size_t residual_tc_workspace_bytes(int64_t rows, int64_t kdim, int64_t ncols) {
  using namespace rtc;
  if (!residual_tc_supported(rows, kdim, ncols)) return 0;
  return align_up((size_t)rows * sizeof(int), 1024) + align_up(residual_tc_digits_bytes(rows, kdim), 1024) +
         residual_tc_apply_bytes(rows, kdim, ncols);
}

int residual_tc_prepare(const float4* M, int64_t ldm, int rows, int kdim, int* rowexp, unsigned char* digits,
                        cudaStream_t s) {
  using namespace rtc;
  if (!residual_tc_supported(rows, kdim, 1)) return MGT_ERR_UNSUPPORTED;
  if (!M || !rowexp || !digits || ((uintptr_t)digits & 15)) return MGT_ERR_ARG;
  const int nch = (kdim + KCC - 1) / KCC;
  count_launch(2);
  rowexp_kernel<<<(rows + 7) / 8, 256, 0, s>>>(M, ldm, rows, kdim, rowexp);
  digitize_kernel<<<dim3(nch, (rows + BM - 1) / BM), 256, 0, s>>>(M, ldm, rows, kdim, rowexp, digits, nch);
  return cudaGetLastError() == cudaSuccess ? MGT_OK : MGT_ERR_CUDA;
}

int residual_tc_apply(const unsigned char* digits, const int* rowexp, int rows, int kdim, const double2* X,
                      int64_t ldx, int ncols, const double2* B, int64_t ldb, double2* R, int64_t ldr, void* work,
                      size_t work_bytes, cudaStream_t s) {
  using namespace rtc;
  if (!residual_tc_supported(rows, kdim, ncols)) return MGT_ERR_UNSUPPORTED;
  if (!digits || !rowexp || ((uintptr_t)digits & 15)) return MGT_ERR_ARG;
  TcResWs w(work, rows, kdim, ncols);
  if (!work || work_bytes < w.total) return MGT_ERR_WORKSPACE;
  static OncePerDevice once;
  once([] {
    cudaFuncSetAttribute(residual_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes());
  });
  if (cudaMemsetAsync(w.status, 0, sizeof(int), s) != cudaSuccess) return MGT_ERR_CUDA;
  // column exponents start far below any real one (0x80808080)
  if (cudaMemsetAsync(w.colexp, 0x80, (size_t)ncols * sizeof(int), s) != cudaSuccess) return MGT_ERR_CUDA;
  count_launch(2);
  colexp_kernel<<<dim3((ncols + 31) / 32, std::min(64, (kdim + 7) / 8)), 256, 0, s>>>(X, ldx, kdim, ncols, w.colexp);
  const int64_t nb = (int64_t)w.nch * KCC * w.ctiles * BNC;
  bdigits_kernel<<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(X, ldx, kdim, ncols, w.colexp, w.bdig, w.nch, w.ctiles);
  count_launch();
  // column tiles of one row tile are neighbours in the launch order, so the
  // second reads the row tile's digit slices from L2
  dim3 grid(w.ctiles, (rows + BM - 1) / BM, w.splits);
  residual_tc_kernel<<<grid, THREADS, smem_bytes(), s>>>(digits, rows, rowexp, w.colexp, w.bdig, w.nch, ncols,
                                                           w.cps, B, ldb, R, ldr, w.partial, w.status);
  if (w.splits > 1) {
    const int64_t tot = (int64_t)rows * ncols;
    count_launch();
    tc_reduce_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(w.partial, w.splits, rows, ncols, B, ldb, R, ldr);
  }
  return cudaGetLastError() == cudaSuccess ? MGT_OK : MGT_ERR_CUDA;
}

size_t residual_tc_split(void* work, int64_t rows, int64_t kdim, int** rowexp, unsigned char** digits, char** aw) {
  using namespace rtc;
  char* b = (char*)work;
  const size_t d_off = align_up((size_t)rows * sizeof(int), 1024);
  const size_t a_off = d_off + align_up(residual_tc_digits_bytes(rows, kdim), 1024);
  if (rowexp) *rowexp = (int*)b;
  if (digits) *digits = (unsigned char*)(b + d_off);
  if (aw) *aw = b + a_off;
  return a_off;
}

int residual_tc(const float4* M, int64_t ldm, int rows, int kdim, const double2* X, int64_t ldx, int ncols,
                const double2* B, int64_t ldb, double2* R, int64_t ldr, void* work, size_t work_bytes,
                cudaStream_t s) {
  if (!residual_tc_supported(rows, kdim, ncols)) return MGT_ERR_UNSUPPORTED;
  if (!work || work_bytes < residual_tc_workspace_bytes(rows, kdim, ncols)) return MGT_ERR_WORKSPACE;
  int* rowexp;
  unsigned char* digits;
  char* aw;
  const size_t a_off = residual_tc_split(work, rows, kdim, &rowexp, &digits, &aw);
  int e = residual_tc_prepare(M, ldm, rows, kdim, rowexp, digits, s);
  if (e != MGT_OK) return e;
  return residual_tc_apply(digits, rowexp, rows, kdim, X, ldx, ncols, B, ldb, R, ldr, aw, work_bytes - a_off, s);
}


}  // namespace mgt
