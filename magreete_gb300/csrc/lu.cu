// K2/K3: blocked right-looking complex LU with partial pivoting, and the
// matching multi-RHS triangular solves.
//
// Per panel of NB columns (the ?getrf loop that torch.linalg.solve reaches
// in solve(), Transmission2D.py:230 / Transmission3D.py:205):
//   1. lu_panel_kernel: one cooperative launch factors the (m x NB) panel.
//      Each CTA keeps a contiguous chunk of panel rows in shared memory; per
//      column it publishes its local pivot candidate (value, row, row
//      contents) and the owner of the diagonal row publishes that row; one
//      grid barrier; every CTA then picks the same global pivot (largest
//      |re|+|im|, lowest row on ties, as LAPACK's i?amax), swaps, scales and
//      applies the rank-1 update to its own rows.  One barrier per column.
//   2. lu_swap_trsm_kernel: applies the panel's row interchanges to every
//      column outside the panel (one gather/scatter of at most 2*NB rows per
//      column) and solves L11 U12 = A12 for the columns right of the panel.
//   3. trailing update A22 -= L21 U12 (a complex GEMM, gemm.cu).
#include <algorithm>
#include <atomic>
#include <mutex>

#include "common.cuh"
#include "gemm.cuh"
#include "gemm_tc.cuh"
#include "diag.cuh"

namespace mgt {

constexpr int kMaxPanelBlocks = 160;
constexpr int kPanelThreads = 256;
constexpr int kPanelRowsTarget = 256;   // default rows per CTA the panel aims for
constexpr size_t kPanelSmemBudget = 220 * 1024;
constexpr int kNBmax = 64;
// one published record per (column parity, CTA): header + candidate row + diagonal row
constexpr size_t kRecHeader = 64;
constexpr size_t kRecBytes = (kRecHeader + 2 * kNBmax * sizeof(double2) + 127) & ~size_t(127);

// Workspace layout (byte offsets), identical for both element types.
struct LuWsLayout {
  size_t status = 8;      // 2 x i32: error, info
  size_t nslot = 16;      // 2 x i32: slots written by the last panel of each slot set
  size_t epoch = 40;      // u64: factorisation counter (bumped on the device, never cleared)
  size_t slots = 64;      // 2 sets x 2*NBmax x int2 (pos, src)
  size_t records;         // 2 x kMaxPanelBlocks x kRecBytes
  size_t inv;             // 2 x NBmax x NBmax complex: inverses of a 128-wide block's diagonal blocks
  size_t uinv;            // NBmax x NBmax complex64: U11^-1, then L11^-1, of the last tile-pivoting panel
  size_t total;
  LuWsLayout() {
    records = (slots + 2 * 2 * kNBmax * sizeof(int2) + 127) & ~size_t(127);
    inv = records + 2 * (size_t)kMaxPanelBlocks * kRecBytes;
    uinv = inv + 2 * (size_t)kNBmax * kNBmax * sizeof(double2);
    total = uinv + 2 * (size_t)kNBmax * kNBmax * sizeof(float2);
  }
};

struct PanelWs {
  int* status;
  int* nslot;
  unsigned long long* epoch;
  int2* slots;
  unsigned char* records;
};

// slot set 0 or 1: two panels' interchanges can be pending at once (lookahead)
static PanelWs panel_ws(void* work, int set = 0) {
  LuWsLayout L;
  char* b = (char*)work;
  PanelWs w;
  w.status = (int*)(b + L.status);
  w.nslot = (int*)(b + L.nslot) + set;
  w.epoch = (unsigned long long*)(b + L.epoch);
  w.slots = (int2*)(b + L.slots) + set * 2 * kNBmax;
  w.records = (unsigned char*)(b + L.records);
  return w;
}

__device__ __forceinline__ bool better(double v, int i, double bv, int bi) {
  return v > bv || (v == bv && i >= 0 && (bi < 0 || i < bi));
}

__device__ __forceinline__ void st_release_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// Panel factorisation with partial pivoting, one cooperative launch.
//
// Each CTA holds a contiguous chunk of panel rows in shared memory.  Per
// column every CTA publishes a record -- its best local pivot candidate
// (|re|+|im|, row, row contents) and, if it owns the diagonal row, that row --
// and releases it with a 64-bit sequence number unique to (factorisation,
// column).  Warp 0 of every CTA then polls all records with acquire loads
// until each carries the expected number: the records are the barrier, so a
// column costs one publish and one poll instead of a barrier plus two reads.
// Records alternate between two buffers by column parity; a CTA can only
// overwrite a buffer after every CTA has published (and so finished reading)
// the column in between.  Polls are bounded; on expiry the kernel records
// MGT_ERR_TIMEOUT and returns.
template <typename T, int NB>
__global__ void __launch_bounds__(kPanelThreads)
lu_panel_kernel(cplx<T>* __restrict__ A, int64_t lda, int m, int w, int j0, int rows_per_cta,
                int32_t* __restrict__ perm, PanelWs ws) {
  // record sequence numbers: unique per (factorisation, column) even when the
  // launch is replayed from a CUDA graph, because the epoch is bumped on the device
  const unsigned long long seq0 = (*(volatile unsigned long long*)ws.epoch << 24) + (unsigned long long)j0 + 1;
  using V = cplx<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* S = reinterpret_cast<V*>(smem_raw);
  __shared__ V U[NB];
  __shared__ V RC[NB];
  __shared__ double red_val[kPanelThreads / 32];
  __shared__ int red_idx[kPanelThreads / 32];
  __shared__ int s_best, s_p, s_wb, s_fail;
  __shared__ int s_piv[NB];
  __shared__ int slot_pos[2 * NB], slot_src[2 * NB];
  __shared__ int s_nslot;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nwarps = kPanelThreads / 32;
  const int G = gridDim.x, bid = blockIdx.x;
  const int r0 = bid * rows_per_cta;
  const int r1 = min(m, r0 + rows_per_cta);
  const int nr = max(0, r1 - r0);

  for (int idx = tid; idx < nr * NB; idx += kPanelThreads) {
    int rr = idx / NB, cc = idx - rr * NB;
    S[idx] = cc < w ? A[(int64_t)(r0 + rr) * lda + cc] : czero<V>();
  }
  if (tid == 0) s_fail = 0;
  __syncthreads();

  for (int c = 0; c < w; ++c) {
    const int buf = c & 1;
    const unsigned long long seq = seq0 + (unsigned long long)c;
    unsigned char* my = ws.records + ((size_t)buf * kMaxPanelBlocks + bid) * kRecBytes;
    // ---- 1. local pivot candidate (rows i >= c of this chunk)
    double best = -1.0;
    int bidx = -1;
    for (int i = max(r0, c) + tid; i < r1; i += kPanelThreads) {
      double v = (double)cabs1(S[(i - r0) * NB + c]);
      if (v > best) { best = v; bidx = i; }
    }
#pragma unroll
    for (int off = 16; off; off >>= 1) {
      double ov = __shfl_down_sync(0xffffffffu, best, off);
      int oi = __shfl_down_sync(0xffffffffu, bidx, off);
      if (better(ov, oi, best, bidx)) { best = ov; bidx = oi; }
    }
    if (lane == 0) { red_val[warp] = best; red_idx[warp] = bidx; }
    __syncthreads();
    if (warp == 0) {
      best = lane < nwarps ? red_val[lane] : -1.0;
      bidx = lane < nwarps ? red_idx[lane] : -1;
#pragma unroll
      for (int off = 16; off; off >>= 1) {
        double ov = __shfl_down_sync(0xffffffffu, best, off);
        int oi = __shfl_down_sync(0xffffffffu, bidx, off);
        if (better(ov, oi, best, bidx)) { best = ov; bidx = oi; }
      }
      if (lane == 0) {
        s_best = bidx;
        *reinterpret_cast<double*>(my + 8) = best;
        *reinterpret_cast<int*>(my + 16) = bidx;
      }
    }
    __syncthreads();
    // ---- 2. publish: candidate row, the diagonal row (owner), then the sequence number
    {
      const int bi = s_best;
      V* cand = reinterpret_cast<V*>(my + kRecHeader);
      V* rowc = cand + NB;
      if (bi >= 0)
        for (int k = tid; k < w; k += kPanelThreads) cand[k] = S[(bi - r0) * NB + k];
      if (c >= r0 && c < r1)
        for (int k = tid; k < w; k += kPanelThreads) rowc[k] = S[(c - r0) * NB + k];
    }
    __syncthreads();
    if (tid == 0) {
      __threadfence();
      st_release_u64(reinterpret_cast<unsigned long long*>(my), seq);
    }
    // ---- 3. poll every CTA's record for this column, pick the global pivot
    if (warp == 0) {
      unsigned seen = 0;   // bit j: record lane + 32 j observed
      const int per = (G + 31) / 32;
      const unsigned want = (per >= 32) ? 0xffffffffu : ((1u << per) - 1u);
      unsigned it = 0;
      bool ok = true;
      while (true) {
        for (int j = 0; j < per; ++j) {
          const int q = lane + 32 * j;
          if (q >= G) { seen |= 1u << j; continue; }
          if (seen & (1u << j)) continue;
          const unsigned char* rq = ws.records + ((size_t)buf * kMaxPanelBlocks + q) * kRecBytes;
          if (ld_acquire_u64(reinterpret_cast<const unsigned long long*>(rq)) == seq) seen |= 1u << j;
        }
        if (__all_sync(0xffffffffu, seen == want)) break;
        if (++it > kSpinLimit) { ok = false; break; }
        if (it > 32) __nanosleep(32);
      }
      double bv = -1.0;
      int bi = -1, bb = -1;
      if (ok) {
        for (int q = lane; q < G; q += 32) {
          const unsigned char* rq = ws.records + ((size_t)buf * kMaxPanelBlocks + q) * kRecBytes;
          double v = __ldcg(reinterpret_cast<const double*>(rq + 8));
          int i = __ldcg(reinterpret_cast<const int*>(rq + 16));
          if (better(v, i, bv, bi)) { bv = v; bi = i; bb = q; }
        }
#pragma unroll
        for (int off = 16; off; off >>= 1) {
          double ov = __shfl_down_sync(0xffffffffu, bv, off);
          int oi = __shfl_down_sync(0xffffffffu, bi, off);
          int ob = __shfl_down_sync(0xffffffffu, bb, off);
          if (better(ov, oi, bv, bi)) { bv = ov; bi = oi; bb = ob; }
        }
      }
      if (lane == 0) {
        s_p = bi;
        s_wb = bb;
        if (!ok) { s_fail = 1; atomicExch(ws.status, MGT_ERR_TIMEOUT); }
      }
    }
    __syncthreads();
    if (s_fail) return;
    // No valid candidate anywhere (the column is all NaN): keep row c in place.
    const int p = s_p >= 0 ? s_p : c, wb = s_p >= 0 ? s_wb : -1;
    const int owner = c / rows_per_cta;
    const V* rec_w = reinterpret_cast<const V*>(ws.records + ((size_t)buf * kMaxPanelBlocks + max(wb, 0)) * kRecBytes +
                                                kRecHeader);
    const V* rec_o = reinterpret_cast<const V*>(ws.records + ((size_t)buf * kMaxPanelBlocks + owner) * kRecBytes +
                                                kRecHeader) + NB;
    for (int k = tid; k < NB; k += kPanelThreads) {
      V rc = k < w ? ldcg(rec_o + k) : czero<V>();
      RC[k] = rc;
      U[k] = (k < w && wb >= 0) ? ldcg(rec_w + k) : rc;
    }
    __syncthreads();
    const V piv = U[c];
    const bool nz = (piv.x != 0 || piv.y != 0);
    if (nz && p != c) {
      if (p >= r0 && p < r1)
        for (int k = tid; k < w; k += kPanelThreads) S[(p - r0) * NB + k] = RC[k];
      if (c >= r0 && c < r1)
        for (int k = tid; k < w; k += kPanelThreads) S[(c - r0) * NB + k] = U[k];
    }
    if (bid == 0 && tid == 0) {
      const int pe = nz ? p : c;
      s_piv[c] = pe;
      if (pe != c) {
        int a = perm[j0 + c], b = perm[j0 + pe];
        perm[j0 + c] = b;
        perm[j0 + pe] = a;
      }
      if (!nz && ws.status[1] == 0) ws.status[1] = j0 + c + 1;
    }
    __syncthreads();
    // ---- 4. scale the column below the diagonal and update the rest of the panel
    const int ibeg = max(r0, c + 1);
    if (nz) {
      const V inv = crecip(piv);
      for (int i = ibeg + tid; i < r1; i += kPanelThreads) {
        V* e = &S[(i - r0) * NB + c];
        *e = cmul(*e, inv);
      }
    }
    __syncthreads();
    const int rows = r1 - ibeg, cols = w - c - 1;
    if (rows > 0 && cols > 0) {
      for (int idx = tid; idx < rows * cols; idx += kPanelThreads) {
        int ii = idx / cols, kk = idx - ii * cols;
        int i = ibeg + ii, k = c + 1 + kk;
        V l = S[(i - r0) * NB + c];
        cfms(S[(i - r0) * NB + k], l, U[k]);
      }
    }
    __syncthreads();
  }

  for (int idx = tid; idx < nr * NB; idx += kPanelThreads) {
    int rr = idx / NB, cc = idx - rr * NB;
    if (cc < w) A[(int64_t)(r0 + rr) * lda + cc] = S[idx];
  }

  // Net effect of the panel's interchanges on the rows they touch: after
  // them, panel row slot_pos[q] holds the row that was at slot_src[q].
  if (bid == 0 && warp == 0) {
    for (int s = lane; s < NB; s += 32) { slot_pos[s] = s; slot_src[s] = s; }
    if (lane == 0) s_nslot = NB;
    __syncwarp();
    for (int s = 0; s < w; ++s) {
      const int pv = s_piv[s];
      if (pv == s) continue;
      int slot = -1;
      if (pv < NB) {
        slot = pv;
      } else {
        const int ns = s_nslot;
        for (int base = NB; base < ns && slot < 0; base += 32) {
          int q = base + lane;
          unsigned hit = __ballot_sync(0xffffffffu, q < ns && slot_pos[q] == pv);
          if (hit) slot = base + __ffs(hit) - 1;
        }
        if (slot < 0) {
          slot = ns;
          if (lane == 0) { slot_pos[ns] = pv; slot_src[ns] = pv; s_nslot = ns + 1; }
        }
      }
      __syncwarp();
      if (lane == 0) { int t = slot_src[s]; slot_src[s] = slot_src[slot]; slot_src[slot] = t; }
      __syncwarp();
    }
    const int ns = s_nslot;
    for (int q = lane; q < ns; q += 32) ws.slots[q] = make_int2(slot_pos[q], slot_src[q]);
    if (lane == 0) *ws.nslot = ns;
  }
}

// Register-resident panel factorisation, one row per thread (at most 256 rows
// per CTA).  A thread keeps the unfinished part of its row in registers,
// shifted so that the current column is always a[0]: every register index is
// a compile-time constant while the column loop stays a loop (small code that
// stays in the instruction cache).  Finished columns (L or U values) go to the
// thread's row of the shared-memory tile sL, which also stages the coalesced
// load and store of the panel.
//
// Pivot search without floating-point compares (FP64 is slow on this part):
// the bits of a non-negative float / double are ordered like its value, so
// |re|+|im| is compared as an unsigned key (bits + 1; 0 = no candidate, NaN
// never a candidate), ties going to the lowest row -- LAPACK's i?amax rule.
//
// Exchange per column: each CTA publishes its best candidate row (and the
// owner of row c publishes row c) in its record, then one flag word.  For
// complex64 the flag word carries the candidate itself -- [tag:8 | row+1:24 |
// key:32], tag = ((j0 + c) mod 128) + 1 -- so the pivot is known as soon as
// every flag has been seen; flags are cleared when a factorisation starts, and
// the previous value of a record's flag (the column two back) never carries
// the current tag.  complex128 keeps the 64-bit sequence flag (factorisation
// epoch, column) with the candidate in the record header.
template <typename T>
struct PanelKey;
template <>
struct PanelKey<float> {
  using K = unsigned;
  static constexpr bool kPacked = true;
  __device__ static K key(float v) {
    const unsigned u = __float_as_uint(v);
    return u <= 0x7F800000u ? u + 1u : 0u;   // +0 .. +inf; NaN and negatives excluded
  }
};
template <>
struct PanelKey<double> {
  using K = unsigned long long;
  static constexpr bool kPacked = false;
  __device__ static K key(double v) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(v);
    return u <= 0x7FF0000000000000ull ? u + 1ull : 0ull;
  }
};

// Warp-wide argmax of (key, row): largest key, lowest row; every lane gets it.
__device__ __forceinline__ void warp_argmax(unsigned& k, int& i) {
  const unsigned m = __reduce_max_sync(0xffffffffu, k);
  i = (int)__reduce_min_sync(0xffffffffu, k == m ? (unsigned)i : 0x7fffffffu);
  k = m;
}
__device__ __forceinline__ void warp_argmax(unsigned long long& k, int& i) {
#pragma unroll
  for (int off = 16; off; off >>= 1) {
    const unsigned long long ok = __shfl_xor_sync(0xffffffffu, k, off);
    const int oi = __shfl_xor_sync(0xffffffffu, i, off);
    if (ok > k || (ok == k && oi < i)) { k = ok; i = oi; }
  }
}

__device__ __forceinline__ unsigned long long pack_flag(unsigned tag, int idx, unsigned key) {
  return ((unsigned long long)tag << 56) | ((unsigned long long)(unsigned)(idx + 1) << 32) | (unsigned long long)key;
}

template <typename T, int NB>
__global__ void __launch_bounds__(kPanelThreads, 1)
lu_panel_reg_kernel(cplx<T>* __restrict__ A, int64_t lda, int m, int w, int j0, int rows_per_cta,
                    int32_t* __restrict__ perm, PanelWs ws) {
  using V = cplx<T>;
  using PK = PanelKey<T>;
  using K = typename PK::K;
  constexpr int LD = NB + 1;                 // padded row of sL (bank spread)
  constexpr int kNone = 0x7fffffff;
  constexpr int kChunk = NB < 16 ? NB : 16;   // live-column granularity of the register loops
  extern __shared__ __align__(16) unsigned char panel_smem[];
  V* sL = reinterpret_cast<V*>(panel_smem);
  __shared__ V U[2 * NB];                    // pivot row, zero beyond w
  __shared__ V RC[2 * NB];                   // row c before the interchange, zero beyond w
  __shared__ K red_key[kPanelThreads / 32];
  __shared__ int red_idx[kPanelThreads / 32];
  __shared__ K s_bkey;
  __shared__ int s_best, s_p, s_fail;
  __shared__ int s_piv[NB];
  __shared__ int slot_pos[2 * NB], slot_src[2 * NB];
  __shared__ int s_nslot;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int nwarps = kPanelThreads / 32;
  const int G = gridDim.x, bid = blockIdx.x;
  const int r0 = bid * rows_per_cta;
  const int nr = max(0, min(m, r0 + rows_per_cta) - r0);
  const int row = r0 + tid;
  const bool have = tid < nr;
  const unsigned long long seq0 = (*(volatile unsigned long long*)ws.epoch << 24) + (unsigned long long)j0 + 1;

  for (int i = tid; i < 2 * NB; i += kPanelThreads) {
    U[i] = czero<V>();
    RC[i] = czero<V>();
  }
  for (int i = tid; i < nr * NB; i += kPanelThreads) {
    const int r = i / NB, k = i % NB;
    sL[r * LD + k] = k < w ? A[(int64_t)(r0 + r) * lda + k] : czero<V>();
  }
  if (tid == 0) s_fail = 0;
  __syncthreads();
  V a[NB];
#pragma unroll
  for (int k = 0; k < NB; ++k) a[k] = have ? sL[tid * LD + k] : czero<V>();

  for (int c = 0; c < w; ++c) {
    const int buf = c & 1;
    unsigned char* my = ws.records + ((size_t)buf * kMaxPanelBlocks + bid) * kRecBytes;
    // ---- 1. this CTA's candidate
    K key = (have && row >= c) ? PK::key(cabs1(a[0])) : K(0);
    int bidx = key ? row : kNone;
    warp_argmax(key, bidx);
    if (lane == 0) { red_key[warp] = key; red_idx[warp] = bidx; }
    __syncthreads();
    if (warp == 0) {
      key = lane < nwarps ? red_key[lane] : K(0);
      bidx = lane < nwarps ? red_idx[lane] : kNone;
      warp_argmax(key, bidx);
      if (lane == 0) {
        s_best = key ? bidx : -1;
        s_bkey = key;
        if (!PK::kPacked) {
          *reinterpret_cast<K*>(my + 8) = key;
          *reinterpret_cast<int*>(my + 16) = key ? bidx : -1;
        }
      }
    }
    __syncthreads();
    // ---- 2. publish the candidate row and (owner) row c: the row's thread
    // puts its registers into its sL row, then its warp copies the row out
    const int tb = s_best >= 0 ? s_best - r0 : -1;
    const int tc = (c >= r0 && c < r0 + nr) ? c - r0 : -1;
    {
      const bool wb = tb >= 0 && (tb >> 5) == warp;
      const bool wc = tc >= 0 && (tc >> 5) == warp;
      if (wb || wc) {
        if (tid == tb || tid == tc) {
          // branch-free: columns past the panel go to the row's pad column (index NB)
#pragma unroll
          for (int k = 0; k < NB; ++k) sL[tid * LD + min(c + k, NB)] = a[k];
        }
        __syncwarp();
        V* rec = reinterpret_cast<V*>(my + kRecHeader);
        if (wb)
          for (int k = lane; k < w; k += 32) rec[k] = sL[tb * LD + k];
        if (wc)
          for (int k = lane; k < w; k += 32) rec[NB + k] = sL[tc * LD + k];
      }
    }
    __syncthreads();
    const unsigned tag = (unsigned)((j0 + c) & 127) + 1u;
    // the release store orders every row write of the CTA before it: the
    // writes precede the barrier above, which thread 0 has passed (PTX
    // release patterns are cumulative over causality order)
    if (tid == 0) {
      if (PK::kPacked)
        st_release_u64(reinterpret_cast<unsigned long long*>(my), pack_flag(tag, s_best, (unsigned)s_bkey));
      else
        st_release_u64(reinterpret_cast<unsigned long long*>(my), seq0 + (unsigned long long)c);
    }
    // ---- 3. warp 0 waits for every CTA's flag and picks the global pivot
    if (warp == 0) {
      constexpr int kPer = (kMaxPanelBlocks + 31) / 32;
      unsigned seen = 0;
      const int per = (G + 31) / 32;
      const unsigned want = (1u << per) - 1u;
      unsigned it = 0;
      bool ok = true;
      K bk = 0;                 // this lane's best candidate so far
      int bi = kNone;
      while (true) {
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
          const int q = lane + 32 * j;
          if (j >= per || (seen & (1u << j))) continue;
          if (q >= G) { seen |= 1u << j; continue; }
          const unsigned char* rq = ws.records + ((size_t)buf * kMaxPanelBlocks + q) * kRecBytes;
          const unsigned long long f = ld_acquire_u64(reinterpret_cast<const unsigned long long*>(rq));
          K k2;
          int i2;
          if (PK::kPacked) {
            if ((unsigned)(f >> 56) != tag) continue;
            k2 = (K)(unsigned)f;
            i2 = (int)((f >> 32) & 0xFFFFFFu) - 1;
          } else {
            if (f != seq0 + (unsigned long long)c) continue;
            k2 = __ldcg(reinterpret_cast<const K*>(rq + 8));
            i2 = __ldcg(reinterpret_cast<const int*>(rq + 16));
          }
          seen |= 1u << j;
          if (!k2) i2 = kNone;
          if (k2 > bk || (k2 == bk && i2 < bi)) { bk = k2; bi = i2; }
        }
        if (__all_sync(0xffffffffu, seen == want)) break;
        if (++it > kSpinLimit) { ok = false; break; }
        if (it > 16) __nanosleep(20);
      }
      if (ok) warp_argmax(bk, bi);
      if (lane == 0) {
        s_p = bk ? bi : -1;
        if (!ok) { s_fail = 1; atomicExch(ws.status, MGT_ERR_TIMEOUT); }
      }
    }
    __syncthreads();
    if (s_fail) return;
    const int p = s_p >= 0 ? s_p : c;
    const int wbk = s_p >= 0 ? s_p / rows_per_cta : -1;
    const int owner = c / rows_per_cta;
    // ---- 4. pivot row and row c from the records
    if (tid < w) {
      const V* rec_w = reinterpret_cast<const V*>(ws.records + ((size_t)buf * kMaxPanelBlocks + max(wbk, 0)) *
                                                  kRecBytes + kRecHeader);
      const V* rec_o = reinterpret_cast<const V*>(ws.records + ((size_t)buf * kMaxPanelBlocks + owner) *
                                                  kRecBytes + kRecHeader) + NB;
      const V rc = ldcg(rec_o + tid);
      RC[tid] = rc;
      U[tid] = wbk >= 0 ? ldcg(rec_w + tid) : rc;
    }
    __syncthreads();
    const V piv = U[c];
    const bool nz = (piv.x != 0 || piv.y != 0);
    // ---- 5. interchange rows c and p: finished columns cooperatively, the rest in registers
    if (nz && p != c) {
      const int tp = (p >= r0 && p < r0 + nr) ? p - r0 : -1;
      if (tid < c) {
        if (tp >= 0) sL[tp * LD + tid] = RC[tid];
        if (tc >= 0) sL[tc * LD + tid] = U[tid];
      }
      if (tid == tp || tid == tc) {
        const V* src = tid == tp ? RC : U;
#pragma unroll
        for (int kc = 0; kc < NB; kc += kChunk) {
          if (kc > 0 && c + kc >= w) break;
#pragma unroll
          for (int k = kc; k < kc + kChunk; ++k) a[k] = src[c + k];
        }
      }
    }
    if (bid == 0 && tid == 0) {
      s_piv[c] = nz ? p : c;
      if (!nz && ws.status[1] == 0) ws.status[1] = j0 + c + 1;
    }
    // ---- 6. scale and rank-1 update in registers, retire column c, shift
    if (have && row > c && nz) {
      const V l = cmul(a[0], crecip(piv));
      a[0] = l;
      // whole chunks of live columns; U is zero beyond w, so the tail of a chunk is a no-op
#pragma unroll
      for (int kc = 0; kc < NB; kc += kChunk) {
        if (kc > 0 && c + kc >= w) break;
#pragma unroll
        for (int k = (kc ? kc : 1); k < kc + kChunk; ++k) cfms(a[k], l, U[c + k]);
      }
    }
    if (have) sL[tid * LD + c] = a[0];
#pragma unroll
    for (int kc = 0; kc < NB; kc += kChunk) {
      if (kc > 0 && c + kc >= w) break;
#pragma unroll
      for (int k = kc; k < kc + kChunk && k + 1 < NB; ++k) a[k] = a[k + 1];
    }
  }
  __syncthreads();
  for (int i = tid; i < nr * NB; i += kPanelThreads) {
    const int r = i / NB, k = i % NB;
    if (k < w) A[(int64_t)(r0 + r) * lda + k] = sL[r * LD + k];
  }

  if (bid == 0 && warp == 0) {
    for (int s2 = lane; s2 < NB; s2 += 32) { slot_pos[s2] = s2; slot_src[s2] = s2; }
    if (lane == 0) s_nslot = NB;
    __syncwarp();
    for (int s2 = 0; s2 < w; ++s2) {
      const int pv = s_piv[s2];
      if (pv == s2) continue;
      int slot = -1;
      if (pv < NB) {
        slot = pv;
      } else {
        const int ns = s_nslot;
        for (int base = NB; base < ns && slot < 0; base += 32) {
          int q = base + lane;
          unsigned hit = __ballot_sync(0xffffffffu, q < ns && slot_pos[q] == pv);
          if (hit) slot = base + __ffs(hit) - 1;
        }
        if (slot < 0) {
          slot = ns;
          if (lane == 0) { slot_pos[ns] = pv; slot_src[ns] = pv; s_nslot = ns + 1; }
        }
      }
      __syncwarp();
      if (lane == 0) { int t2 = slot_src[s2]; slot_src[s2] = slot_src[slot]; slot_src[slot] = t2; }
      __syncwarp();
    }
    const int ns = s_nslot;
    for (int q = lane; q < ns; q += 32) ws.slots[q] = make_int2(slot_pos[q], slot_src[q]);
    if (lane == 0) *ws.nslot = ns;
    // the panel's interchanges applied to perm in one gather / scatter
    int32_t pv[2 * NB / 32];
#pragma unroll
    for (int j = 0; j < 2 * NB / 32; ++j) {
      const int q = lane + 32 * j;
      if (q < ns) pv[j] = perm[j0 + slot_src[q]];
    }
    __syncwarp();
#pragma unroll
    for (int j = 0; j < 2 * NB / 32; ++j) {
      const int q = lane + 32 * j;
      if (q < ns) perm[j0 + slot_pos[q]] = pv[j];
    }
  }
}

constexpr size_t reg_panel_smem(int nb, size_t elem) { return (size_t)kPanelThreads * (nb + 1) * elem; }

// Cluster variant of the register-resident panel, for panels whose CTAs fit
// in one thread-block cluster (at most 16): the exchange goes through
// distributed shared memory instead of L2.  Per column each CTA stores its
// candidate (key, row) into every CTA's table (st.shared::cluster), one
// hardware cluster barrier makes all tables complete, every CTA picks the
// same pivot, and the pivot row and row c are read straight from the owning
// CTAs' shared memory.  Candidate rows and tables alternate between two
// buffers by column parity, so one barrier per column suffices: a CTA writes
// buffer b again only after the next column's barrier, which every CTA
// reaches after its reads of buffer b.  All CTAs run the same barrier
// sequence (no early exit), and a final barrier keeps every CTA's shared
// memory alive until the others have read it.
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ uint32_t cluster_map(uint32_t a, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}
__device__ __forceinline__ void cluster_st_u32(uint32_t a, uint32_t v) {
  asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}
__device__ __forceinline__ void cluster_st_u64(uint32_t a, unsigned long long v) {
  asm volatile("st.shared::cluster.u64 [%0], %1;" ::"r"(a), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long cluster_ld_u64(uint32_t a) {
  unsigned long long v;
  asm volatile("ld.shared::cluster.u64 %0, [%1];" : "=l"(v) : "r"(a) : "memory");
  return v;
}
__device__ __forceinline__ void cluster_barrier() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

constexpr int kMaxClusterCtas = 16;

template <int NB>
__global__ void __launch_bounds__(kPanelThreads, 1)
lu_panel_cluster_kernel(float2* __restrict__ A, int64_t lda, int m, int w, int j0, int rows_per_cta,
                        int32_t* __restrict__ perm, PanelWs ws) {
  using T = float;
  using V = float2;
  using PK = PanelKey<T>;
  using K = typename PK::K;
  constexpr int LD = NB + 1;
  constexpr int kNone = 0x7fffffff;
  constexpr int kChunk = NB < 16 ? NB : 16;
  extern __shared__ __align__(16) unsigned char panel_smem[];
  V* sL = reinterpret_cast<V*>(panel_smem);
  __shared__ V U[2 * NB];
  __shared__ V RC[2 * NB];
  __shared__ __align__(16) V rowbuf[2][NB];        // this CTA's candidate row, per column parity
  __shared__ __align__(16) V rcbuf[2][NB];         // row c (owner CTA), per column parity
  __shared__ unsigned long long ctab[2][kMaxClusterCtas];   // every CTA's candidate: key << 32 | row + 1
  __shared__ K red_key[kPanelThreads / 32];
  __shared__ int red_idx[kPanelThreads / 32];
  __shared__ K s_bkey;
  __shared__ int s_best, s_p;
  __shared__ int s_piv[NB];
  __shared__ int slot_pos[2 * NB], slot_src[2 * NB];
  __shared__ int s_nslot;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int nwarps = kPanelThreads / 32;
  const int G = gridDim.x;
  const int bid = (int)cluster_rank();             // one cluster spans the grid
  const int r0 = bid * rows_per_cta;
  const int nr = max(0, min(m, r0 + rows_per_cta) - r0);
  const int row = r0 + tid;
  const bool have = tid < nr;

  for (int i = tid; i < 2 * NB; i += kPanelThreads) {
    U[i] = czero<V>();
    RC[i] = czero<V>();
  }
  for (int i = tid; i < nr * NB; i += kPanelThreads) {
    const int r = i / NB, k = i % NB;
    sL[r * LD + k] = k < w ? A[(int64_t)(r0 + r) * lda + k] : czero<V>();
  }
  __syncthreads();
  V a[NB];
#pragma unroll
  for (int k = 0; k < NB; ++k) a[k] = have ? sL[tid * LD + k] : czero<V>();

  for (int c = 0; c < w; ++c) {
    const int buf = c & 1;
    // ---- 1. this CTA's candidate
    K key = (have && row >= c) ? PK::key(cabs1(a[0])) : K(0);
    int bidx = key ? row : kNone;
    warp_argmax(key, bidx);
    if (lane == 0) { red_key[warp] = key; red_idx[warp] = bidx; }
    __syncthreads();
    if (warp == 0) {
      key = lane < nwarps ? red_key[lane] : K(0);
      bidx = lane < nwarps ? red_idx[lane] : kNone;
      warp_argmax(key, bidx);
      if (lane == 0) {
        s_best = key ? bidx : -1;
        s_bkey = key;
      }
    }
    __syncthreads();
    // ---- 2. candidate row and (owner) row c into this CTA's buffers; the
    // candidate into every CTA's table
    const int tb = s_best >= 0 ? s_best - r0 : -1;
    const int tc = (c >= r0 && c < r0 + nr) ? c - r0 : -1;
    {
      const bool wb = tb >= 0 && (tb >> 5) == warp;
      const bool wc = tc >= 0 && (tc >> 5) == warp;
      if (wb || wc) {
        if (tid == tb || tid == tc) {
#pragma unroll
          for (int k = 0; k < NB; ++k) sL[tid * LD + min(c + k, NB)] = a[k];
        }
        __syncwarp();
        if (wb)
          for (int k = lane; k < NB; k += 32) rowbuf[buf][k] = k < w ? sL[tb * LD + k] : czero<V>();
        if (wc)
          for (int k = lane; k < NB; k += 32) rcbuf[buf][k] = k < w ? sL[tc * LD + k] : czero<V>();
      }
    }
    if (warp == 1 && lane < G) {
      const unsigned long long ent = ((unsigned long long)(unsigned)s_bkey << 32) | (unsigned)(s_best + 1);
      cluster_st_u64(cluster_map(smem_addr(&ctab[buf][bid]), (uint32_t)lane), ent);
    }
    cluster_barrier();
    // ---- 3. the global pivot, the same in every CTA
    if (warp == 0) {
      K bk = 0;
      int bi = kNone;
      if (lane < G) {
        const unsigned long long ent = ctab[buf][lane];
        bk = (K)(ent >> 32);
        bi = bk ? (int)(unsigned)(ent & 0xffffffffu) - 1 : kNone;
      }
      warp_argmax(bk, bi);
      if (lane == 0) s_p = bk ? bi : -1;
    }
    __syncthreads();
    const int p = s_p >= 0 ? s_p : c;
    const int wbk = s_p >= 0 ? s_p / rows_per_cta : -1;
    const int owner = c / rows_per_cta;
    // ---- 4. pivot row and row c from the owning CTAs' shared memory
    for (int i = tid; i < 2 * NB; i += kPanelThreads) {
      V rc = czero<V>(), u = czero<V>();
      if (i < w) {
        const unsigned long long vr = cluster_ld_u64(cluster_map(smem_addr(&rcbuf[buf][i]), (uint32_t)owner));
        rc = make_float2(__uint_as_float((unsigned)vr), __uint_as_float((unsigned)(vr >> 32)));
        if (wbk >= 0) {
          const unsigned long long vu = cluster_ld_u64(cluster_map(smem_addr(&rowbuf[buf][i]), (uint32_t)wbk));
          u = make_float2(__uint_as_float((unsigned)vu), __uint_as_float((unsigned)(vu >> 32)));
        } else {
          u = rc;
        }
      }
      RC[i] = rc;
      U[i] = u;
    }
    __syncthreads();
    const V piv = U[c];
    const bool nz = (piv.x != 0 || piv.y != 0);
    // ---- 5. interchange rows c and p
    if (nz && p != c) {
      const int tp = (p >= r0 && p < r0 + nr) ? p - r0 : -1;
      if (tid < c) {
        if (tp >= 0) sL[tp * LD + tid] = RC[tid];
        if (tc >= 0) sL[tc * LD + tid] = U[tid];
      }
      if (tid == tp || tid == tc) {
        const V* src = tid == tp ? RC : U;
#pragma unroll
        for (int kc = 0; kc < NB; kc += kChunk) {
          if (kc > 0 && c + kc >= w) break;
#pragma unroll
          for (int k = kc; k < kc + kChunk; ++k) a[k] = src[c + k];
        }
      }
    }
    if (bid == 0 && tid == 0) {
      s_piv[c] = nz ? p : c;
      if (!nz && ws.status[1] == 0) ws.status[1] = j0 + c + 1;
    }
    // ---- 6. scale and rank-1 update in registers, retire column c, shift
    if (have && row > c && nz) {
      const V l = cmul(a[0], crecip(piv));
      a[0] = l;
#pragma unroll
      for (int kc = 0; kc < NB; kc += kChunk) {
        if (kc > 0 && c + kc >= w) break;
#pragma unroll
        for (int k = (kc ? kc : 1); k < kc + kChunk; ++k) cfms(a[k], l, U[c + k]);
      }
    }
    if (have) sL[tid * LD + c] = a[0];
#pragma unroll
    for (int kc = 0; kc < NB; kc += kChunk) {
      if (kc > 0 && c + kc >= w) break;
#pragma unroll
      for (int k = kc; k < kc + kChunk && k + 1 < NB; ++k) a[k] = a[k + 1];
    }
  }
  __syncthreads();
  for (int i = tid; i < nr * NB; i += kPanelThreads) {
    const int r = i / NB, k = i % NB;
    if (k < w) A[(int64_t)(r0 + r) * lda + k] = sL[r * LD + k];
  }
  if (bid == 0 && warp == 0) {
    for (int s2 = lane; s2 < NB; s2 += 32) { slot_pos[s2] = s2; slot_src[s2] = s2; }
    if (lane == 0) s_nslot = NB;
    __syncwarp();
    for (int s2 = 0; s2 < w; ++s2) {
      const int pv = s_piv[s2];
      if (pv == s2) continue;
      int slot = -1;
      if (pv < NB) {
        slot = pv;
      } else {
        const int ns = s_nslot;
        for (int base = NB; base < ns && slot < 0; base += 32) {
          int q = base + lane;
          unsigned hit = __ballot_sync(0xffffffffu, q < ns && slot_pos[q] == pv);
          if (hit) slot = base + __ffs(hit) - 1;
        }
        if (slot < 0) {
          slot = ns;
          if (lane == 0) { slot_pos[ns] = pv; slot_src[ns] = pv; s_nslot = ns + 1; }
        }
      }
      __syncwarp();
      if (lane == 0) { int t2 = slot_src[s2]; slot_src[s2] = slot_src[slot]; slot_src[slot] = t2; }
      __syncwarp();
    }
    const int ns = s_nslot;
    for (int q = lane; q < ns; q += 32) ws.slots[q] = make_int2(slot_pos[q], slot_src[q]);
    if (lane == 0) *ws.nslot = ns;
    int32_t pv[2 * NB / 32];
#pragma unroll
    for (int j = 0; j < 2 * NB / 32; ++j) {
      const int q = lane + 32 * j;
      if (q < ns) pv[j] = perm[j0 + slot_src[q]];
    }
    __syncwarp();
#pragma unroll
    for (int j = 0; j < 2 * NB / 32; ++j) {
      const int q = lane + 32 * j;
      if (q < ns) perm[j0 + slot_pos[q]] = pv[j];
    }
  }
  cluster_barrier();   // no CTA leaves while another may still read its shared memory
}

constexpr int kSwapCols = 32;

// run-time tuning knobs (set by the autotuner; see mgt_set_tuning)
static std::atomic<int> g_panel_rows{kPanelRowsTarget};
static std::atomic<int> g_outer_block{128};
// complex64 tensor-core LU with tile pivoting: pair 128-wide blocks (one
// K = 256 trailing update for both) while the trailing order is at least this
static std::atomic<int> g_wide_min{8192};
static std::atomic<int> g_panel_max_ctas{0};     // 0: one per SM
static std::atomic<int> g_cooperative{1};        // panel launched with the cooperative attribute
static std::atomic<int> g_panel_reg{1};          // register-resident panel: 0 never, 1 complex64, 2 both
static std::atomic<int> g_lookahead{1};          // tensor-core LU: next block's panels beside the update
static std::atomic<int> g_fused_right{1};        // tensor-core LU: one fused pass for a block's right columns

// Row interchanges for the columns outside the panel, then (right of the
// panel) U12 = L11^-1 A12 by forward substitution with the unit lower L11.
template <typename T, int NB>
__global__ void __launch_bounds__(256)
lu_swap_trsm_kernel(cplx<T>* __restrict__ A, int64_t lda, int n, int j0, int w, int left_begin, int left_end,
                    int right_begin, int right_end, PanelWs ws, int do_trsm, const cplx<T>* __restrict__ Linv) {
  using V = cplx<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* buf = reinterpret_cast<V*>(smem_raw);   // [2*NB][kSwapCols]
  V* L = buf + 2 * NB * kSwapCols;            // [NB][NB]
  const int tid = threadIdx.x;
  // columns [left_begin, left_end) left of the panel, [right_begin, right_end) right of it
  const int nleft_blocks = max(0, left_end - left_begin + kSwapCols - 1) / kSwapCols;
  const bool right_cols = (int)blockIdx.x >= nleft_blocks;
  const bool right = right_cols && do_trsm;   // columns right of the panel that get the solve
  const int col0 = right_cols ? right_begin + ((int)blockIdx.x - nleft_blocks) * kSwapCols
                              : left_begin + (int)blockIdx.x * kSwapCols;
  const int colend = right_cols ? right_end : left_end;
  const int ncols = min(kSwapCols, colend - col0);
  const int m = n - j0;
  const int ns = min(*ws.nslot, 2 * NB);
  // gather rows slot_src[q] (all slots: the top w rows are needed by the solve)
  // asynchronous copies: every load of this stage in flight at once
  for (int idx = tid; idx < ns * kSwapCols; idx += blockDim.x) {
    int q = idx / kSwapCols, cc = idx - q * kSwapCols;
    int2 sl = ws.slots[q];
    bool inb = sl.x >= 0 && sl.x < m && sl.y >= 0 && sl.y < m;
    bool need = inb && ((sl.x != sl.y) || (right && sl.x < w));
    if (cc < ncols && need)
      cp_async_elem<(int)sizeof(V)>(buf + q * kSwapCols + cc, A + (int64_t)(j0 + sl.y) * lda + col0 + cc, true);
  }
  if (right) {
    // L11 from the factor, or (tile pivoting) its inverse from the tile kernel
    for (int idx = tid; idx < w * w; idx += blockDim.x) {
      int i = idx / w, k = idx - i * w;
      cp_async_elem<(int)sizeof(V)>(L + i * NB + k, Linv ? Linv + i * NB + k : A + (int64_t)(j0 + i) * lda + j0 + k,
                                    true);
    }
  }
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();
  if (right && Linv) {
    // U12 = L11^-1 X: thread = (column cc, rows i0 + 8 m), products independent
    // across threads (no chain over the rows)
    const int cc = tid & 31, i0 = tid >> 5;
    V acc[NB / 8];
#pragma unroll
    for (int m = 0; m < NB / 8; ++m) acc[m] = czero<V>();
    for (int k = 0; k < w; ++k) {
      const V xk = buf[k * kSwapCols + cc];
#pragma unroll
      for (int m = 0; m < NB / 8; ++m) cfma(acc[m], L[(i0 + 8 * m) * NB + k], xk);
    }
    __syncthreads();
#pragma unroll
    for (int m = 0; m < NB / 8; ++m)
      if (i0 + 8 * m < w && cc < kSwapCols) buf[(i0 + 8 * m) * kSwapCols + cc] = acc[m];
    __syncthreads();
  } else if (right) {
    // 8 lanes per column: lane = col_local * 8 + t8, 4 columns per warp
    const int warp = tid >> 5, lane = tid & 31;
    const int cc = warp * 4 + (lane >> 3), t8 = lane & 7;
    if (cc < kSwapCols) {
      for (int k = 0; k < w - 1; ++k) {
        __syncwarp();
        const V xk = buf[k * kSwapCols + cc];
        for (int i = k + 1 + t8; i < w; i += 8) cfms(buf[i * kSwapCols + cc], L[i * NB + k], xk);
      }
    }
    __syncthreads();
  }
  // scatter: moved rows, and (right of the panel) the solved top w rows
  for (int idx = tid; idx < ns * kSwapCols; idx += blockDim.x) {
    int q = idx / kSwapCols, cc = idx - q * kSwapCols;
    int2 sl = ws.slots[q];
    bool inb = sl.x >= 0 && sl.x < m && sl.y >= 0 && sl.y < m;
    bool moved = sl.x != sl.y;
    bool top = right && sl.x < w;
    if (cc < ncols && inb && (moved || top)) A[(int64_t)(j0 + sl.x) * lda + col0 + cc] = buf[q * kSwapCols + cc];
  }
}

// Second inner panel of a 128-wide block, columns right of the block:
// rows j1 .. j1+wb of those columns get the first inner panel's update
// (B -= L_ba U_a) and then U12 = L_bb^-1 B.  The row interchanges of the
// second panel have already been applied to every column.
template <typename T, int NB>
__global__ void __launch_bounds__(256)
lu_preupdate_trsm_kernel(cplx<T>* __restrict__ A, int64_t lda, int n, int J0, int wa, int j1, int wb, int col_begin) {
  using V = cplx<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* buf = reinterpret_cast<V*>(smem_raw);    // [NB][kSwapCols]
  V* Lba = buf + NB * kSwapCols;               // [NB][NB + 1]
  V* Ua = Lba + NB * (NB + 1);                 // [NB][kSwapCols]
  const int tid = threadIdx.x;
  const int col0 = col_begin + blockIdx.x * kSwapCols;
  const int ncols = min(kSwapCols, n - col0);
  for (int idx = tid; idx < wb * kSwapCols; idx += 256) {
    int r = idx / kSwapCols, cc = idx - r * kSwapCols;
    const bool ok = cc < ncols;
    cp_async_elem<(int)sizeof(V)>(buf + r * kSwapCols + cc, ok ? A + (int64_t)(j1 + r) * lda + col0 + cc : A, ok);
  }
  for (int idx = tid; idx < wb * wa; idx += 256) {
    int r = idx / wa, k = idx - r * wa;
    cp_async_elem<(int)sizeof(V)>(Lba + r * (NB + 1) + k, A + (int64_t)(j1 + r) * lda + J0 + k, true);
  }
  for (int idx = tid; idx < wa * kSwapCols; idx += 256) {
    int k = idx / kSwapCols, cc = idx - k * kSwapCols;
    const bool ok = cc < ncols;
    cp_async_elem<(int)sizeof(V)>(Ua + k * kSwapCols + cc, ok ? A + (int64_t)(J0 + k) * lda + col0 + cc : A, ok);
  }
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();
  // buf -= Lba * Ua: thread owns column cc = tid % 32 and rows tid / 32 + 8 q
  {
    const int cc = tid & 31, rq = tid >> 5;
    for (int r = rq; r < wb; r += 8) {
      V acc = buf[r * kSwapCols + cc];
      for (int k = 0; k < wa; ++k) cfms(acc, Lba[r * (NB + 1) + k], Ua[k * kSwapCols + cc]);
      buf[r * kSwapCols + cc] = acc;
    }
  }
  __syncthreads();
  // L_bb (unit lower) into the Lba area, then forward substitution
  for (int idx = tid; idx < wb * wb; idx += 256) {
    int i = idx / wb, k = idx - i * wb;
    Lba[i * (NB + 1) + k] = A[(int64_t)(j1 + i) * lda + j1 + k];
  }
  __syncthreads();
  {
    const int warp = tid >> 5, lane = tid & 31;
    const int cc = warp * 4 + (lane >> 3), t8 = lane & 7;
    for (int k = 0; k < wb - 1; ++k) {
      __syncwarp();
      const V xk = buf[k * kSwapCols + cc];
      for (int i = k + 1 + t8; i < wb; i += 8) cfms(buf[i * kSwapCols + cc], Lba[i * (NB + 1) + k], xk);
    }
  }
  __syncthreads();
  for (int idx = tid; idx < wb * kSwapCols; idx += 256) {
    int r = idx / kSwapCols, cc = idx - r * kSwapCols;
    if (cc < ncols) A[(int64_t)(j1 + r) * lda + col0 + cc] = buf[r * kSwapCols + cc];
  }
}

template <typename T>
int lower_block_inverses(const cplx<T>* F, int64_t ldf, int n, cplx<T>* Inv, cudaStream_t s);

// dynamic shared memory of lu_block_right_kernel: block rows, moved rows, one operator
template <int NB>
constexpr size_t block_right_smem(size_t elem) {
  return ((size_t)2 * NB * kSwapCols + (size_t)4 * NB * kSwapCols + (size_t)NB * (NB + 1)) * elem;
}

// Columns right of a 128-wide block whose inner panels sit at J0 (width wa)
// and j1 = J0 + wa (width wb), in one pass per 32 columns: both panels' row
// interchanges (slot sets A and B, composed), then U_A = L_AA^-1 X_A,
// X_B -= L_BA U_A and U_B = L_BB^-1 X_B with the diagonal blocks' inverses
// precomputed (Inv[0] = L_AA^-1, Inv[1] = L_BB^-1).  The same arithmetic as
// the two swap passes and the pre-update pass it replaces, with the
// triangular solves as products with the inverses.
template <typename T, int NB>
__global__ void __launch_bounds__(256)
lu_block_right_kernel(cplx<T>* __restrict__ A, int64_t lda, int n, int J0, int wa, int wb, int col_begin,
                      PanelWs wsA, PanelWs wsB, const cplx<T>* __restrict__ Inv) {
  using V = cplx<T>;
  constexpr int CW = kSwapCols;
  constexpr int MAXF = 4 * NB;                 // moved rows below the block (both slot sets)
  static_assert(NB == 64 && CW == 32 && 256 == 4 * NB, "thread tiling: 32 x 2 rows, 8 x 4 columns");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* Tb = reinterpret_cast<V*>(smem_raw);      // [2 NB][CW] the block's rows
  V* Fr = Tb + 2 * NB * CW;                    // [MAXF][CW] moved rows below the block
  V* Lb = Fr + MAXF * CW;                      // [NB][NB + 1] operator of the current step
  __shared__ int tsrc[2 * NB];                 // source (rel J0) of each block row
  __shared__ int fpos[MAXF], fsrc[MAXF];       // moved rows below the block: position, source (rel J0)
  __shared__ int s_nf;
  const int tid = threadIdx.x;
  const int W = wa + wb;
  const int col0 = col_begin + blockIdx.x * CW;
  const int ncols = min(CW, n - col0);
  const int m = n - J0;
  const int nsA = min(*wsA.nslot, 2 * NB);
  const int nsB = wb > 0 ? min(*wsB.nslot, 2 * NB) : 0;
  // source (rel J0) of position x (rel J0) after panel A's interchanges
  auto srcA = [&](int x) -> int {
    if (x < NB) return x < nsA ? wsA.slots[x].y : x;
    for (int q = NB; q < nsA; ++q)
      if (wsA.slots[q].x == x) return wsA.slots[q].y;
    return x;
  };
  // source (rel J0) of position p (rel J0) after both panels' interchanges
  auto src_both = [&](int p) -> int {
    int mid = p;
    if (wb > 0 && p >= wa) {
      const int y = p - wa;
      if (y < NB) {
        if (y < nsB) mid = wsB.slots[y].y + wa;
      } else {
        for (int q = NB; q < nsB; ++q)
          if (wsB.slots[q].x == y) { mid = wsB.slots[q].y + wa; break; }
      }
    }
    return srcA(mid);
  };
  if (tid == 0) s_nf = 0;
  __syncthreads();
  // positions below the block that either panel touches: A's (rel J0) and B's (rel j1)
  for (int q = tid; q < nsA + nsB; q += blockDim.x) {
    const bool isA = q < nsA;
    const int2 sl = isA ? wsA.slots[q] : wsB.slots[q - nsA];
    const int p = isA ? sl.x : sl.x + wa;
    if (p < W || p >= m) continue;
    bool dup = false;
    if (!isA)   // a position in both lists is taken from A's
      for (int r = 0; r < nsA && !dup; ++r) dup = wsA.slots[r].x == p;
    if (!dup) {
      const int k = atomicAdd(&s_nf, 1);
      if (k < MAXF) fpos[k] = p;
    }
  }
  for (int r = tid; r < W; r += blockDim.x) tsrc[r] = src_both(r);
  __syncthreads();
  const int nf = min(s_nf, MAXF);
  for (int f = tid; f < nf; f += blockDim.x) fsrc[f] = src_both(fpos[f]);
  __syncthreads();
  // gather every source before anything is written (asynchronous copies, all in flight)
  for (int idx = tid; idx < 2 * NB * CW; idx += blockDim.x) {
    const int r = idx / CW, c = idx - r * CW;
    const bool ok = r < W && c < ncols;
    cp_async_elem<(int)sizeof(V)>(Tb + idx, ok ? A + (int64_t)(J0 + tsrc[r]) * lda + col0 + c : A, ok);
  }
  for (int idx = tid; idx < nf * CW; idx += blockDim.x) {
    const int f = idx / CW, c = idx - f * CW;
    if (c < ncols) cp_async_elem<(int)sizeof(V)>(Fr + idx, A + (int64_t)(J0 + fsrc[f]) * lda + col0 + c, true);
  }
  for (int idx = tid; idx < NB * NB; idx += blockDim.x) {
    const int r = idx / NB, k = idx - r * NB;
    cp_async_elem<(int)sizeof(V)>(Lb + r * (NB + 1) + k, Inv + idx, true);
  }
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();
  for (int idx = tid; idx < nf * CW; idx += blockDim.x) {
    const int f = idx / CW, c = idx - f * CW;
    if (c < ncols) A[(int64_t)(J0 + fpos[f]) * lda + col0 + c] = Fr[idx];
  }
  // Y (NB rows of Tb from row0) = Lb * Y, or Y -= Lb * X (X = the first NB
  // rows); each thread a 2 x 4 tile: rows 2 tr, 2 tr + 1, columns tc + 8 j
  auto apply = [&](int row0, bool sub) {
    const int tr = tid >> 3, tc = tid & 7;
    const V* X = sub ? Tb : Tb + row0 * CW;
    V acc[2][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] = sub ? Tb[(row0 + 2 * tr + i) * CW + tc + 8 * j] : czero<V>();
#pragma unroll 4
    for (int k = 0; k < NB; ++k) {
      const V l0 = Lb[(2 * tr) * (NB + 1) + k], l1 = Lb[(2 * tr + 1) * (NB + 1) + k];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const V x = X[k * CW + tc + 8 * j];
        if (sub) {
          cfms(acc[0][j], l0, x);
          cfms(acc[1][j], l1, x);
        } else {
          cfma(acc[0][j], l0, x);
          cfma(acc[1][j], l1, x);
        }
      }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) Tb[(row0 + 2 * tr + i) * CW + tc + 8 * j] = acc[i][j];
    __syncthreads();
  };
  apply(0, false);                                   // U_A = L_AA^-1 X_A
  if (wb > 0) {
    for (int idx = tid; idx < NB * NB; idx += blockDim.x) {
      const int r = idx / NB, k = idx - r * NB;
      const bool ok = r < wb && k < wa;
      cp_async_elem<(int)sizeof(V)>(Lb + r * (NB + 1) + k, ok ? A + (int64_t)(J0 + wa + r) * lda + J0 + k : A, ok);
    }
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();
    apply(NB, true);                                 // X_B -= L_BA U_A
    for (int idx = tid; idx < NB * NB; idx += blockDim.x) {
      const int r = idx / NB, k = idx - r * NB;
      cp_async_elem<(int)sizeof(V)>(Lb + r * (NB + 1) + k, Inv + NB * NB + idx, true);
    }
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();
    apply(NB, false);                                // U_B = L_BB^-1 X_B
  }
  for (int idx = tid; idx < W * CW; idx += blockDim.x) {
    const int r = idx / CW, c = idx - r * CW;
    const int rr = r < wa ? r : NB + (r - wa);
    if (c < ncols) A[(int64_t)(J0 + r) * lda + col0 + c] = Tb[rr * CW + c];
  }
}

// perm = identity; the factorisation epoch moves on by one; the panel records'
// flags are cleared (the complex64 panel's short column tags rely on it)
__global__ void lu_start_kernel(int32_t* perm, int n, unsigned long long* epoch, unsigned char* records) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) perm[i] = i;
  if (i == 0) *epoch += 1;
  for (int r = i; r < 2 * kMaxPanelBlocks; r += gridDim.x * blockDim.x)
    *reinterpret_cast<unsigned long long*>(records + (size_t)r * kRecBytes) = 0ull;
}

static int num_sms() { return device_sm_count(); }

// Trailing update: tensor cores (tcgen05 TF32x3) for complex64 when a plan is
// given, SIMT otherwise (complex128, or no tensor-core scratch).
struct TcLU {
  TcPlan plan;
  CUtensorMap cmap;   // the whole matrix being factored
};
static int trailing_update(const TcLU* tc, int M, int N, int K, const double2* A, int64_t lda, const double2* B,
                           int64_t ldb, double2* C, int64_t ldc, int, int*, cudaStream_t s, int) {
  (void)tc;
  return gemm_sub<double>(M, N, K, A, lda, B, ldb, C, ldc, s);
}
static int trailing_update(const TcLU* tc, int M, int N, int K, const float2* A, int64_t lda, const float2* B,
                           int64_t ldb, float2* C, int64_t ldc, int c0, int* status, cudaStream_t s, int max_ctas) {
  if (tc) return gemm_sub_tc(tc->plan, tc->cmap, M, N, K, A, lda, B, ldb, 2 * c0, c0, status, s, max_ctas);
  return gemm_sub<float>(M, N, K, A, lda, B, ldb, C, ldc, s);
}

static std::atomic<int> g_panel_cluster{1};     // complex64 panels of <= 16 CTAs as one cluster

// Options of one factorisation: the process-wide tuning values, overridden
// by the caller's mgt_lu_options where given.
struct LuOpts {
  int pivoting = MGT_PIVOT_PARTIAL;
  int panel_rows, outer_block, panel_max_ctas, cooperative, panel_reg, lookahead, fused_right, panel_cluster;
  int wide_min;
  LuOpts() {
    panel_rows = g_panel_rows.load(std::memory_order_relaxed);
    outer_block = g_outer_block.load(std::memory_order_relaxed);
    panel_max_ctas = g_panel_max_ctas.load(std::memory_order_relaxed);
    cooperative = g_cooperative.load(std::memory_order_relaxed);
    panel_reg = g_panel_reg.load(std::memory_order_relaxed);
    lookahead = g_lookahead.load(std::memory_order_relaxed);
    fused_right = g_fused_right.load(std::memory_order_relaxed);
    panel_cluster = g_panel_cluster.load(std::memory_order_relaxed);
    wide_min = g_wide_min.load(std::memory_order_relaxed);
  }
};

static int resolve_lu_options(const mgt_lu_options* o, LuOpts* r) {
  if (!o) return MGT_OK;
  if (o->size < (int32_t)sizeof(mgt_lu_options)) return MGT_ERR_ARG;
  if (o->pivoting != MGT_PIVOT_PARTIAL && o->pivoting != MGT_PIVOT_TILE) return MGT_ERR_ARG;
  r->pivoting = o->pivoting;
  if (o->panel_rows > 0) {
    if (o->panel_rows < 32 || o->panel_rows > 4096) return MGT_ERR_ARG;
    r->panel_rows = o->panel_rows;
  }
  if (o->panel_max_ctas > 0) r->panel_max_ctas = std::min(o->panel_max_ctas, 4096);
  if (o->cooperative >= 0) r->cooperative = o->cooperative ? 1 : 0;
  if (o->lookahead >= 0) r->lookahead = o->lookahead ? 1 : 0;
  if (o->outer_block > 0) {
    if (o->outer_block != 64 && o->outer_block != 128) return MGT_ERR_ARG;
    r->outer_block = o->outer_block;
  }
  return MGT_OK;
}

// ---------------------------------------------------------------- tile-pivoting panel (complex64)
//
// MGT_PIVOT_TILE: the pivots of a 64-column panel are chosen among the rows
// of its diagonal tile.  lu_tile_kernel (one CTA) factors the w x w tile with
// partial pivoting among the tile's rows, records the interchanges in the slot
// format of the panel kernels (the swap kernels then apply them to the other
// columns) and in perm, and writes U11^-1; lu_l21_kernel solves every row below
// the tile, L21 = A21 U11^-1, with no exchange between CTAs.  The system
// matrices of this engine rarely need a pivot from outside the tile (LAPACK
// swaps a few rows in a thousand there); the growth that remains is what
// iterative refinement absorbs.
constexpr int kTileLD = 65;   // padded row stride of the tile in shared memory
// dynamic shared memory of lu_tile_kernel: the tile by row and by position,
// two inversion scratch blocks, the staged candidate rows
constexpr int kCandLD = 128;  // a staged candidate row: columns 4 (j + k) + g < 128
constexpr size_t kTileSmem = (2 * 64 * kTileLD + 2 * 32 * 33 + 2 * 8 * kCandLD) * sizeof(float2);

// 1/z for the tile's pivots: Smith's scaling with two correctly rounded
// reciprocals instead of three divisions (each result within a few ulp of
// the quotient; the LU is only FP32-accurate and the mixed method's
// refinement certifies the solution)
__device__ __forceinline__ float2 crecip_tile(float2 z) {
  if (fabsf(z.x) >= fabsf(z.y)) {
    const float r = z.y * __frcp_rn(z.x), inv = __frcp_rn(fmaf(z.y, r, z.x));
    return make_float2(inv, -r * inv);
  }
  const float r = z.x * __frcp_rn(z.y), inv = __frcp_rn(fmaf(z.x, r, z.y));
  return make_float2(r * inv, -inv);
}

// One level of the recursion, blocks of h = 2^LH rows: the (up to 8) items of
// a thread are interleaved inside the k loop, so their dependent chains of
// multiply-adds overlap (item = (block q, row i, column j), upper items first)
template <int LH>
__device__ __forceinline__ void tile_inv_level(float2* T, float2* S1, float2* S2, int tid) {
  constexpr int h = 1 << LH, per = h * h, tot = 32 * h, M = (2 * tot + 255) / 256;
  int qi[M], ii[M], jj[M];
  bool val[M], up[M];
  float2 acc[M];
#pragma unroll
  for (int m = 0; m < M; ++m) {
    const int e = tid + 256 * m;
    val[m] = e < 2 * tot;
    up[m] = e < tot;
    const int f = up[m] ? e : e - tot;
    qi[m] = f >> (2 * LH);
    ii[m] = (f >> LH) & (h - 1);
    jj[m] = f & (h - 1);
  }
  // step 1: S1 = A^-1 B (upper), S2 = B A^-1 (lower; A^-1 unit lower, diagonal 1)
#pragma unroll
  for (int m = 0; m < M; ++m) {
    const int b = 2 * h * qi[m];
    acc[m] = (val[m] && !up[m]) ? T[(b + h + ii[m]) * kTileLD + b + jj[m]] : make_float2(0.f, 0.f);
  }
#pragma unroll 4
  for (int k = 0; k < h; ++k) {
#pragma unroll
    for (int m = 0; m < M; ++m) {
      const int b = 2 * h * qi[m];
      if (val[m] && up[m] && k >= ii[m])
        cfma(acc[m], T[(b + ii[m]) * kTileLD + b + k], T[(b + k) * kTileLD + b + h + jj[m]]);
      if (val[m] && !up[m] && k > jj[m])
        cfma(acc[m], T[(b + h + ii[m]) * kTileLD + b + k], T[(b + k) * kTileLD + b + jj[m]]);
    }
  }
#pragma unroll
  for (int m = 0; m < M; ++m)
    if (val[m]) (up[m] ? S1 : S2)[qi[m] * per + ii[m] * h + jj[m]] = acc[m];
  __syncthreads();
  // step 2: B <- -(S1 C^-1) (upper), B <- -(C^-1 S2) (lower)
#pragma unroll
  for (int m = 0; m < M; ++m)
    acc[m] = (val[m] && !up[m]) ? S2[qi[m] * per + ii[m] * h + jj[m]] : make_float2(0.f, 0.f);
#pragma unroll 4
  for (int k = 0; k < h; ++k) {
#pragma unroll
    for (int m = 0; m < M; ++m) {
      const int b = 2 * h * qi[m];
      if (val[m] && up[m] && k <= jj[m])
        cfma(acc[m], S1[qi[m] * per + ii[m] * h + k], T[(b + h + k) * kTileLD + b + h + jj[m]]);
      if (val[m] && !up[m] && k < ii[m])
        cfma(acc[m], T[(b + h + ii[m]) * kTileLD + b + h + k], S2[qi[m] * per + k * h + jj[m]]);
    }
  }
#pragma unroll
  for (int m = 0; m < M; ++m) {
    if (!val[m]) continue;
    const int b = 2 * h * qi[m];
    const float2 v = make_float2(-acc[m].x, -acc[m].y);
    if (up[m]) T[(b + ii[m]) * kTileLD + b + h + jj[m]] = v;
    else T[(b + h + ii[m]) * kTileLD + b + jj[m]] = v;
  }
  __syncthreads();
}

// In-place inverses of the upper triangle U (diagonal included) and of the
// unit lower triangle L (strict lower part) of the 64 x 64 tile T, by block
// recursion: for a block [[A, B], [0, C]] of U, the off-diagonal block of the
// inverse is -(A^-1 B) C^-1; for [[A, 0], [B, C]] of L it is -C^-1 (B A^-1).
// Level h combines 32 / h pairs of inverted h x h blocks; 256 threads.
// A zero diagonal entry of U inverts to zero (the factorisation has already
// recorded it as a zero pivot).
__device__ void tile_triangular_inverses(float2* T, float2* S1, float2* S2, int tid) {
  for (int i = tid; i < 64; i += 256) {
    const float2 u = T[i * kTileLD + i];
    T[i * kTileLD + i] = (u.x != 0.f || u.y != 0.f) ? crecip_tile(u) : make_float2(0.f, 0.f);
  }
  __syncthreads();
  tile_inv_level<0>(T, S1, S2, tid);
  tile_inv_level<1>(T, S1, S2, tid);
  tile_inv_level<2>(T, S1, S2, tid);
  tile_inv_level<3>(T, S1, S2, tid);
  tile_inv_level<4>(T, S1, S2, tid);
  tile_inv_level<5>(T, S1, S2, tid);
}

// One CTA of 256 threads; thread (r, g) = (tid / 4, tid % 4) holds the
// columns g, g + 4, ... of tile row r in registers, a[k] = column 4 (j + k) + g
// after j shifts (every fourth column), so register indices stay compile-time
// constants and no loop has a data-dependent bound.  Per column c, with one
// block barrier: the holders of column c bid |re| + |im| (lowest tile row on
// ties); each warp's best row stages itself in cand[warp] before the barrier;
// after it every thread reads the eight bids, the winner retires (its staged
// row is row c of U), and the other rows compute their multiplier and update.
// Rows never move between threads: the row chosen at column c goes to
// position c, which gives the interchange slots directly.  Then all warps
// invert U11 and L11 in place, for the rows below (L21 = A21 U11^-1) and the
// columns to the right (U12 = L11^-1 A12).
__global__ void __launch_bounds__(256, 1)
lu_tile_kernel(float2* __restrict__ A, int64_t lda, int w, int j0, int32_t* __restrict__ perm, PanelWs ws,
               float2* __restrict__ Uinv, float2* __restrict__ Linv) {
  // A: the tile's top-left element (row j0, column j0); w <= 64
  extern __shared__ __align__(16) unsigned char tile_smem[];
  float2* T = reinterpret_cast<float2*>(tile_smem);    // [64][kTileLD]: the tile, then the multipliers by tile row
  float2* F = T + 64 * kTileLD;                         // [64][kTileLD], row q = position q
  float2* S1 = F + 64 * kTileLD;
  float2* S2 = S1 + 32 * 33;
  float2* cand = S2 + 32 * 33;                          // [2][8][kCandLD]: each warp's best row, by column parity
  __shared__ uint32_t s_key[2][8];
  __shared__ int s_row[2][8];
  __shared__ float2 s_inv[2][8];                       // 1 / each warp's candidate pivot
  __shared__ int s_piv[64];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int r = tid >> 2, g = tid & 3;
  for (int idx = tid; idx < 64 * 64; idx += 256) {
    const int i = idx >> 6, k = idx & 63;
    const bool in = i < w && k < w;
    cp_async_elem<8>(T + i * kTileLD + k, in ? A + (int64_t)i * lda + k : A, in);
  }
  cp_async_commit();
  if (tid < 64) s_piv[tid] = tid;
  cp_async_wait<0>();
  __syncthreads();
  float2 a[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) a[k] = T[r * kTileLD + 4 * k + g];
  bool active = r < w;
  for (int j = 0; j < 16 && 4 * j < w; ++j) {
    // not unrolled: u only selects threads, and one copy of the column body
    // keeps the loop within the instruction cache
#pragma unroll 1
    for (int u = 0; u < 4; ++u) {
      const int c = 4 * j + u;
      if (c >= w) break;
      const int buf = c & 1;
      float2* cb = cand + buf * 8 * kCandLD;
      // bid: key 0 = no bid; +1 keeps the rows of a zero column valid bidders
      const uint32_t key = (active && g == u) ? __float_as_uint(fabsf(a[0].x) + fabsf(a[0].y)) + 1u : 0u;
      const uint32_t mx = __reduce_max_sync(0xffffffffu, key);
      const uint32_t ml = __reduce_min_sync(0xffffffffu, (key == mx && mx != 0u) ? (uint32_t)lane : 32u);
      if (mx != 0u && (lane >> 2) == (int)(ml >> 2)) {
#pragma unroll
        for (int k = 0; k < 16; ++k) cb[warp * kCandLD + 4 * (j + k) + g] = a[k];
        // the candidate's reciprocal before the barrier, off the chain after it
        if (g == u) {
          const bool z = a[0].x == 0.f && a[0].y == 0.f;
          s_inv[buf][warp] = z ? make_float2(0.f, 0.f) : crecip_tile(a[0]);
        }
      }
      if (lane == 0) {
        s_key[buf][warp] = mx;
        s_row[buf][warp] = warp * 8 + (int)(ml >> 2);
      }
      __syncthreads();
      // the winning warp: largest bid, lowest warp (lowest rows) on ties; lanes
      // 0..7 read one bid each and two warp reductions decide
      const uint32_t kq = lane < 8 ? s_key[buf][lane] : 0u;
      const uint32_t kmax = __reduce_max_sync(0xffffffffu, kq);
      const int best = (int)__reduce_min_sync(0xffffffffu, (lane < 8 && kq == kmax) ? (uint32_t)lane : 8u);
      const int p = s_row[buf][best];
      const float2* prow = cb + best * kCandLD;
      const float2 pinv = s_inv[buf][best];
      if (r == p) {
        if (g == 0) {
          s_piv[c] = r;
          const float2 piv = prow[c];
          if (piv.x == 0.f && piv.y == 0.f && ws.status[1] == 0) ws.status[1] = j0 + c + 1;
        }
        active = false;
      }
      float2 l = g == u ? cmul(a[0], pinv) : make_float2(0.f, 0.f);
      l.x = __shfl_sync(0xffffffffu, l.x, (lane & ~3) | u);
      l.y = __shfl_sync(0xffffffffu, l.y, (lane & ~3) | u);
      if (active) {
        if (g == u) T[r * kTileLD + c] = l;
#pragma unroll
        for (int k = 0; k < 16; ++k) cfms(a[k], l, prow[4 * (j + k) + g]);
      }
      // row c of U (read from the staged row until the next column's barrier)
      if (tid < 64 && tid >= c) F[c * kTileLD + tid] = prow[tid];
    }
#pragma unroll
    for (int k = 0; k < 15; ++k) a[k] = a[k + 1];
  }
  __syncthreads();
  // the multipliers in position order (position q holds tile row s_piv[q]);
  // identity beyond w (the last panel)
  for (int idx = tid; idx < 64 * 64; idx += 256) {
    const int q = idx >> 6, k = idx & 63;
    if (q >= w) F[q * kTileLD + k] = make_float2(q == k ? 1.f : 0.f, 0.f);
    else if (k < q) F[q * kTileLD + k] = T[s_piv[q] * kTileLD + k];
  }
  __syncthreads();
  for (int idx = tid; idx < 64 * 64; idx += 256) {
    const int q = idx >> 6, k = idx & 63;
    if (q < w && k < w) A[(int64_t)q * lda + k] = F[q * kTileLD + k];
  }
  if (warp == 0) {
    for (int q = lane; q < kNBmax; q += 32) ws.slots[q] = make_int2(q, q < w ? s_piv[q] : q);
    if (lane == 0) *ws.nslot = kNBmax;
    int32_t pv[2];
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int q = lane + 32 * j;
      if (q < w) pv[j] = perm[j0 + s_piv[q]];
    }
    __syncwarp();
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int q = lane + 32 * j;
      if (q < w) perm[j0 + q] = pv[j];
    }
  }
  __syncthreads();
  tile_triangular_inverses(F, S1, S2, tid);
  for (int idx = tid; idx < 64 * 64; idx += 256) {
    const int i = idx >> 6, k = idx & 63;
    const float2 v = F[i * kTileLD + k];
    const bool inw = i < w && k < w;
    Uinv[idx] = (inw && k >= i) ? v : make_float2(0.f, 0.f);
    Linv[idx] = (inw && k < i) ? v : make_float2(i == k ? 1.f : 0.f, 0.f);
  }
}

// Rows below the first tile of a 128-wide block (tile pivoting), fused:
// L21 = A21 U11^-1 on the first panel's w columns, then the second panel's wb
// columns A22 -= L21 U12 (U12: the first panel's rows of those columns,
// already solved).  32 rows per CTA, thread = (row, every eighth column).
__global__ void __launch_bounds__(256)
lu_l21_update_kernel(float2* __restrict__ A, int64_t lda, int rows, int w, int wb, const float2* __restrict__ Uinv,
                     const float2* __restrict__ U12) {
  // A: first row below the tile, first column of the panel; U12: the panel's
  // first row, first column of the second panel
  extern __shared__ __align__(16) unsigned char fused_smem[];
  float2* Ui = reinterpret_cast<float2*>(fused_smem);   // [64][64]
  float2* Us = Ui + 64 * 64;                             // [64][64] U12
  float2* Ar = Us + 64 * 64;                             // [32][64] A21, then L21
  float2* Cr = Ar + 32 * 64;                             // [32][64] A22
  const int tid = threadIdx.x, r0 = blockIdx.x * 32;
  for (int idx = tid; idx < 64 * 32; idx += 256) cp_async_elem<16>(Ui + 2 * idx, Uinv + 2 * idx, true);
  for (int idx = tid; idx < 64 * 64; idx += 256) {
    const int k = idx >> 6, c = idx & 63;
    const bool in = k < w && c < wb;
    cp_async_elem<8>(Us + idx, in ? U12 + (int64_t)k * lda + c : U12, in);
  }
  for (int idx = tid; idx < 32 * 64; idx += 256) {
    const int r = idx >> 6, k = idx & 63;
    const bool ra = r0 + r < rows && k < w, rc = r0 + r < rows && k < wb;
    cp_async_elem<8>(Ar + idx, ra ? A + (int64_t)(r0 + r) * lda + k : A, ra);
    cp_async_elem<8>(Cr + idx, rc ? A + (int64_t)(r0 + r) * lda + w + k : A, rc);
  }
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();
  const int r = tid >> 3, g = tid & 7;
  float2 acc[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) acc[q] = make_float2(0.f, 0.f);
  for (int i = 0; i < w; ++i) {
    const float2 a = Ar[r * 64 + i];
#pragma unroll
    for (int q = 0; q < 8; ++q) cfma(acc[q], a, Ui[i * 64 + g + 8 * q]);
  }
  __syncthreads();   // every thread has read its row of A21
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int k = g + 8 * q;
    Ar[r * 64 + k] = acc[q];
    if (r0 + r < rows && k < w) A[(int64_t)(r0 + r) * lda + k] = acc[q];
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < 8; ++q) acc[q] = Cr[r * 64 + g + 8 * q];
  for (int k = 0; k < w; ++k) {
    const float2 l = Ar[r * 64 + k];
#pragma unroll
    for (int q = 0; q < 8; ++q) cfms(acc[q], l, Us[k * 64 + g + 8 * q]);
  }
  if (r0 + r < rows) {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int c = g + 8 * q;
      if (c < wb) A[(int64_t)(r0 + r) * lda + w + c] = acc[q];
    }
  }
}
constexpr size_t kL21UpdateSmem = (2 * 64 * 64 + 2 * 32 * 64) * sizeof(float2);

// The interchanges of tile t (rows 64 t .., position q holds tile row
// perm[64 t + q] - 64 t: rows move only within their tile) on the columns
// left of the tile's outer block, which the panels left alone.  Block
// (32 columns, tile): gather the tile's rows through shared memory, write
// them back in order.
__global__ void __launch_bounds__(256)
lu_tile_left_perm_kernel(float2* __restrict__ A, int64_t lda, int n, const int32_t* __restrict__ perm, int outer) {
  __shared__ float2 buf[64][33];
  const int j0 = blockIdx.y * 64, w = min(64, n - j0);
  const int jb = j0 / outer * outer, c0 = blockIdx.x * 32;
  if (c0 >= jb) return;
  const int ncols = min(32, jb - c0);
  const int tid = threadIdx.x;
  for (int idx = tid; idx < w * 32; idx += 256) {
    const int q = idx >> 5, cc = idx & 31;
    const int src = perm[j0 + q] - j0;
    if (cc < ncols && src >= 0 && src < w) buf[q][cc] = A[(int64_t)(j0 + src) * lda + c0 + cc];
  }
  __syncthreads();
  for (int idx = tid; idx < w * 32; idx += 256) {
    const int q = idx >> 5, cc = idx & 31;
    const int src = perm[j0 + q] - j0;
    if (cc < ncols && src >= 0 && src < w && src != q) A[(int64_t)(j0 + q) * lda + c0 + cc] = buf[q][cc];
  }
}

// Rows below the tile: A21 <- A21 U11^-1 (w columns), 32 rows per CTA; the
// operands are staged with asynchronous copies (all in flight at once).
__global__ void __launch_bounds__(256)
lu_l21_kernel(float2* __restrict__ A, int64_t lda, int rows, int w, const float2* __restrict__ Uinv) {
  // A: first row below the tile, first column of the panel
  __shared__ __align__(16) float2 Ui[64 * 64];
  __shared__ __align__(16) float2 Ar[32 * 64];
  const int tid = threadIdx.x, r0 = blockIdx.x * 32;
  for (int idx = tid; idx < 64 * 32; idx += 256) cp_async_elem<16>(Ui + 2 * idx, Uinv + 2 * idx, true);
  for (int idx = tid; idx < 32 * 64; idx += 256) {
    const int r = idx >> 6, k = idx & 63;
    const bool in = r0 + r < rows && k < w;
    cp_async_elem<8>(Ar + idx, in ? A + (int64_t)(r0 + r) * lda + k : A, in);
  }
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();
  const int r = tid >> 3, g = tid & 7;
  float2 acc[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) acc[q] = make_float2(0.f, 0.f);
  for (int i = 0; i < w; ++i) {
    const float2 a = Ar[r * 64 + i];
#pragma unroll
    for (int q = 0; q < 8; ++q) cfma(acc[q], a, Ui[i * 64 + g + 8 * q]);
  }
  if (r0 + r < rows) {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int k = g + 8 * q;
      if (k < w) A[(int64_t)(r0 + r) * lda + k] = acc[q];
    }
  }
}

// Largest cluster of register panel CTAs the device schedules (16, 8 or 0).
static int cluster_panel_max() {
  static int cmax_dev[kMaxDevices];
  static OncePerDevice once;
  const int dev = current_device();
  once([dev] {
    int& cmax = cmax_dev[dev];
    const size_t smem = reg_panel_smem(64, sizeof(float2));
    cmax = 0;
    if (cudaFuncSetAttribute(lu_panel_cluster_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
      return;
    cudaFuncSetAttribute(lu_panel_cluster_kernel<64>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    for (int size : {kMaxClusterCtas, 8}) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(size);
      cfg.blockDim = dim3(kPanelThreads);
      cfg.dynamicSmemBytes = smem;
      cudaLaunchAttribute a[1];
      a[0].id = cudaLaunchAttributeClusterDimension;
      a[0].val.clusterDim.x = size;
      a[0].val.clusterDim.y = 1;
      a[0].val.clusterDim.z = 1;
      cfg.attrs = a;
      cfg.numAttrs = 1;
      int clusters = 0;
      if (cudaOccupancyMaxActiveClusters(&clusters, lu_panel_cluster_kernel<64>, &cfg) == cudaSuccess && clusters > 0) {
        cmax = size;
        break;
      }
    }
    cudaGetLastError();
  });
  return cmax_dev[dev];
}

int set_sym_assembly(int v);
int get_sym_assembly();

// Per-thread side stream and fork / join events for the lookahead update.
struct SideStream {
  cudaStream_t s = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  int device = -1;
};
static SideStream* side_stream() {
  thread_local SideStream ss;
  int dev = 0;
  cudaGetDevice(&dev);
  if (ss.device != dev) {
    if (cudaStreamCreateWithFlags(&ss.s, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ss.fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ss.join, cudaEventDisableTiming) != cudaSuccess)
      return nullptr;
    ss.device = dev;
  }
  return &ss;
}

template <typename T, int NB>
static int lu_factor_impl(cplx<T>* A, int n, int64_t lda, int32_t* perm, void* work, cudaStream_t s,
                          const LuOpts& opt, const TcLU* tc = nullptr) {
  using V = cplx<T>;
  static OncePerDevice once;
  once([] {
    cudaFuncSetAttribute(lu_panel_kernel<T, NB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPanelSmemBudget);
    cudaFuncSetAttribute(lu_swap_trsm_kernel<T, NB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)((2 * NB * kSwapCols + NB * NB) * sizeof(V)));
    cudaFuncSetAttribute(lu_panel_reg_kernel<T, NB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)reg_panel_smem(NB, sizeof(V)));
    cudaFuncSetAttribute(lu_tile_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTileSmem);
    cudaFuncSetAttribute(lu_l21_update_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kL21UpdateSmem);
  });
  PanelWs ws = panel_ws(work);
  if (cudaMemsetAsync(work, 0, 32, s) != cudaSuccess) return MGT_ERR_CUDA;   // status, nslot
  lu_start_kernel<<<(n + 255) / 256, 256, 0, s>>>(perm, n, ws.epoch, ws.records);
  count_launch();
  const int sms = std::min(num_sms(), kMaxPanelBlocks);
  const size_t sm2 = (2 * NB * kSwapCols + NB * NB) * sizeof(V);
  // CTAs of the panel kernel for a panel of m rows
  auto panel_ctas = [&](int m) -> int {
    const int64_t min_g_smem = ((int64_t)m * NB * (int64_t)sizeof(V) + kPanelSmemBudget - 1) / kPanelSmemBudget;
    const int rows_target = opt.panel_rows;
    int G = (int)std::max<int64_t>({1, (m + rows_target - 1) / rows_target, min_g_smem});
    const int gmax = opt.panel_max_ctas;
    return std::min(G, gmax > 0 ? std::min(gmax, sms) : sms);
  };
  // factor columns [j0, j0+w) over rows [j0, n); the interchanges go to slot set `set`
  auto panel_only = [&](int j0, int w, int set, bool with_l21 = true) -> int {
    if constexpr (sizeof(T) == 4) {
      if (opt.pivoting == MGT_PIVOT_TILE) {
        LuWsLayout Lw;
        float2* Ui = reinterpret_cast<float2*>((char*)work + Lw.uinv);
        // L11^-1 where the fused right-column pass reads the block's diagonal inverses
        float2* Li = reinterpret_cast<float2*>((char*)work + Lw.inv) + (size_t)set * kNBmax * kNBmax;
        lu_tile_kernel<<<1, 256, kTileSmem, s>>>(A + (int64_t)j0 * lda + j0, lda, w, j0, perm, panel_ws(work, set),
                                                  Ui, Li);
        count_launch();
        const int below = n - j0 - w;
        if (below > 0 && with_l21) {
          lu_l21_kernel<<<(below + 31) / 32, 256, 0, s>>>(A + (int64_t)(j0 + w) * lda + j0, lda, below, w, Ui);
          count_launch();
        }
        return cudaGetLastError() == cudaSuccess ? MGT_OK : MGT_ERR_CUDA;
      }
    }
    const int m = n - j0;
    const int G = panel_ctas(m);
    int rpc = (m + G - 1) / G;
    size_t smem = (size_t)rpc * NB * sizeof(V);
    if (smem > kPanelSmemBudget) return MGT_ERR_UNSUPPORTED;
    PanelWs pw = panel_ws(work, set);
    V* P = A + (int64_t)j0 * lda + j0;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(G);
    cfg.blockDim = dim3(kPanelThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    // Without the attribute (CUDA-graph capture of concurrent branches) the
    // caller keeps the panels' total CTA count within the SM count instead.
    cfg.numAttrs = opt.cooperative ? 1 : 0;
    // up to one row per thread: the register-resident kernel, as one thread-
    // block cluster (exchange in distributed shared memory) when it fits
    cudaError_t le;
    const int reg_mode = opt.panel_reg;
    bool launched = false;
    if constexpr (sizeof(T) == 4) {
      const int cmax = cluster_panel_max();
      if (rpc <= kPanelThreads && reg_mode != 0 && G <= cmax && opt.panel_cluster) {
        cudaLaunchConfig_t cc = cfg;
        cudaLaunchAttribute ca[1];
        ca[0].id = cudaLaunchAttributeClusterDimension;
        ca[0].val.clusterDim.x = G;
        ca[0].val.clusterDim.y = 1;
        ca[0].val.clusterDim.z = 1;
        cc.attrs = ca;
        cc.numAttrs = 1;
        cc.dynamicSmemBytes = reg_panel_smem(NB, sizeof(V));
        le = cudaLaunchKernelEx(&cc, lu_panel_cluster_kernel<NB>, P, lda, m, w, j0, rpc, perm, pw);
        launched = true;
      }
    }
    if (launched) {
    } else if (rpc <= kPanelThreads && (reg_mode == 2 || (reg_mode == 1 && sizeof(T) == 4))) {
      cfg.dynamicSmemBytes = reg_panel_smem(NB, sizeof(V));
      le = cudaLaunchKernelEx(&cfg, lu_panel_reg_kernel<T, NB>, P, lda, m, w, j0, rpc, perm, pw);
    } else {
      le = cudaLaunchKernelEx(&cfg, lu_panel_kernel<T, NB>, P, lda, m, w, j0, rpc, perm, pw);
    }
    if (le != cudaSuccess) return MGT_ERR_CUDA;
    count_launch();
    return MGT_OK;
  };
  // apply the interchanges of the panel at j0 (slot set `set`) to columns
  // [left_begin, left_end) and [right_begin, right_end); with do_trsm the
  // latter also get U12 = L11^-1 A12 on the panel's rows
  auto swap = [&](cudaStream_t st, int j0, int w, int set, int left_begin, int left_end, int right_begin,
                  int right_end, int do_trsm) {
    const int nleft = left_end > left_begin ? (left_end - left_begin + kSwapCols - 1) / kSwapCols : 0;
    const int nright = right_end > right_begin ? (right_end - right_begin + kSwapCols - 1) / kSwapCols : 0;
    if (nleft + nright > 0) {
      // tile pivoting: the tile kernel left L11^-1 of this panel in slot `set`
      const V* Linv = nullptr;
      if (opt.pivoting == MGT_PIVOT_TILE && do_trsm)
        Linv = reinterpret_cast<const V*>((char*)work + LuWsLayout().inv) + (size_t)set * kNBmax * kNBmax;
      lu_swap_trsm_kernel<T, NB><<<nleft + nright, 256, sm2, st>>>(A, lda, n, j0, w, left_begin, left_end,
                                                                    right_begin, right_end, panel_ws(work, set),
                                                                    do_trsm, Linv);
      count_launch();
    }
  };
  // Tile pivoting moves rows only within their 64-row tile, and nothing reads
  // a tile's L entries left of its outer block again before the end: those
  // columns take the tile's interchanges in one pass at the end
  // (lu_tile_left_perm_kernel) instead of once per panel.
  const bool defer_left = opt.pivoting == MGT_PIVOT_TILE;
  auto finish = [&](int outer) -> int {
    if constexpr (sizeof(T) == 4) {
      if (defer_left && n > NB) {
        lu_tile_left_perm_kernel<<<dim3((n + kSwapCols - 1) / kSwapCols, (n + NB - 1) / NB), 256, 0, s>>>(
            reinterpret_cast<float2*>(A), lda, n, perm, outer);
        count_launch();
      }
    } else {
      (void)outer;
    }
    return cudaGetLastError() == cudaSuccess ? MGT_OK : MGT_ERR_CUDA;
  };
  // one inner panel, then its interchanges on every other column
  auto panel_step = [&](int j0, int w, int do_trsm) -> int {
    int e = panel_only(j0, w, 0);
    if (e == MGT_OK) swap(s, j0, w, 0, defer_left ? j0 : 0, j0, j0 + w, n, do_trsm);
    return e;
  };
  auto update_on = [&](cudaStream_t st, int r0, int c0, int k0, int K, int rows, int cols, bool dominant,
                       int max_ctas) -> int {
    // A[r0:r0+rows, c0:c0+cols] -= A[r0:, k0:k0+K] * A[k0:k0+K, c0:]
    if (rows <= 0 || cols <= 0) return MGT_OK;
    if (dominant) dom_begin(st);
    int e;
    if (dominant)
      e = trailing_update(tc, rows, cols, K, A + (int64_t)r0 * lda + k0, lda, A + (int64_t)k0 * lda + c0, lda,
                          A + (int64_t)r0 * lda + c0, lda, c0, ws.status, st, max_ctas);
    else
      e = gemm_sub<T>(rows, cols, K, A + (int64_t)r0 * lda + k0, lda, A + (int64_t)k0 * lda + c0, lda,
                      A + (int64_t)r0 * lda + c0, lda, st);
    // algorithmic work of C -= A B: 8 rows cols K real flops; C read + written once, A and B read once
    if (dominant)
      dom_end(st, 8.0 * rows * (double)cols * K,
              sizeof(V) * (2.0 * rows * (double)cols + (double)rows * K + (double)K * cols));
    return e;
  };
  auto update = [&](int r0, int c0, int k0, int K, int rows, int cols, bool dominant) -> int {
    return update_on(s, r0, c0, k0, K, rows, cols, dominant, 0);
  };
  if (tc == nullptr || opt.outer_block == NB) {
    for (int j0 = 0; j0 < n; j0 += NB) {
      const int w = std::min(NB, n - j0);
      int e = panel_step(j0, w, 1);
      if (e == MGT_OK) e = update(j0 + w, j0 + w, j0, w, n - j0 - w, n - j0 - w, true);
      if (e != MGT_OK) return e;
    }
    return finish(NB);
  }
  // tensor-core path: 128-wide outer blocks made of two 64-wide inner panels,
  // so that the trailing update runs with K = 128 (half the C traffic per flop)
  static OncePerDevice once2;
  const size_t sm3 = (NB * kSwapCols + NB * (NB + 1) + NB * kSwapCols) * sizeof(V);
  once2([sm3] {
    cudaFuncSetAttribute(lu_preupdate_trsm_kernel<T, NB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm3);
    if constexpr (sizeof(T) == 4)
      cudaFuncSetAttribute(lu_block_right_kernel<T, NB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)block_right_smem<NB>(sizeof(V)));
  });
  // Lookahead (cooperative panels, not under stream capture): the trailing
  // update of block J0 first brings the next block's columns up to date, then
  // the rest of it runs on a side stream (its first columns with the CTAs
  // capped to leave the next panels their SMs, the others on every SM), while
  // this stream factors the next block's two inner panels and applies their
  // interchanges to the columns the side stream does not touch.  The
  // far-right interchanges, the second panel's pre-update and the U12 solve
  // follow once the side stream has finished.
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(s, &cap);
  SideStream* side = nullptr;
  if (opt.lookahead && (opt.cooperative || opt.pivoting == MGT_PIVOT_TILE) && cap == cudaStreamCaptureStatusNone)
    side = side_stream();
  // the two inner panels of the block at J0 and everything up to (not
  // including) the columns at or right of `far`: interchanges on the left,
  // the second panel's columns brought up to date
  auto block_panels = [&](int J0, int far) -> int {
    const int W = std::min(2 * NB, n - J0), wa = std::min(NB, W), wb = W - wa, j1 = J0 + wa;
    // tile pivoting: the rows below the first tile get L21 together with the
    // second panel's update, once the swap kernel has solved U12
    const bool fuse = defer_left && sizeof(T) == 4 && wb > 0;
    int e = panel_only(J0, wa, 0, !fuse);
    if (e != MGT_OK) return e;
    // (tile pivoting) columns left of J0 wait for the final pass; the
    // second panel's rows of the first panel's columns (L_BA, read by the
    // right-column pass) are swapped here
    swap(s, J0, wa, 0, defer_left ? J0 : 0, J0, j1, std::min(far, J0 + W), 1);
    if (wb > 0) {
      if (fuse) {
        if constexpr (sizeof(T) == 4) {
          const float2* Ui = reinterpret_cast<const float2*>((char*)work + LuWsLayout().uinv);
          lu_l21_update_kernel<<<(n - j1 + 31) / 32, 256, kL21UpdateSmem, s>>>(
              reinterpret_cast<float2*>(A) + (int64_t)j1 * lda + J0, lda, n - j1, wa, wb, Ui,
              reinterpret_cast<const float2*>(A) + (int64_t)J0 * lda + j1);
          count_launch();
        }
      } else {
        e = update(j1, j1, J0, wa, n - j1, wb, false);
      }
      if (e == MGT_OK) e = panel_only(j1, wb, 1);
      if (e != MGT_OK) return e;
      swap(s, j1, wb, 1, defer_left ? J0 : 0, j1, 0, 0, 0);
    }
    return MGT_OK;
  };
  // the far-right columns [J0 + W, n) of the block at J0: both panels'
  // interchanges, the first panel's solve, the second panel's pre-update + solve
  auto block_right = [&](int J0) {
    const int W = std::min(2 * NB, n - J0), wa = std::min(NB, W), wb = W - wa, j1 = J0 + wa;
    const int right = n - J0 - W;
    if (right <= 0) return;
    if constexpr (sizeof(T) == 4) {
      if (wb > 0 && opt.fused_right) {
        V* Inv = reinterpret_cast<V*>((char*)work + LuWsLayout().inv);
        // tile pivoting: the tile kernels left both diagonal blocks' inverses there
        if (opt.pivoting != MGT_PIVOT_TILE) lower_block_inverses<T>(A + (int64_t)J0 * lda + J0, lda, W, Inv, s);
        lu_block_right_kernel<T, NB><<<(right + kSwapCols - 1) / kSwapCols, 256, block_right_smem<NB>(sizeof(V)), s>>>(
            A, lda, n, J0, wa, wb, J0 + W, panel_ws(work, 0), panel_ws(work, 1), Inv);
        count_launch();
        return;
      }
    }
    swap(s, J0, wa, 0, 0, 0, J0 + W, n, 1);
    if (wb > 0) {
      swap(s, j1, wb, 1, 0, 0, J0 + W, n, 0);
      lu_preupdate_trsm_kernel<T, NB><<<(right + kSwapCols - 1) / kSwapCols, 256, sm3, s>>>(A, lda, n, J0, wa, j1,
                                                                                           wb, J0 + W);
      count_launch();
    }
  };
  auto lookahead_update = [&](int J0, int W, int P0, int WN, int rest, cudaStream_t s2) -> int {
    if constexpr (sizeof(T) == 4) {
      const int M = n - P0;
      const float2* L21 = reinterpret_cast<const float2*>(A + (int64_t)P0 * lda + J0);
      const float2* U12 = reinterpret_cast<const float2*>(A + (int64_t)J0 * lda + P0);
      dom_begin(s);
      int e = tc_split_a(tc->plan, M, W, L21, lda, s);
      if (e == MGT_OK) e = tc_split_b(tc->plan, WN, W, U12, lda, s);
      if (e == MGT_OK) e = tc_gemm(tc->plan, tc->cmap, M, WN, W, 2 * P0, P0, ws.status, s);
      dom_end(s, 8.0 * M * (double)WN * W, sizeof(V) * (2.0 * M * (double)WN + (double)M * W + (double)W * WN));
      if (e != MGT_OK) return e;
      if (cudaEventRecord(side->fork, s) != cudaSuccess || cudaStreamWaitEvent(s2, side->fork, 0) != cudaSuccess)
        return MGT_ERR_CUDA;
      // the rest's B split on the side stream too (this stream touches no
      // split buffer before the join)
      dom_begin(s2);
      e = tc_split_b(tc->plan, rest, W, U12 + WN, lda, s2);
      // the first columns beside the next block's panels, on the SMs they
      // leave free; the rest, by when the panels should be done, on every SM
      // (a persistent launch keeps the SMs it started on)
      const bool tile = opt.pivoting == MGT_PIVOT_TILE;
      const int reserve = tile ? 16 : panel_ctas(M);
      const double t_pan = tile ? 3e-4 : 2.0 * NB * 4.5e-6 + 1e-4;
      const double head = t_pan * 3e14 * (sms - reserve) / sms / (8.0 * M * (double)W);
      const int c1 = (int)std::min<double>(rest, (std::floor(head / (2 * NB)) + 1) * (2 * NB));
      if (e == MGT_OK)
        e = tc_gemm(tc->plan, tc->cmap, M, c1, W, 2 * (P0 + WN), P0, ws.status, s2, std::max(1, sms - reserve));
      if (e == MGT_OK && c1 < rest)
        e = tc_gemm(tc->plan, tc->cmap, M, rest - c1, W, 2 * (P0 + WN + c1), P0, ws.status, s2, 0, c1);
      dom_end(s2, 8.0 * M * (double)rest * W, sizeof(V) * (2.0 * M * (double)rest + (double)W * rest));
      // once forked, the join is recorded whatever happened
      const bool joined = cudaEventRecord(side->join, s2) == cudaSuccess;
      return e != MGT_OK ? e : (joined ? MGT_OK : MGT_ERR_CUDA);
    } else {
      (void)J0; (void)W; (void)P0; (void)WN; (void)rest; (void)s2;
      return MGT_ERR_UNSUPPORTED;
    }
  };
  // Paired blocks (tile pivoting, while the trailing order is at least
  // opt.wide_min): once block X at P0 is factored and its right-column
  // pass done, X's update goes only to the next block Y's columns (every row
  // below X) and to Y's rows of the columns right of Y; Y is factored, and
  // the columns right of Y then take the update of both blocks as one
  // product with K = 256 (half the C traffic per flop of two K = 128
  // updates).  Tile pivoting moves Y's rows only within Y's tiles, every one
  // of which already carries X's update.
  auto pair_update = [&](int X0, int Y0, int WY) -> int {
    if constexpr (sizeof(T) == 4) {
      const int KX = Y0 - X0, M = n - Y0, far0 = Y0 + WY, nfar = n - far0;
      const float2* L21 = reinterpret_cast<const float2*>(A + (int64_t)Y0 * lda + X0);
      const float2* U12 = reinterpret_cast<const float2*>(A + (int64_t)X0 * lda + Y0);
      dom_begin(s);
      int e = tc_split_a(tc->plan, M, KX, L21, lda, s);
      if (e == MGT_OK) e = tc_split_b(tc->plan, WY + nfar, KX, U12, lda, s);
      if (e == MGT_OK) e = tc_gemm(tc->plan, tc->cmap, M, WY, KX, 2 * Y0, Y0, ws.status, s);
      // Y's rows are the first WY rows of the split L21
      if (e == MGT_OK && nfar > 0)
        e = tc_gemm(tc->plan, tc->cmap, WY, nfar, KX, 2 * far0, Y0, ws.status, s, 0, WY);
      const double cells = (double)M * WY + (double)WY * nfar;
      dom_end(s, 8.0 * cells * KX, sizeof(V) * (2.0 * cells + (double)M * KX + (double)KX * (WY + nfar)));
      return e;
    } else {
      (void)X0; (void)Y0; (void)WY;
      return MGT_ERR_UNSUPPORTED;
    }
  };
  if constexpr (sizeof(T) != 4) side = nullptr;   // the tensor-core path is complex64 only
  const bool pairs = sizeof(T) == 4 && opt.pivoting == MGT_PIVOT_TILE && opt.wide_min > 0;
  int e = block_panels(0, n);
  if (e != MGT_OK) return e;
  block_right(0);
  // the factored columns [K0, K0 + KW) (one block, or a pair) whose update of
  // the trailing matrix is pending
  int K0 = 0, KW = std::min(2 * NB, n);
  while (K0 + KW < n) {
    const int P0 = K0 + KW;                      // next block
    const int WN = std::min(2 * NB, n - P0);
    const int rest = n - P0 - WN;
    // the side update takes the SMs the panels leave free only for about the
    // panels' time (lookahead_update), so the overlap pays whenever there is
    // a rest, unless partial-pivoting panels would leave it too few SMs
    const bool overlap = side != nullptr && rest > 0 &&
                         (opt.pivoting == MGT_PIVOT_TILE || sms - panel_ctas(n - P0) >= 16);
    if (!overlap) {
      e = update(P0, P0, K0, KW, n - P0, n - P0, true);
      if (e == MGT_OK) e = block_panels(P0, n);
      if (e != MGT_OK) return e;
    } else {
      // A[P0:, P0:] -= L21 U12 of the pending columns: the operand splits (the
      // rows of L21 are permuted by the next panels' interchanges) and the
      // next block's columns here; the rest of the update on the side stream
      e = lookahead_update(K0, KW, P0, WN, rest, side->s);
      if (e == MGT_OK) e = block_panels(P0, P0 + WN);
      // always join: nothing of the side stream may outlive this call
      if (cudaStreamWaitEvent(s, side->join, 0) != cudaSuccess && e == MGT_OK) e = MGT_ERR_CUDA;
      if (e != MGT_OK) return e;
    }
    block_right(P0);
    K0 = P0;
    KW = WN;
    const int Y0 = P0 + WN, WY = std::min(2 * NB, n - Y0);
    if (pairs && WN == 2 * NB && WY == 2 * NB && n - P0 >= opt.wide_min) {
      e = pair_update(P0, Y0, WY);
      if (e == MGT_OK) e = block_panels(Y0, n);
      if (e != MGT_OK) return e;
      block_right(Y0);
      KW = WN + WY;
    }
  }
  return finish(2 * NB);
}

// ---------------------------------------------------------------- solves

constexpr int kTrsmCols = 32;

// In-place solve of a bs x bs triangular block against bs rows of X
// (all columns): lower unit (forward) or upper non-unit (backward).
template <typename T, int BS, bool UPPER>
__global__ void __launch_bounds__(256)
trsm_block_kernel(const cplx<T>* __restrict__ F, int64_t ldf, int row0, int bs, cplx<T>* __restrict__ X,
                  int64_t ldx, int nrhs) {
  using V = cplx<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* Ts = reinterpret_cast<V*>(smem_raw);   // [BS][BS]
  V* Xs = Ts + BS * BS;                       // [BS][kTrsmCols]
  __shared__ V dinv[BS];
  const int tid = threadIdx.x;
  const int col0 = blockIdx.x * kTrsmCols;
  const int ncols = min(kTrsmCols, nrhs - col0);
  for (int idx = tid; idx < bs * bs; idx += blockDim.x) {
    int i = idx / bs, k = idx - i * bs;
    Ts[i * BS + k] = F[(int64_t)(row0 + i) * ldf + row0 + k];
  }
  for (int idx = tid; idx < bs * kTrsmCols; idx += blockDim.x) {
    int i = idx / kTrsmCols, cc = idx - i * kTrsmCols;
    if (cc < ncols) Xs[i * kTrsmCols + cc] = X[(int64_t)(row0 + i) * ldx + col0 + cc];
  }
  __syncthreads();
  if (UPPER) {
    for (int i = tid; i < bs; i += blockDim.x) dinv[i] = crecip(Ts[i * BS + i]);
    __syncthreads();
  }
  const int warp = tid >> 5, lane = tid & 31;
  const int cc = warp * 4 + (lane >> 3), t8 = lane & 7;
  if (cc < kTrsmCols) {
    if (!UPPER) {
      for (int k = 0; k < bs - 1; ++k) {
        __syncwarp();
        const V xk = Xs[k * kTrsmCols + cc];
        for (int i = k + 1 + t8; i < bs; i += 8) cfms(Xs[i * kTrsmCols + cc], Ts[i * BS + k], xk);
      }
    } else {
      for (int k = bs - 1; k >= 0; --k) {
        __syncwarp();
        if (t8 == 0) Xs[k * kTrsmCols + cc] = cmul(Xs[k * kTrsmCols + cc], dinv[k]);
        __syncwarp();
        const V xk = Xs[k * kTrsmCols + cc];
        for (int i = t8; i < k; i += 8) cfms(Xs[i * kTrsmCols + cc], Ts[i * BS + k], xk);
      }
    }
  }
  __syncthreads();
  for (int idx = tid; idx < bs * kTrsmCols; idx += blockDim.x) {
    int i = idx / kTrsmCols, c2 = idx - i * kTrsmCols;
    if (c2 < ncols) X[(int64_t)(row0 + i) * ldx + col0 + c2] = Xs[i * kTrsmCols + c2];
  }
}

template <typename V>
__global__ void permute_rows_kernel(const V* __restrict__ B, int64_t ldb, const int32_t* __restrict__ perm,
                                    V* __restrict__ X, int64_t ldx, int n, int nrhs) {
  int i = blockIdx.y;
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && c < nrhs) X[(int64_t)i * ldx + c] = B[(int64_t)perm[i] * ldb + c];
}

template <typename T, bool UPPER>
int tri_solve(const cplx<T>* F, int64_t ldf, cplx<T>* X, int64_t ldx, int n, int nrhs, void* work, int* status,
              cudaStream_t s);
size_t tri_solve_workspace_bytes(int64_t n, int64_t nrhs, size_t elem);

template <typename T>
static int lu_solve_impl(const cplx<T>* LU, int n, int64_t lda, const int32_t* perm, const cplx<T>* B,
                         int64_t ldb, cplx<T>* X, int64_t ldx, int nrhs, cudaStream_t s, void* work = nullptr) {
  using V = cplx<T>;
  if (work) {
    // persistent flag-ordered triangular solves (one launch per triangle and 64 columns)
    int* status = (int*)((char*)work + 128);
    if (cudaMemsetAsync(status, 0, 2 * sizeof(int), s) != cudaSuccess) return MGT_ERR_CUDA;
    dim3 pg((nrhs + 127) / 128, n);
    if (n > 65535) return MGT_ERR_UNSUPPORTED;
    permute_rows_kernel<V><<<pg, 128, 0, s>>>(B, ldb, perm, X, ldx, n, nrhs);
    count_launch();
    int e = tri_solve<T, false>(LU, lda, X, ldx, n, nrhs, work, status, s);
    if (e == MGT_OK) e = tri_solve<T, true>(LU, lda, X, ldx, n, nrhs, work, status, s);
    return e;
  }
  constexpr int BS = 64;
  static OncePerDevice once;
  const size_t smem = (BS * BS + BS * kTrsmCols) * sizeof(V);
  once([smem] {
    cudaFuncSetAttribute(trsm_block_kernel<T, BS, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(trsm_block_kernel<T, BS, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  });
  if (n > 65535) return MGT_ERR_UNSUPPORTED;
  dim3 pg((nrhs + 127) / 128, n);
  permute_rows_kernel<V><<<pg, 128, 0, s>>>(B, ldb, perm, X, ldx, n, nrhs);
  count_launch();
  const int cblocks = (nrhs + kTrsmCols - 1) / kTrsmCols;
  for (int r0 = 0; r0 < n; r0 += BS) {
    int bs = std::min(BS, n - r0);
    trsm_block_kernel<T, BS, false><<<cblocks, 256, smem, s>>>(LU, lda, r0, bs, X, ldx, nrhs);
    count_launch();
    int rem = n - r0 - bs;
    if (rem > 0) {
      int e = gemm_sub<T>(rem, nrhs, bs, LU + (int64_t)(r0 + bs) * lda + r0, lda, X + (int64_t)r0 * ldx, ldx,
                          X + (int64_t)(r0 + bs) * ldx, ldx, s);
      if (e != MGT_OK) return e;
    }
  }
  const int nblk = (n + BS - 1) / BS;
  for (int b = nblk - 1; b >= 0; --b) {
    int r0 = b * BS, bs = std::min(BS, n - r0);
    trsm_block_kernel<T, BS, true><<<cblocks, 256, smem, s>>>(LU, lda, r0, bs, X, ldx, nrhs);
    count_launch();
    if (r0 > 0) {
      int e = gemm_sub<T>(r0, nrhs, bs, LU + r0, lda, X + (int64_t)r0 * ldx, ldx, X, ldx, s);
      if (e != MGT_OK) return e;
    }
  }
  return cudaGetLastError() == cudaSuccess ? MGT_OK : MGT_ERR_CUDA;
}

}  // namespace mgt

using namespace mgt;

// Below this order the complex64 trailing update stays on the SIMT pipes.
constexpr int64_t kTcMinN = 256;

static size_t tc_region_offset() { return (LuWsLayout().total + 1023) & ~size_t(1023); }

extern "C" int mgt_lu_workspace_bytes(int dtype, int64_t n, size_t* bytes) {
  if (!bytes || n <= 0 || (dtype != MGT_C128 && dtype != MGT_C64)) return MGT_ERR_ARG;
  *bytes = LuWsLayout().total;
  if (dtype == MGT_C64 && n >= kTcMinN) *bytes = tc_region_offset() + tc_scratch_bytes(n);
  return MGT_OK;
}

extern "C" int mgt_lu_factor_ex(int dtype, void* A, int64_t n, int64_t lda, int32_t* perm, void* work,
                                size_t work_bytes, const mgt_lu_options* options, void* stream) {
  if (!A || !perm || !work || n <= 0 || lda < n || n > (1 << 20)) return MGT_ERR_ARG;
  if (work_bytes < LuWsLayout().total) return MGT_ERR_WORKSPACE;
  LuOpts opt;
  int e = resolve_lu_options(options, &opt);
  if (e != MGT_OK) return e;
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == MGT_C128) {
    if (opt.pivoting != MGT_PIVOT_PARTIAL) return MGT_ERR_UNSUPPORTED;
    return lu_factor_impl<double, 32>((double2*)A, (int)n, lda, perm, work, s, opt);
  }
  if (dtype == MGT_C64) {
    // tensor-core trailing update when the workspace holds its split buffers,
    // the rows are 16-byte aligned (even lda) and the driver exposes TMA maps
    if (n >= kTcMinN && (lda & 1) == 0 && work_bytes >= tc_region_offset() + tc_scratch_bytes(n) && tc_available()) {
      TcLU tc;
      e = tc.plan.init((char*)work + tc_region_offset(), n);
      if (e == MGT_OK) e = tc_make_cmap(&tc.cmap, (float2*)A, n, n, lda);
      if (e == MGT_OK) return lu_factor_impl<float, 64>((float2*)A, (int)n, lda, perm, work, s, opt, &tc);
    }
    return lu_factor_impl<float, 64>((float2*)A, (int)n, lda, perm, work, s, opt);
  }
  return MGT_ERR_ARG;
}

extern "C" int mgt_lu_factor(int dtype, void* A, int64_t n, int64_t lda, int32_t* perm, void* work,
                             size_t work_bytes, void* stream) {
  return mgt_lu_factor_ex(dtype, A, n, lda, perm, work, work_bytes, nullptr, stream);
}

extern "C" int mgt_lu_solve_workspace_bytes(int dtype, int64_t n, int64_t nrhs, size_t* bytes) {
  if (!bytes || n <= 0 || nrhs <= 0 || (dtype != MGT_C128 && dtype != MGT_C64)) return MGT_ERR_ARG;
  *bytes = tri_solve_workspace_bytes(n, nrhs, dtype == MGT_C128 ? sizeof(double2) : sizeof(float2));
  return MGT_OK;
}

extern "C" int mgt_lu_solve(int dtype, const void* LU, int64_t n, int64_t lda, const int32_t* perm,
                            const void* B, int64_t ldb, void* X, int64_t ldx, int64_t nrhs, void* work,
                            size_t work_bytes, void* stream) {
  if (!LU || !perm || !B || !X || n <= 0 || nrhs <= 0 || lda < n || ldb < nrhs || ldx < nrhs) return MGT_ERR_ARG;
  if (B == X) return MGT_ERR_ARG;
  if (work && work_bytes < tri_solve_workspace_bytes(n, nrhs, dtype == MGT_C128 ? sizeof(double2) : sizeof(float2)))
    return MGT_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == MGT_C128)
    return lu_solve_impl<double>((const double2*)LU, (int)n, lda, perm, (const double2*)B, ldb, (double2*)X, ldx,
                                 (int)nrhs, s, work);
  if (dtype == MGT_C64)
    return lu_solve_impl<float>((const float2*)LU, (int)n, lda, perm, (const float2*)B, ldb, (float2*)X, ldx,
                                (int)nrhs, s, work);
  return MGT_ERR_ARG;
}

extern "C" int mgt_workspace_status(void* work, int32_t out[2], void* stream) {
  if (!work || !out) return MGT_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  LuWsLayout L;
  int32_t* st = (int32_t*)((char*)work + L.status);
  if (cudaMemcpyAsync(out, st, 2 * sizeof(int32_t), cudaMemcpyDeviceToHost, s) != cudaSuccess) return MGT_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return MGT_ERR_CUDA;
  if (cudaMemsetAsync(st, 0, 2 * sizeof(int32_t), s) != cudaSuccess) return MGT_ERR_CUDA;
  return MGT_OK;
}

// ---------------------------------------------------------------- no-allocation LU entry point
//
// mgt_lu_factor_static: the same LU as mgt_lu_factor, but its scratch space
// (panel pivot candidates, pivot-row broadcast buffers, grid-barrier counters
// and status words) lives in the file-scope device array below instead of a
// caller-provided workspace.  It exists for callers that cannot obtain device
// memory at call time: a C or Fortran host that binds only this library (no
// torch caching allocator or other pool to ask for a workspace) and whose
// process policy forbids cudaMalloc after start-up, or a process that has
// already reserved all device memory into its own pool.
//
// The array takes kStaticLuScratchBytes (1 MiB) of device memory on every GPU
// that loads the library, until the process exits.  Every call on a device
// shares it: the call clears the barrier counters and status words it needs
// at zero before it starts, and two calls whose GPU work overlaps (different
// streams, or different host threads) race on it and corrupt each other --
// serialise them.  The first call on each device looks up the array's device
// address with cudaGetSymbolAddress (the host-side name of a __device__ array
// is not a device address); make that first call before any stream capture.

namespace mgt {
constexpr size_t kStaticLuScratchBytes = size_t(1) << 20;
constexpr int64_t kStaticLuMaxN = 65536;
static __device__ __align__(256) unsigned char g_lu_static_scratch[kStaticLuScratchBytes];

static int static_lu_scratch(void** out) {
  static std::mutex mu;
  static void* per_device[64] = {};
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return MGT_ERR_CUDA;
  std::lock_guard<std::mutex> lk(mu);
  if (!per_device[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_lu_static_scratch) != cudaSuccess || !p) return MGT_ERR_CUDA;
    per_device[dev] = p;
  }
  *out = per_device[dev];
  return MGT_OK;
}
}  // namespace mgt

extern "C" int mgt_lu_factor_static(int dtype, void* A, int64_t n, int64_t lda, int32_t* perm, int32_t* info,
                                    void* stream) {
  if (!A || !perm || n <= 0 || lda < n) return MGT_ERR_ARG;
  if (dtype != MGT_C128 && dtype != MGT_C64) return MGT_ERR_ARG;
  if (n > kStaticLuMaxN) return MGT_ERR_UNSUPPORTED;
  if (LuWsLayout().total > kStaticLuScratchBytes) return MGT_ERR_WORKSPACE;
  void* work = nullptr;
  int e = static_lu_scratch(&work);
  if (e != MGT_OK) return e;
  cudaStream_t s = (cudaStream_t)stream;
  const LuOpts opt;
  e = dtype == MGT_C128 ? lu_factor_impl<double, 32>((double2*)A, (int)n, lda, perm, work, s, opt)
                        : lu_factor_impl<float, 64>((float2*)A, (int)n, lda, perm, work, s, opt);
  if (e != MGT_OK) return e;
  if (info) {
    LuWsLayout L;
    if (cudaMemcpyAsync(info, (char*)work + L.status, 2 * sizeof(int32_t), cudaMemcpyDeviceToDevice, s) !=
        cudaSuccess)
      return MGT_ERR_CUDA;
  }
  return MGT_OK;
}

extern "C" int mgt_set_tuning(int key, int value) {
  if (key == MGT_TUNE_PANEL_ROWS) {
    if (value < 32 || value > 4096) return MGT_ERR_ARG;
    g_panel_rows.store(value);
    return MGT_OK;
  }
  if (key == MGT_TUNE_OUTER_BLOCK) {
    if (value != 64 && value != 128) return MGT_ERR_ARG;
    g_outer_block.store(value);
    return MGT_OK;
  }
  if (key == MGT_TUNE_PANEL_MAX_CTAS) {
    if (value < 0 || value > 4096) return MGT_ERR_ARG;
    g_panel_max_ctas.store(value);
    return MGT_OK;
  }
  if (key == MGT_TUNE_COOPERATIVE) {
    g_cooperative.store(value ? 1 : 0);
    return MGT_OK;
  }
  if (key == MGT_TUNE_PANEL_REGISTERS) {
    if (value < 0 || value > 2) return MGT_ERR_ARG;
    g_panel_reg.store(value);
    return MGT_OK;
  }
  if (key == MGT_TUNE_TC_PRECISION) return tc_set_mode(value);
  if (key == MGT_TUNE_LOOKAHEAD) {
    g_lookahead.store(value ? 1 : 0);
    return MGT_OK;
  }
  if (key == MGT_TUNE_FUSED_RIGHT) {
    g_fused_right.store(value ? 1 : 0);
    return MGT_OK;
  }
  if (key == MGT_TUNE_PANEL_CLUSTER) {
    g_panel_cluster.store(value ? 1 : 0);
    return MGT_OK;
  }
  if (key == MGT_TUNE_SYM_ASSEMBLY) return set_sym_assembly(value);
  if (key == MGT_TUNE_WIDE_UPDATE) {
    if (value < 0) return MGT_ERR_ARG;
    g_wide_min.store(value);
    return MGT_OK;
  }
  return MGT_ERR_ARG;
}

extern "C" int mgt_get_tuning(int key) {
  if (key == MGT_TUNE_PANEL_ROWS) return g_panel_rows.load();
  if (key == MGT_TUNE_OUTER_BLOCK) return g_outer_block.load();
  if (key == MGT_TUNE_PANEL_MAX_CTAS) return g_panel_max_ctas.load();
  if (key == MGT_TUNE_COOPERATIVE) return g_cooperative.load();
  if (key == MGT_TUNE_PANEL_REGISTERS) return g_panel_reg.load();
  if (key == MGT_TUNE_TC_PRECISION) return tc_get_mode();
  if (key == MGT_TUNE_LOOKAHEAD) return g_lookahead.load();
  if (key == MGT_TUNE_FUSED_RIGHT) return g_fused_right.load();
  if (key == MGT_TUNE_PANEL_CLUSTER) return g_panel_cluster.load();
  if (key == MGT_TUNE_SYM_ASSEMBLY) return get_sym_assembly();
  if (key == MGT_TUNE_WIDE_UPDATE) return g_wide_min.load();
  return MGT_ERR_ARG;
}
