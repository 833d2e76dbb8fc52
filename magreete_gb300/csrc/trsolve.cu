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
#include <mutex>

#include "common.cuh"
#include "diag.cuh"

namespace mgt {

constexpr int kTB = 64;      // block rows
constexpr int kTG = 16;      // right-hand-side columns per chain (independent column groups), narrow
constexpr int kTGWide = 64;  // wide chains: complex64, large n (more work per loaded block, fewer chains)
constexpr int kWideMinN = 20000;

// register tile of one thread in a 64 x TG block: TR rows x 4 columns
template <int TG> struct TriTile;
template <> struct TriTile<16> { static constexpr int TR = 1, TC = 4, TPR = 4; };    // 64 x 4 threads
template <> struct TriTile<64> { static constexpr int TR = 4, TC = 4, TPR = 16; };   // 16 x 16 threads

__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Factor blocks staged per CTA: two (the next block loads during the current
// product) for complex64, one for complex128 (shared memory).
template <typename T> constexpr int tri_nbuf() { return sizeof(T) == 4 ? 2 : 1; }

// Row stride of the right-hand sides in diag_inverse_kernel: the four lanes
// of a column group read rows r..r+3, and a stride of 72 complex64 (an odd
// multiple of 64 bytes) puts those rows on different banks (with 64 they
// shared one: 4-way conflicts on every access).
constexpr int kInvLd = kTB + 8;

// Inverse of every 64 x 64 diagonal block of the unit lower (or upper) factor:
// one CTA per block, identity right-hand sides, substitution in shared memory.
// Warp w owns columns 8w..8w+7 of the inverse, which is lower (upper)
// triangular: the steps above (below) those columns multiply exact zeros and
// are skipped.
template <typename T, bool UPPER>
__global__ void __launch_bounds__(256)
diag_inverse_kernel(const cplx<T>* __restrict__ F, int64_t ldf, int n, cplx<T>* __restrict__ Inv) {
  using V = cplx<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* Ts = reinterpret_cast<V*>(smem_raw);          // [kTB][kTB + 1]
  V* Xs = Ts + kTB * (kTB + 1);                      // [kTB][kInvLd]
  __shared__ V dinv[kTB];
  const int tid = threadIdx.x, i = blockIdx.x;
  const int r0 = i * kTB, rb = min(kTB, n - r0);
  for (int idx = tid; idx < kTB * kTB; idx += 256) {
    int r = idx >> 6, c = idx & 63;
    const bool ok = r < rb && c < rb;
    cp_async_elem<(int)sizeof(V)>(Ts + r * (kTB + 1) + c, ok ? F + (int64_t)(r0 + r) * ldf + r0 + c : F, ok);
    V e = czero<V>();
    if (r == c) e.x = 1;
    Xs[r * kInvLd + c] = e;
  }
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();
  if (UPPER)
    for (int r = tid; r < kTB; r += 256) dinv[r] = r < rb ? crecip(Ts[r * (kTB + 1) + r]) : czero<V>();
  __syncthreads();
  const int warp = tid >> 5, lane = tid & 31;
  const int col = warp * 8 + (lane >> 2), t4 = lane & 3;   // 4 lanes per column, 64 columns
  if (!UPPER) {
    for (int kk = warp * 8; kk < rb - 1; ++kk) {
      __syncwarp();
      const V xk = Xs[kk * kInvLd + col];
      for (int r = kk + 1 + t4; r < rb; r += 4) cfms(Xs[r * kInvLd + col], Ts[r * (kTB + 1) + kk], xk);
    }
  } else {
    for (int kk = min(rb - 1, warp * 8 + 7); kk >= 0; --kk) {
      __syncwarp();
      if (t4 == 0) Xs[kk * kInvLd + col] = cmul(Xs[kk * kInvLd + col], dinv[kk]);
      __syncwarp();
      const V xk = Xs[kk * kInvLd + col];
      for (int r = t4; r < kk; r += 4) cfms(Xs[r * kInvLd + col], Ts[r * (kTB + 1) + kk], xk);
    }
  }
  __syncthreads();
  V* out = Inv + (int64_t)i * kTB * kTB;
  for (int idx = tid; idx < kTB * kTB; idx += 256) out[idx] = Xs[(idx >> 6) * kInvLd + (idx & 63)];
}

// W_i = Inv_i F_(i, j): the inverted diagonal block times the factor block of
// the last dependency j of block row i (j = i - 1 for L, i + 1 for U), so
// that the solve can form Inv_i (B_i - all other products) before block j
// is done and needs only X_i = Z - W_i X_j after it.  One CTA per block row,
// thread = (4 rows, 4 columns) of W_i.
template <typename T, bool UPPER>
__global__ void __launch_bounds__(256)
chain_factor_kernel(const cplx<T>* __restrict__ F, int64_t ldf, int n, const cplx<T>* __restrict__ Inv,
                    cplx<T>* __restrict__ W) {
  using V = cplx<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* Is = reinterpret_cast<V*>(smem_raw);   // [kTB][kTB + 1]
  V* Fs = Is + kTB * (kTB + 1);              // [kTB][kTB + 1]
  const int tid = threadIdx.x, i = blockIdx.x, nb = gridDim.x;
  const int j = UPPER ? i + 1 : i - 1;
  if (j < 0 || j >= nb) return;
  const int r0 = i * kTB, rb = min(kTB, n - r0), c0 = j * kTB, cb = min(kTB, n - c0);
  const V* inv = Inv + (int64_t)i * kTB * kTB;
  for (int idx = tid; idx < kTB * kTB; idx += 256) {
    const int r = idx >> 6, c = idx & 63;
    cp_async_elem<(int)sizeof(V)>(Is + r * (kTB + 1) + c, inv + idx, true);
    const bool ok = r < rb && c < cb;
    cp_async_elem<(int)sizeof(V)>(Fs + r * (kTB + 1) + c, ok ? F + (int64_t)(r0 + r) * ldf + c0 + c : F, ok);
  }
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();
  const int tr = tid >> 4, tc = tid & 15;   // rows 4 tr .., columns tc + 16 q
  V acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[a][q] = czero<V>();
  for (int k = 0; k < kTB; ++k) {
    V f[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) f[q] = Fs[k * (kTB + 1) + tc + 16 * q];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const V x = Is[(4 * tr + a) * (kTB + 1) + k];
#pragma unroll
      for (int q = 0; q < 4; ++q) cfma(acc[a][q], x, f[q]);
    }
  }
  V* out = W + (int64_t)i * kTB * kTB;
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int q = 0; q < 4; ++q) out[(4 * tr + a) * kTB + tc + 16 * q] = acc[a][q];
}

// acc (64 x TG, a TR x TC tile per thread: rows TR tr + i, columns tc + TPR j)
// -= A (64 x 64, smem, padded) * Y (64 x TG, smem)
template <int TG, typename V>
__device__ __forceinline__ void block_gemm_sub(V (&acc)[TriTile<TG>::TR][TriTile<TG>::TC], const V* As, const V* Ys,
                                               int tr, int tc) {
  constexpr int TR = TriTile<TG>::TR, TC = TriTile<TG>::TC, TPR = TriTile<TG>::TPR;
#pragma unroll 4
  for (int kk = 0; kk < kTB; ++kk) {
    V a[TR], y[TC];
#pragma unroll
    for (int i = 0; i < TR; ++i) a[i] = As[(TR * tr + i) * (kTB + 1) + kk];
#pragma unroll
    for (int j = 0; j < TC; ++j) y[j] = Ys[kk * TG + tc + TPR * j];
#pragma unroll
    for (int i = 0; i < TR; ++i)
#pragma unroll
      for (int j = 0; j < TC; ++j) cfms(acc[i][j], a[i], y[j]);
  }
}

// Stage st of work item (block row i, ndep dependencies) into buf: for
// st < ndep - 1 the factor block of dependency st (it does not depend on the
// flag), then the inverted diagonal block (full 64 x 64; the only stage when
// ndep = 0), then W_i = Inv_i F_(i, last dependency).
template <bool UPPER, typename V>
__device__ __forceinline__ void tri_stage(V* buf, int st, int ndep, const V* __restrict__ F, int64_t ldf,
                                          const V* __restrict__ Inv, const V* __restrict__ W, int i, int nb, int n,
                                          int r0, int rb, int tid) {
  if (ndep > 0 && st == ndep) {
    const V* w = W + (int64_t)i * kTB * kTB;
    for (int idx = tid; idx < kTB * kTB; idx += 256)
      cp_async_elem<(int)sizeof(V)>(buf + (idx >> 6) * (kTB + 1) + (idx & 63), w + idx, true);
  } else if (st < ndep - 1) {
    const int j = UPPER ? nb - 1 - st : st;
    const int c0 = j * kTB, cb = min(kTB, n - c0);
    for (int idx = tid; idx < kTB * kTB; idx += 256) {
      const int r = idx >> 6, c = idx & 63;
      const bool ok = r < rb && c < cb;
      cp_async_elem<(int)sizeof(V)>(buf + r * (kTB + 1) + c, ok ? F + (int64_t)(r0 + r) * ldf + c0 + c : F, ok);
    }
  } else {
    const V* inv = Inv + (int64_t)i * kTB * kTB;
    for (int idx = tid; idx < kTB * kTB; idx += 256)
      cp_async_elem<(int)sizeof(V)>(buf + (idx >> 6) * (kTB + 1) + (idx & 63), inv + idx, true);
  }
  cp_async_commit();
}

// Persistent solve of one triangle.  Work items (block row, column group) are
// claimed in dependency order; groups are independent chains.  An item's
// stages are the factor blocks it depends on, then its inverted diagonal
// block; each is copied asynchronously, and with two buffers the next stage
// loads while the current block product runs.
// Split sums: each (block row, group) is `parts` items, claimed helpers
// first.  Helper p >= 1 sums the products of dependencies
// [last - (p+1) dper, last - p dper) into its slot of `part` and releases its
// flag in `hflags`; the main item (p = 0) sums the dper dependencies before
// the last, adds the helpers' slots, then solves as above.  A row's long sum
// of block products is thus spread over `parts` CTAs.  Every item waits only
// on items claimed before it, so progress is guaranteed as before.
template <typename T, bool UPPER, int TG>
__global__ void __launch_bounds__(256)
tri_solve_kernel(const cplx<T>* __restrict__ F, int64_t ldf, const cplx<T>* __restrict__ Inv,
                 const cplx<T>* __restrict__ W, cplx<T>* __restrict__ X, int64_t ldx, int n, int ncols,
                 unsigned* counter, unsigned* flags, const unsigned* epoch_ptr, int* status, int parts, int dper,
                 cplx<T>* __restrict__ part, unsigned* hflags) {
  // flag value of this solve: bumped on the device before the launch, so a
  // replay from a CUDA graph never sees the previous run's flags as ready
  const unsigned epoch = *(volatile const unsigned*)epoch_ptr;
  using V = cplx<T>;
  constexpr int TR = TriTile<TG>::TR, TC = TriTile<TG>::TC, TPR = TriTile<TG>::TPR;
  constexpr int NBUF = tri_nbuf<T>();
  constexpr int kAs = kTB * (kTB + 1);               // one padded 64 x 64 block
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* Asb = reinterpret_cast<V*>(smem_raw);          // NBUF x [kTB][kTB + 1]
  V* Ys = Asb + NBUF * kAs;                          // [kTB][TG]
  __shared__ unsigned s_item;
  __shared__ int s_fail;
  const int tid = threadIdx.x, tr = tid / TPR, tc = tid % TPR;
  const int nb = (n + kTB - 1) / kTB, ng = (ncols + TG - 1) / TG;
  const unsigned items = (unsigned)nb * ng * parts;
  while (true) {
    if (tid == 0) { s_item = atomicAdd(counter, 1u); s_fail = 0; }
    __syncthreads();
    const unsigned k = s_item;
    if (k >= items) break;
    const unsigned rg = k / parts;
    const int p = parts - 1 - (int)(k % parts);   // helpers (p >= 1, farthest first), then the main item
    const int kr = (int)(rg / ng), g = (int)(rg % ng);
    const int i = UPPER ? nb - 1 - kr : kr;
    const int r0 = i * kTB, rb = min(kTB, n - r0), cg = g * TG;
    unsigned* gflags = flags + (size_t)g * nb;
    // dependencies in completion order: ascending for L, descending for U.
    // All but the last are applied as they complete; then Z = Inv_i acc is
    // formed before the last one is done, and after it X_i = Z - W_i X_last:
    // one product on the chain from block to block instead of two.
    const int ndep = UPPER ? nb - 1 - i : i;
    // dependencies [dlo(q), dhi(q)) of part q (the last one, ndep - 1, is the main item's)
    auto dlo = [&](int q) { return max(0, ndep - 1 - (q + 1) * dper); };
    auto dhi = [&](int q) { return max(0, ndep - 1 - q * dper); };
    const size_t slot = ((size_t)i * ng + g) * (parts - 1);   // + q - 1 for helper q
    auto stage = [&](V* buf, int st) { tri_stage<UPPER>(buf, st, ndep, F, ldf, Inv, W, i, nb, n, r0, rb, tid); };
    auto bufof = [&](int st) { return Asb + (NBUF == 2 ? (st & 1) * kAs : 0); };
    // wait for dependency d's completion flag and stage its rows of X in Ys
    auto take_dep = [&](int d) -> bool {
      const int j = UPPER ? nb - 1 - d : d;
      const int c0 = j * kTB, cb = min(kTB, n - c0);
      if (tid == 0) {
        unsigned it = 0;
        while (ld_acquire_u32(gflags + j) != epoch) {
          if (++it > kSpinLimit) { s_fail = 1; atomicExch(status, MGT_ERR_TIMEOUT); break; }
          if (it > 64) __nanosleep(32);
        }
      }
      __syncthreads();
      if (s_fail) return false;
      for (int idx = tid; idx < kTB * TG; idx += 256) {
        int r = idx / TG, c = idx % TG;
        Ys[idx] = (r < cb && cg + c < ncols) ? ldcg(X + (int64_t)(c0 + r) * ldx + cg + c) : czero<V>();
      }
      __syncthreads();
      return true;
    };
    V acc[TR][TC];
    if (p > 0) {
      // helper: -(sum of its dependencies' products) into its slot
      const int lo = dlo(p), hi = dhi(p);
      if (lo >= hi) {
        __syncthreads();   // every thread has read s_item before it is claimed again
        continue;
      }
#pragma unroll
      for (int a = 0; a < TR; ++a)
#pragma unroll
        for (int b = 0; b < TC; ++b) acc[a][b] = czero<V>();
      stage(bufof(lo), lo);
      for (int d = lo; d < hi; ++d) {
        const bool next = d + 1 < hi;
        if (NBUF == 2 && next) stage(bufof(d + 1), d + 1);
        if (NBUF == 2 && next) cp_async_wait<1>(); else cp_async_wait<0>();
        if (!take_dep(d)) {
          cp_async_wait<0>();
          return;
        }
        block_gemm_sub<TG>(acc, bufof(d), Ys, tr, tc);
        __syncthreads();
        if (NBUF == 1 && next) stage(bufof(d + 1), d + 1);
      }
      V* out = part + (slot + p - 1) * (size_t)(kTB * TG);
#pragma unroll
      for (int a = 0; a < TR; ++a)
#pragma unroll
        for (int b = 0; b < TC; ++b) out[(TR * tr + a) * TG + tc + TPR * b] = acc[a][b];
      __threadfence();
      __syncthreads();
      if (tid == 0) st_release_u32(hflags + slot + p - 1, epoch);
      continue;
    }
#pragma unroll
    for (int a = 0; a < TR; ++a)
#pragma unroll
      for (int b = 0; b < TC; ++b) {
        const int r = TR * tr + a, c = cg + tc + TPR * b;
        acc[a][b] = (r < rb && c < ncols) ? X[(int64_t)(r0 + r) * ldx + c] : czero<V>();
      }
    const int d0 = dlo(0);
    stage(bufof(d0), d0);
    for (int d = d0; d < ndep - 1; ++d) {
      if (NBUF == 2) stage(bufof(d + 1), d + 1);
      if (NBUF == 2) cp_async_wait<1>(); else cp_async_wait<0>();
      if (!take_dep(d)) {
        cp_async_wait<0>();
        return;
      }
      block_gemm_sub<TG>(acc, bufof(d), Ys, tr, tc);
      __syncthreads();
      if (NBUF == 1) stage(bufof(d + 1), d + 1);
    }
    // the helpers' sums (helpers beyond the first empty one are empty too)
    for (int q = 1; q < parts && dlo(q) < dhi(q); ++q) {
      if (tid == 0) {
        unsigned it = 0;
        while (ld_acquire_u32(hflags + slot + q - 1) != epoch) {
          if (++it > kSpinLimit) { s_fail = 1; atomicExch(status, MGT_ERR_TIMEOUT); break; }
          if (it > 64) __nanosleep(32);
        }
      }
      __syncthreads();
      if (s_fail) {
        cp_async_wait<0>();
        return;
      }
      const V* in = part + (slot + q - 1) * (size_t)(kTB * TG);
#pragma unroll
      for (int a = 0; a < TR; ++a)
#pragma unroll
        for (int b = 0; b < TC; ++b) {
          const V v = ldcg(in + (TR * tr + a) * TG + tc + TPR * b);
          acc[a][b].x += v.x;
          acc[a][b].y += v.y;
        }
    }
    // Z = Inv_i * acc (Inv_i is stage max(ndep - 1, 0)); W_i loads meanwhile
    const int sinv = ndep > 0 ? ndep - 1 : 0;
    if (NBUF == 2 && ndep > 0) {
      stage(bufof(ndep), ndep);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
#pragma unroll
    for (int a = 0; a < TR; ++a)
#pragma unroll
      for (int b = 0; b < TC; ++b) Ys[(TR * tr + a) * TG + tc + TPR * b] = acc[a][b];
    __syncthreads();
    V out[TR][TC];
#pragma unroll
    for (int a = 0; a < TR; ++a)
#pragma unroll
      for (int b = 0; b < TC; ++b) out[a][b] = czero<V>();
    block_gemm_sub<TG>(out, bufof(sinv), Ys, tr, tc);   // out = -Z
#pragma unroll
    for (int a = 0; a < TR; ++a)
#pragma unroll
      for (int b = 0; b < TC; ++b) {
        out[a][b].x = -out[a][b].x;
        out[a][b].y = -out[a][b].y;
      }
    __syncthreads();
    if (ndep > 0) {
      if (NBUF == 1) stage(bufof(ndep), ndep);
      cp_async_wait<0>();
      if (!take_dep(ndep - 1)) return;
      block_gemm_sub<TG>(out, bufof(ndep), Ys, tr, tc);   // X_i = Z - W_i X_last
    }
#pragma unroll
    for (int a = 0; a < TR; ++a)
#pragma unroll
      for (int b = 0; b < TC; ++b) {
        const int r = TR * tr + a, c = cg + tc + TPR * b;
        if (r < rb && c < ncols) X[(int64_t)(r0 + r) * ldx + c] = out[a][b];
      }
    __threadfence();
    __syncthreads();
    if (tid == 0) st_release_u32(gflags + i, epoch);
  }
}

// counter = 0 for the work-item claims; every completion flag of this solve
// cleared and the completion mark set to 1.  The workspace is allocated by the
// caller and may hold anything (a freed permutation holds every small
// integer), so nothing of the protocol may depend on its previous contents.
__global__ void tri_start_kernel(unsigned* counter, unsigned* mark, unsigned* flags, int nflags) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    *counter = 0;
    *mark = 1;
  }
  for (int f = i; f < nflags; f += gridDim.x * blockDim.x) flags[f] = 0;
}

// Items per (block row, column group): the main item and its helpers, for a
// solve of nb block rows (the last rows' sums then take about nb / parts
// block products in a row instead of nb)
static int tri_parts(int64_t nb) { return nb >= 64 ? 4 : 1; }

// Workspace of one triangular solve: counter, completion mark and status
// (256 B); completion flags (groups x blocks) followed by the helpers' flags
// (groups x blocks x (parts - 1)); inverted diagonal blocks (L and U); chain
// factors W (L and U); the helpers' partial sums (64 x group width each).
// Sized for the narrow groups (the most flags); a solve in wide groups fits.
struct TriWs {
  size_t flags = 256, inv, wch, part, total;
  TriWs(int64_t n, int64_t nrhs, size_t elem) {
    const int64_t nb = (n + kTB - 1) / kTB, ng = (nrhs + kTG - 1) / kTG, P = tri_parts(nb);
    inv = flags + (((size_t)(nb * ng * P) * sizeof(unsigned) + 255) & ~size_t(255));
    wch = inv + 2 * (size_t)nb * kTB * kTB * elem;
    part = wch + 2 * (size_t)nb * kTB * kTB * elem;
    const int64_t cols = (nrhs + kTGWide - 1) / kTGWide * kTGWide;   // >= groups x group width
    total = part + (size_t)(nb * (P - 1)) * kTB * cols * elem;
  }
};

size_t tri_solve_workspace_bytes(int64_t n, int64_t nrhs, size_t elem) { return TriWs(n, nrhs, elem).total; }

static int resident_ctas(const void* kern, size_t smem) {
  int dev = 0, sms = 1, per = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, 256, smem);
  return std::max(1, sms * std::max(1, per));
}

// In-place X = T^-1 X (T = unit lower or upper part of F), nrhs columns.
template <typename T, bool UPPER>
int tri_solve(const cplx<T>* F, int64_t ldf, cplx<T>* X, int64_t ldx, int n, int nrhs, void* work, int* status,
              cudaStream_t s) {
  using V = cplx<T>;
  const size_t smem_inv = (size_t)(kTB * (kTB + 1) + kTB * kInvLd) * sizeof(V);
  const size_t smem = (size_t)(tri_nbuf<T>() * kTB * (kTB + 1) + kTB * kTG) * sizeof(V);
  const size_t smem_w = (size_t)(tri_nbuf<T>() * kTB * (kTB + 1) + kTB * kTGWide) * sizeof(V);
  const size_t smem_cf = (size_t)(2 * kTB * (kTB + 1)) * sizeof(V);
  // resident-CTA caps per device (set with the device's function attributes)
  static int max_ctas_dev[kMaxDevices], max_ctas_w_dev[kMaxDevices];
  static OncePerDevice once;
  const int dev = current_device();
  once([smem, smem_w, smem_inv, smem_cf, dev] {
    int& max_ctas = max_ctas_dev[dev];
    int& max_ctas_w = max_ctas_w_dev[dev];
    cudaFuncSetAttribute(diag_inverse_kernel<T, UPPER>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_inv);
    cudaFuncSetAttribute(chain_factor_kernel<T, UPPER>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_cf);
    cudaFuncSetAttribute(tri_solve_kernel<T, UPPER, kTG>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    // at most two CTAs per SM: the block row on the dependency chain shares its
    // SM with fewer off-chain products (n = 12000, 64 RHS: 5.15 -> 4.80 ms per
    // complex64 LU solve against the three that fit)
    max_ctas = std::min(resident_ctas((const void*)tri_solve_kernel<T, UPPER, kTG>, smem), 2 * device_sm_count());
    if constexpr (sizeof(T) == 4) {
      cudaFuncSetAttribute(tri_solve_kernel<T, UPPER, kTGWide>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem_w);
      max_ctas_w = std::min(resident_ctas((const void*)tri_solve_kernel<T, UPPER, kTGWide>, smem_w),
                            2 * device_sm_count());
    }
  });
  // wide column groups where block rows alone give enough parallelism
  const bool wide = sizeof(T) == 4 && n >= kWideMinN;
  const int tg = wide ? kTGWide : kTG;
  const int nb = (n + kTB - 1) / kTB, ng = (nrhs + tg - 1) / tg;
  const int parts = tri_parts(nb);
  const int dper = parts > 1 ? (nb - 1 + parts - 1) / parts : std::max(1, nb);   // parts x dper >= nb - 1
  const TriWs L(n, nrhs, sizeof(V));
  unsigned* counter = (unsigned*)work;
  unsigned* flags = (unsigned*)((char*)work + L.flags);
  unsigned* hflags = flags + (size_t)nb * ng;
  // inverted diagonal blocks (L, then U), then the chain factors W (L, then U)
  V* inv = (V*)((char*)work + L.inv) + (UPPER ? (size_t)nb * kTB * kTB : 0);
  V* wch = (V*)((char*)work + L.wch) + (UPPER ? (size_t)nb * kTB * kTB : 0);
  V* part = (V*)((char*)work + L.part);
  count_launch(2);
  diag_inverse_kernel<T, UPPER><<<nb, 256, smem_inv, s>>>(F, ldf, n, inv);
  chain_factor_kernel<T, UPPER><<<nb, 256, smem_cf, s>>>(F, ldf, n, inv, wch);
  unsigned* epoch = counter + 1;   // completion mark, set by tri_start_kernel
  const int nflags = nb * ng * parts;
  const int64_t items = (int64_t)nb * ng * parts;
  count_launch();
  tri_start_kernel<<<std::max(1, std::min(nflags, 1 << 16) / 256 + 1), 256, 0, s>>>(counter, epoch, flags, nflags);
  count_launch();
  if constexpr (sizeof(T) == 4) {
    if (wide) {
      const int grid = (int)std::min<int64_t>(items, std::max(1, max_ctas_w_dev[dev]));
      tri_solve_kernel<T, UPPER, kTGWide><<<grid, 256, smem_w, s>>>(F, ldf, inv, wch, X, ldx, n, nrhs, counter,
                                                                     flags, epoch, status, parts, dper, part,
                                                                     hflags);
      return cudaGetLastError() == cudaSuccess ? MGT_OK : MGT_ERR_CUDA;
    }
  }
  {
    const int grid = (int)std::min<int64_t>(items, std::max(1, max_ctas_dev[dev]));
    tri_solve_kernel<T, UPPER, kTG><<<grid, 256, smem, s>>>(F, ldf, inv, wch, X, ldx, n, nrhs, counter, flags,
                                                             epoch, status, parts, dper, part, hflags);
  }
  return cudaGetLastError() == cudaSuccess ? MGT_OK : MGT_ERR_CUDA;
}

// Inverses of the 64 x 64 diagonal blocks of a unit lower factor of order n
// (rows / columns at F), written to Inv[block][64][64]; the LU uses it for the
// two inner panels of a 128-wide block.
template <typename T>
int lower_block_inverses(const cplx<T>* F, int64_t ldf, int n, cplx<T>* Inv, cudaStream_t s) {
  using V = cplx<T>;
  const size_t smem_inv = (size_t)(kTB * (kTB + 1) + kTB * kInvLd) * sizeof(V);
  static OncePerDevice once;
  once([smem_inv] {
    cudaFuncSetAttribute(diag_inverse_kernel<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_inv);
  });
  count_launch();
  diag_inverse_kernel<T, false><<<(n + kTB - 1) / kTB, 256, smem_inv, s>>>(F, ldf, n, Inv);
  return cudaGetLastError() == cudaSuccess ? MGT_OK : MGT_ERR_CUDA;
}
template int lower_block_inverses<float>(const float2*, int64_t, int, float2*, cudaStream_t);

template int tri_solve<double, false>(const double2*, int64_t, double2*, int64_t, int, int, void*, int*, cudaStream_t);
template int tri_solve<double, true>(const double2*, int64_t, double2*, int64_t, int, int, void*, int*, cudaStream_t);
template int tri_solve<float, false>(const float2*, int64_t, float2*, int64_t, int, int, void*, int*, cudaStream_t);
template int tri_solve<float, true>(const float2*, int64_t, float2*, int64_t, int, int, void*, int*, cudaStream_t);

}  // namespace mgt
