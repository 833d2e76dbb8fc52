// K4: double-float residual R = B - M X and the mixed-precision refinement
// driver (complex64 LU + double-float residual -> complex128 accuracy).
//
// The reference solves once in complex128 (torch.linalg.solve in solve(),
// Transmission2D.py:230, Transmission3D.py:205).  Here the factorisation runs
// in complex64 and classical iterative refinement (Wilkinson; Moler 1967)
// recovers FP64 accuracy: x += LU^-1 (b - M x), with the residual formed in
// double-float arithmetic from a double-float copy of M.
#include <algorithm>
#include <mutex>

#include "common.cuh"
#include "df.cuh"
#include "diag.cuh"
#include "residual_tc.cuh"

namespace mgt {

constexpr int kResRPT = 2;              // rows of R per thread
constexpr int kResRows = 16 * kResRPT;  // rows of R per CTA
constexpr int kResK = 16;               // K chunk staged in shared memory
// Columns of R per launch.  Two 94-register CTAs of 64 columns per SM beat
// one 156-register CTA of 128 columns once K is split (GB300, n = 12000,
// 128 right-hand sides: 29.9 vs 31.1 ms).
constexpr int kResCols = 64;

// Each thread owns rows {ty + 16 i : i < kResRPT} and columns {tx + 16 j : j < RT}.
template <int RT>
__global__ void __launch_bounds__(256)
residual_df_kernel(const float4* __restrict__ M, int64_t ldm, const float4* __restrict__ Xs, int64_t ldxs,
                   const double2* __restrict__ B, int64_t ldb, double2* __restrict__ R, int64_t ldr, int n,
                   int kdim, int ncols, int col_base, int k_per_split, double2* __restrict__ partial) {
  constexpr int RPT = kResRPT;
  __shared__ float4 Ms[kResRows][kResK + 1];
  __shared__ float4 Xsh[kResK][16 * RT];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int row0 = blockIdx.x * kResRows;
  float4 acc[RPT][RT];
#pragma unroll
  for (int i = 0; i < RPT; ++i)
#pragma unroll
    for (int j = 0; j < RT; ++j) acc[i][j] = make_float4(0.f, 0.f, 0.f, 0.f);
  // split-K (partial != null): this CTA covers K range [kbeg, kend) and
  // writes its joined sum to partial[blockIdx.y]
  const int kbeg = blockIdx.y * k_per_split, kend = min(kdim, kbeg + k_per_split);
  for (int k0 = kbeg; k0 < kend; k0 += kResK) {
#pragma unroll
    for (int q = 0; q < RPT; ++q) {
      int idx = tid + 256 * q;
      int r = idx >> 4, kk = idx & 15;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (row0 + r < n && k0 + kk < kend) v = M[(int64_t)(row0 + r) * ldm + k0 + kk];
      Ms[r][kk] = v;
    }
    for (int idx = tid; idx < kResK * 16 * RT; idx += 256) {
      int kk = idx / (16 * RT), c = idx - kk * (16 * RT);
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (k0 + kk < kend && c < ncols) v = Xs[(int64_t)(k0 + kk) * ldxs + col_base + c];
      Xsh[kk][c] = v;
    }
    __syncthreads();
#pragma unroll 2
    for (int kk = 0; kk < kResK; ++kk) {
      float4 a[RPT];
#pragma unroll
      for (int i = 0; i < RPT; ++i) a[i] = Ms[ty + 16 * i][kk];
#pragma unroll
      for (int j = 0; j < RT; ++j) {
        const float4 x = Xsh[kk][tx + 16 * j];
#pragma unroll
        for (int i = 0; i < RPT; ++i) df_cmac(acc[i][j], a[i], x);
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < RPT; ++i) {
    int r = row0 + ty + 16 * i;
    if (r >= n) continue;
#pragma unroll
    for (int j = 0; j < RT; ++j) {
      int c = tx + 16 * j;
      if (c < ncols) {
        double2 mx = df_join(acc[i][j]);
        if (partial) {
          partial[((int64_t)blockIdx.y * n + r) * ncols + c] = mx;
        } else {
          double2 b = B ? B[(int64_t)r * ldb + col_base + c] : make_double2(0.0, 0.0);
          R[(int64_t)r * ldr + col_base + c] = make_double2(b.x - mx.x, b.y - mx.y);
        }
      }
    }
  }
}

__global__ void split_df_kernel(const double2* __restrict__ X, int64_t ldx, float4* __restrict__ Y, int64_t ldy,
                                int n, int ncols) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)n * ncols) return;
  int r = (int)(idx / ncols), c = (int)(idx - (int64_t)r * ncols);
  Y[(int64_t)r * ldy + c] = df_split(X[(int64_t)r * ldx + c]);
}

__global__ void c128_to_c64_kernel(const double2* __restrict__ X, int64_t ldx, float2* __restrict__ Y, int64_t ldy,
                                   int n, int ncols) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)n * ncols) return;
  int r = (int)(idx / ncols), c = (int)(idx - (int64_t)r * ncols);
  double2 v = X[(int64_t)r * ldx + c];
  Y[(int64_t)r * ldy + c] = make_float2((float)v.x, (float)v.y);
}

// X (complex128) = Y (complex64) when assign, X += Y otherwise
__global__ void c64_into_c128_kernel(const float2* __restrict__ Y, int64_t ldy, double2* __restrict__ X, int64_t ldx,
                                     int n, int ncols, int assign) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)n * ncols) return;
  int r = (int)(idx / ncols), c = (int)(idx - (int64_t)r * ncols);
  float2 y = Y[(int64_t)r * ldy + c];
  double2* x = X + (int64_t)r * ldx + c;
  if (assign) *x = make_double2(y.x, y.y);
  else *x = make_double2(x->x + (double)y.x, x->y + (double)y.y);
}

// out[slot] += sum |X|^2 (slot 0 or 1); FP64 accumulation per thread, then atomics
__global__ void sumsq_kernel(const double2* __restrict__ X, int64_t ldx, int n, int ncols, double* out) {
  double s = 0.0;
  int64_t total = (int64_t)n * ncols;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int r = (int)(idx / ncols), c = (int)(idx - (int64_t)r * ncols);
    double2 v = X[(int64_t)r * ldx + c];
    s = fma(v.x, v.x, fma(v.y, v.y, s));
  }
#pragma unroll
  for (int off = 16; off; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
  __shared__ double red[8];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    atomicAdd(out, t);
  }
}

template <int RT>
static void launch_residual(const float4* M, int64_t ldm, const float4* Xs, int64_t ldxs, const double2* B,
                            int64_t ldb, double2* R, int64_t ldr, int n, int kdim, int ncols, int col_base,
                            int ksplit, int kps, double2* partial, cudaStream_t s) {
  count_launch();
  dim3 grid((n + kResRows - 1) / kResRows, ksplit);
  residual_df_kernel<RT><<<grid, 256, 0, s>>>(M, ldm, Xs, ldxs, B, ldb, R, ldr, n, kdim, ncols, col_base, kps,
                                              partial);
}

// resident CTAs per SM of residual_df_kernel<RT> (1 when no device answers)
template <int RT>
static int residual_occupancy() {
  static int occ[kMaxDevices];
  static OncePerDevice once;
  const int dev = current_device();
  once([dev] {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, residual_df_kernel<RT>, 256, 0) == cudaSuccess && b > 0)
      occ[dev] = b;
    else {
      occ[dev] = 1;
      cudaGetLastError();
    }
  });
  return occ[dev];
}

// R = B - sum of the split-K partials (FP64)
__global__ void residual_reduce_kernel(const double2* __restrict__ partial, int ksplit, int n, int ncols,
                                       const double2* __restrict__ B, int64_t ldb, double2* __restrict__ R,
                                       int64_t ldr, int col_base) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)n * ncols) return;
  const int r = (int)(idx / ncols), c = (int)(idx - (int64_t)r * ncols);
  double2 acc = B ? B[(int64_t)r * ldb + col_base + c] : make_double2(0.0, 0.0);
  for (int q = 0; q < ksplit; ++q) {
    const double2 v = partial[(int64_t)q * n * ncols + idx];
    acc.x -= v.x;
    acc.y -= v.y;
  }
  R[(int64_t)r * ldr + col_base + c] = acc;
}

static int res_num_sms() { return device_sm_count(); }

// K splits of a rows x kdim residual over ncols (<= kResCols) columns.
// Many short CTAs balance the SMs better than a few long ones: the split
// aims for at least six waves of CTAs, then takes the first split whose last
// wave is at least 97% full (else the fullest), at most 16 splits of at
// least 256 columns of K each.  Measured on GB300 (64 columns): n = 2000
// 1.12 -> 0.47 ms, 12000 19.5 -> 15.5 ms, 27000 81.6 -> 75 ms.
int residual_ksplit(int rows, int kdim, int ncols) {
  if (rows <= 0 || kdim <= 0) return 1;
  const int nc = std::min(std::max(ncols, 1), kResCols);
  const int occ = nc <= 16 ? residual_occupancy<1>() : nc <= 32 ? residual_occupancy<2>() : residual_occupancy<4>();
  const int64_t slots = (int64_t)res_num_sms() * occ;
  const int64_t rb = (rows + kResRows - 1) / kResRows;
  const int kmax = std::max(1, std::min(16, kdim / 256));
  const int lo = (int)std::min<int64_t>(kmax, std::max<int64_t>(1, (6 * slots + rb - 1) / rb));
  int best = lo;
  double best_fill = 0.0;
  for (int ks = lo; ks <= kmax; ++ks) {
    const int64_t ctas = rb * ks, waves = (ctas + slots - 1) / slots;
    const double fill = (double)ctas / (double)(waves * slots);
    if (fill >= 0.97) return ks;
    if (fill > best_fill) { best_fill = fill; best = ks; }
  }
  return best;
}

// complex128 elements of the split-K partial buffer for a rows x kdim residual
// with nrhs right-hand sides
int64_t residual_partial_elems(int64_t rows, int64_t kdim, int64_t nrhs) {
  if (rows <= 0 || kdim <= 0 || nrhs <= 0 || rows > (1 << 30) || kdim > (1 << 30)) return 0;
  const int nc = (int)std::min<int64_t>(nrhs, kResCols);
  const int ks = residual_ksplit((int)rows, (int)kdim, nc);
  return ks > 1 ? (int64_t)ks * rows * nc : 0;
}

// R (rows x nrhs) = B - M Xs, M (rows x kdim) double-float, Xs (kdim x nrhs,
// leading dimension ldxs) the double-float copy of X; B may be null (zero).
// Columns go in tiles of kResCols.  With a partial buffer (partial_elems
// complex128) the K range is split across CTAs: residual_ksplit splits,
// fewer if the buffer holds fewer than splits x rows x min(nrhs, kResCols).
int residual_rect(const float4* M, int64_t ldm, const float4* Xs, int64_t ldxs, const double2* B, int64_t ldb,
                  double2* R, int64_t ldr, int rows, int kdim, int nrhs, cudaStream_t s, double2* partial,
                  int64_t partial_elems) {
  const int ncmax = std::min(nrhs, kResCols);
  int ksplit = partial ? residual_ksplit(rows, kdim, ncmax) : 1;
  // never more splits than the partial buffer holds
  const int64_t per_split = (int64_t)rows * ncmax;
  if (per_split > 0) ksplit = (int)std::max<int64_t>(1, std::min<int64_t>(ksplit, partial_elems / per_split));
  const int kps = ksplit > 1 ? (((kdim + ksplit - 1) / ksplit + kResK - 1) / kResK) * kResK : kdim;
  double2* part = ksplit > 1 ? partial : nullptr;
  for (int c0 = 0; c0 < nrhs; c0 += kResCols) {
    int nc = std::min(kResCols, nrhs - c0);
    int rt = (nc + 15) / 16;
    switch (rt) {
      case 1: launch_residual<1>(M, ldm, Xs, ldxs, B, ldb, R, ldr, rows, kdim, nc, c0, ksplit, kps, part, s); break;
      case 2: launch_residual<2>(M, ldm, Xs, ldxs, B, ldb, R, ldr, rows, kdim, nc, c0, ksplit, kps, part, s); break;
      default: launch_residual<4>(M, ldm, Xs, ldxs, B, ldb, R, ldr, rows, kdim, nc, c0, ksplit, kps, part, s); break;
    }
    if (part) {
      const int64_t tot = (int64_t)rows * nc;
      count_launch();
      residual_reduce_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(part, ksplit, rows, nc, B, ldb, R, ldr,
                                                                           c0);
    }
  }
  return cudaGetLastError() == cudaSuccess ? MGT_OK : MGT_ERR_CUDA;
}

// Xs (n x ncols, leading dimension ldy) = double-float split of X
int split_df(const double2* X, int64_t ldx, float4* Xs, int64_t ldy, int n, int ncols, cudaStream_t s) {
  int64_t tot = (int64_t)n * ncols;
  if (tot <= 0) return MGT_OK;
  count_launch();
  split_df_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(X, ldx, Xs, ldy, n, ncols);
  return cudaGetLastError() == cudaSuccess ? MGT_OK : MGT_ERR_CUDA;
}

static int residual_impl(const float4* M, int64_t ldm, const double2* X, int64_t ldx, const double2* B, int64_t ldb,
                         double2* R, int64_t ldr, int n, int nrhs, float4* Xs, double2* part, int64_t part_elems,
                         cudaStream_t s) {
  int e = split_df(X, ldx, Xs, nrhs, n, nrhs, s);
  if (e != MGT_OK) return e;
  return residual_rect(M, ldm, Xs, nrhs, B, ldb, R, ldr, n, n, nrhs, s, part, part_elems);
}

size_t tri_solve_workspace_bytes(int64_t n, int64_t nrhs, size_t elem);

// refinement workspace layout: the residual runs on the tensor cores
// (residual_tc.cu) where the device and shape allow, in double-float on the
// FP32 pipes otherwise
struct RefineWs {
  bool tc;        // tensor-core residual
  float4* Xs;     // (double-float residual) n x nrhs double-float copy of X
  double2* Rr;    // n x nrhs residual
  float2* R32;    // n x nrhs complex64 residual / right-hand side
  float2* D32;    // n x nrhs complex64 correction
  double* norms;  // [0] = ||B||^2, [1] = ||R||^2
  void* tri;      // triangular-solve flags
  double2* part;  // (double-float residual) split-K partial sums
  int64_t part_elems;
  int* rowexp;    // (tensor-core residual) row exponents of M
  unsigned char* digits;   // (tensor-core residual) digits of M
  void* tcw;      // (tensor-core residual) one application's workspace
  size_t tcw_bytes;
  size_t total;
  RefineWs(void* base, int64_t n, int64_t r) {
    char* b = (char*)base;
    size_t off = 0;
    auto take = [&](size_t bytes) { char* p = b ? b + off : nullptr; off += (bytes + 255) & ~size_t(255); return p; };
    tc = residual_tc_supported(n, n, r);
    rowexp = nullptr;
    digits = nullptr;
    if (tc) {
      // M's row exponents and digits first: their place does not depend on
      // nrhs, so a workspace prepared once serves solves of fewer columns
      rowexp = (int*)take(n * sizeof(int));
      off = (off + 1023) & ~size_t(1023);
      digits = (unsigned char*)take(residual_tc_digits_bytes(n, n));
      off = (off + 1023) & ~size_t(1023);
    }
    Rr = (double2*)take(n * r * sizeof(double2));
    R32 = (float2*)take(n * r * sizeof(float2));
    D32 = (float2*)take(n * r * sizeof(float2));
    norms = (double*)take(2 * sizeof(double));
    tri = take(tri_solve_workspace_bytes(n, r, sizeof(float2)));
    Xs = nullptr;
    part = nullptr;
    part_elems = 0;
    tcw = nullptr;
    tcw_bytes = 0;
    if (tc) {
      off = (off + 1023) & ~size_t(1023);
      tcw_bytes = residual_tc_apply_bytes(n, n, r);
      tcw = take(tcw_bytes);
    } else {
      Xs = (float4*)take(n * r * sizeof(float4));
      part_elems = residual_partial_elems(n, n, r);
      part = (double2*)take(part_elems * sizeof(double2));
    }
    total = off;
  }
  // Rr = B - M X; prepared: the row exponents and digits of this M are in
  // the workspace already (an earlier residual of the same solve, or
  // mgt_refine_prepare); M may then be null
  int residual(const float4* M, int64_t ldm, const double2* X, int64_t ldx, const double2* B, int64_t ldb, int n,
               int nr, bool prepared, cudaStream_t s) {
    if (tc) {
      if (!prepared) {
        int e = residual_tc_prepare(M, ldm, n, n, rowexp, digits, s);
        if (e != MGT_OK) return e;
      }
      return residual_tc_apply(digits, rowexp, n, n, X, ldx, nr, B, ldb, Rr, nr, tcw, tcw_bytes, s);
    }
    return residual_impl(M, ldm, X, ldx, B, ldb, Rr, nr, n, nr, Xs, part, part_elems, s);
  }
  // device status word of the tensor-core residual (MGT_OK or MGT_ERR_TIMEOUT), or null
  int* status() const { return tc ? (int*)tcw : nullptr; }
};

}  // namespace mgt

using namespace mgt;

extern "C" int mgt_lu_solve(int dtype, const void* LU, int64_t n, int64_t lda, const int32_t* perm,
                            const void* B, int64_t ldb, void* X, int64_t ldx, int64_t nrhs, void* work,
                            size_t work_bytes, void* stream);

extern "C" int mgt_residual_workspace_bytes(int64_t n, int64_t nrhs, size_t* bytes) {
  if (!bytes || n <= 0 || nrhs <= 0) return MGT_ERR_ARG;
  const size_t df = (((size_t)n * nrhs * sizeof(float4) + 255) & ~size_t(255)) +
                    residual_partial_elems(n, n, nrhs) * sizeof(double2) + 256;
  *bytes = std::max(df, residual_tc_workspace_bytes(n, n, nrhs));
  return MGT_OK;
}

extern "C" int mgt_residual(const void* M, int64_t n, int64_t ldm, const void* X, int64_t ldx, const void* B,
                            int64_t ldb, void* R, int64_t ldr, int64_t nrhs, void* work, size_t work_bytes,
                            void* stream) {
  if (!M || !X || !B || !R || !work || n <= 0 || nrhs <= 0 || ldm < n || ldx < nrhs || ldb < nrhs || ldr < nrhs)
    return MGT_ERR_ARG;
  if (n > (1 << 30)) return MGT_ERR_WORKSPACE;
  // tensor cores when the workspace holds their buffers
  if (residual_tc_supported(n, n, nrhs) && work_bytes >= residual_tc_workspace_bytes(n, n, nrhs))
    return residual_tc((const float4*)M, ldm, (int)n, (int)n, (const double2*)X, ldx, (int)nrhs, (const double2*)B,
                       ldb, (double2*)R, ldr, work, work_bytes, (cudaStream_t)stream);
  if (work_bytes < (size_t)n * nrhs * sizeof(float4)) return MGT_ERR_WORKSPACE;
  // split-K partials after the double-float copy of X, as far as the workspace holds them
  const size_t xs_bytes = ((size_t)n * nrhs * sizeof(float4) + 255) & ~size_t(255);
  double2* part = nullptr;
  int64_t part_elems = 0;
  if (work_bytes > xs_bytes) {
    part = (double2*)((char*)work + xs_bytes);
    part_elems = (int64_t)((work_bytes - xs_bytes) / sizeof(double2));
  }
  return residual_impl((const float4*)M, ldm, (const double2*)X, ldx, (const double2*)B, ldb, (double2*)R, ldr,
                       (int)n, (int)nrhs, (float4*)work, part, part_elems, (cudaStream_t)stream);
}

extern "C" int mgt_residual_prepare(const void* M, int64_t n, int64_t ldm, void* work, size_t work_bytes,
                                    void* stream) {
  if (!M || !work || n <= 0 || ldm < n) return MGT_ERR_ARG;
  if (n > (1 << 30)) return MGT_ERR_WORKSPACE;
  if (!residual_tc_supported(n, n, 1)) return MGT_ERR_UNSUPPORTED;
  int* rowexp;
  unsigned char* digits;
  if (work_bytes < residual_tc_split(work, n, n, &rowexp, &digits, nullptr)) return MGT_ERR_WORKSPACE;
  return residual_tc_prepare((const float4*)M, ldm, (int)n, (int)n, rowexp, digits, (cudaStream_t)stream);
}

extern "C" int mgt_residual_apply(int64_t n, const void* X, int64_t ldx, const void* B, int64_t ldb, void* R,
                                  int64_t ldr, int64_t nrhs, void* work, size_t work_bytes, void* stream) {
  if (!X || !B || !R || !work || n <= 0 || nrhs <= 0 || ldx < nrhs || ldb < nrhs || ldr < nrhs) return MGT_ERR_ARG;
  if (n > (1 << 30)) return MGT_ERR_WORKSPACE;
  if (!residual_tc_supported(n, n, nrhs)) return MGT_ERR_UNSUPPORTED;
  if (work_bytes < residual_tc_workspace_bytes(n, n, nrhs)) return MGT_ERR_WORKSPACE;
  int* rowexp;
  unsigned char* digits;
  char* aw;
  const size_t a_off = residual_tc_split(work, n, n, &rowexp, &digits, &aw);
  return residual_tc_apply(digits, rowexp, (int)n, (int)n, (const double2*)X, ldx, (int)nrhs, (const double2*)B, ldb,
                           (double2*)R, ldr, aw, work_bytes - a_off, (cudaStream_t)stream);
}

extern "C" int mgt_refine_workspace_bytes(int64_t n, int64_t nrhs, size_t* bytes) {
  if (!bytes || n <= 0 || nrhs <= 0) return MGT_ERR_ARG;
  *bytes = RefineWs(nullptr, n, nrhs).total;
  return MGT_OK;
}

extern "C" int mgt_solve_refined(const void* M, int64_t ldm, const void* LU, int64_t ldlu, const int32_t* perm,
                                 int64_t n, const void* B, int64_t ldb, void* X, int64_t ldx, int64_t nrhs,
                                 double tol, int max_iter, void* work, size_t work_bytes, int* iters,
                                 double* rel_res, void* stream) {
  if (!LU || !perm || !B || !X || !work || n <= 0 || nrhs <= 0 || (M && ldm < n) || ldlu < n || ldb < nrhs ||
      ldx < nrhs || max_iter < 0)
    return MGT_ERR_ARG;
  RefineWs w(work, n, nrhs);
  if (!M && !w.tc) return MGT_ERR_ARG;   // prepared digits exist only for the tensor-core residual
  if (work_bytes < w.total) return MGT_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  const int nn = (int)n, nr = (int)nrhs;
  const int64_t tot = n * nrhs;
  const unsigned eg = (unsigned)((tot + 255) / 256);
  const double2* Bd = (const double2*)B;
  double2* Xd = (double2*)X;
  double h[2];
  if (cudaMemsetAsync(w.norms, 0, 2 * sizeof(double), s) != cudaSuccess) return MGT_ERR_CUDA;
  count_launch();
  sumsq_kernel<<<std::min<int64_t>(1024, (tot + 255) / 256), 256, 0, s>>>(Bd, ldb, nn, nr, w.norms);
  // x0 = LU^-1 b in complex64
  count_launch();
  c128_to_c64_kernel<<<eg, 256, 0, s>>>(Bd, ldb, w.R32, nr, nn, nr);
  const size_t tri_bytes = tri_solve_workspace_bytes(n, nrhs, sizeof(float2));
  int e = mgt_lu_solve(MGT_C64, LU, n, ldlu, perm, w.R32, nr, w.D32, nr, nrhs, w.tri, tri_bytes, stream);
  if (e != MGT_OK) return e;
  count_launch();
  c64_into_c128_kernel<<<eg, 256, 0, s>>>(w.D32, nr, Xd, ldx, nn, nr, 1);
  double prev = 0.0, rel = 0.0;
  int it = 0;
  int dev_status = MGT_OK;
  for (;; ++it) {
    e = w.residual((const float4*)M, ldm, Xd, ldx, Bd, ldb, nn, nr, it > 0 || !M, s);
    if (e != MGT_OK) return e;
    if (cudaMemsetAsync(w.norms + 1, 0, sizeof(double), s) != cudaSuccess) return MGT_ERR_CUDA;
    count_launch();
    sumsq_kernel<<<std::min<int64_t>(1024, (tot + 255) / 256), 256, 0, s>>>(w.Rr, nr, nn, nr, w.norms + 1);
    if (cudaMemcpyAsync(h, w.norms, 2 * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess) return MGT_ERR_CUDA;
    if (w.status() &&
        cudaMemcpyAsync(&dev_status, w.status(), sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess)
      return MGT_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return MGT_ERR_CUDA;
    if (dev_status != MGT_OK) return dev_status;
    rel = h[0] > 0 ? sqrt(h[1] / h[0]) : sqrt(h[1]);
    if (rel <= tol || it >= max_iter) break;
    if (it > 0 && !(rel < 0.9 * prev)) break;  // stagnation or divergence
    prev = rel;
    count_launch();
    c128_to_c64_kernel<<<eg, 256, 0, s>>>(w.Rr, nr, w.R32, nr, nn, nr);
    e = mgt_lu_solve(MGT_C64, LU, n, ldlu, perm, w.R32, nr, w.D32, nr, nrhs, w.tri, tri_bytes, stream);
    if (e != MGT_OK) return e;
    count_launch();
    c64_into_c128_kernel<<<eg, 256, 0, s>>>(w.D32, nr, Xd, ldx, nn, nr, 0);
  }
  if (iters) *iters = it;
  if (rel_res) *rel_res = rel;
  if (cudaGetLastError() != cudaSuccess) return MGT_ERR_CUDA;
  return (rel <= tol && rel == rel) ? MGT_OK : MGT_ERR_NOT_CONVERGED;
}

// ---------------------------------------------------------------- DOS dots

__global__ void column_dots_kernel(const double2* __restrict__ A, int64_t lda, const double2* __restrict__ B,
                                   int64_t ldb, int n, int ncols, int rows_per_block, double2* out) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncols) return;
  int r0 = blockIdx.y * rows_per_block, r1 = min(n, r0 + rows_per_block);
  double2 acc = make_double2(0.0, 0.0);
  for (int r = r0; r < r1; ++r) cfma(acc, A[(int64_t)r * lda + c], B[(int64_t)r * ldb + c]);
  atomicAdd(&out[c].x, acc.x);
  atomicAdd(&out[c].y, acc.y);
}

extern "C" int mgt_column_dots(const void* A, int64_t lda, const void* B, int64_t ldb, int64_t n, int64_t ncols,
                               void* out, void* stream) {
  if (!A || !B || !out || n <= 0 || ncols <= 0 || lda < ncols || ldb < ncols) return MGT_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemsetAsync(out, 0, ncols * sizeof(double2), s) != cudaSuccess) return MGT_ERR_CUDA;
  int rpb = 64;
  dim3 grid((unsigned)((ncols + 127) / 128), (unsigned)((n + rpb - 1) / rpb));
  if (grid.y > 65535) { rpb = (int)((n + 65534) / 65535); grid.y = (unsigned)((n + rpb - 1) / rpb); }
  count_launch();
  column_dots_kernel<<<grid, 128, 0, s>>>((const double2*)A, lda, (const double2*)B, ldb, (int)n, (int)ncols, rpb,
                                          (double2*)out);
  return cudaGetLastError() == cudaSuccess ? MGT_OK : MGT_ERR_CUDA;
}

extern "C" int mgt_refine_prepare(const void* M, int64_t ldm, int64_t n, int64_t nrhs, void* work, size_t work_bytes,
                                  void* stream) {
  if (!M || !work || n <= 0 || nrhs <= 0 || ldm < n) return MGT_ERR_ARG;
  RefineWs w(work, n, nrhs);
  if (!w.tc) return MGT_ERR_UNSUPPORTED;
  if (work_bytes < w.total) return MGT_ERR_WORKSPACE;
  return residual_tc_prepare((const float4*)M, ldm, (int)n, (int)n, w.rowexp, w.digits, (cudaStream_t)stream);
}

// ---------------------------------------------------------------- stream-ordered refinement steps
//
// The same refinement as mgt_solve_refined, split into steps that only
// enqueue work (no host synchronisation), so that a whole solve can be
// captured into a CUDA graph.  The caller decides how many corrections to
// run and reads the final norms afterwards.

extern "C" int mgt_refine_start(const void* LU, int64_t ldlu, const int32_t* perm, int64_t n, const void* B,
                                int64_t ldb, void* X, int64_t ldx, int64_t nrhs, void* work, size_t work_bytes,
                                void* stream) {
  if (!LU || !perm || !B || !X || !work || n <= 0 || nrhs <= 0 || ldlu < n || ldb < nrhs || ldx < nrhs)
    return MGT_ERR_ARG;
  RefineWs w(work, n, nrhs);
  if (work_bytes < w.total) return MGT_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  const int nn = (int)n, nr = (int)nrhs;
  const unsigned eg = (unsigned)((n * nrhs + 255) / 256);
  count_launch();
  c128_to_c64_kernel<<<eg, 256, 0, s>>>((const double2*)B, ldb, w.R32, nr, nn, nr);
  int e = mgt_lu_solve(MGT_C64, LU, n, ldlu, perm, w.R32, nr, w.D32, nr, nrhs, w.tri,
                       tri_solve_workspace_bytes(n, nrhs, sizeof(float2)), stream);
  if (e != MGT_OK) return e;
  count_launch();
  c64_into_c128_kernel<<<eg, 256, 0, s>>>(w.D32, nr, (double2*)X, ldx, nn, nr, 1);
  return cudaGetLastError() == cudaSuccess ? MGT_OK : MGT_ERR_CUDA;
}

extern "C" int mgt_refine_correct(const void* M, int64_t ldm, const void* LU, int64_t ldlu, const int32_t* perm,
                                  int64_t n, const void* B, int64_t ldb, void* X, int64_t ldx, int64_t nrhs,
                                  void* work, size_t work_bytes, void* stream) {
  if (!LU || !perm || !B || !X || !work || n <= 0 || nrhs <= 0 || (M && ldm < n) || ldlu < n || ldb < nrhs ||
      ldx < nrhs)
    return MGT_ERR_ARG;
  RefineWs w(work, n, nrhs);
  if (!M && !w.tc) return MGT_ERR_ARG;
  if (work_bytes < w.total) return MGT_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  const int nn = (int)n, nr = (int)nrhs;
  const unsigned eg = (unsigned)((n * nrhs + 255) / 256);
  int e = w.residual((const float4*)M, ldm, (const double2*)X, ldx, (const double2*)B, ldb, nn, nr, !M, s);
  if (e != MGT_OK) return e;
  count_launch();
  c128_to_c64_kernel<<<eg, 256, 0, s>>>(w.Rr, nr, w.R32, nr, nn, nr);
  e = mgt_lu_solve(MGT_C64, LU, n, ldlu, perm, w.R32, nr, w.D32, nr, nrhs, w.tri,
                   tri_solve_workspace_bytes(n, nrhs, sizeof(float2)), stream);
  if (e != MGT_OK) return e;
  count_launch();
  c64_into_c128_kernel<<<eg, 256, 0, s>>>(w.D32, nr, (double2*)X, ldx, nn, nr, 0);
  return cudaGetLastError() == cudaSuccess ? MGT_OK : MGT_ERR_CUDA;
}

extern "C" int mgt_refine_norms(const void* M, int64_t ldm, int64_t n, const void* B, int64_t ldb, const void* X,
                                int64_t ldx, int64_t nrhs, void* work, size_t work_bytes, double* norms_dev,
                                void* stream) {
  if (!B || !X || !work || !norms_dev || n <= 0 || nrhs <= 0 || (M && ldm < n) || ldb < nrhs || ldx < nrhs)
    return MGT_ERR_ARG;
  RefineWs w(work, n, nrhs);
  if (!M && !w.tc) return MGT_ERR_ARG;
  if (work_bytes < w.total) return MGT_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  const int nn = (int)n, nr = (int)nrhs;
  const int64_t tot = n * nrhs;
  int e = w.residual((const float4*)M, ldm, (const double2*)X, ldx, (const double2*)B, ldb, nn, nr, !M, s);
  if (e != MGT_OK) return e;
  if (cudaMemsetAsync(norms_dev, 0, 2 * sizeof(double), s) != cudaSuccess) return MGT_ERR_CUDA;
  count_launch(2);
  sumsq_kernel<<<(unsigned)std::min<int64_t>(1024, (tot + 255) / 256), 256, 0, s>>>((const double2*)B, ldb, nn, nr,
                                                                                   norms_dev);
  sumsq_kernel<<<(unsigned)std::min<int64_t>(1024, (tot + 255) / 256), 256, 0, s>>>(w.Rr, nr, nn, nr, norms_dev + 1);
  return cudaGetLastError() == cudaSuccess ? MGT_OK : MGT_ERR_CUDA;
}
