// K5: matrix-free propagation to detectors.
//
// out[m*d+a, r] = coef * sum_j sum_b G_ab(t_m - s_j) Ek[j*d+b, r] + E0[m*d+a, r]
//
// The reference builds the dense (d*M x d*N) G0(points) and multiplies
// (propagate(): Transmission2D.py:190, :701; Transmission3D.py:163, :675).
// Here each CTA owns 16 detectors and all (up to 64) right-hand-side
// columns of one source range: it evaluates the 16 x 8 Green's blocks of a
// source chunk in FP64 into shared memory, stages the matching Ek rows, and
// contracts in FP64.  Source ranges are split across CTAs for parallelism; a
// second kernel sums the partials in FP64 and applies coef and E0.  That is
// the plain method.  The fast method (MGT_CDF) assembles the propagator rows
// in FP64 once, stored double-float, and contracts them with the residual
// kernel in double-float on the FP32 pipes: each Green's block is evaluated
// once for all right-hand sides, and the FP64 evaluation no longer stalls the
// contraction.
#include <algorithm>
#include <mutex>
#include <type_traits>

#include "common.cuh"
#include "df.cuh"
#include "green.cuh"
#include "diag.cuh"
#include "residual_tc.cuh"

namespace mgt {

constexpr int kPT = 16;      // detectors per CTA
constexpr int kPJ = 8;       // sources per chunk
constexpr int kPCols = 64;   // right-hand-side columns per launch

template <bool DF> struct Acc;
template <> struct Acc<false> {
  using S = double2;   // staged operand
  using A = double2;   // accumulator
  __device__ static S from(double2 v) { return v; }
  __device__ static A zero() { return make_double2(0.0, 0.0); }
  __device__ static void mac(A& acc, S a, S b) { cfma(acc, a, b); }
  __device__ static double2 out(A a) { return a; }
};
template <> struct Acc<true> {
  using S = float4;
  using A = float4;
  __device__ static S from(double2 v) { return df_split(v); }
  __device__ static A zero() { return make_float4(0.f, 0.f, 0.f, 0.f); }
  __device__ static void mac(A& acc, S a, S b) { df_cmac(acc, a, b); }
  __device__ static double2 out(A a) { return df_join(a); }
};

template <int KIND, int RT, bool DF>
__global__ void __launch_bounds__(256)
propagate_partial_kernel(const double* __restrict__ tgt, int nt, const double* __restrict__ src, int ns, double k0,
                         bool regularize, double radius, const double2* __restrict__ Ek, int64_t ld_ek, int ncols,
                         int src_per_split, double2* __restrict__ partial) {
  constexpr int d = Kind<KIND>::d, dim = Kind<KIND>::dim;
  constexpr int ROWS = kPT * d, KC = kPJ * d;
  using P = Acc<DF>;
  using S = typename P::S;
  __shared__ S Gs[ROWS][KC + 1];
  __shared__ S Es[KC][16 * RT];
  __shared__ double tpos[kPT][dim];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int t0 = blockIdx.x * kPT;
  const int sbeg = blockIdx.y * src_per_split, send = min(ns, sbeg + src_per_split);
  if (tid < kPT * dim) {
    int tt = tid / dim, c = tid - tt * dim;
    tpos[tt][c] = (t0 + tt < nt) ? tgt[(int64_t)(t0 + tt) * dim + c] : 0.0;
  }
  typename P::A acc[d][RT];
#pragma unroll
  for (int i = 0; i < d; ++i)
#pragma unroll
    for (int j = 0; j < RT; ++j) acc[i][j] = P::zero();
  __syncthreads();
  for (int sj0 = sbeg; sj0 < send; sj0 += kPJ) {
    if (tid < kPT * kPJ) {
      const int tt = tid / kPJ, jj = tid - tt * kPJ, j = sj0 + jj;
      double2 g[d * d];
      if (t0 + tt < nt && j < send) {
        double r[dim];
#pragma unroll
        for (int c = 0; c < dim; ++c) r[c] = tpos[tt][c] - src[(int64_t)j * dim + c];
        if (!green_block<KIND>(r, k0, regularize, radius, g)) {
          const double nan = __longlong_as_double(0x7ff8000000000000ll);
#pragma unroll
          for (int e = 0; e < d * d; ++e) g[e] = make_double2(nan, nan);
        }
      } else {
#pragma unroll
        for (int e = 0; e < d * d; ++e) g[e] = make_double2(0.0, 0.0);
      }
#pragma unroll
      for (int a = 0; a < d; ++a)
#pragma unroll
        for (int b = 0; b < d; ++b) Gs[tt * d + a][jj * d + b] = P::from(g[a * d + b]);
    }
    for (int idx = tid; idx < KC * 16 * RT; idx += 256) {
      int kk = idx / (16 * RT), c = idx - kk * (16 * RT);
      int64_t row = (int64_t)sj0 * d + kk;
      double2 v = make_double2(0.0, 0.0);
      if (row < (int64_t)send * d && c < ncols) v = Ek[row * ld_ek + c];
      Es[kk][c] = P::from(v);
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < KC; ++kk) {
      S a[d];
#pragma unroll
      for (int i = 0; i < d; ++i) a[i] = Gs[ty + 16 * i][kk];
#pragma unroll
      for (int j = 0; j < RT; ++j) {
        S x = Es[kk][tx + 16 * j];
#pragma unroll
        for (int i = 0; i < d; ++i) P::mac(acc[i][j], a[i], x);
      }
    }
    __syncthreads();
  }
  const int64_t nrows = (int64_t)nt * d;
  double2* part = partial + (int64_t)blockIdx.y * nrows * ncols;
#pragma unroll
  for (int i = 0; i < d; ++i) {
    int64_t row = (int64_t)t0 * d + ty + 16 * i;
    if (row >= nrows) continue;
#pragma unroll
    for (int j = 0; j < RT; ++j) {
      int c = tx + 16 * j;
      if (c < ncols) part[row * ncols + c] = P::out(acc[i][j]);
    }
  }
}

__global__ void propagate_reduce_kernel(const double2* __restrict__ partial, int nsplit, int64_t nrows, int ncols,
                                        double2 coef, const double2* __restrict__ E0, int64_t ld_e0,
                                        double2* __restrict__ out, int64_t ld_out) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nrows * ncols) return;
  int64_t r = idx / ncols;
  int c = (int)(idx - r * ncols);
  double2 s = make_double2(0.0, 0.0);
  for (int q = 0; q < nsplit; ++q) {
    double2 v = partial[(int64_t)q * nrows * ncols + idx];
    s.x += v.x;
    s.y += v.y;
  }
  double2 o = cmul(coef, s);
  if (E0) {
    double2 e = E0[r * ld_e0 + c];
    o.x += e.x;
    o.y += e.y;
  }
  out[r * ld_out + c] = o;
}

static int sm_count() { return device_sm_count(); }

static int choose_splits(int64_t nt, int64_t ns) {
  int64_t tiles = (nt + kPT - 1) / kPT;
  int64_t want = (2 * sm_count() + tiles - 1) / tiles;
  int64_t maxs = std::max<int64_t>(1, (ns + 63) / 64);
  return (int)std::max<int64_t>(1, std::min<int64_t>({want, maxs, 64}));
}

template <int KIND, int RT, bool DF>
static void launch_partial(dim3 grid, const double* t, int nt, const double* s, int ns, double k0, bool reg,
                           double radius, const double2* Ek, int64_t ld_ek, int ncols, int sps, double2* part,
                           cudaStream_t st) {
  count_launch();
  propagate_partial_kernel<KIND, RT, DF><<<grid, 256, 0, st>>>(t, nt, s, ns, k0, reg, radius, Ek, ld_ek, ncols, sps,
                                                              part);
}

template <int KIND, bool DF>
static void launch_partial_rt(int rt, dim3 grid, const double* t, int nt, const double* s, int ns, double k0,
                              bool reg, double radius, const double2* Ek, int64_t ld_ek, int ncols, int sps,
                              double2* part, cudaStream_t st) {
  switch (rt) {
    case 1: launch_partial<KIND, 1, DF>(grid, t, nt, s, ns, k0, reg, radius, Ek, ld_ek, ncols, sps, part, st); break;
    case 2: launch_partial<KIND, 2, DF>(grid, t, nt, s, ns, k0, reg, radius, Ek, ld_ek, ncols, sps, part, st); break;
    default: launch_partial<KIND, 4, DF>(grid, t, nt, s, ns, k0, reg, radius, Ek, ld_ek, ncols, sps, part, st); break;
  }
}

template <bool DF>
static void launch_partial_kind(int kind, int rt, dim3 grid, const double* t, int nt, const double* s, int ns,
                                double k0, bool reg, double radius, const double2* Ek, int64_t ld_ek, int ncols,
                                int sps, double2* part, cudaStream_t st) {
  switch (kind) {
    case MGT_2D_VECTOR: launch_partial_rt<MGT_2D_VECTOR, DF>(rt, grid, t, nt, s, ns, k0, reg, radius, Ek, ld_ek, ncols, sps, part, st); break;
    case MGT_2D_SCALAR: launch_partial_rt<MGT_2D_SCALAR, DF>(rt, grid, t, nt, s, ns, k0, reg, radius, Ek, ld_ek, ncols, sps, part, st); break;
    case MGT_3D_VECTOR: launch_partial_rt<MGT_3D_VECTOR, DF>(rt, grid, t, nt, s, ns, k0, reg, radius, Ek, ld_ek, ncols, sps, part, st); break;
    default: launch_partial_rt<MGT_3D_SCALAR, DF>(rt, grid, t, nt, s, ns, k0, reg, radius, Ek, ld_ek, ncols, sps, part, st); break;
  }
}

int assemble_propagator_into(int kind, const double* t, int nt, const double* src, int ns, double k0, double2 coef,
                             bool reg, double radius, int nanp, double2 fill, int transpose, void* out, int64_t ld,
                             int dtype, cudaStream_t s);
int residual_rect(const float4* M, int64_t ldm, const float4* Xs, int64_t ldxs, const double2* B, int64_t ldb,
                  double2* R, int64_t ldr, int rows, int kdim, int nrhs, cudaStream_t s, double2* partial,
                  int64_t partial_elems);
int64_t residual_partial_elems(int64_t rows, int64_t kdim, int64_t nrhs);
int split_df(const double2* X, int64_t ldx, float4* Xs, int64_t ldy, int n, int ncols, cudaStream_t s);

// Double-float path: the propagator's detector rows are assembled in chunks
// of at most kPropChunkBytes (as -coef G, double-float) and contracted with
// the double-float copy of Ek by the residual kernel: out = E0 - (-coef G) Ek.
constexpr size_t kPropChunkBytes = size_t(1) << 30;
static int64_t prop_chunk_targets(int64_t nt, int64_t ns, int d) {
  const int64_t row_bytes = (int64_t)d * d * ns * (int64_t)sizeof(float4);   // one target's d rows
  return std::max<int64_t>(1, std::min<int64_t>(nt, (int64_t)kPropChunkBytes / std::max<int64_t>(1, row_bytes)));
}
// workspace: Xs (d ns x nrhs float4) | one chunk of propagator rows | split-K partials
static size_t prop_xs_bytes(int64_t ns, int64_t nrhs, int d) {
  return ((size_t)d * ns * nrhs * sizeof(float4) + 255) & ~size_t(255);
}
static size_t prop_chunk_bytes(int64_t nt, int64_t ns, int d) {
  return ((size_t)prop_chunk_targets(nt, ns, d) * d * d * ns * sizeof(float4) + 255) & ~size_t(255);
}
static size_t prop_part_elems(int64_t nt, int64_t ns, int64_t nrhs, int d) {
  return (size_t)residual_partial_elems(prop_chunk_targets(nt, ns, d) * d, (int64_t)d * ns, nrhs);
}
static size_t prop_df_bytes(int64_t nt, int64_t ns, int64_t nrhs, int d) {
  return prop_xs_bytes(ns, nrhs, d) + prop_chunk_bytes(nt, ns, d) + prop_part_elems(nt, ns, nrhs, d) * sizeof(double2);
}
// tensor-core contraction: one chunk of propagator rows | the residual kernel's workspace
static bool prop_tc_ok(int64_t nt, int64_t ns, int64_t nrhs, int d) {
  return residual_tc_supported(prop_chunk_targets(nt, ns, d) * d, (int64_t)d * ns, nrhs);
}
static size_t prop_tc_bytes(int64_t nt, int64_t ns, int64_t nrhs, int d) {
  if (!prop_tc_ok(nt, ns, nrhs, d)) return 0;
  return prop_chunk_bytes(nt, ns, d) +
         residual_tc_workspace_bytes(prop_chunk_targets(nt, ns, d) * d, (int64_t)d * ns, nrhs) + 1024;
}

static int kind_dim_d(int kind, int* dim) {
  switch (kind) {
    case MGT_2D_VECTOR: *dim = 2; return 2;
    case MGT_2D_SCALAR: *dim = 2; return 1;
    case MGT_3D_VECTOR: *dim = 3; return 3;
    case MGT_3D_SCALAR: *dim = 3; return 1;
    default: return 0;
  }
}

}  // namespace mgt

using namespace mgt;

extern "C" int mgt_propagate_workspace_bytes(int kind, int64_t n_targets, int64_t n_sources, int64_t nrhs,
                                             size_t* bytes) {
  int dim;
  int d = kind_dim_d(kind, &dim);
  if (!bytes || d == 0 || n_targets <= 0 || n_sources <= 0 || nrhs <= 0) return MGT_ERR_ARG;
  int nsplit = choose_splits(n_targets, n_sources);
  // the larger of the two methods' needs: FP64 partial sums, or the
  // double-float copy of Ek plus one chunk of assembled propagator rows
  *bytes = std::max({(size_t)nsplit * n_targets * d * std::min<int64_t>(nrhs, kPCols) * sizeof(double2),
                     prop_df_bytes(n_targets, n_sources, nrhs, d), prop_tc_bytes(n_targets, n_sources, nrhs, d)});
  return MGT_OK;
}

extern "C" int mgt_propagate(int kind, int dtype, const double* targets, int64_t n_targets, const double* sources,
                             int64_t n_sources, double k0, double coef_re, double coef_im, int regularize,
                             double radius, const void* Ek, int64_t ld_ek, const void* E0, int64_t ld_e0, void* out,
                             int64_t ld_out, int64_t nrhs, void* work, size_t work_bytes, void* stream) {
  int dim;
  int d = kind_dim_d(kind, &dim);
  if (d == 0 || !targets || !sources || !Ek || !out || !work || n_targets <= 0 || n_sources <= 0 || nrhs <= 0)
    return MGT_ERR_ARG;
  if (dtype != MGT_C128 && dtype != MGT_CDF) return MGT_ERR_ARG;
  if (ld_ek < nrhs || ld_out < nrhs || (E0 && ld_e0 < nrhs)) return MGT_ERR_ARG;
  if (n_targets > (1 << 28) || n_sources > (1 << 28)) return MGT_ERR_UNSUPPORTED;
  size_t need = 0;
  mgt_propagate_workspace_bytes(kind, n_targets, n_sources, nrhs, &need);
  if (work_bytes < need) return MGT_ERR_WORKSPACE;
  cudaStream_t st = (cudaStream_t)stream;
  const int nt = (int)n_targets, ns = (int)n_sources;
  if (dtype == MGT_CDF && prop_tc_ok(nt, ns, nrhs, d)) {
    // propagator rows (-coef G, double-float) contracted on the tensor cores:
    // out = E0 - (-coef G) Ek; rows with NaN blocks (a detector on a scatterer)
    // come out NaN for the host's fix-up
    const int64_t ct = prop_chunk_targets(nt, ns, d);
    float4* Gc = (float4*)work;
    char* tw = (char*)work + ((prop_chunk_bytes(nt, ns, d) + 1023) & ~size_t(1023));
    const size_t tw_bytes = work_bytes - (size_t)(tw - (char*)work);
    const double2 mcoef = make_double2(-coef_re, -coef_im);
    const double2 nanfill = make_double2(0.0, 0.0);
    int e = MGT_OK;
    for (int64_t t0 = 0; t0 < nt && e == MGT_OK; t0 += ct) {
      const int tc = (int)std::min<int64_t>(ct, nt - t0);
      e = assemble_propagator_into(kind, targets + t0 * dim, tc, sources, ns, k0, mcoef, regularize != 0, radius,
                                   MGT_NAN_KEEP, nanfill, 0, Gc, (int64_t)d * ns, MGT_CDF, st);
      if (e != MGT_OK) break;
      const double2* b = E0 ? (const double2*)E0 + t0 * d * ld_e0 : nullptr;
      e = residual_tc(Gc, (int64_t)d * ns, tc * d, d * ns, (const double2*)Ek, ld_ek, (int)nrhs, b, ld_e0,
                      (double2*)out + t0 * d * ld_out, ld_out, tw, tw_bytes, st);
    }
    return e;
  }
  if (dtype == MGT_CDF) {
    const int64_t ct = prop_chunk_targets(nt, ns, d);
    float4* Xs = (float4*)work;
    float4* Gc = (float4*)((char*)work + prop_xs_bytes(ns, nrhs, d));
    double2* part = (double2*)((char*)Gc + prop_chunk_bytes(nt, ns, d));
    int e = split_df((const double2*)Ek, ld_ek, Xs, nrhs, d * ns, (int)nrhs, st);
    const double2 mcoef = make_double2(-coef_re, -coef_im);
    const double2 nanfill = make_double2(0.0, 0.0);
    for (int64_t t0 = 0; t0 < nt && e == MGT_OK; t0 += ct) {
      const int tc = (int)std::min<int64_t>(ct, nt - t0);
      e = assemble_propagator_into(kind, targets + t0 * dim, tc, sources, ns, k0, mcoef, regularize != 0, radius,
                                   MGT_NAN_KEEP, nanfill, 0, Gc, (int64_t)d * ns, MGT_CDF, st);
      if (e != MGT_OK) break;
      const double2* b = E0 ? (const double2*)E0 + t0 * d * ld_e0 : nullptr;
      e = residual_rect(Gc, (int64_t)d * ns, Xs, nrhs, b, ld_e0, (double2*)out + t0 * d * ld_out, ld_out, tc * d,
                        d * ns, (int)nrhs, st, part, (int64_t)prop_part_elems(nt, ns, nrhs, d));
    }
    return e;
  }
  const int nsplit = choose_splits(n_targets, n_sources);
  const int sps = (ns + nsplit - 1) / nsplit;
  const int tiles = (nt + kPT - 1) / kPT;
  if (tiles > (1 << 30)) return MGT_ERR_UNSUPPORTED;
  double2* part = (double2*)work;
  const double2* ek = (const double2*)Ek;
  const double2* e0 = (const double2*)E0;
  double2* o = (double2*)out;
  const double2 coef = make_double2(coef_re, coef_im);
  for (int64_t c0 = 0; c0 < nrhs; c0 += kPCols) {
    int nc = (int)std::min<int64_t>(kPCols, nrhs - c0);
    int rt = (nc + 15) / 16;
    if (rt == 3) rt = 4;
    dim3 grid(tiles, nsplit);
    if (dtype == MGT_CDF)
      launch_partial_kind<true>(kind, rt, grid, targets, nt, sources, ns, k0, regularize != 0, radius, ek + c0, ld_ek,
                                nc, sps, part, st);
    else
      launch_partial_kind<false>(kind, rt, grid, targets, nt, sources, ns, k0, regularize != 0, radius, ek + c0,
                                 ld_ek, nc, sps, part, st);
    int64_t nrows = (int64_t)nt * d;
    int64_t tot = nrows * nc;
    count_launch();
    propagate_reduce_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(part, nsplit, nrows, nc, coef,
                                                                          e0 ? e0 + c0 : nullptr, ld_e0, o + c0,
                                                                          ld_out);
  }
  return cudaGetLastError() == cudaSuccess ? MGT_OK : MGT_ERR_CUDA;
}
