// K1: Green's-matrix assembly.
//
// One thread per (row point, column point) pair writes that pair's d x d
// block of complex entries; threads of a warp take consecutive column points,
// so each of the d output rows a warp touches is one contiguous run of
// 32*d*16 bytes.  The kernel is store-bandwidth bound for the 3D kinds and
// FP64-pipe bound (Bessel J0/Y0/J1/Y1) for the 2D kinds.
// The Green's blocks themselves are in green.cuh.
#include <atomic>

#include "common.cuh"
#include "df.cuh"
#include "green.cuh"
#include "diag.cuh"

namespace mgt {

constexpr int kAsmThreads = 128;
constexpr int kAsmRows = 4;

struct OutSpec {
  void* p;
  int64_t ld;
  int dtype;
};

__device__ __forceinline__ void store_entry(const OutSpec& o, int64_t row, int64_t col, double2 v) {
  if (!o.p) return;
  if (o.dtype == MGT_C128) reinterpret_cast<double2*>(o.p)[row * o.ld + col] = v;
  else if (o.dtype == MGT_C64) reinterpret_cast<float2*>(o.p)[row * o.ld + col] = make_float2((float)v.x, (float)v.y);
  else reinterpret_cast<float4*>(o.p)[row * o.ld + col] = df_split(v);
}

// System matrix: block (i, j) = -coef * G(r_i - r_j) for i != j,
// (1 - shift) * I for i == j.
template <int KIND>
__global__ void __launch_bounds__(kAsmThreads)
assemble_system_kernel(const double* __restrict__ pts, int n, double k0, double2 coef,
                       double2 diag, OutSpec o1, OutSpec o2) {
  constexpr int dim = Kind<KIND>::dim, d = Kind<KIND>::d;
  int j = blockIdx.x * kAsmThreads + threadIdx.x;
  if (j >= n) return;
  double sj[dim];
#pragma unroll
  for (int c = 0; c < dim; ++c) sj[c] = pts[(int64_t)j * dim + c];
  int i0 = blockIdx.y * kAsmRows;
  for (int ii = 0; ii < kAsmRows; ++ii) {
    int i = i0 + ii;
    if (i >= n) break;
    double2 g[d * d];
    if (i == j) {
#pragma unroll
      for (int a = 0; a < d; ++a)
#pragma unroll
        for (int b = 0; b < d; ++b) g[a * d + b] = (a == b) ? diag : make_double2(0.0, 0.0);
    } else {
      double r[dim];
#pragma unroll
      for (int c = 0; c < dim; ++c) r[c] = pts[(int64_t)i * dim + c] - sj[c];
      // distinct scatterers at the same position give the reference a NaN block
      if (!green_block<KIND>(r, k0, false, 0.0, g)) {
#pragma unroll
        for (int q = 0; q < d * d; ++q)
          g[q] = make_double2(__longlong_as_double(0x7ff8000000000000ll), __longlong_as_double(0x7ff8000000000000ll));
      } else {
#pragma unroll
        for (int q = 0; q < d * d; ++q) {
          double2 v = g[q];
          g[q] = make_double2(-(coef.x * v.x - coef.y * v.y), -(coef.x * v.y + coef.y * v.x));
        }
      }
    }
#pragma unroll
    for (int a = 0; a < d; ++a) {
      int64_t row = (int64_t)i * d + a;
#pragma unroll
      for (int b = 0; b < d; ++b) {
        store_entry(o1, row, (int64_t)j * d + b, g[a * d + b]);
        store_entry(o2, row, (int64_t)j * d + b, g[a * d + b]);
      }
    }
  }
}

// The same matrix from half the Green's blocks: G(-r) = G(r) and every block
// is symmetric, so M is complex-symmetric.  One CTA per 16 x 16 tile of point
// pairs with bj >= bi evaluates each pair once (FP64, into shared memory)
// and writes the tile and, off the diagonal, its mirror image, both as
// contiguous row segments.  Negating r changes neither |r| nor the products
// of its components, so the mirrored values are bitwise those of the lower
// triangle evaluated directly.
constexpr int kSymTP = 16;

template <int KIND>
__global__ void __launch_bounds__(kSymTP * kSymTP)
assemble_system_sym_kernel(const double* __restrict__ pts, int n, double k0, double2 coef, double2 diag,
                           OutSpec o1, OutSpec o2) {
  constexpr int dim = Kind<KIND>::dim, d = Kind<KIND>::d;
  constexpr int TP = kSymTP, W = TP * d;          // tile side in matrix rows / columns
  const int bi = blockIdx.y, bj = blockIdx.x;
  if (bj < bi) return;
  extern __shared__ __align__(16) unsigned char asm_smem[];
  double2* S = reinterpret_cast<double2*>(asm_smem);   // [TP][TP][d * d]
  const int tid = threadIdx.x, p = tid / TP, q = tid % TP;
  const int i = bi * TP + p, j = bj * TP + q;
  double2 g[d * d];
  if (i < n && j < n) {
    if (i == j) {
#pragma unroll
      for (int a = 0; a < d; ++a)
#pragma unroll
        for (int b = 0; b < d; ++b) g[a * d + b] = (a == b) ? diag : make_double2(0.0, 0.0);
    } else {
      double r[dim];
#pragma unroll
      for (int c = 0; c < dim; ++c) r[c] = pts[(int64_t)i * dim + c] - pts[(int64_t)j * dim + c];
      if (!green_block<KIND>(r, k0, false, 0.0, g)) {
#pragma unroll
        for (int e = 0; e < d * d; ++e)
          g[e] = make_double2(__longlong_as_double(0x7ff8000000000000ll), __longlong_as_double(0x7ff8000000000000ll));
      } else {
#pragma unroll
        for (int e = 0; e < d * d; ++e) {
          double2 v = g[e];
          g[e] = make_double2(-(coef.x * v.x - coef.y * v.y), -(coef.x * v.y + coef.y * v.x));
        }
      }
    }
  } else {
#pragma unroll
    for (int e = 0; e < d * d; ++e) g[e] = make_double2(0.0, 0.0);
  }
#pragma unroll
  for (int e = 0; e < d * d; ++e) S[(p * TP + q) * d * d + e] = g[e];
  __syncthreads();
  // tile (bi, bj): row i d + a, column j d + b
  for (int idx = tid; idx < W * W; idx += TP * TP) {
    const int rr = idx / W, cc = idx - rr * W;
    const int pp = rr / d, a = rr - pp * d, qq = cc / d, b = cc - qq * d;
    const int ii = bi * TP + pp, jj = bj * TP + qq;
    if (ii < n && jj < n) {
      const double2 v = S[(pp * TP + qq) * d * d + a * d + b];
      store_entry(o1, (int64_t)ii * d + a, (int64_t)jj * d + b, v);
      store_entry(o2, (int64_t)ii * d + a, (int64_t)jj * d + b, v);
    }
  }
  if (bi == bj) return;
  // mirror tile (bj, bi): row j d + b, column i d + a holds the same value
  for (int idx = tid; idx < W * W; idx += TP * TP) {
    const int rr = idx / W, cc = idx - rr * W;
    const int qq = rr / d, b = rr - qq * d, pp = cc / d, a = cc - pp * d;
    const int ii = bi * TP + pp, jj = bj * TP + qq;
    if (ii < n && jj < n) {
      const double2 v = S[(pp * TP + qq) * d * d + a * d + b];
      store_entry(o1, (int64_t)jj * d + b, (int64_t)ii * d + a, v);
      store_entry(o2, (int64_t)jj * d + b, (int64_t)ii * d + a, v);
    }
  }
}

// Propagator: coef * G(t_i - s_j).  Threads run over the output's column
// points: sources (normal) or targets (transposed output).
template <int KIND, bool TRANSPOSE>
__global__ void __launch_bounds__(kAsmThreads)
assemble_propagator_kernel(const double* __restrict__ tgt, int nt, const double* __restrict__ src,
                           int ns, double k0, double2 coef, bool regularize, double radius,
                           int nan_policy, double2 fill, OutSpec out) {
  constexpr int dim = Kind<KIND>::dim, d = Kind<KIND>::d;
  int ncol = TRANSPOSE ? nt : ns, nrow = TRANSPOSE ? ns : nt;
  int q = blockIdx.x * kAsmThreads + threadIdx.x;
  if (q >= ncol) return;
  const double* colp = TRANSPOSE ? tgt : src;
  const double* rowp = TRANSPOSE ? src : tgt;
  double cq[dim];
#pragma unroll
  for (int c = 0; c < dim; ++c) cq[c] = colp[(int64_t)q * dim + c];
  int p0 = blockIdx.y * kAsmRows;
  for (int pp = 0; pp < kAsmRows; ++pp) {
    int p = p0 + pp;
    if (p >= nrow) break;
    double r[dim];
#pragma unroll
    for (int c = 0; c < dim; ++c) {
      double rp = rowp[(int64_t)p * dim + c];
      r[c] = TRANSPOSE ? (cq[c] - rp) : (rp - cq[c]);  // always target - source
    }
    double2 g[d * d];
    if (green_block<KIND>(r, k0, regularize, radius, g)) {
#pragma unroll
      for (int e = 0; e < d * d; ++e) {
        double2 v = g[e];
        g[e] = make_double2(coef.x * v.x - coef.y * v.y, coef.x * v.y + coef.y * v.x);
      }
    } else {
      double2 bad = nan_policy == MGT_NAN_FILL ? fill
                                               : make_double2(__longlong_as_double(0x7ff8000000000000ll),
                                                              __longlong_as_double(0x7ff8000000000000ll));
#pragma unroll
      for (int e = 0; e < d * d; ++e) g[e] = bad;
    }
#pragma unroll
    for (int a = 0; a < d; ++a) {
      // output row index d*p + a; block entry G_ab (normal) or G_ba (transposed)
#pragma unroll
      for (int b = 0; b < d; ++b)
        store_entry(out, (int64_t)p * d + a, (int64_t)q * d + b, TRANSPOSE ? g[b * d + a] : g[a * d + b]);
    }
  }
}

static std::atomic<int> g_sym_assembly{1};   // assemble from half the Green's blocks

template <int KIND>
static cudaError_t launch_system(const double* pts, int n, double k0, double2 coef, double2 diag,
                                 OutSpec o1, OutSpec o2, cudaStream_t s) {
  if (g_sym_assembly.load(std::memory_order_relaxed)) {
    constexpr int d = Kind<KIND>::d;
    const int nb = (n + kSymTP - 1) / kSymTP;
    if (nb <= 65535) {
      const size_t smem = (size_t)kSymTP * kSymTP * d * d * sizeof(double2);
      assemble_system_sym_kernel<KIND><<<dim3(nb, nb), kSymTP * kSymTP, smem, s>>>(pts, n, k0, coef, diag, o1, o2);
      count_launch();
      return cudaGetLastError();
    }
  }
  dim3 grid((n + kAsmThreads - 1) / kAsmThreads, (n + kAsmRows - 1) / kAsmRows);
  assemble_system_kernel<KIND><<<grid, kAsmThreads, 0, s>>>(pts, n, k0, coef, diag, o1, o2);
  count_launch();
  return cudaGetLastError();
}

int set_sym_assembly(int v) {
  g_sym_assembly.store(v ? 1 : 0);
  return MGT_OK;
}
int get_sym_assembly() { return g_sym_assembly.load(); }

template <int KIND>
static cudaError_t launch_prop(const double* t, int nt, const double* src, int ns, double k0,
                               double2 coef, bool reg, double radius, int nanp, double2 fill,
                               int transpose, OutSpec out, cudaStream_t s) {
  int ncol = transpose ? nt : ns, nrow = transpose ? ns : nt;
  dim3 grid((ncol + kAsmThreads - 1) / kAsmThreads, (nrow + kAsmRows - 1) / kAsmRows);
  count_launch();
  if (transpose)
    assemble_propagator_kernel<KIND, true><<<grid, kAsmThreads, 0, s>>>(t, nt, src, ns, k0, coef, reg, radius, nanp, fill, out);
  else
    assemble_propagator_kernel<KIND, false><<<grid, kAsmThreads, 0, s>>>(t, nt, src, ns, k0, coef, reg, radius, nanp, fill, out);
  return cudaGetLastError();
}

// Propagator blocks into any output format (used by the propagation's
// assembled double-float path).
int assemble_propagator_into(int kind, const double* t, int nt, const double* src, int ns, double k0, double2 coef,
                             bool reg, double radius, int nanp, double2 fill, int transpose, void* out, int64_t ld,
                             int dtype, cudaStream_t s) {
  if (((transpose ? ns : nt) + kAsmRows - 1) / kAsmRows > 65535) return MGT_ERR_UNSUPPORTED;
  OutSpec o{out, ld, dtype};
  cudaError_t e;
  switch (kind) {
    case MGT_2D_VECTOR: e = launch_prop<MGT_2D_VECTOR>(t, nt, src, ns, k0, coef, reg, radius, nanp, fill, transpose, o, s); break;
    case MGT_2D_SCALAR: e = launch_prop<MGT_2D_SCALAR>(t, nt, src, ns, k0, coef, reg, radius, nanp, fill, transpose, o, s); break;
    case MGT_3D_VECTOR: e = launch_prop<MGT_3D_VECTOR>(t, nt, src, ns, k0, coef, reg, radius, nanp, fill, transpose, o, s); break;
    default: e = launch_prop<MGT_3D_SCALAR>(t, nt, src, ns, k0, coef, reg, radius, nanp, fill, transpose, o, s); break;
  }
  return e == cudaSuccess ? MGT_OK : MGT_ERR_CUDA;
}

}  // namespace mgt

using namespace mgt;

static int kind_d(int kind) {
  switch (kind) {
    case MGT_2D_VECTOR: return 2;
    case MGT_3D_VECTOR: return 3;
    case MGT_2D_SCALAR: case MGT_3D_SCALAR: return 1;
    default: return 0;
  }
}

extern "C" int mgt_assemble_system(int kind, const double* points, int64_t n_points, double k0,
                                   double coef_re, double coef_im, double shift_re, double shift_im,
                                   void* out1, int64_t ld1, int dtype1, void* out2, int64_t ld2,
                                   int dtype2, void* stream) {
  int d = kind_d(kind);
  if (d == 0 || !points || n_points <= 0 || n_points > (1 << 30) / 3) return MGT_ERR_ARG;
  if (!out1) return MGT_ERR_ARG;
  if (dtype1 < MGT_C128 || dtype1 > MGT_CDF || ld1 < d * n_points) return MGT_ERR_ARG;
  if (out2 && (dtype2 < MGT_C128 || dtype2 > MGT_CDF || ld2 < d * n_points)) return MGT_ERR_ARG;
  if ((n_points + kAsmRows - 1) / kAsmRows > 65535) return MGT_ERR_UNSUPPORTED;
  cudaStream_t s = (cudaStream_t)stream;
  int n = (int)n_points;
  double2 coef = make_double2(coef_re, coef_im), diag = make_double2(1.0 - shift_re, -shift_im);
  OutSpec o1{out1, ld1, dtype1}, o2{out2, ld2, dtype2};
  cudaError_t e;
  switch (kind) {
    case MGT_2D_VECTOR: e = launch_system<MGT_2D_VECTOR>(points, n, k0, coef, diag, o1, o2, s); break;
    case MGT_2D_SCALAR: e = launch_system<MGT_2D_SCALAR>(points, n, k0, coef, diag, o1, o2, s); break;
    case MGT_3D_VECTOR: e = launch_system<MGT_3D_VECTOR>(points, n, k0, coef, diag, o1, o2, s); break;
    default: e = launch_system<MGT_3D_SCALAR>(points, n, k0, coef, diag, o1, o2, s); break;
  }
  return e == cudaSuccess ? MGT_OK : MGT_ERR_CUDA;
}

extern "C" int mgt_assemble_propagator(int kind, const double* targets, int64_t n_targets,
                                       const double* sources, int64_t n_sources, double k0,
                                       double coef_re, double coef_im, int regularize, double radius,
                                       int nan_policy, double fill_re, double fill_im, int transpose,
                                       void* out_c128, int64_t ld, void* stream) {
  int d = kind_d(kind);
  if (d == 0 || !targets || !sources || !out_c128 || n_targets <= 0 || n_sources <= 0) return MGT_ERR_ARG;
  if (n_targets > (1 << 30) / 3 || n_sources > (1 << 30) / 3) return MGT_ERR_ARG;
  if (nan_policy != MGT_NAN_KEEP && nan_policy != MGT_NAN_FILL) return MGT_ERR_ARG;
  int64_t ncols = transpose ? d * n_targets : d * n_sources;
  if (ld < ncols) return MGT_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  double2 coef = make_double2(coef_re, coef_im), fill = make_double2(fill_re, fill_im);
  return assemble_propagator_into(kind, targets, (int)n_targets, sources, (int)n_sources, k0, coef, regularize != 0,
                                  radius, nan_policy, fill, transpose, out_c128, ld, MGT_C128, s);
}
