// Shared device helpers for the coupled-dipole engine (sm_103a).
//
// Complex numbers are stored interleaved (re, im) exactly like torch
// complex128 / complex64 tensors: double2 / float2.  All matrices are
// row-major with an explicit leading dimension in elements.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <utility>

#include "../../include/magreete_gb300.h"

namespace mgt {

// Kernel attributes (the dynamic shared-memory limit, cluster permissions)
// belong to one device's context, and device properties can differ between
// GPUs: set-up that records them runs once per device, the first time it is
// needed with that device current.
constexpr int kMaxDevices = 64;

inline int current_device() {
  int d = 0;
  if (cudaGetDevice(&d) != cudaSuccess || d < 0 || d >= kMaxDevices) d = 0;
  return d;
}

struct OncePerDevice {
  std::once_flag flags[kMaxDevices];
  template <class F> void operator()(F&& f) { std::call_once(flags[current_device()], std::forward<F>(f)); }
};

// SM count of the current device (cached per device).
inline int device_sm_count() {
  static OncePerDevice once;
  static int sms[kMaxDevices] = {};
  const int d = current_device();
  once([d] {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, d) != cudaSuccess || v <= 0) v = 1;
    sms[d] = v;
  });
  return sms[d];
}

template <typename T> struct CplxOf;
template <> struct CplxOf<double> { using type = double2; };
template <> struct CplxOf<float> { using type = float2; };
template <typename T> using cplx = typename CplxOf<T>::type;

__host__ __device__ inline double2 mkc(double a, double b) { return make_double2(a, b); }
__host__ __device__ inline float2 mkc(float a, float b) { return make_float2(a, b); }

template <typename V> __device__ inline V czero() { V v; v.x = 0; v.y = 0; return v; }

__device__ inline double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ inline float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ inline double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ inline float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ inline double2 cmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ inline float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// acc += a * b
__device__ inline void cfma(double2& acc, double2 a, double2 b) {
  acc.x = fma(a.x, b.x, acc.x); acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y); acc.y = fma(a.y, b.x, acc.y);
}
__device__ inline void cfma(float2& acc, float2 a, float2 b) {
  acc.x = fmaf(a.x, b.x, acc.x); acc.x = fmaf(-a.y, b.y, acc.x);
  acc.y = fmaf(a.x, b.y, acc.y); acc.y = fmaf(a.y, b.x, acc.y);
}
// acc -= a * b
__device__ inline void cfms(double2& acc, double2 a, double2 b) {
  acc.x = fma(-a.x, b.x, acc.x); acc.x = fma(a.y, b.y, acc.x);
  acc.y = fma(-a.x, b.y, acc.y); acc.y = fma(-a.y, b.x, acc.y);
}
__device__ inline void cfms(float2& acc, float2 a, float2 b) {
  acc.x = fmaf(-a.x, b.x, acc.x); acc.x = fmaf(a.y, b.y, acc.x);
  acc.y = fmaf(-a.x, b.y, acc.y); acc.y = fmaf(-a.y, b.x, acc.y);
}
// |re| + |im|: the pivot magnitude LAPACK's i?amax uses
__device__ inline double cabs1(double2 a) { return fabs(a.x) + fabs(a.y); }
__device__ inline float cabs1(float2 a) { return fabsf(a.x) + fabsf(a.y); }

// 1/z with Smith's scaling (avoids overflow of |z|^2 for large entries)
__device__ inline double2 crecip(double2 z) {
  if (fabs(z.x) >= fabs(z.y)) {
    double r = z.y / z.x, d = z.x + z.y * r;
    return make_double2(1.0 / d, -r / d);
  }
  double r = z.x / z.y, d = z.y + z.x * r;
  return make_double2(r / d, -1.0 / d);
}
__device__ inline float2 crecip(float2 z) {
  if (fabsf(z.x) >= fabsf(z.y)) {
    float r = z.y / z.x, d = z.x + z.y * r;
    return make_float2(1.0f / d, -r / d);
  }
  float r = z.x / z.y, d = z.y + z.x * r;
  return make_float2(r / d, -1.0f / d);
}

__device__ inline double2 to_c64(double2 v) { return v; }
__device__ inline float2 to_c32(double2 v) { return make_float2((float)v.x, (float)v.y); }

// Loads that bypass L1: used for data another SM wrote (after a grid barrier).
__device__ inline double2 ldcg(const double2* p) { return __ldcg(p); }
__device__ inline float2 ldcg(const float2* p) { return __ldcg(p); }

// One element (8 or 16 bytes) copied global -> shared without passing through
// registers (sm_80 cp.async); zero-filled, with nothing read, when !ok.
template <int BYTES>
__device__ __forceinline__ void cp_async_elem(void* dst, const void* src, bool ok) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  const int sz = ok ? BYTES : 0;
  if constexpr (BYTES == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(src), "r"(sz) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;" ::"r"(d), "l"(src), "n"(BYTES), "r"(sz) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Iteration limit of every device-side spin wait (about a few seconds with
// the back-off below).  A wait that runs out records MGT_ERR_TIMEOUT in the
// status word and the kernel returns instead of hanging.
constexpr unsigned kSpinLimit = 1u << 24;

struct GridBarrier {
  unsigned* count;   // arrivals in the current generation
  unsigned* gen;     // generation counter
};

// Grid-wide barrier for a cooperative launch, with a bounded wait.
// Returns false (and sets *status) if the wait ran out.
__device__ inline bool grid_sync(GridBarrier b, int* status) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    unsigned nblocks = gridDim.x * gridDim.y * gridDim.z;
    volatile unsigned* vgen = b.gen;
    unsigned g = *vgen;
    __threadfence();
    unsigned arrived = atomicAdd(b.count, 1u);
    if (arrived == nblocks - 1) {
      *b.count = 0;
      __threadfence();
      atomicAdd(b.gen, 1u);
    } else {
      unsigned it = 0;
      while (*vgen == g) {
        if (++it > kSpinLimit) { atomicExch(status, MGT_ERR_TIMEOUT); ok = 0; break; }
        if (it > 64) __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok != 0;
}

}  // namespace mgt
