// Green's-function blocks, evaluated in FP64 (shared by assembly and the
// matrix-free propagate).
//
// Formulas (r = t - s, R = |r|, P = r r^T / R^2):
//   2D TE  (Transmission2D.py:63-91): (i/4)[(I-P) H0(kR) - (I-2P) H1(kR)/(kR)]
//   2D TM  (Transmission2D.py:595-618): (i/4) H0(kR)
//   3D vec (Transmission3D.py:47-77): [I - P - (I-3P)(1/(ikR) + 1/(kR)^2)] e^{ikR}/(4 pi R)
//   3D sca (Transmission3D.py:573-601): e^{ikR}/(4 pi R)
// with H_nu = J_nu + i Y_nu evaluated by CUDA's double-precision j0/y0/j1/y1.
#pragma once
#include "common.cuh"

namespace mgt {

template <int KIND> struct Kind;
template <> struct Kind<MGT_2D_VECTOR> { static constexpr int dim = 2, d = 2; };
template <> struct Kind<MGT_2D_SCALAR> { static constexpr int dim = 2, d = 1; };
template <> struct Kind<MGT_3D_VECTOR> { static constexpr int dim = 3, d = 3; };
template <> struct Kind<MGT_3D_SCALAR> { static constexpr int dim = 3, d = 1; };

// d x d Green's block for separation r (row-major in g).  Returns false where
// the reference's value is NaN: R == 0, or R (k*R for the 2D TE kind) below
// `radius` when regularising.
template <int KIND>
__device__ __forceinline__ bool green_block(const double* r, double k0, bool regularize,
                                            double radius, double2* g) {
  constexpr double kPi = 3.14159265358979323846;
  if constexpr (KIND == MGT_2D_VECTOR) {
    double R2 = r[0] * r[0] + r[1] * r[1];
    double kR = k0 * sqrt(R2);
    if (regularize && kR < radius) kR = 0.0;
    if (R2 == 0.0 || kR == 0.0) return false;
    double inv = 1.0 / kR;
    double h0r = j0(kR), h0i = y0(kR);
    double h1r = j1(kR) * inv, h1i = y1(kR) * inv;
    double invR2 = 1.0 / R2;
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int b = 0; b < 2; ++b) {
        double P = r[a] * r[b] * invR2;
        double e = (a == b) ? 1.0 : 0.0;
        double c0 = e - P, c1 = e - 2.0 * P;
        double tr = c0 * h0r - c1 * h1r, ti = c0 * h0i - c1 * h1i;
        g[a * 2 + b] = make_double2(-0.25 * ti, 0.25 * tr);  // (i/4) * t
      }
    return true;
  } else if constexpr (KIND == MGT_2D_SCALAR) {
    double R = sqrt(r[0] * r[0] + r[1] * r[1]);
    if (regularize && R < radius) R = 0.0;
    if (R == 0.0) return false;
    double kR = k0 * R;
    g[0] = make_double2(-0.25 * y0(kR), 0.25 * j0(kR));
    return true;
  } else if constexpr (KIND == MGT_3D_VECTOR) {
    double R2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    double R = sqrt(R2);
    double invR2 = 1.0 / R2;
    if (regularize && R < radius) R = 0.0;
    if (R2 == 0.0 || R == 0.0) return false;
    double kR = k0 * R, inv = 1.0 / kR;
    double s, c;
    sincos(kR, &s, &c);
    double amp = 1.0 / (4.0 * kPi * R);
    double er = c * amp, ei = s * amp;
    // f = 1/(ikR) + 1/(kR)^2 = inv^2 - i inv
    double fr = inv * inv, fi = -inv;
    // diagonal coefficient (1 - f), projector coefficient -(1 - 3 f)
    double dr = 1.0 - fr, di = -fi;
    double pr = -(1.0 - 3.0 * fr), pi = 3.0 * fi;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        double P = r[a] * r[b] * invR2;
        double tr = P * pr + ((a == b) ? dr : 0.0);
        double ti = P * pi + ((a == b) ? di : 0.0);
        g[a * 3 + b] = make_double2(tr * er - ti * ei, tr * ei + ti * er);
      }
    return true;
  } else {
    double R = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    if (regularize && R < radius) R = 0.0;
    if (R == 0.0) return false;
    double kR = k0 * R, s, c;
    sincos(kR, &s, &c);
    double amp = 1.0 / (4.0 * kPi * R);
    g[0] = make_double2(c * amp, s * amp);
    return true;
  }
}

}  // namespace mgt
