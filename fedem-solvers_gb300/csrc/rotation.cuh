// rotation.cuh -- 3x4 position matrices and finite rotations on the device,
// shared by the element, increment and joint kernels.
#pragma once

namespace fgpu {

// 3x4 position matrices, column-major: T[r + 3c]; o = a o b
__device__ inline void compose34(const double* a, const double* b, double* o) {
#pragma unroll
  for (int c = 0; c < 4; ++c)
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      double s = a[r] * b[3 * c] + a[r + 3] * b[3 * c + 1] + a[r + 6] * b[3 * c + 2];
      if (c == 3) s += a[r + 9];
      o[r + 3 * c] = s;
    }
}

__device__ inline void crossd(const double* a, const double* b, double* c) {
  double x = a[1] * b[2] - a[2] * b[1], y = a[2] * b[0] - a[0] * b[2], z = a[0] * b[1] - a[1] * b[0];
  c[0] = x; c[1] = y; c[2] = z;
}

// rotation tensor from a rotation vector through a unit quaternion
// (rotationModule.f90:355-370,393-436).  For half angles below epsTh2 = 5e-4
// the reference interpolates sin(h)/h linearly (sinEpsOverEps = sin(epsTh2)/epsTh2,
// evaluated on the host); cos(h) is then its Taylor series to h^6 (the next
// term is below 1e-30), which spares the FP64 sine/cosine on the usual small
// increments.  The quaternion is normalised twice, by one reciprocal square
// root each.
__device__ inline void rotvecToMat(const double* rv, double sinEpsOverEps, double* R /* col-major 3x3 */) {
  const double epsTh2 = 0.0005;
  double thh = 0.5 * sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
  double cthh, fac;
  if (thh < epsTh2) {
    const double h2 = thh * thh;
    cthh = 1.0 - h2 * (0.5 - h2 * (1.0 / 24.0 - h2 * (1.0 / 720.0)));
    double f1 = thh / epsTh2;
    fac = f1 * sinEpsOverEps + 1.0 - f1;
  } else {
    double sthh;
    sincos(thh, &sthh, &cthh);
    fac = sthh / thh;
  }
  double q0 = cthh, q1 = rv[0] * fac * 0.5, q2 = rv[1] * fac * 0.5, q3 = rv[2] * fac * 0.5;
  double inv = rsqrt(q0 * q0 + q1 * q1 + q2 * q2 + q3 * q3);
  q0 *= inv; q1 *= inv; q2 *= inv; q3 *= inv;
  inv = rsqrt(q0 * q0 + q1 * q1 + q2 * q2 + q3 * q3);
  q0 *= inv; q1 *= inv; q2 *= inv; q3 *= inv;
  R[0] = 2.0 * (q1 * q1 + q0 * q0) - 1.0;
  R[4] = 2.0 * (q2 * q2 + q0 * q0) - 1.0;
  R[8] = 2.0 * (q3 * q3 + q0 * q0) - 1.0;
  R[3] = 2.0 * (q1 * q2 - q3 * q0);
  R[6] = 2.0 * (q1 * q3 + q2 * q0);
  R[7] = 2.0 * (q2 * q3 - q1 * q0);
  R[1] = 2.0 * (q2 * q1 + q3 * q0);
  R[2] = 2.0 * (q3 * q1 - q2 * q0);
  R[5] = 2.0 * (q3 * q2 + q1 * q0);
}

}  // namespace fgpu
