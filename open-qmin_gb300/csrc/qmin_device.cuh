// Device-side Q-tensor algebra shared by the qmin_gb300 kernels.  Every
// function is templated on the storage/arithmetic type T (double for the FP64
// form, float for the FP32 form).  Formulas follow open-Qmin's
// inc/qTensorFunctions.h, src/forces/lcForces.h and
// src/forces/landauDeGennesLCBoundary.h, written here from the functionals
// they implement.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

namespace qmin {

template <class T> struct V5 { T c[5]; };

// derivative of tr Q^2, tr Q^3, (tr Q^2)^2 w.r.t. (q0..q4) (qTensorFunctions.h:73-107)
// and the phase force f = -(a dTrQ2 + b dTrQ3 + c d(TrQ2)^2), a = A/2, b = B/3, c = C/4
// (landauDeGennesLCDistortionTerms.cpp:23-38).  With s = tr Q^2 / 2,
// d(TrQ2)^2 = 4 s dTrQ2, so a dTrQ2 + c d(TrQ2)^2 = (a + 4 c s) dTrQ2: one
// factor instead of two products per component (about a third fewer FP64
// operations, which bound the FP64 force kernels on GB300).
template <class T>
__device__ __forceinline__ void phase_force(T a, T b, T c, const T *q, T *f)
{
    const T q0 = q[0], q1 = q[1], q2 = q[2], q3 = q[3], q4 = q[4];
    const T s = q0 * q0 + q1 * q1 + q2 * q2 + q3 * q3 + q4 * q4 + q0 * q3;
    const T g = a + T(4) * c * s;
    const T d2[5] = {T(2) * (T(2) * q0 + q3), T(4) * q1, T(4) * q2, T(2) * (q0 + T(2) * q3), T(4) * q4};
    const T d3[5] = {T(-3) * (-q1 * q1 + q3 * q3 + q4 * q4 + T(2) * q0 * q3),
                     T(6) * (q0 * q1 + q1 * q3 + q2 * q4),
                     T(-6) * q2 * q3 + T(6) * q1 * q4,
                     T(-3) * (q0 * q0 - q1 * q1 + q2 * q2 + T(2) * q0 * q3),
                     T(6) * q1 * q2 - T(6) * q0 * q4};
#pragma unroll
    for (int k = 0; k < 5; ++k) f[k] = -(g * d2[k]) - b * d3[k];
}

// f = phase force - e for a site with distortion (or other) term e, in the
// fewest FP64 operations: the constant factors of dTrQ2 and dTrQ3 folded into
// 2 (a + 4 c s) and 3 b, 6 b (loop-invariant), e entering the FMA chains.
//   f0 = -2 g u0 + 3 b X0 - e0,  u0 = 2 q0 + q3,  X0 = -q1^2 + q3^2 + q4^2 + 2 q0 q3
//   f1 = -4 g q1 - 6 b X1 - e1,  X1 = q0 q1 + q1 q3 + q2 q4
//   f2 = -4 g q2 - 6 b X2 - e2,  X2 = q1 q4 - q2 q3
//   f3 = -2 g u3 + 3 b X3 - e3,  u3 = q0 + 2 q3,  X3 = q0^2 - q1^2 + q2^2 + 2 q0 q3
//   f4 = -4 g q4 - 6 b X4 - e4,  X4 = q1 q2 - q0 q4
template <class T>
__device__ __forceinline__ void phase_force_sub(T a, T b, T c, const T *q, const T *e, T *f)
{
    const T q0 = q[0], q1 = q[1], q2 = q[2], q3 = q[3], q4 = q[4];
    // s = q0^2 + q1^2 + q2^2 + q3^2 + q4^2 + q0 q3
    const T s = fma(q0, q0 + q3, fma(q1, q1, fma(q2, q2, fma(q3, q3, q4 * q4))));
    const T g2 = fma(T(8) * c, s, T(2) * a), g4 = g2 + g2;
    const T b3 = T(3) * b, b6 = T(6) * b;
    const T u0 = fma(T(2), q0, q3), u3 = fma(T(2), q3, q0);
    const T w = fma(q0 + q0, q3, -(q1 * q1));  // 2 q0 q3 - q1^2
    const T X0 = fma(q3, q3, fma(q4, q4, w));
    const T X1 = fma(q0, q1, fma(q1, q3, q2 * q4));
    const T X2 = fma(q1, q4, -(q2 * q3));
    const T X3 = fma(q0, q0, fma(q2, q2, w));
    const T X4 = fma(q1, q2, -(q0 * q4));
    f[0] = fma(b3, X0, fma(-g2, u0, -e[0]));
    f[1] = fma(-b6, X1, fma(-g4, q1, -e[1]));
    f[2] = fma(-b6, X2, fma(-g4, q2, -e[2]));
    f[3] = fma(b3, X3, fma(-g2, u3, -e[3]));
    f[4] = fma(-b6, X4, fma(-g4, q4, -e[4]));
}

// lcForce::bulkL1Force cross terms (lcForces.h:26-37): S0 += S0+S3, S3 += S0+S3, S1,S2,S4 *= 2
template <class T>
__device__ __forceinline__ void l1_cross(T *s)
{
    const T cross = s[0] + s[3];
    s[0] += cross;
    s[1] *= T(2);
    s[2] *= T(2);
    s[3] += cross;
    s[4] *= T(2);
}

// correctForceFromMetric (landauDeGennesLC.cpp:137-160)
template <class T>
__device__ __forceinline__ void metric(T *f)
{
    const T f0 = f[0], f3 = f[3];
    f[0] = (T(2) / T(3)) * (T(2) * f0 - f3);
    f[3] = (T(2) / T(3)) * (T(2) * f3 - f0);
}

// the metric applied twice (M^2 = (4/9) [[5, -4], [-4, 5]] on (f0, f3)): what a
// type-0 site gets in CPU mode when no field term sits between the two
template <class T>
__device__ __forceinline__ void metric2(T *f)
{
    const T f0 = f[0], f3 = f[3];
    f[0] = (T(20) / T(9)) * f0 - (T(16) / T(9)) * f3;
    f[3] = (T(20) / T(9)) * f3 - (T(16) / T(9)) * f0;
}

// QT-metric dot product dotVec (inc/functions.h:140-147)
template <class T>
__device__ __forceinline__ T dot_qt(const T *x, const T *y)
{
    T s = x[0] * y[0] + x[1] * y[1] + x[2] * y[2] + x[3] * y[3] + x[4] * y[4];
    return s + x[0] * y[3];
}

// acc += (F.F, v.v, F.v) in the QT metric, accumulated inside the FMA chains
// (x.y = x0 (y0 + y3) + x1 y1 + x2 y2 + x3 y3 + x4 y4, the y0 + y3 of v shared)
template <class T>
__device__ __forceinline__ void dot3_acc(const T *f, const T *v, T *acc)
{
    const T fs = f[0] + f[3], vs = v[0] + v[3];
    acc[0] = fma(f[0], fs, fma(f[1], f[1], fma(f[2], f[2], fma(f[3], f[3], fma(f[4], f[4], acc[0])))));
    acc[1] = fma(v[0], vs, fma(v[1], v[1], fma(v[2], v[2], fma(v[3], v[3], fma(v[4], v[4], acc[1])))));
    acc[2] = fma(f[0], vs, fma(f[1], v[1], fma(f[2], v[2], fma(f[3], v[3], fma(f[4], v[4], acc[2])))));
}

template <class T>
__device__ __forceinline__ T tr_q2(const T *q)
{
    return T(2) * (q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3] + q[4] * q[4] + q[0] * q[3]);
}

template <class T>
__device__ __forceinline__ T tr_q3(const T *q)
{
    return T(-3) * ((-(q[1] * q[1]) + q[3] * q[3] + q[4] * q[4]) * q[0] + q[0] * q[0] * q[3] - q[1] * q[1] * q[3] +
                    q[2] * q[2] * q[3] - T(2) * q[1] * q[2] * q[4]);
}

// Fournier-Galatola degenerate planar anchoring (landauDeGennesLCBoundary.h:44-72, W1 = W2 = W):
// with Qt = Q + S0/2 I, w = Qt nu, s = nu.w, the planar-projected deviation is
// D = nu w^T + w nu^T - s nu nu^T and E = W tr D^2 + W (tr Q^2 - 3 S0^2 / 2)^2.
// dE/dQt = 2 W D, mapped to (q0..q4) with Qzz = -q0 - q3.
template <class T>
__device__ __forceinline__ void planar_D(const T *q, const T *nu, T S0, T D[6])
{
    const T h = T(0.5) * S0;
    const T Qxx = q[0] + h, Qyy = q[3] + h, Qzz = -q[0] - q[3] + h;
    const T w0 = Qxx * nu[0] + q[1] * nu[1] + q[2] * nu[2];
    const T w1 = q[1] * nu[0] + Qyy * nu[1] + q[4] * nu[2];
    const T w2 = q[2] * nu[0] + q[4] * nu[1] + Qzz * nu[2];
    const T s = nu[0] * w0 + nu[1] * w1 + nu[2] * w2;
    D[0] = T(2) * nu[0] * w0 - s * nu[0] * nu[0];                // xx
    D[1] = nu[0] * w1 + w0 * nu[1] - s * nu[0] * nu[1];          // xy
    D[2] = nu[0] * w2 + w0 * nu[2] - s * nu[0] * nu[2];          // xz
    D[3] = T(2) * nu[1] * w1 - s * nu[1] * nu[1];                // yy
    D[4] = nu[1] * w2 + w1 * nu[2] - s * nu[1] * nu[2];          // yz
    D[5] = T(2) * nu[2] * w2 - s * nu[2] * nu[2];                // zz
}

// force on an LC site q from one object neighbour with stored tensor qb
// (computeBoundaryForce, landauDeGennesLCBoundary.h:26-74), added into f
template <class T>
__device__ __forceinline__ void anchoring_force_add(int kind, T W, T S0, const T *q, const T *qb, T *f)
{
    if (kind == 0) {
        T d[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) d[k] = T(2) * (q[k] - qb[k]);
        T ans[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) ans[k] = T(2) * d[k];
        ans[0] += d[3];
        ans[3] += d[0];
#pragma unroll
        for (int k = 0; k < 5; ++k) f[k] += -W * ans[k];
    } else {
        T D[6];
        planar_D(q, qb, S0, D);
        const T sq = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3] + q[4] * q[4] + q[0] * q[3];
        const T c2 = T(3) * (S0 * S0) - T(4) * sq;
        f[0] += T(2) * W * (T(2) * q[0] + q[3]) * c2 - T(2) * W * (D[0] - D[5]);
        f[1] += T(4) * W * q[1] * c2 - T(4) * W * D[1];
        f[2] += T(4) * W * q[2] * c2 - T(4) * W * D[2];
        f[3] += T(2) * W * (q[0] + T(2) * q[3]) * c2 - T(2) * W * (D[3] - D[5]);
        f[4] += T(4) * W * q[4] * c2 - T(4) * W * D[4];
    }
}

// computeBoundaryEnergy (landauDeGennesLCBoundary.h:77-124)
template <class T>
__device__ __forceinline__ T anchoring_energy(int kind, T W, T S0, const T *q, const T *qb)
{
    if (kind == 0) {
        T d[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) d[k] = q[k] - qb[k];
        return W * tr_q2(d);
    }
    T D[6];
    planar_D(q, qb, S0, D);
    const T e1 = D[0] * D[0] + D[3] * D[3] + D[5] * D[5] + T(2) * (D[1] * D[1] + D[2] * D[2] + D[4] * D[4]);
    const T e2 = T(3) * (S0 * S0) -
                 T(4) * (q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[0] * q[3] + q[3] * q[3] + q[4] * q[4]);
    return W * e1 + T(0.25) * W * e2 * e2;
}

}  // namespace qmin
