// pb_device.cuh -- device-side camera model, robust loss and per-observation linearisation.
//
// Projection: frame pinhole with Brown-Conrady distortion (OpenCV tangential convention)
// as stated in the reference's src/internal/BundleAdjustProjection.h:58-91.
// Linearisation: src/internal/BundleAdjustPlaMatrixProjection.cpp:176-285 with the reference
// point parameterisation of the online Schur path (:216-262, BundleAdjustPlaMatrixAssembly.cpp:24-40):
//   rotation increment  C2W' = D E(w)^T D C2W, D = diag(1,-1,-1), E = Rx Ry Rz
//   centre increment    C' = C + dC (world frame), or the 2-DoF gauge tangent for the scale camera
//   point increment     X' = X + s(X) dX, s(X) = (|X|/1000) / atan(|X|/1000)
// and, for problems with control points, the plain parameterisation (:208-214): rotation columns
// Jw x (X - C) of a world-frame rotation vector, C2W' = Exp(w) C2W, and X' = X + dX.  The two
// rotation charts agree to first order up to the sign of the first component.
// The projection, residual and robust cost are always evaluated in FP64; the Jacobians are
// produced in the arithmetic type T of the kernel (float on the mixed path).
#pragma once

#include <cuda_runtime.h>

#include "pb_internal.h"

namespace pb {

struct DCam {
    double R[9];
    double C[3];
    double fx, fy, cx, cy, k1, k2, k3, p1, p2, su, sv;
    bool flip;
};

__device__ __forceinline__ void load_cam(const double* __restrict__ c, DCam& k) {
#pragma unroll
    for (int i = 0; i < 9; ++i) k.R[i] = __ldg(c + i);
#pragma unroll
    for (int i = 0; i < 3; ++i) k.C[i] = __ldg(c + 9 + i);
    k.fx = __ldg(c + 12); k.fy = __ldg(c + 13); k.cx = __ldg(c + 14); k.cy = __ldg(c + 15);
    k.k1 = __ldg(c + 16); k.k2 = __ldg(c + 17); k.k3 = __ldg(c + 18); k.p1 = __ldg(c + 19); k.p2 = __ldg(c + 20);
    k.su = __ldg(c + 21) < 0.0 ? -1.0 : 1.0;
    k.sv = __ldg(c + 22) < 0.0 ? -1.0 : 1.0;
    k.flip = __ldg(c + 23) != 0.0;
}

struct Proj {
    double px, py;       // pixel
    double x, y, r2, radial, xd, yd, zc, iz;
    double d0, d1, d2;   // X - C
};

// FP64 projection; false when the point is not in front (forward depth <= 1e-9) or not finite.
__device__ __forceinline__ bool project64(const DCam& c, double X0, double X1, double X2, Proj& p) {
    p.d0 = X0 - c.C[0];
    p.d1 = X1 - c.C[1];
    p.d2 = X2 - c.C[2];
    const double xc = c.R[0] * p.d0 + c.R[3] * p.d1 + c.R[6] * p.d2;
    const double yc = c.R[1] * p.d0 + c.R[4] * p.d1 + c.R[7] * p.d2;
    const double zc = c.R[2] * p.d0 + c.R[5] * p.d1 + c.R[8] * p.d2;
    const double fwd = c.flip ? -zc : zc;
    if (!(fwd > 1e-9)) return false;
    const double iz = 1.0 / zc;
    const double x = xc * iz, y = yc * iz;
    const double r2 = x * x + y * y;
    const double radial = 1.0 + r2 * (c.k1 + r2 * (c.k2 + r2 * c.k3));
    const double xy2 = 2.0 * x * y;
    const double xd = x * radial + c.p1 * xy2 + c.p2 * (r2 + 2.0 * x * x);
    const double yd = y * radial + c.p1 * (r2 + 2.0 * y * y) + c.p2 * xy2;
    p.px = c.su * c.fx * xd + c.cx;
    p.py = c.sv * c.fy * yd + c.cy;
    p.x = x; p.y = y; p.r2 = r2; p.radial = radial; p.xd = xd; p.yd = yd; p.zc = zc; p.iz = iz;
    return isfinite(p.px) && isfinite(p.py);
}

// evaluateImageRobustLoss (BundleAdjustPlaMatrixProjection.cpp:75-109) in FP64.
__device__ __forceinline__ bool robust_loss(double s, int loss, double scale, double& cost, double& weight) {
    if (!(s >= 0.0) || !isfinite(s)) return false;
    if (loss == 0) { cost = 0.5 * s; weight = 1.0; return true; }
    const double c2 = scale * scale;
    if (loss == 1) {
        if (s <= c2) { cost = 0.5 * s; weight = 1.0; return true; }
        const double n = sqrt(s);
        cost = scale * n - 0.5 * c2;
        weight = scale / n;
        return true;
    }
    const double ratio = s / c2;
    cost = 0.5 * c2 * log1p(ratio);
    weight = 1.0 / (1.0 + ratio);
    return true;
}

// First and second derivatives d1 = rho'(s), d2 = rho''(s) of the robust cost of robust_loss
// (the normal weight is 2 rho'(s)).  Used by the exact Hessian of the backward pass.
__device__ __forceinline__ void robust_derivatives(double s, int loss, double scale, double& d1, double& d2) {
    d1 = 0.5;
    d2 = 0.0;
    if (loss == 0) return;
    const double c2 = scale * scale;
    if (loss == 1) {
        if (s <= c2) return;
        const double n = sqrt(s);
        d1 = 0.5 * scale / n;
        d2 = -0.25 * scale / (n * s);
        return;
    }
    const double q = 1.0 / (1.0 + s / c2);
    d1 = 0.5 * q;
    d2 = -0.5 * q * q / c2;
}

// Control-point residual of a track point (linearizeControlPoint,
// BundleAdjustPlaMatrixConstraints.cpp:90-116): r = sqrt(weight) W (X - P) from a record
// [sqrt(weight) W (9, row-major), P (3)], Huber on |r|^2 with the control-point delta
// (finishRobust, :17-29).  False when the cost is not finite.
__device__ __forceinline__ bool cp_eval(const double* __restrict__ rec, double X0, double X1, double X2, double delta,
                                        double* r, double& cost, double& weight) {
    const double d0 = X0 - rec[9], d1 = X1 - rec[10], d2 = X2 - rec[11];
    for (int a = 0; a < 3; ++a) r[a] = rec[a * 3] * d0 + rec[a * 3 + 1] * d1 + rec[a * 3 + 2] * d2;
    const double sq = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    double c = 0.0, w = 0.0;
    if (!isfinite(sq)) return false;
    if (sq <= delta * delta) {
        c = 0.5 * sq;
        w = 1.0;
    } else {
        const double n = sqrt(sq);
        c = delta * n - 0.5 * delta * delta;
        w = delta / n;
    }
    cost = c;
    weight = w;
    return isfinite(c) && isfinite(w);
}

__device__ __forceinline__ double point_scale(double X0, double X1, double X2) {
    const double len = sqrt(X0 * X0 + X1 * X1 + X2 * X2) / 1000.0;
    if (!isfinite(len) || len == 0.0) return 1.0;
    return len / atan(len);
}

template <typename T>
struct Lin {
    T r0, r1;
    T Jp[6];            // 2x3 point Jacobian (row-major, scaled)
    T Jc[12];           // 2x6 pose Jacobian (row-major)
    T Ji[2 * kMaxNI];   // 2 x ni intrinsic Jacobian (row-major, compact columns)
    T w;                // normal weight
    double cost;        // robust cost (FP64)
    double rd0, rd1;    // residual (FP64)
    double wd;          // normal weight (FP64)
};

// Intrinsic Jacobian column `col` of the parameter block [fx, log(fy/fx), cx, cy, k1, k2, k3, p1,
// p2] (referenceIntrinsicParameterJacobian, BundleAdjustPlaMatrixProjection.cpp:228-262).
template <typename U>
__device__ __forceinline__ void intrinsic_column(int col, U x, U y, U r2, U xd, U yd, U su, U sv, U sfx, U sfy,
                                                 U aspect, U& ju, U& jv) {
    ju = U(0);
    jv = U(0);
    switch (col) {
        case 0: ju = su * xd; jv = sv * yd * aspect; break;
        case 1: jv = sfy * yd; break;
        case 2: ju = U(1); break;
        case 3: jv = U(1); break;
        case 4: ju = sfx * x * r2; jv = sfy * y * r2; break;
        case 5: ju = sfx * x * r2 * r2; jv = sfy * y * r2 * r2; break;
        case 6: ju = sfx * x * r2 * r2 * r2; jv = sfy * y * r2 * r2 * r2; break;
        case 7: ju = sfx * U(2) * x * y; jv = sfy * (r2 + U(2) * y * y); break;
        case 8: ju = sfx * (r2 + U(2) * x * x); jv = sfy * U(2) * x * y; break;
        default: break;
    }
}

// Linearises one observation; s64 is the point step scale s(X) of its track.  `tangent` selects the gauge tangent centre columns (basis: two
// world-frame directions in gb[0..5]); `plain` the rotation columns of the plain parameterisation.
// Returns false on an invalid projection or loss.
// With `grad`, also writes the observation's gradient -J^T w r in FP64: pose [0, 6), point
// [6, 9), intrinsic columns [9, 9 + ni).  On the FP64 path it comes from the FP64 Jacobian; on
// the FP32 path from the FP64 projection through v = R (dpi/dx_c)^T (w r), so that the gradient
// (and the fixed point of the mixed solve) does not carry the FP32 rounding of the Jacobian.
template <typename T>
__device__ __forceinline__ bool linearize_obs(const DCam& c, double X0, double X1, double X2, double s64, double u,
                                              double v, double wobs, int loss, double lscale, bool tangent,
                                              bool plain, const double* __restrict__ gb, int ni,
                                              const int* __restrict__ cols, bool want_jacobian, Lin<T>& L,
                                              double* grad = nullptr) {
    Proj p;
    if (!project64(c, X0, X1, X2, p)) return false;
    const double r0 = p.px - u, r1 = p.py - v;
    double cost, rw;
    if (!robust_loss(wobs * (r0 * r0 + r1 * r1), loss, lscale, cost, rw)) return false;
    L.cost = cost;
    L.rd0 = r0;
    L.rd1 = r1;
    L.wd = wobs * rw;
    L.r0 = static_cast<T>(r0);
    L.r1 = static_cast<T>(r1);
    L.w = static_cast<T>(wobs * rw);
    if (!isfinite(cost) || !isfinite(wobs * rw)) return false;
    if (!want_jacobian) return true;
    const T x = static_cast<T>(p.x), y = static_cast<T>(p.y), r2 = static_cast<T>(p.r2);
    const T radial = static_cast<T>(p.radial);
    const T k1 = static_cast<T>(c.k1), k2 = static_cast<T>(c.k2), k3 = static_cast<T>(c.k3);
    const T p1 = static_cast<T>(c.p1), p2 = static_cast<T>(c.p2);
    const T sfx = static_cast<T>(c.su * c.fx), sfy = static_cast<T>(c.sv * c.fy);
    const T dr = k1 + r2 * (T(2) * k2 + T(3) * k3 * r2);
    const T dxd_dx = radial + T(2) * x * x * dr + T(2) * p1 * y + T(6) * p2 * x;
    const T dxd_dy = T(2) * x * y * dr + T(2) * p1 * x + T(2) * p2 * y;
    const T dyd_dx = dxd_dy;
    const T dyd_dy = radial + T(2) * y * y * dr + T(6) * p1 * y + T(2) * p2 * x;
    const T iz = static_cast<T>(p.iz);
    const T du_dx = sfx * dxd_dx, du_dy = sfx * dxd_dy, dv_dx = sfy * dyd_dx, dv_dy = sfy * dyd_dy;
    const T dc[6] = {du_dx * iz, du_dy * iz, -(du_dx * x + du_dy * y) * iz,
                     dv_dx * iz, dv_dy * iz, -(dv_dx * x + dv_dy * y) * iz};
    T R[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) R[i] = static_cast<T>(c.R[i]);
    const T d0 = static_cast<T>(p.d0), d1 = static_cast<T>(p.d1), d2 = static_cast<T>(p.d2);
    const T s = static_cast<T>(s64);
    const T rs0 = plain ? T(-1) : T(1);
#pragma unroll
    for (int pa = 0; pa < 2; ++pa) {
        // world point Jacobian: dpi/dXw = dpi/dxc * R^T
        const T jw0 = dc[pa * 3 + 0] * R[0] + dc[pa * 3 + 1] * R[1] + dc[pa * 3 + 2] * R[2];
        const T jw1 = dc[pa * 3 + 0] * R[3] + dc[pa * 3 + 1] * R[4] + dc[pa * 3 + 2] * R[5];
        const T jw2 = dc[pa * 3 + 0] * R[6] + dc[pa * 3 + 1] * R[7] + dc[pa * 3 + 2] * R[8];
        // rotation columns of the target parameterisation: s_k * Jw (e_k x d), s = (1,-1,-1)
        L.Jc[pa * 6 + 0] = rs0 * (jw2 * d1 - jw1 * d2);
        L.Jc[pa * 6 + 1] = jw2 * d0 - jw0 * d2;
        L.Jc[pa * 6 + 2] = jw0 * d1 - jw1 * d0;
        if (tangent) {
            L.Jc[pa * 6 + 3] = -(jw0 * static_cast<T>(gb[0]) + jw1 * static_cast<T>(gb[1]) + jw2 * static_cast<T>(gb[2]));
            L.Jc[pa * 6 + 4] = -(jw0 * static_cast<T>(gb[3]) + jw1 * static_cast<T>(gb[4]) + jw2 * static_cast<T>(gb[5]));
            L.Jc[pa * 6 + 5] = T(0);
        } else {
            L.Jc[pa * 6 + 3] = -jw0;
            L.Jc[pa * 6 + 4] = -jw1;
            L.Jc[pa * 6 + 5] = -jw2;
        }
        L.Jp[pa * 3 + 0] = jw0 * s;
        L.Jp[pa * 3 + 1] = jw1 * s;
        L.Jp[pa * 3 + 2] = jw2 * s;
    }
    const T xd = static_cast<T>(p.xd), yd = static_cast<T>(p.yd);
    const T aspect = static_cast<T>(c.fx > 0.0 ? c.fy / c.fx : 1.0);
    const T su = static_cast<T>(c.su), sv = static_cast<T>(c.sv);
    for (int k = 0; k < ni; ++k) intrinsic_column<T>(cols[k], x, y, r2, xd, yd, su, sv, sfx, sfy, aspect, L.Ji[k],
                                                     L.Ji[kMaxNI + k]);
    if (grad) {
        const double w = L.wd;
        if (sizeof(T) == sizeof(double)) {
            for (int a = 0; a < 6; ++a)
                grad[a] = -w * (static_cast<double>(L.Jc[a]) * r0 + static_cast<double>(L.Jc[6 + a]) * r1);
            for (int a = 0; a < 3; ++a)
                grad[6 + a] = -w * (static_cast<double>(L.Jp[a]) * r0 + static_cast<double>(L.Jp[3 + a]) * r1);
            for (int a = 0; a < ni; ++a)
                grad[9 + a] = -w * (static_cast<double>(L.Ji[a]) * r0 + static_cast<double>(L.Ji[kMaxNI + a]) * r1);
        } else {
            const double wr0 = w * r0, wr1 = w * r1;
            const double gx = p.x, gy = p.y, gr2 = p.r2;
            const double gdr = c.k1 + gr2 * (2.0 * c.k2 + 3.0 * c.k3 * gr2);
            const double gxx = p.radial + 2.0 * gx * gx * gdr + 2.0 * c.p1 * gy + 6.0 * c.p2 * gx;
            const double gxy = 2.0 * gx * gy * gdr + 2.0 * c.p1 * gx + 2.0 * c.p2 * gy;
            const double gyy = p.radial + 2.0 * gy * gy * gdr + 6.0 * c.p1 * gy + 2.0 * c.p2 * gx;
            const double gsfx = c.su * c.fx, gsfy = c.sv * c.fy;
            const double a0 = gsfx * wr0, a1 = gsfy * wr1;
            // t = (dpi/dx_c)^T (w r); v = R t is J_world^T (w r)
            const double tx = (a0 * gxx + a1 * gxy) * p.iz;
            const double ty = (a0 * gxy + a1 * gyy) * p.iz;
            const double tz = -(tx * gx + ty * gy);
            const double v0 = c.R[0] * tx + c.R[1] * ty + c.R[2] * tz;
            const double v1 = c.R[3] * tx + c.R[4] * ty + c.R[5] * tz;
            const double v2 = c.R[6] * tx + c.R[7] * ty + c.R[8] * tz;
            grad[0] = plain ? v2 * p.d1 - v1 * p.d2 : -(v2 * p.d1 - v1 * p.d2);
            grad[1] = -(v2 * p.d0 - v0 * p.d2);
            grad[2] = -(v0 * p.d1 - v1 * p.d0);
            if (tangent) {
                grad[3] = v0 * gb[0] + v1 * gb[1] + v2 * gb[2];
                grad[4] = v0 * gb[3] + v1 * gb[4] + v2 * gb[5];
                grad[5] = 0.0;
            } else {
                grad[3] = v0;
                grad[4] = v1;
                grad[5] = v2;
            }
            grad[6] = -s64 * v0;
            grad[7] = -s64 * v1;
            grad[8] = -s64 * v2;
            const double gaspect = c.fx > 0.0 ? c.fy / c.fx : 1.0;
            for (int k = 0; k < ni; ++k) {
                double ju, jv;
                intrinsic_column<double>(cols[k], gx, gy, gr2, p.xd, p.yd, c.su, c.sv, gsfx, gsfy, gaspect, ju, jv);
                grad[9 + k] = -(ju * wr0 + jv * wr1);
            }
        }
    }
    return true;
}

// Float-float numbers (hi + lo, |lo| <= ulp(hi)/2) for the compensated FP32 arithmetic of the
// mixed path: products use the exact FMA residual (Dekker / Ogita-Rump-Oishi "TwoProduct"),
// sums the Knuth "TwoSum"; about 44 significant bits, all on the FP32 pipe.
struct ff {
    float hi, lo;
};

__device__ __forceinline__ ff ff_make(double d) {
    const float h = static_cast<float>(d);
    return {h, static_cast<float>(d - static_cast<double>(h))};
}
// __fmul_rn / __fadd_rn are never contracted into an FMA, which the error-free transformations
// below depend on.
__device__ __forceinline__ ff ff_norm(float s, float e) {
    const float h = __fadd_rn(s, e);
    return {h, __fadd_rn(e, -__fadd_rn(h, -s))};
}
__device__ __forceinline__ ff operator*(ff a, ff b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return ff_norm(p, e);
}
__device__ __forceinline__ ff operator*(float a, ff b) {
    const float p = __fmul_rn(a, b.hi);
    float e = fmaf(a, b.hi, -p);
    e = fmaf(a, b.lo, e);
    return ff_norm(p, e);
}
__device__ __forceinline__ ff operator+(ff a, ff b) {
    const float s = __fadd_rn(a.hi, b.hi);
    const float bp = __fadd_rn(s, -a.hi);
    const float e = __fadd_rn(__fadd_rn(a.hi, -__fadd_rn(s, -bp)), __fadd_rn(b.hi, -bp)) + (a.lo + b.lo);
    return ff_norm(s, e);
}
__device__ __forceinline__ ff operator-(ff a) { return {-a.hi, -a.lo}; }

// Value type of the reduced-system terms: float-float on the FP32 path, double on the FP64 path.
template <typename T>
struct ValueOf;
template <>
struct ValueOf<float> {
    using type = ff;
    __device__ static __forceinline__ ff make(double d) { return ff_make(d); }
    __device__ static __forceinline__ ff zero() { return {0.f, 0.f}; }
};
template <>
struct ValueOf<double> {
    using type = double;
    __device__ static __forceinline__ double make(double d) { return d; }
    __device__ static __forceinline__ double zero() { return 0.0; }
};

// Two-sum compensated accumulator (FP32 path) / plain FP64 accumulator.
template <typename T>
struct Acc;

template <>
struct Acc<double> {
    using part_type = double;  // partial sums written by the assembly
    double s = 0.0;
    __device__ __forceinline__ void add(double v) { s += v; }
    __device__ __forceinline__ void add_prod(double a, double b) { s = fma(a, b, s); }
    __device__ __forceinline__ double value() const { return s; }
    __device__ __forceinline__ double value64() const { return s; }
    __device__ __forceinline__ void merge(const Acc<double>& o) { s += o.s; }
    __device__ __forceinline__ void merge_part(double v) { s += v; }
    __device__ __forceinline__ double part() const { return s; }
};

template <>
struct Acc<float> {
    float hi = 0.f, lo = 0.f;
    __device__ __forceinline__ void add(float v) {
        const float s = __fadd_rn(hi, v);
        const float bp = __fadd_rn(s, -hi);
        const float e = __fadd_rn(__fadd_rn(hi, -__fadd_rn(s, -bp)), __fadd_rn(v, -bp));
        hi = s;
        lo += e;
    }
    __device__ __forceinline__ void add_prod(float a, float b) {
        const float p = __fmul_rn(a, b);
        const float pe = fmaf(a, b, -p);
        add(p);
        lo += pe;
    }
    __device__ __forceinline__ float value() const { return hi + lo; }
    __device__ __forceinline__ double value64() const { return static_cast<double>(hi) + static_cast<double>(lo); }
    __device__ __forceinline__ void merge(const Acc<float>& o) {
        add(o.hi);
        lo += o.lo;
    }
    __device__ __forceinline__ void add(ff v) {
        add(v.hi);
        lo += v.lo;
    }
    using part_type = float2;  // (hi, lo) pair: the partial keeps the compensation term
    __device__ __forceinline__ void merge_part(float2 v) {
        add(v.x);
        lo += v.y;
    }
    __device__ __forceinline__ float2 part() const { return make_float2(hi, lo); }
};

// acc += a * b, the product's rounding error carried into the compensation term (FP32 path) /
// one FMA (FP64 path).
__device__ __forceinline__ void acc_fma(Acc<float>& acc, ff a, ff b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    acc.add(p);
    acc.lo += e;
}
__device__ __forceinline__ void acc_fma(Acc<float>& acc, float a, ff b) {
    const float p = __fmul_rn(a, b.hi);
    float e = fmaf(a, b.hi, -p);
    e = fmaf(a, b.lo, e);
    acc.add(p);
    acc.lo += e;
}
__device__ __forceinline__ void acc_fma(Acc<double>& acc, double a, double b) { acc.s = fma(a, b, acc.s); }

// Sum of the accumulators of a warp into lane 0 by a fixed shuffle tree (deterministic order).
__device__ __forceinline__ void warp_merge(Acc<double>& acc) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc.s += __shfl_down_sync(0xffffffffu, acc.s, o);
}
__device__ __forceinline__ void warp_merge(Acc<float>& acc) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float h = __shfl_down_sync(0xffffffffu, acc.hi, o);
        const float l = __shfl_down_sync(0xffffffffu, acc.lo, o);
        acc.merge_part(make_float2(h, l));
    }
}

// exact product of two floats as a float-float
__device__ __forceinline__ ff two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return {p, fmaf(a, b, -p)};
}
__device__ __forceinline__ double two_prod(double a, double b) { return a * b; }

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// ---------------------------------------------------------------- float-float linearisation
// The mixed path's robust weight and gradient in float-float arithmetic.  FP64 runs at a small
// fraction of the FP32 rate on this part, and the robust weight, the cost and the gradient chain
// of every observation were most of the FP64 work of the assembly.  The projection and residual
// stay FP64; the rest runs on the FP32 pipe with ~44 significant bits.  (A float-float projection
// was measured too: its ~3e-10 px residual error put a noise floor into the reduced right-hand
// side near convergence and cost ~30% more CG iterations than it saved.)  The reciprocal and
// reciprocal square root take one Newton-Raphson step from the FP32 hardware approximation, with
// the correction term evaluated in float-float (the double-word division scheme of Joldes,
// Muller and Popescu, "Tight and rigorous error bounds for basic building blocks of double-word
// arithmetic", ACM TOMS 2017).  Inputs are float-float copies of the effective cameras, point
// scales and observation weights, written when the FP64 state changes.

__host__ __device__ __forceinline__ float2 ff_pack(double d) {
    const float h = static_cast<float>(d);
    return make_float2(h, static_cast<float>(d - static_cast<double>(h)));
}
__device__ __forceinline__ ff ffl(float2 v) { return {v.x, v.y}; }
__device__ __forceinline__ ff ff_sub(ff a, ff b) { return a + (-b); }
__device__ __forceinline__ ff ff_twice(ff a) { return {2.f * a.hi, 2.f * a.lo}; }  // exact
__device__ __forceinline__ ff ff_one() { return {1.f, 0.f}; }
__device__ __forceinline__ bool ff_le(ff a, ff b) { return a.hi < b.hi || (a.hi == b.hi && a.lo <= b.lo); }

// 1 / a: r = RN(1 / a.hi), then r + r (1 - a r) with the residual 1 - a r in float-float.
__device__ __forceinline__ ff ff_recip(ff a) {
    const float r = __frcp_rn(a.hi);
    const ff e = ff_sub(ff_one(), r * a);
    return ff_norm(r, __fmul_rn(r, e.hi));
}
// 1 / sqrt(a), a > 0: y = rsqrt(a.hi), then y + y (1 - a y^2) / 2 with the residual in float-float.
__device__ __forceinline__ ff ff_rsqrt(ff a) {
    const float y = rsqrtf(a.hi);
    const ff e = ff_sub(ff_one(), a * two_prod(y, y));
    return ff_norm(y, __fmul_rn(0.5f * y, e.hi));
}

// Float-float camera record: R (9), C (3), fx, fy, cx, cy, k1, k2, k3, p1, p2 (11), then the
// signs su, sv and the depth flip as plain floats.
constexpr int kCamFF = 24;
__host__ __device__ __forceinline__ void camera_ff(const double* c, float2* out) {
    for (int i = 0; i < 21; ++i) out[i] = ff_pack(c[i]);
    out[21] = make_float2(c[21] < 0.0 ? -1.f : 1.f, 0.f);
    out[22] = make_float2(c[22] < 0.0 ? -1.f : 1.f, 0.f);
    out[23] = make_float2(c[23] != 0.0 ? 1.f : 0.f, 0.f);
}

struct LinFF {
    float Jc[12];          // 2x6 pose Jacobian (FP32)
    float Jp[6];           // 2x3 point Jacobian, scaled (FP32)
    float Ji[2 * kMaxNI];  // 2 x ni intrinsic Jacobian (FP32)
    ff r0, r1, w;          // residual and normal weight
    ff g[9 + kMaxNI];      // -J^T w r: pose [0, 6), point [6, 9), intrinsic [9, 9 + ni)
};

// Intrinsic Jacobian column `col` (as intrinsic_column) in float-float.
__device__ __forceinline__ void intrinsic_column_ff(int col, ff x, ff y, ff r2, ff xd, ff yd, float su, float sv,
                                                    ff sfx, ff sfy, ff aspect, ff& ju, ff& jv) {
    const ff z = {0.f, 0.f};
    ju = z;
    jv = z;
    switch (col) {
        case 0: ju = su * xd; jv = (sv * yd) * aspect; break;
        case 1: jv = sfy * yd; break;
        case 2: ju = ff_one(); break;
        case 3: jv = ff_one(); break;
        case 4: ju = sfx * (x * r2); jv = sfy * (y * r2); break;
        case 5: { const ff r4 = r2 * r2; ju = sfx * (x * r4); jv = sfy * (y * r4); break; }
        case 6: { const ff r6 = r2 * r2 * r2; ju = sfx * (x * r6); jv = sfy * (y * r6); break; }
        case 7: ju = sfx * ff_twice(x * y); jv = sfy * (r2 + ff_twice(y * y)); break;
        case 8: ju = sfx * (r2 + ff_twice(x * x)); jv = sfy * ff_twice(x * y); break;
        default: break;
    }
}

// linearize_obs of the mixed path (same Jacobian columns, same robust weight).  The projection
// and residual stay FP64 (p: project64 of the observation): the residual is a small difference
// of pixel coordinates, and its absolute accuracy sets the noise floor of the gradient near
// convergence, where the reduced right-hand side shrinks towards it.  Everything after the
// residual -- the robust weight and the gradient -J^T w r -- runs in float-float, and the cost is
// not evaluated.  cam: the camera's float-float record (kCamFF values); s: the point's step scale;
// wobs: the observation weight; gb: the FP64 gauge tangent basis (read for the tangent camera only).
__device__ __forceinline__ bool linearize_obs_ff(const Proj& p, double u, double v, const float2* __restrict__ cam,
                                                 ff s, ff wobs, int loss, ff lscale, bool tangent, bool plain,
                                                 const double* __restrict__ gb, int ni, const int* __restrict__ cols,
                                                 LinFF& L) {
    ff R[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) R[i] = ffl(cam[i]);
    const ff d0 = ff_make(p.d0), d1 = ff_make(p.d1), d2 = ff_make(p.d2);
    const ff iz = ff_make(p.iz);
    const ff x = ff_make(p.x), y = ff_make(p.y), r2 = ff_make(p.r2), radial = ff_make(p.radial);
    const ff xd = ff_make(p.xd), yd = ff_make(p.yd);
    const ff k1 = ffl(cam[16]), k2 = ffl(cam[17]), k3 = ffl(cam[18]), p1 = ffl(cam[19]), p2 = ffl(cam[20]);
    const float su = cam[21].x, sv = cam[22].x;
    const ff fx = ffl(cam[12]), fy = ffl(cam[13]);
    const ff sfx = su * fx, sfy = sv * fy;
    const ff r0 = ff_make(p.px - u), r1 = ff_make(p.py - v);
    // evaluateImageRobustLoss weight (BundleAdjustPlaMatrixProjection.cpp:75-109)
    const ff sq = wobs * (r0 * r0 + r1 * r1);
    if (!(sq.hi >= 0.f) || !isfinite(sq.hi)) return false;
    ff rw = ff_one();
    if (loss == 1) {
        if (!ff_le(sq, lscale * lscale)) rw = lscale * ff_rsqrt(sq);
    } else if (loss == 2) {
        const ff c2 = lscale * lscale;
        rw = c2 * ff_recip(c2 + sq);
    }
    const ff w = wobs * rw;
    if (!isfinite(w.hi)) return false;
    L.r0 = r0;
    L.r1 = r1;
    L.w = w;
    // FP32 Jacobians from the leading parts (the formulas of linearize_obs)
    const float fx_ = x.hi, fy_ = y.hi, fr2 = r2.hi, frad = radial.hi;
    const float fk1 = k1.hi, fk2 = k2.hi, fk3 = k3.hi, fp1 = p1.hi, fp2 = p2.hi;
    const float fsfx = sfx.hi, fsfy = sfy.hi, fiz = iz.hi;
    const float dr = fk1 + fr2 * (2.f * fk2 + 3.f * fk3 * fr2);
    const float dxd_dx = frad + 2.f * fx_ * fx_ * dr + 2.f * fp1 * fy_ + 6.f * fp2 * fx_;
    const float dxd_dy = 2.f * fx_ * fy_ * dr + 2.f * fp1 * fx_ + 2.f * fp2 * fy_;
    const float dyd_dy = frad + 2.f * fy_ * fy_ * dr + 6.f * fp1 * fy_ + 2.f * fp2 * fx_;
    const float du_dx = fsfx * dxd_dx, du_dy = fsfx * dxd_dy, dv_dx = fsfy * dxd_dy, dv_dy = fsfy * dyd_dy;
    const float dc[6] = {du_dx * fiz, du_dy * fiz, -(du_dx * fx_ + du_dy * fy_) * fiz,
                         dv_dx * fiz, dv_dy * fiz, -(dv_dx * fx_ + dv_dy * fy_) * fiz};
    const float fd0 = d0.hi, fd1 = d1.hi, fd2 = d2.hi, fs = s.hi;
    const float rs0 = plain ? -1.f : 1.f;
#pragma unroll
    for (int pa = 0; pa < 2; ++pa) {
        const float jw0 = dc[pa * 3] * R[0].hi + dc[pa * 3 + 1] * R[1].hi + dc[pa * 3 + 2] * R[2].hi;
        const float jw1 = dc[pa * 3] * R[3].hi + dc[pa * 3 + 1] * R[4].hi + dc[pa * 3 + 2] * R[5].hi;
        const float jw2 = dc[pa * 3] * R[6].hi + dc[pa * 3 + 1] * R[7].hi + dc[pa * 3 + 2] * R[8].hi;
        L.Jc[pa * 6 + 0] = rs0 * (jw2 * fd1 - jw1 * fd2);
        L.Jc[pa * 6 + 1] = jw2 * fd0 - jw0 * fd2;
        L.Jc[pa * 6 + 2] = jw0 * fd1 - jw1 * fd0;
        if (tangent) {
            L.Jc[pa * 6 + 3] = -(jw0 * static_cast<float>(gb[0]) + jw1 * static_cast<float>(gb[1]) +
                                 jw2 * static_cast<float>(gb[2]));
            L.Jc[pa * 6 + 4] = -(jw0 * static_cast<float>(gb[3]) + jw1 * static_cast<float>(gb[4]) +
                                 jw2 * static_cast<float>(gb[5]));
            L.Jc[pa * 6 + 5] = 0.f;
        } else {
            L.Jc[pa * 6 + 3] = -jw0;
            L.Jc[pa * 6 + 4] = -jw1;
            L.Jc[pa * 6 + 5] = -jw2;
        }
        L.Jp[pa * 3 + 0] = jw0 * fs;
        L.Jp[pa * 3 + 1] = jw1 * fs;
        L.Jp[pa * 3 + 2] = jw2 * fs;
    }
    const ff aspect = fx.hi > 0.f ? fy * ff_recip(fx) : ff_one();
    for (int k = 0; k < ni; ++k)
        intrinsic_column<float>(cols[k], fx_, fy_, fr2, xd.hi, yd.hi, su, sv, fsfx, fsfy, aspect.hi, L.Ji[k],
                                L.Ji[kMaxNI + k]);
    // gradient -J^T (w r) through v = R (dpi/dx_c)^T (w r), in float-float
    const ff wr0 = w * r0, wr1 = w * r1;
    const ff gdr = k1 + r2 * (ff_twice(k2) + 3.f * (k3 * r2));
    const ff gxx = radial + ff_twice(x * x) * gdr + ff_twice(p1 * y) + 6.f * (p2 * x);
    const ff gxy = ff_twice(x * y) * gdr + ff_twice(p1 * x) + ff_twice(p2 * y);
    const ff gyy = radial + ff_twice(y * y) * gdr + 6.f * (p1 * y) + ff_twice(p2 * x);
    const ff a0 = sfx * wr0, a1 = sfy * wr1;
    const ff tx = (a0 * gxx + a1 * gxy) * iz;
    const ff ty = (a0 * gxy + a1 * gyy) * iz;
    const ff tz = -(tx * x + ty * y);
    const ff v0 = R[0] * tx + R[1] * ty + R[2] * tz;
    const ff v1 = R[3] * tx + R[4] * ty + R[5] * tz;
    const ff v2 = R[6] * tx + R[7] * ty + R[8] * tz;
    const ff g0 = ff_sub(v2 * d1, v1 * d2);
    L.g[0] = plain ? g0 : -g0;
    L.g[1] = -ff_sub(v2 * d0, v0 * d2);
    L.g[2] = -ff_sub(v0 * d1, v1 * d0);
    if (tangent) {
        L.g[3] = v0 * ff_make(gb[0]) + v1 * ff_make(gb[1]) + v2 * ff_make(gb[2]);
        L.g[4] = v0 * ff_make(gb[3]) + v1 * ff_make(gb[4]) + v2 * ff_make(gb[5]);
        L.g[5] = {0.f, 0.f};
    } else {
        L.g[3] = v0;
        L.g[4] = v1;
        L.g[5] = v2;
    }
    L.g[6] = -(s * v0);
    L.g[7] = -(s * v1);
    L.g[8] = -(s * v2);
    for (int k = 0; k < ni; ++k) {
        ff ju, jv;
        intrinsic_column_ff(cols[k], x, y, r2, xd, yd, su, sv, sfx, sfy, aspect, ju, jv);
        L.g[9 + k] = -(ju * wr0 + jv * wr1);
    }
    return true;
}

}  // namespace pb
