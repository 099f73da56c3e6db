// Rel-rod shape factors (diffsims/utils/shape_factor_models.py), their
// derivatives, and the precession rotation average -- shared by the forward
// orientation kernel and the adjoint kernels.
//
// Every function is a template over a constant block C that provides:
//   int shape, prec;                       model and precession mode
//   double width, minima, phi, int_step;   w, minima_number, phi (rad), breakpoint spacing
//   float width_f, mw_f, mfac_f, sigma_f, phi_f, int_step_f;
//     (mw = n / w, mfac = pi n / |w|, sigma = pi / w)
#pragma once
#include <type_traits>

#include "common.cuh"

namespace ds {

constexpr float SHAPE_PI_F = 3.14159265358979f;
constexpr double SHAPE_PI = 3.14159265358979323846;

// Breakpoint spacing of the precession average per model: the kinks of
// linear at 0 and +-w, the zeros of sinc at multiples of w/n, feature-scale
// grids of the smooth models (w/2n for sin2c and atanc, w/pi for lorentzian);
// 0 = no breakpoints.
inline double precession_breakpoint_step(int shape, double width, double minima) {
    const double aw = fabs(width), n = minima;
    switch (shape) {
        case DS_SHAPE_LINEAR: return aw;
        case DS_SHAPE_SINC: return n > 0 ? aw / n : 0.0;
        case DS_SHAPE_SIN2C:
        case DS_SHAPE_ATANC: return n > 0 ? aw / (2.0 * n) : 0.0;
        case DS_SHAPE_LORENTZIAN: return aw / SHAPE_PI;
        default: return 0.0;
    }
}

// FP32 precession average below this -> redone in FP64.  Measured against a
// tight adaptive quadrature on random (s0, r phi) over the selection band,
// FP32 max relative error per decade of the average: linear (a small
// difference of O(1) terms near the band edge) 3e-5 at 1e-5..1e-4, 7e-6 at
// 1e-3..1e-2, 2e-6 above; sin2c 8e-6 at 1e-3..1e-2, 5e-6 above; sinc 3e-6
// above 1e-3; atanc and lorentzian ~1e-6 above 1e-4.
// The forward kernels take the linear model's average from its FP32 closed
// form (simulate_kernel.cuh), accurate to 7.4e-7 down to 1e-10: only
// averages below that are redone in FP64.
inline float precession_fp64_threshold_quadrature(int shape);
inline float precession_fp64_threshold(int shape) {
    return shape == DS_SHAPE_LINEAR ? 1e-10f : precession_fp64_threshold_quadrature(shape);
}
// FP32 quadrature (the adjoint kernels, and every model but linear forward)
inline float precession_fp64_threshold_quadrature(int shape) {
    switch (shape) {
        case DS_SHAPE_LINEAR:
        case DS_SHAPE_SIN2C: return 1e-2f;
        case DS_SHAPE_SINC: return 1e-3f;
        default: return 1e-4f;
    }
}

// ----------------------------------------------------------- the models ----
// FP32, one excitation error.
template <class C>
__device__ inline float shape_base_f32(const C &c, float s) {
    switch (c.shape) {
        case DS_SHAPE_LINEAR: {  // :52-73
            const float v = __fdiv_rn(c.width_f - fabsf(s), c.width_f);
            return v > 0.f ? v : 0.f;
        }
        case DS_SHAPE_SINC:    // :76-101 (s = 0 -> 0)
        case DS_SHAPE_SIN2C: { // :104-123
            const float x = s * c.mw_f;  // minima_number * s / width
            float v = 0.f;
            if (x != 0.f) v = fabsf(sinpif(x - rintf(x))) / (SHAPE_PI_F * fabsf(x));
            return c.shape == DS_SHAPE_SIN2C ? v * v : v;
        }
        case DS_SHAPE_ATANC: {  // :126-151 (s = 0 -> 1)
            const float y = c.mfac_f * s;
            return y == 0.f ? 1.f : atanf(y) / y;
        }
        case DS_SHAPE_LORENTZIAN: {  // :154-180 = 1 / (1 + (pi s / w)^2)
            const float x = c.sigma_f * s;
            return __frcp_rn(fmaf(x, x, 1.f));  // the correctly rounded reciprocal: = 1.f / (...)
        }
        default:
            return 1.f;  // binary, :33-49
    }
}

// FP64, direct transcription.
template <class C>
__device__ inline double shape_base_f64(const C &c, double s) {
    switch (c.shape) {
        case DS_SHAPE_LINEAR: {
            double v = 1 - fabs(s) / c.width;
            return v < 0 ? 0.0 : v;
        }
        case DS_SHAPE_SINC:
        case DS_SHAPE_SIN2C: {
            double fac = SHAPE_PI * c.minima / c.width;
            double den = fac * s;
            double v = den != 0 ? fabs(sin(fac * s) / den) : 0.0;
            return c.shape == DS_SHAPE_SIN2C ? v * v : v;
        }
        case DS_SHAPE_ATANC: {
            double fac = SHAPE_PI * c.minima / fabs(c.width);
            double y = fac * s;
            return y == 0 ? 1.0 : atan(y) / y;
        }
        case DS_SHAPE_LORENTZIAN: {
            double sigma = SHAPE_PI / c.width;
            return sigma / (SHAPE_PI * (sigma * sigma * s * s + 1)) * c.width;
        }
        default:
            return 1.0;
    }
}

// d f / d s (zero where the model is flat or at its isolated points:
// s = 0 of sinc, the cut-off of linear).
template <typename T, class C>
__device__ inline T shape_deriv(const C &c, T s) {
    switch (c.shape) {
        case DS_SHAPE_LINEAR: {
            const T w = (T)c.width;
            const T v = (T)1 - fabs(s) / w;
            if (!(v > (T)0) || s == (T)0) return (T)0;
            return s > (T)0 ? -(T)1 / w : (T)1 / w;
        }
        case DS_SHAPE_SINC:
        case DS_SHAPE_SIN2C: {
            const T fac = (T)(SHAPE_PI * c.minima / c.width);
            const T x = fac * s;
            if (x == (T)0) return (T)0;
            const T sx = sin(x), cx = cos(x);
            const T q = sx / x;                       // sin x / x
            const T dq = (x * cx - sx) / (x * x);     // d/dx (sin x / x)
            if (c.shape == DS_SHAPE_SIN2C) return (T)2 * q * dq * fac;
            return (q < (T)0 ? -dq : dq) * fac;       // |sin x / x|
        }
        case DS_SHAPE_ATANC: {
            const T fac = (T)(SHAPE_PI * c.minima / fabs(c.width));
            const T y = fac * s;
            if (y == (T)0) return (T)0;
            return (y / ((T)1 + y * y) - atan(y)) / (y * y) * fac;
        }
        case DS_SHAPE_LORENTZIAN: {
            const T sg = (T)(SHAPE_PI / c.width);
            const T d = (T)1 + sg * sg * s * s;
            return -(T)2 * sg * sg * s / (d * d);
        }
        default:
            return (T)0;
    }
}

// ------------------------------------------- precession rotation average ----
// shf(s0, r) = (1/2pi) int_0^2pi f(s0 + r phi cos t) dt
//            = (1/pi)  int_0^pi  f(s0 + a cos t) dt,  a = r phi
// (diffsims/utils/shape_factor_models.py:222-268 evaluates it per spot with an
// adaptive quadrature).  Here: the s-range [s0 - a, s0 + a] is cut at the
// multiples of a per-model spacing h (the kinks of linear at 0 and +-w, the
// zeros of sinc at multiples of w/n, and a feature-scale grid for the smooth
// models), each cut maps to t = acos((k h - s0) / a), and every piece gets an
// 8-point Gauss-Legendre rule in t.  On one piece the integrand is analytic
// in t, so the rule's error is ~1e-7 relative or below for every model at the
// chosen spacings (checked against a tight adaptive quadrature).  linear
// pieces outside |s| < w are zero and skipped.  With GRAD the same nodes also
// give d shf / d s0 = (1/pi) int f'(.) dt and d shf / d a = (1/pi) int f'(.) cos t dt
// (f is continuous at the cuts, so moving them adds nothing).  The nodes of a
// piece come in pairs mid +- d: cos(mid +- d) = cos mid cos d -+ sin mid sin d,
// one sincos per pair.
//
// 8-point Gauss-Legendre rule on [-1, 1]: the positive roots of P_8 and
// their weights.
template <typename T>
__device__ __forceinline__ T gl8_x(int i) {
    const T x[4] = {(T)0.18343464249564978, (T)0.525532409916329, (T)0.7966664774136267, (T)0.9602898564975362};
    return x[i];
}
template <typename T>
__device__ __forceinline__ T gl8_w(int i) {
    const T w[4] = {(T)0.36268378337836166, (T)0.3137066458778869, (T)0.22238103445337443,
                    (T)0.10122853629037706};
    return w[i];
}

__device__ __forceinline__ void sincos_t(float x, float *s, float *c) { sincosf(x, s, c); }
__device__ __forceinline__ void sincos_t(double x, double *s, double *c) { sincos(x, s, c); }
__device__ __forceinline__ void sincospi_t(float x, float *s, float *c) { sincospif(x, s, c); }
__device__ __forceinline__ void sincospi_t(double x, double *s, double *c) { sincospi(x, s, c); }
__device__ __forceinline__ float sinpi_t(float x) { return sinpif(x); }
__device__ __forceinline__ double sinpi_t(double x) { return sinpi(x); }

// The per-model constants in the quadrature's type, formed once per spot
// (not per node): w, n / w, pi n / |w|, pi / w.
template <typename T>
struct ShapeK {
    T w, mw, mfac, sigma;
};
template <class C>
__device__ __forceinline__ ShapeK<float> shape_k(const C &c, float) {
    return {c.width_f, c.mw_f, c.mfac_f, c.sigma_f};
}
template <class C>
__device__ __forceinline__ ShapeK<double> shape_k(const C &c, double) {
    return {c.width, c.minima / c.width, SHAPE_PI * c.minima / fabs(c.width), SHAPE_PI / c.width};
}

// Model SHAPE at s: value, and with GRAD the derivative d f / d s.
template <int SHAPE, bool GRAD, typename T>
__device__ __forceinline__ T shape_vd(const ShapeK<T> &K, T s, T &df) {
    const T PI_T = (T)SHAPE_PI;
    if (SHAPE == DS_SHAPE_LINEAR) {
        const T w = K.w;
        const T v = (w - fabs(s)) / w;
        if (GRAD) df = (v > (T)0 && s != (T)0) ? (s > (T)0 ? -(T)1 / w : (T)1 / w) : (T)0;
        return v > (T)0 ? v : (T)0;
    } else if (SHAPE == DS_SHAPE_SINC || SHAPE == DS_SHAPE_SIN2C) {
        const T x = s * K.mw;  // x = n s / w, u = pi x
        if (x == (T)0) {
            if (GRAD) df = (T)0;
            return (T)0;
        }
        const T m = rint(x);
        const T t = x - m;
        const T u = PI_T * x;
        if (!GRAD) {
            const T g = sinpi_t(t) / u;  // +-sin(u) / u: the sign does not matter here
            return (SHAPE == DS_SHAPE_SIN2C) ? g * g : fabs(g);
        }
        // sin(pi (t + m)) = (-1)^m sin(pi t), likewise cos
        const T sg = ((long long)m & 1) ? (T)-1 : (T)1;
        T sn, cs;
        sincospi_t(t, &sn, &cs);
        const T ru = (T)1 / u;
        const T g = sg * sn * ru;                       // sin u / u
        const T dg = (sg * cs - g) * ru * (PI_T * K.mw);  // d/ds (sin u / u)
        df = (SHAPE == DS_SHAPE_SIN2C) ? (T)2 * g * dg : (g < (T)0 ? -dg : dg);
        return (SHAPE == DS_SHAPE_SIN2C) ? g * g : fabs(g);
    } else if (SHAPE == DS_SHAPE_ATANC) {
        const T y = K.mfac * s;
        if (y == (T)0) {
            if (GRAD) df = (T)0;
            return (T)1;
        }
        const T f = atan(y) / y;
        if (GRAD) df = ((T)1 / ((T)1 + y * y) - f) / y * K.mfac;
        return f;
    } else if (SHAPE == DS_SHAPE_LORENTZIAN) {
        const T x = K.sigma * s;
        const T f = (T)1 / ((T)1 + x * x);
        if (GRAD) df = -(T)2 * x * K.sigma * f * f;
        return f;
    } else {
        if (GRAD) df = (T)0;
        return (T)1;
    }
}

// The linear model's rotation average in closed form (FP64):
//   (1 / pi) int_0^pi max(0, 1 - |s0 + a cos t| / w) dt,  a > 0, w > 0.
// On each of [0, w] and [-w, 0] the integrand is 1 -/+ (s0 + a cos t) / w
// between the angles t(b) = acos((b - s0) / a) of the interval's ends, so the
// integral is (1 -/+ s0 / w) dt -/+ (a / w) d(sin t).  Evaluated stably:
// every angle is held as x or pi - x (x <= pi / 2) from the exactly summed
// distance of b to the nearer end of [s0 - a, s0 + a] (t = 2 asin(sqrt(d /
// 2a))), range ends are exactly 0 or pi, and a piece that ends where the
// integrand vanishes (t_e at b = +/-w) is written about that angle:
//   (a / w) [sin t_e (1 - cos D) +/- cos t_e (D - sin D)],  D its length,
// with 1 - cos D = 2 sin^2(D / 2) and D - sin D by its Taylor series for
// small D: no difference of nearly equal terms, so small averages (spots
// that graze the support) keep their relative accuracy (<= 1e-10 against
// 50-digit arithmetic, averages from 1e-19 to 1).  Sines and cosines come
// from the half-angle values q = sin(x / 2), p = cos(x / 2) of each angle,
// so a call costs three FP64 asin and square roots.
struct PrecAngle {
    double x;     // t = x (near 0) or pi - x (near pi), x = 2 asin(q) in [0, pi]
    double q, p;  // sin(x / 2), cos(x / 2)
    bool top;
    bool inside;  // b strictly inside (s0 - a, s0 + a)
};

// D - sin D, with sin D = 2 h cos(D / 2) from h = sin(D / 2)
__device__ __forceinline__ double d_minus_sin(double d, double h) {
    if (d < 0.25) {
        const double d2 = d * d;
        return d * d2 * (1.0 / 6 - d2 * (1.0 / 120 - d2 * (1.0 / 5040 - d2 * (1.0 / 362880 - d2 / 39916800.0))));
    }
    return d - 2.0 * h * sqrt((1.0 - h) * (1.0 + h));
}

// sin and cos of the angle from its half-angle values: sin t = 2 q p,
// cos t = 1 - 2 q^2 (negated for t = pi - x); no trigonometric call
__device__ __forceinline__ void prec_sc(const PrecAngle &A, double &sn, double &cs) {
    sn = 2.0 * A.q * A.p;
    const double c = (1.0 - A.q) * (1.0 + A.q) - A.q * A.q;
    cs = A.top ? c : -c;
}

__device__ inline double linear_precession_closed(double s0, double a, double w) {
    const double PI = SHAPE_PI;
    // s0 + a = hi + hl and s0 - a = lo + ll exactly (two-sum)
    const double hi = s0 + a, hb = hi - s0, hl = (s0 - (hi - hb)) + (a - hb);
    const double lo = s0 - a, lb = lo - s0, ll = (s0 - (lo - lb)) + (-a - lb);
    auto angle = [&](double b) {
        PrecAngle A;
        const double dt = (hi - b) + hl;  // (s0 + a) - b
        const double db = (b - lo) - ll;  // b - (s0 - a)
        A.inside = dt > 0.0 && db > 0.0;
        A.top = dt <= db;
        A.q = A.inside ? fmin(1.0, sqrt((A.top ? dt : db) / (2.0 * a))) : 0.0;
        A.p = sqrt((1.0 - A.q) * (1.0 + A.q));
        A.x = A.inside ? 2.0 * asin(A.q) : 0.0;
        return A;
    };
    // t(B) - t(A), and h = sin of its half from the half-angle values
    auto diff = [&](const PrecAngle &A, const PrecAngle &B, double &h) {
        const double sa = A.top ? A.q : A.p, ca = A.top ? A.p : A.q;  // sin, cos of t(A) / 2
        const double sb = B.top ? B.q : B.p, cb = B.top ? B.p : B.q;
        h = sb * ca - cb * sa;
        if (A.top && B.top) return B.x - A.x;
        if (!A.top && !B.top) return A.x - B.x;
        if (A.top) return (PI - B.x) - A.x;
        return B.x - (PI - A.x);
    };
    const PrecAngle Tw = angle(w), T0 = angle(0.0), Tm = angle(-w);
    double tot = 0.0, h, se, ce, s1, c1;
    double d = diff(Tw, T0, h);  // [0, w]: (w - s) / w
    if (d > 0.0) {
        if (Tw.inside) {
            prec_sc(Tw, se, ce);
            tot += (a / w) * (se * 2.0 * h * h + ce * d_minus_sin(d, h));
        } else {
            prec_sc(T0, s1, c1);
            prec_sc(Tw, se, ce);
            tot += ((w - s0) / w) * d - (a / w) * (s1 - se);
        }
    }
    d = diff(T0, Tm, h);  // [-w, 0]: (w + s) / w
    if (d > 0.0) {
        if (Tm.inside) {
            prec_sc(Tm, se, ce);
            tot += (a / w) * (se * 2.0 * h * h - ce * d_minus_sin(d, h));
        } else {
            prec_sc(Tm, se, ce);
            prec_sc(T0, s1, c1);
            tot += ((w + s0) / w) * d + (a / w) * (se - s1);
        }
    }
    return tot / PI;
}

template <typename T, bool GRAD, int SHAPE, class C>
__device__ __forceinline__ T precession_average_impl(const C &c, T s0h, T s0l, T a, T *ds0, T *da) {
    const T PI_T = (T)SHAPE_PI;
    const T s0 = s0h + s0l;
    const ShapeK<T> K = shape_k(c, s0);
    T dfd;
    if (!(a > (T)0)) {
        const T v = shape_vd<SHAPE, GRAD>(K, s0, dfd);
        if (GRAD) { *ds0 = dfd; *da = (T)0; }
        return v;
    }
    if constexpr (SHAPE == DS_SHAPE_LINEAR && !GRAD && std::is_same<T, double>::value) {
        if (K.w > 0.0) return linear_precession_closed(s0, a, K.w);
    }
    const T h = (T)c.int_step;
    const T w = K.w;
    const T lo = s0 - a, hi = s0 + a;
    const bool clip = SHAPE == DS_SHAPE_LINEAR && w > (T)0;
    T kf = (h > (T)0 && h < (T)INFINITY) ? ceil(lo / h) : (T)INFINITY;
    T th_prev = PI_T, s_prev = lo, sum = (T)0, g0 = (T)0, g1 = (T)0;
    for (;;) {
        const T sk = kf * h;
        const bool last = !(sk < hi);
        const T s_next = last ? hi : sk;
        const T th = last ? (T)0 : acos(fmin(fmax((sk - s0) / a, (T)-1), (T)1));
        if (th_prev > th && !(clip && (s_next <= -w || s_prev >= w))) {
            const T mid = (T)0.5 * (th + th_prev), half = (T)0.5 * (th_prev - th);
            T sm, cm;
            sincos_t(mid, &sm, &cm);
            T acc = (T)0, a0 = (T)0, a1 = (T)0;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                T sd, cd;
                sincos_t(half * gl8_x<T>(i), &sd, &cd);
                const T c1 = cm * cd - sm * sd, c2 = cm * cd + sm * sd;  // cos(mid + d), cos(mid - d)
                T d1, d2;
                const T f1 = shape_vd<SHAPE, GRAD>(K, fma(a, c1, s0h) + s0l, d1);
                const T f2 = shape_vd<SHAPE, GRAD>(K, fma(a, c2, s0h) + s0l, d2);
                acc = fma(gl8_w<T>(i), f1 + f2, acc);
                if (GRAD) {
                    a0 = fma(gl8_w<T>(i), d1 + d2, a0);
                    a1 = fma(gl8_w<T>(i), d1 * c1 + d2 * c2, a1);
                }
            }
            sum = fma(half, acc, sum);
            if (GRAD) {
                g0 = fma(half, a0, g0);
                g1 = fma(half, a1, g1);
            }
        }
        if (last) break;
        th_prev = th;
        s_prev = s_next;
        kf += (T)1;
    }
    if (GRAD) {
        *ds0 = g0 / PI_T;
        *da = g1 / PI_T;
    }
    return sum / PI_T;
}

// s0 = s0h + s0l (a pair in FP32, s0l = 0 in FP64).  Returns shf; with GRAD
// also *ds0 and *da.  Inlined form (for kernels with few live registers at
// the call) and an out-of-line form (precession_average) for the forward
// kernel, whose variants without the average must not pay its registers.
template <typename T, bool GRAD, class C>
__device__ __forceinline__ T precession_average_inline(const C &c, T s0h, T s0l, T a, T *ds0, T *da) {
    switch (c.shape) {
        case DS_SHAPE_LINEAR: return precession_average_impl<T, GRAD, DS_SHAPE_LINEAR>(c, s0h, s0l, a, ds0, da);
        case DS_SHAPE_SINC: return precession_average_impl<T, GRAD, DS_SHAPE_SINC>(c, s0h, s0l, a, ds0, da);
        case DS_SHAPE_SIN2C: return precession_average_impl<T, GRAD, DS_SHAPE_SIN2C>(c, s0h, s0l, a, ds0, da);
        case DS_SHAPE_ATANC: return precession_average_impl<T, GRAD, DS_SHAPE_ATANC>(c, s0h, s0l, a, ds0, da);
        case DS_SHAPE_LORENTZIAN: return precession_average_impl<T, GRAD, DS_SHAPE_LORENTZIAN>(c, s0h, s0l, a, ds0, da);
        default:
            if (GRAD) { *ds0 = (T)0; *da = (T)0; }
            return (T)1;
    }
}

template <typename T, bool GRAD, class C>
__device__ __noinline__ T precession_average(const C &c, T s0h, T s0l, T a, T *ds0, T *da) {
    return precession_average_inline<T, GRAD>(c, s0h, s0l, a, ds0, da);
}

// lorentzian_precession (:183-219) and its partial derivatives, FP64.
template <class C>
__device__ inline double lorentzian_precession_grad(const C &c, double s, double r, double &dsf_ds, double &dsf_dr) {
    const double sig = SHAPE_PI / c.width;
    const double u = sig * sig * (r * r * c.phi * c.phi - s * s) + 1;
    const double z = sqrt(u * u + 4 * sig * sig * s * s);
    const double Q = 2 * (u + z) / (z * z);
    const double f = (sig / SHAPE_PI) * sqrt(Q);
    // dQ = 2 [(du + dz) / z^2 - 2 (u + z) dz / z^3],  dz = (u du + 4 sig^2 s ds) / z
    auto dQ = [&](double du, double dz) { return 2 * ((du + dz) / (z * z) - 2 * (u + z) * dz / (z * z * z)); };
    const double k = f > 0 ? (sig / SHAPE_PI) * 0.5 / sqrt(Q) : 0.0;
    {
        const double du = -2 * sig * sig * s;
        const double dz = (u * du + 4 * sig * sig * s) / z;
        dsf_ds = k * dQ(du, dz);
    }
    {
        const double du = 2 * sig * sig * r * c.phi * c.phi;
        const double dz = u * du / z;
        dsf_dr = k * dQ(du, dz);
    }
    return f;
}

}  // namespace ds
