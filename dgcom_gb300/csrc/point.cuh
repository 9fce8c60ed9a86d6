// Point functions of the stage: the pieces each kernel applies per node,
// per face node or per subcell, shared by the forward kernels
// (kernels.cuh), their reverse (adjoint_kernels.cuh, adjoint_point.cuh)
// and, compiled for the host without DGSWE_FAST, by the unit test of the
// reverse functions. Included inside nothing: it opens dgswe::DGSWE_NS
// itself, DGSWE_NS and DGSWE_FAST being set by the translation unit.
#pragma once

#include <math.h>
#include <stdint.h>

#include "device.hpp"
#include "fp64_bits.hpp"

#if defined(__CUDACC__)
#define DG_PT __host__ __device__ __forceinline__
#else
#define DG_PT inline
#endif

// The FAST arithmetic in device code; a host compilation (the unit test)
// takes the IEEE operations
#if DGSWE_FAST && defined(__CUDA_ARCH__)
#define DGSWE_FAST_PATH 1
#else
#define DGSWE_FAST_PATH 0
#endif

namespace dgswe {
namespace DGSWE_NS {

constexpr int kWetDry = 0, kEntropyStable = 1, kEntropyConservative = 2;
constexpr int kBcWall = 0, kBcNodeTides = 2, kBcParent = 3;
constexpr int kIncomingWave = 1;

// ---------------------------------------------------------------------------
// arithmetic
//
// Every compare, minimum and maximum of doubles on the per-node paths goes
// through fp:: (fp64_bits.hpp): the same result on the integer pipes, which
// leaves the FP64 pipe, the stage's bound, to arithmetic.

using fp::lmax;
using fp::lmin;

// Square roots and reciprocals. DGSWE_FAST: faithful (within an ulp of the
// correctly rounded value) from a single-precision seed refined in FP64,
// ≈ 5 FP64-pipe operations against ≈ 8 for sqrt and ≈ 5 for 1/y measured
// on GB300; the float views of the seed are built on the integer pipes,
// since F2F conversions run on the FP64 pipe. Arguments outside the seed's
// range (zero, subnormal, negative, huge, non-finite) take the IEEE
// operation. Otherwise, and always without DGSWE_FAST, the IEEE operation.
#if DGSWE_FAST_PATH
// The float at or below a positive double in [2^-126, 2^128): the exponent
// rebiased, the mantissa truncated
__device__ __forceinline__ float f32_seed(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    return __uint_as_float((unsigned int)(b >> 29) - (896u << 23));
}
// The double of a positive normal float
__device__ __forceinline__ double f64_of(float f) {
    return __longlong_as_double(
        (long long)(((unsigned long long)__float_as_uint(f) << 29) + (896ull << 52)));
}
#endif

DG_PT double vsqrt(double x) {
#if DGSWE_FAST_PATH
    const int64_t b = fp::bits(x);
    if (b < 0x3810000000000000ll || b >= 0x47E0000000000000ll) return sqrt(x);  // 2^-126, 2^127
    const float r0 = rsqrtf(f32_seed(x));
    const double h0 = f64_of(0.5f * r0);  // 1/(2√x), single precision
    double c = x * f64_of(r0);
    c = fma(h0, fma(-c, c, x), c);     // relative error ≈ 2^-42
    return fma(h0, fma(-c, c, x), c);  // ≈ 2^-63 before the last rounding
#else
    return sqrt(x);
#endif
}

DG_PT double vrcp(double y) {
#if DGSWE_FAST_PATH
    const int64_t b = fp::bits(y);
    if (b < 0x3820000000000000ll || b >= 0x47C0000000000000ll) return 1.0 / y;  // 2^-125, 2^125
    double r = f64_of(__frcp_rn(f32_seed(y)));
    double e = fma(-y, r, 1.0);
    r = fma(r, e, r);  // Newton: relative error ≈ 2^-44
    e = fma(-y, r, 1.0);
    return fma(r, e, r);
#else
    return 1.0 / y;
#endif
}

DG_PT double vdiv(double x, double y) {
#if DGSWE_FAST_PATH
    return x * vrcp(y);
#else
    return x / y;
#endif
}

struct Q {
    double h, hu, hv, u, v, b;
};
struct Sd {
    double h, u, v, b;
};
struct F3 {
    double h, hu, hv;
};

DG_PT Sd side(const Q& q) { return {q.h, q.u, q.v, q.b}; }

// node velocity (src/flux/swe_2d_entropy.rs:106-116)
DG_PT void node_velocity(double h, double hu, double hv, double h_min,
                                              double& u, double& v) {
    const bool wet = fp::gt(h, h_min);
    const double inv_h = vrcp(h);
    u = wet ? hu * inv_h : 0.0;
    v = wet ? hv * inv_h : 0.0;
}

// Two-point flux F#(q_l, q_r)·m (src/flux/swe_2d_entropy.rs:140-160)
DG_PT F3 wflux(const Q& l, const Q& r, double m0, double m1, double g) {
    const double mass = 0.5 * ((l.hu + r.hu) * m0 + (l.hv + r.hv) * m1);
    const double pressure = (0.5 * g) * (l.h * r.h);
    const double u_avg = 0.5 * (l.u + r.u), v_avg = 0.5 * (l.v + r.v);
    return {mass, mass * u_avg + pressure * m0, mass * v_avg + pressure * m1};
}

// HLL in face-aligned components with Einfeldt speeds
// (src/flux/swe_2d.rs:277-375); l/r: depth, normal and tangential momentum,
// and the velocities (zero on a dry side)
DG_PT F3 hll_aligned(double h_l, double hun_l, double hut_l, double un_l,
                                          double ut_l, double h_r, double hun_r, double hut_r,
                                          double un_r, double ut_r, double g, double sqrt_g,
                                          double half_g, double h_min) {
    const bool dry = fp::le(h_l, h_min) && fp::le(h_r, h_min);
    const double sh_l = vsqrt(fp::max0(h_l)), sh_r = vsqrt(fp::max0(h_r));
    const double c_l = sqrt_g * sh_l, c_r = sqrt_g * sh_r;
    const double sh_sum = sh_l + sh_r;
    const bool roe = fp::gt(sh_sum, 1e-10);
    const double h_roe = 0.5 * (h_l + h_r);
    const double un_roe = roe ? vdiv(sh_l * un_l + sh_r * un_r, sh_sum) : 0.0;
    const double c_roe = roe ? vsqrt(g * h_roe) : 0.0;
    const double s_l = fp::gt(h_l, h_min) ? lmin(un_l - c_l, un_roe - c_roe) : un_r - 2.0 * c_r;
    const double s_r = fp::gt(h_r, h_min) ? lmax(un_r + c_r, un_roe + c_roe) : un_l + 2.0 * c_l;
    const double fl_h = h_l * un_l, fl_hu = h_l * un_l * un_l + half_g * h_l * h_l,
                 fl_hv = h_l * un_l * ut_l;
    const double fr_h = h_r * un_r, fr_hu = h_r * un_r * un_r + half_g * h_r * h_r,
                 fr_hv = h_r * un_r * ut_r;
    const double inv_ds = vrcp(s_r - s_l);
    const double s_lr = s_l * s_r;
    const double st_h = inv_ds * (s_r * fl_h - s_l * fr_h + s_lr * (h_r - h_l));
    const double st_hu = inv_ds * (s_r * fl_hu - s_l * fr_hu + s_lr * (hun_r - hun_l));
    const double st_hv = inv_ds * (s_r * fl_hv - s_l * fr_hv + s_lr * (hut_r - hut_l));
    const bool from_l = fp::ge0(s_l), from_r = fp::le0(s_r);
    F3 f;
    f.h = dry ? 0.0 : (from_l ? fl_h : (from_r ? fr_h : st_h));
    f.hu = dry ? 0.0 : (from_l ? fl_hu : (from_r ? fr_hu : st_hu));
    f.hv = dry ? 0.0 : (from_l ? fl_hv : (from_r ? fr_hv : st_hv));
    return f;
}

// wall_ram_pressure (src/solver/rhs/swe_2d_split_form.rs:147-156)
DG_PT double wall_ram(double h, double un, double sill, double g) {
    un = fp::max0(un);
    const double head = un * un * (0.5 / g);
    const double ram = (1.0 - head / sill) * h * un * (2.0 * un + sqrt(g * h));
    return fp::gt(sill, head) ? ram : 0.0;
}

// hydrostatic_hll (src/solver/rhs/swe_2d_split_form.rs:336-402) along m with
// |m| = norm and m/|m| = (nx, ny): the flux seen from side a and from side b
DG_PT void hydro_hll(const Sd& qa, const Sd& qb, double m0, double m1,
                                          double norm, double nx, double ny, double g,
                                          double sqrt_g, double half_g, double h_min, F3& fa,
                                          F3& fb) {
    const double b_face = lmax(qa.b, qb.b);
    const double hs_a = fp::max0(qa.h + qa.b - b_face);
    const double hs_b = fp::max0(qb.h + qb.b - b_face);
    const bool wet_a = fp::gt(qa.h, h_min), wet_b = fp::gt(qb.h, h_min);
    const double ua = wet_a ? qa.u : 0.0, va = wet_a ? qa.v : 0.0;
    const double ub = wet_b ? qb.u : 0.0, vb = wet_b ? qb.v : 0.0;
    const double un_a = ua * nx + va * ny, ut_a = -ua * ny + va * nx;
    const double un_b = ub * nx + vb * ny, ut_b = -ub * ny + vb * nx;
    const bool sw_a = fp::gt(hs_a, h_min), sw_b = fp::gt(hs_b, h_min);
    const F3 r = hll_aligned(hs_a, hs_a * un_a, hs_a * ut_a, sw_a ? un_a : 0.0, sw_a ? ut_a : 0.0,
                             hs_b, hs_b * un_b, hs_b * ut_b, sw_b ? un_b : 0.0, sw_b ? ut_b : 0.0,
                             g, sqrt_g, half_g, h_min);
    // rotate back (src/flux/swe_2d.rs:38-44), times |m|
    const double f_h = norm * r.h;
    const double f_hu = norm * (r.hu * nx - r.hv * ny);
    const double f_hv = norm * (r.hu * ny + r.hv * nx);
    const bool hll_dry = fp::le(hs_a, h_min) && fp::le(hs_b, h_min);
    const double hsa = hll_dry ? 0.0 : hs_a, hsb = hll_dry ? 0.0 : hs_b;
    double wall_a = 0.0, wall_b = 0.0;
    if (hll_dry) {
        if (wet_a) wall_a = wall_ram(qa.h, qa.u * nx + qa.v * ny, b_face - (qa.h + qa.b), g);
        if (wet_b)
            wall_b = wall_ram(qb.h, -1.0 * (qb.u * nx + qb.v * ny), b_face - (qb.h + qb.b), g);
    }
    const double dp_a = half_g * (qa.h * qa.h - hsa * hsa) + wall_a;
    const double dp_b = half_g * (qb.h * qb.h - hsb * hsb) + wall_b;
    fa = {f_h, f_hu + dp_a * m0, f_hv + dp_a * m1};
    fb = {f_h, f_hu + dp_b * m0, f_hv + dp_b * m1};
}

// HarmonicTide::elevation (src/boundary/harmonic_tide.rs:124-136)
DG_PT double tide_elevation(const Condition& c, double t) {
    double tide = 0.0;
    for (int i = 0; i < c.n_constituents; ++i) {
        const Constituent& k = c.c[i];
        const double f = k.f + k.f_rate * t;
        const double u_deg = k.u_deg + k.u_rate_deg * t;
        const double offset = (k.v0_deg + u_deg) * (M_PI / 180.0);
        tide += f * k.amplitude * cos(k.omega * t + k.phase + offset);
    }
    double ramp = 1.0;
    if (fp::gt0(c.ramp)) {
        double tau = t / c.ramp;
        tau = fp::lt0(tau) ? 0.0 : (fp::gt(tau, 1.0) ? 1.0 : tau);
        ramp = tau * tau * (3.0 - 2.0 * tau);
    }
    return c.mean + ramp * tide;
}


// ---------------------------------------------------------------------------
// damping and the wet/dry correction

// The reference's cube root (src/source/swe_2d/friction.rs:39-70)
DG_PT double ref_cbrt(double x) {
    if (!(x >= 2.2250738585072014e-308 && x <= 1.7976931348623157e308)) return cbrt(x);
    const unsigned long long bits = (unsigned long long)fp::bits(x);
    double y = fp::from_bits((int64_t)(bits / 3ull + 0x2A9F7893782DA1CEull));
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const double y3 = y * y * y;
        y += y * ((x - y3) / (2.0 * y3 + x));
    }
    return y;
}

// Manning's rate g n² |u| / h^{4/3} at a floored depth h
DG_PT double manning_rate(double g_n2, double h, double speed) {
#if DGSWE_FAST_PATH
    // h^{-1/3} from a single-precision seed (relative error δ ≈ 2^-22) and
    // one step of third order, z ← z(1 + e/3 + 2e²/9) with e = 1 − h z³
    // (error ≈ 5δ³ ≈ 2^-61); then the rate is g n² |u| z⁴, no division
    const int64_t b = fp::bits(h);
    double z = (b >= 0x3820000000000000ll && b < 0x47C0000000000000ll)  // 2^-125, 2^125
                   ? f64_of(rcbrtf(f32_seed(h)))
                   : 1.0 / cbrt(h);
    const double e = fma(-h, z * z * z, 1.0);
    z = fma(z * e, fma(e, 2.0 / 9.0, 1.0 / 3.0), z);
    const double z2 = z * z;
    return g_n2 * speed * (z2 * z2);
#else
    return g_n2 * speed / (ref_cbrt(h) * h);
#endif
}

struct DampIn {
    double h, hu, hv, u, v;  // the RHS input (u, v: node velocity)
};

// damp_node (src/solver/algorithms/wetting_drying.rs:324-357)
DG_PT void damp(const Physics& P, double g_n2, double h, double& hu,
                                     double& hv, const DampIn& from, double dt) {
    if (fp::le0(h)) {
        hu = 0.0;
        hv = 0.0;
        return;
    }
    double rate = 0.0;
    if (P.friction) {
        double u, v;
        if (P.has_wet_dry) {
            // desingularized_velocity (wetting_drying.rs:115-130): the node
            // velocity where h ≥ h_dry (> h_min)
            if (fp::le0(from.h)) {
                u = v = 0.0;
            } else if (fp::ge(from.h, P.h_dry)) {
                if (fp::gt(P.h_dry, P.h_min)) {
                    u = from.u;
                    v = from.v;
                } else {
                    const double inv = 1.0 / from.h;
                    u = from.hu * inv;
                    v = from.hv * inv;
                }
            } else {
                const double r = from.h / P.h_dry;
                const double factor =
                    1.4142135623730951 * r / (P.h_dry * sqrt(1.0 + r * r * r * r));
                u = factor * from.hu;
                v = factor * from.hv;
            }
        } else {
            // SWEState2D::velocity (src/solver/state/swe_2d.rs:54-61)
            const double h_reg = lmax(from.h, P.h_min);
            const double inv_d = 1.0 / (from.h * from.h + h_reg * h_reg);
            const double factor = 2.0 * from.h * inv_d;
            u = from.hu * factor;
            v = from.hv * factor;
        }
        const double speed = vsqrt(u * u + v * v);
        if (fp::gt0(speed)) rate += manning_rate(g_n2, lmax(h, P.manning_h_min), speed);
    }
    if (P.has_wet_dry && fp::lt(h, P.h_dry)) {
        // thin_layer_rate (wetting_drying.rs:135-146); h > 0 here
        const double excess = P.h_dry / h - 1.0;
        rate += excess * excess / P.relaxation_time;
    }
    const double factor = vrcp(1.0 + dt * rate);
    hu *= factor;
    hv *= factor;
}

// correct_node (src/solver/algorithms/wetting_drying.rs:148-165)
DG_PT void correct_node(const Physics& P, double h, double& hu, double& hv) {
    if (fp::le0(h)) {
        hu = 0.0;
        hv = 0.0;
        return;
    }
    if (fp::lt(h, P.h_dry)) {
        const double r = h / P.h_dry;
        const double factor = 1.4142135623730951 * r / (P.h_dry * sqrt(1.0 + r * r * r * r));
        hu = h * (factor * hu);
        hv = h * (factor * hv);
    }
    // |hu| > h·u_max; the square root only near the cap. First a test on
    // the exponent fields alone (integer pipes): with E the biased exponent,
    // |m| < √2·2^(max(E_hu, E_hv) − 1022) and h·u_max ≥ 2^(E_h + E_u − 2046)
    // for normal h and u_max, so max(E_hu, E_hv) + 1025 ≤ E_h + E_u means
    // |m|² < 0.99·cap² and the exact test below would be false.
    const int e_h = (int)((fp::bits(h) >> 52) & 0x7FF);
    const int e_u = (int)((fp::bits(P.max_velocity) >> 52) & 0x7FF);
    const int e_hu = (int)((fp::bits(hu) >> 52) & 0x7FF), e_hv = (int)((fp::bits(hv) >> 52) & 0x7FF);
    if (e_h >= 1 && e_u >= 1 && (e_hu > e_hv ? e_hu : e_hv) + 1025 <= e_h + e_u) return;
    const double m2 = hu * hu + hv * hv;
    const double cap = P.max_velocity * h;
    if (fp::gt(m2, 0.99 * (cap * cap))) {
        const double momentum = sqrt(m2);
        if (fp::gt(momentum, cap)) {
            const double scale = cap / momentum;
            hu *= scale;
            hv *= scale;
        }
    }
}


// limited_slope with SlopeDistances (src/solver/rhs/swe_2d_split_form.rs:168-203)
DG_PT double limited_slope(double q0, double q1, double q2, double ic,
                                                double im, double ip) {
    const double dm = q1 - q0, dp = q2 - q1;
    const bool extremum = fp::le0(dm * dp);
    const double central = (q2 - q0) * ic;
    const double bound = fp::min_nn(fabs(dm * im), fabs(dp * ip));
    const double sign = fp::lt0(central) ? -1.0 : 1.0;
    return extremum ? 0.0 : sign * fp::min_nn(fabs(central), bound);
}

// reconstruct_subcell (src/solver/rhs/swe_2d_split_form.rs:279-317)
DG_PT void reconstruct(const Sd& m, const Sd& c, const Sd& p, double x0,
                                            double x1, double x2, double xl, double xr,
                                            double h_dry, Sd& left, Sd& right) {
    const double e0 = m.h + m.b, e1 = c.h + c.b, e2 = p.h + p.b;
    double ws = -INFINITY;
    ws = (fp::ge(m.h, h_dry) && fp::gt(e0, ws)) ? e0 : ws;
    ws = (fp::ge(c.h, h_dry) && fp::gt(e1, ws)) ? e1 : ws;
    ws = (fp::ge(p.h, h_dry) && fp::gt(e2, ws)) ? e2 : ws;
    const bool flooding = (fp::lt(m.h, h_dry) && fp::lt(e0, ws)) ||
                          (fp::lt(c.h, h_dry) && fp::lt(e1, ws)) ||
                          (fp::lt(p.h, h_dry) && fp::lt(e2, ws));
    const double fm = x1 - xl, fpd = xr - x1;
    const double ic = vrcp(x2 - x0);
    const double im = vrcp(fp::gt0(fm) ? fm : 0.5 * (x1 - x0));
    const double ip = vrcp(fp::gt0(fpd) ? fpd : 0.5 * (x2 - x1));
    const double s_h = limited_slope(m.h, c.h, p.h, ic, im, ip);
    const double s_eta = flooding ? 0.0 : limited_slope(e0, e1, e2, ic, im, ip);
    const double s_u = limited_slope(m.u, c.u, p.u, ic, im, ip);
    const double s_v = limited_slope(m.v, c.v, p.v, ic, im, ip);
    double d = xl - x1;
    double hh = fp::max0(c.h + s_h * d);
    left = {hh, c.u + s_u * d, c.v + s_v * d, e1 + s_eta * d - hh};
    d = xr - x1;
    hh = fp::max0(c.h + s_h * d);
    right = {hh, c.u + s_u * d, c.v + s_v * d, e1 + s_eta * d - hh};
}


// node_reference_rate (swe_2d.rs:1346-1357) with the mean's ¼ folded into
// the metric table m (¼∇r, ¼∇s, ¼|∇r|, ¼|∇s|): a power-of-two scaling, so
// lr + ls here has exactly the bits of ¼(lr + ls) from unscaled metrics
DG_PT double node_rate(double h, double u, double v, const double* m,
                                            double g) {
    const double c = vsqrt(g * fp::max0(h));
    const double lr = fabs(u * m[0] + v * m[1]) + c * m[4];
    const double ls = fabs(u * m[2] + v * m[3]) + c * m[5];
    return lr + ls;
}

using fp::f32_trunc;

// node_rate in single precision from truncated inputs (the metric m already
// truncated: f32_trunc of the double table), and its error scale
// B = (|u| + |v| + c)·(m4 + m5): each term of the rate (|u·m0 + v·m1|,
// c·m4, …) is within 2^-20 of its magnitude (truncation < 2^-23 per input,
// rounding 2^-24 per operation), and the magnitudes sum to at most B since
// |m0|, |m1| ≤ m4 and |m2|, |m3| ≤ m5; so |node_rate − r| ≤ 2^-20·B, less
// terms of the size of 2^-126 from values below the float range
DG_PT void node_rate_f32(double h, double u, double v, const float* m, float g32, float& r,
                         float& bound) {
    const float h32 = f32_trunc(h), u32 = f32_trunc(u), v32 = f32_trunc(v);
    const float m0 = m[0], m1 = m[1], m2 = m[2], m3 = m[3], m4 = m[4], m5 = m[5];
    const float c = sqrtf(g32 * h32);
    r = (fabsf(u32 * m0 + v32 * m1) + c * m4) + (fabsf(u32 * m2 + v32 * m3) + c * m5);
    bound = (fabsf(u32) + fabsf(v32) + c) * (m4 + m5);
}

// The interior velocity of BCContext2D (velocity_simple): (hu, hv)/h where
// h > h_min, else 0
DG_PT void interior_velocity(const Q& qi, double h_min, double& u, double& v) {
    u = 0.0;
    v = 0.0;
    if (fp::gt(qi.h, h_min)) {
        const double inv = 1.0 / qi.h;
        u = qi.hu * inv;
        v = qi.hv * inv;
    }
}

// Reflective2D mirror ghost (src/boundary/boundary_2d.rs:271-283) of the
// interior node qi with velocity (u, v)
DG_PT Q wall_ghost(const Q& qi, double u, double v, double nx, double ny, double wall_h_min,
                   double h_min) {
    double ghu = 0.0, ghv = 0.0;
    if (!fp::le(qi.h, wall_h_min)) {
        const double un = u * nx + v * ny;
        ghu = qi.h * (u - 2.0 * un * nx);
        ghv = qi.h * (v - 2.0 * un * ny);
    }
    Q qe;
    qe.h = qi.h;
    qe.hu = ghu;
    qe.hv = ghv;
    qe.b = qi.b;
    node_velocity(qe.h, ghu, ghv, h_min, qe.u, qe.v);
    return qe;
}

// characteristic_state (src/boundary/characteristic.rs:481-520): the
// boundary state from the interior node qi and the external depth and
// normal and tangential velocity, with its node velocity
DG_PT Q characteristic_state_ext(const Q& qi, double h_e, double un_e, double ut_e, double nx,
                                 double ny, double g, double h_min) {
    const double h_i = fmax(qi.h, 0.0);
    double un_i = 0.0, ut_i = 0.0;
    if (h_i > h_min) {
        const double ui = qi.hu / h_i, vi = qi.hv / h_i;
        un_i = ui * nx + vi * ny;
        ut_i = -ui * ny + vi * nx;
    }
    const double c_i = sqrt(g * h_i), c_e = sqrt(g * h_e);
    const double w_out = un_i + 2.0 * c_i, w_in = un_e - 2.0 * c_e;
    const bool wi = h_i > h_min, we = h_e > h_min;
    double h_b, un_b;
    if (!wi && !we) {
        h_b = 0.0;
        un_b = 0.0;
    } else if (wi && un_i >= c_i) {
        h_b = h_i;
        un_b = un_i;
    } else if (we && un_e <= -c_e) {
        h_b = h_e;
        un_b = un_e;
    } else if (wi && !we) {
        const double cc = fmax(w_out / 3.0, 0.0);
        h_b = cc * cc / g;
        un_b = cc;
    } else if (!wi && we) {
        const double cc = fmax(-w_in / 3.0, 0.0);
        h_b = cc * cc / g;
        un_b = -cc;
    } else {
        const double cc = fmax(0.25 * (w_out - w_in), 0.0);
        h_b = cc * cc / g;
        un_b = 0.5 * (w_out + w_in);
    }
    const double ut_b = un_b > 0.0 ? ut_i : ut_e;
    const double ub = un_b * nx - ut_b * ny, vb = un_b * ny + ut_b * nx;
    Q qb;
    qb.h = h_b;
    qb.hu = h_b * ub;
    qb.hv = h_b * vb;
    qb.b = qi.b;
    node_velocity(qb.h, qb.hu, qb.hv, h_min, qb.u, qb.v);
    return qb;
}

// CharacteristicOBC's boundary state (src/boundary/characteristic.rs:411-437)
// for elevation-only external data: the interior node qi (velocity u, v)
// and the external elevation eta
DG_PT Q characteristic_state(const Q& qi, double u, double v, double eta, double nx, double ny,
                             int elevation_only, double g, double h_min) {
    const double bathy = qi.b;
    const double h_e = fmax(eta - bathy, 0.0);
    double un_e = 0.0;
    if (elevation_only == kIncomingWave) un_e = 2.0 * (sqrt(g * fmax(-bathy, 0.0)) - sqrt(g * h_e));
    const double ut_e = -u * ny + v * nx;
    return characteristic_state_ext(qi, h_e, un_e, ut_e, nx, ny, g, h_min);
}

// tidal_ramp (src/boundary/harmonic_tide.rs:24-32): τ²(3 − 2τ), τ = t/duration in [0, 1]
DG_PT double tidal_ramp(double t, double duration) {
    if (!fp::gt0(duration)) return 1.0;
    double tau = t / duration;
    tau = fp::lt0(tau) ? 0.0 : (fp::gt(tau, 1.0) ? 1.0 : tau);
    return tau * tau * (3.0 - 2.0 * tau);
}

// OceanModelState's external state at a slot over the child bed `bed`
// (src/boundary/ocean_nesting.rs:565-600, 833-880): the snapshots'
// Lagrange weights at t (TimeStencil::new, src/io/field_series.rs:41-81;
// linear, or cubic through up to four), Σ w·values (parent_term), the ramp,
// the datum shift and the transport scaling (parent_state). `series` is the
// slot's [n_times][3] ζ, u, v. t outside the times takes the nearest end
// (the host refuses such runs beforehand).
DG_PT void parent_state_at(const double* times, int n, int cubic, const float* series, double t,
                           double ramp_duration, double reference_level, int velocity,
                           double max_ratio, double parent_depth, double bed, double& eta,
                           double& u, double& v, bool& has_uv) {
    int idx[4] = {0, 0, 0, 0};
    double w[4] = {1.0, 0.0, 0.0, 0.0};
    int len = 1;
    if (n > 1) {
        if (!fp::ge(t, times[0])) {
            idx[0] = 0;
        } else if (!fp::le(t, times[n - 1])) {
            idx[0] = n - 1;
        } else {
            // the first index whose time is ≥ t, within [1, n − 1]
            int lo = 0, hi = n;
            while (lo < hi) {
                const int mid = (lo + hi) / 2;
                if (fp::lt(times[mid], t)) lo = mid + 1;
                else hi = mid;
            }
            const int i1 = lo < 1 ? 1 : (lo > n - 1 ? n - 1 : lo);
            const int i0 = i1 - 1;
            if (t == times[i0]) {
                idx[0] = i0;
            } else if (t == times[i1]) {
                idx[0] = i1;
            } else {
                const int a0 = cubic ? (i0 > 0 ? i0 - 1 : 0) : i0;
                const int a1 = cubic ? (i1 + 1 < n - 1 ? i1 + 1 : n - 1) : i1;
                len = a1 - a0 + 1;
                for (int s = 0; s < len; ++s) {
                    const int a = a0 + s;
                    double p = 1.0;
                    bool first = true;
                    for (int b = a0; b <= a1; ++b) {
                        if (b == a) continue;
                        const double x = (t - times[b]) / (times[a] - times[b]);
                        p = first ? x : p * x;
                        first = false;
                    }
                    idx[s] = a;
                    w[s] = p;
                }
            }
        }
    }
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int k = 0; k < len; ++k) {
        const float* q = series + 3 * idx[k];
        s0 += w[k] * (double)q[0];
        s1 += w[k] * (double)q[1];
        s2 += w[k] * (double)q[2];
    }
    const double ramp = tidal_ramp(t, ramp_duration);
    const double zeta = ramp * s0;
    u = ramp * s1;
    v = ramp * s2;
    eta = zeta + ramp * reference_level;
    has_uv = velocity != 0;
    if (has_uv && max_ratio > 0.0 && fp::finite(parent_depth)) {
        const double d_parent = zeta + parent_depth, d_child = eta - bed;
        if (fp::gt0(d_parent) && fp::gt0(d_child)) {
            double ratio = d_parent / d_child;
            const double lo = 1.0 / max_ratio;
            ratio = fp::lt(ratio, lo) ? lo : (fp::gt(ratio, max_ratio) ? max_ratio : ratio);
            u *= ratio;
            v *= ratio;
        }
    }
}

// BoundaryTides' external state at a slot (tide_term, tide_level,
// tide_state: src/boundary/tidal_atlas.rs:1078-1131) over the child bed
// `bed`: η, and (u, v) if the tides carry velocity (has_uv)
DG_PT void node_tide_state(const double* omega, const double* f_rate, const double* coef, int n,
                           double t, double ramp_duration, double mean, int velocity,
                           double max_ratio, double source_depth, double bed, double& eta,
                           double& u, double& v, bool& has_uv) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int j = 0; j < n; ++j) {
        const double f = 1.0 + f_rate[j] * t;
        const double x = omega[j] * t;
        const double cs = cos(x), sn = sin(x);
        const double* c = coef + 6 * j;
        s0 += f * (c[0] * cs + c[1] * sn);
        s1 += f * (c[2] * cs + c[3] * sn);
        s2 += f * (c[4] * cs + c[5] * sn);
    }
    const double ramp = tidal_ramp(t, ramp_duration);
    eta = mean + ramp * s0;
    u = ramp * s1;
    v = ramp * s2;
    has_uv = velocity != 0;
    if (has_uv && max_ratio > 0.0) {
        const double d_source = source_depth + eta, d_child = eta - bed;
        if (fp::gt0(source_depth) && fp::gt0(d_source) && fp::gt0(d_child)) {
            double ratio = d_source / d_child;
            const double lo = 1.0 / max_ratio;
            ratio = fp::lt(ratio, lo) ? lo : (fp::gt(ratio, max_ratio) ? max_ratio : ratio);
            u *= ratio;
            v *= ratio;
        }
    }
}

// ---------------------------------------------------------------------------
// the weather (GriddedAtmosphere2D, src/source/swe_2d/gridded_atmosphere.rs)

// The linear TimeStencil (src/io/field_series.rs:41-81,
// TimeInterpolation::Linear) of the weather's snapshot times at Unix time
// tu: one snapshot at a snapshot's own time, else the bracketing two with
// their Lagrange weights. A time outside the snapshots takes the nearest
// end (the host refuses runs there, where the reference panics).
DG_PT int weather_weights(const double* times, int n, double tu, int idx[2], double w[2]) {
    idx[0] = 0;
    idx[1] = 0;
    w[0] = 1.0;
    w[1] = 0.0;
    if (n <= 1) return 1;
    if (!fp::ge(tu, times[0])) return 1;
    if (!fp::le(tu, times[n - 1])) {
        idx[0] = n - 1;
        return 1;
    }
    // the first index whose time is ≥ tu, within [1, n − 1]
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) / 2;
        if (fp::lt(times[mid], tu)) lo = mid + 1;
        else hi = mid;
    }
    const int i1 = lo < 1 ? 1 : (lo > n - 1 ? n - 1 : lo);
    const int i0 = i1 - 1;
    if (tu == times[i0]) {
        idx[0] = i0;
        return 1;
    }
    if (tu == times[i1]) {
        idx[0] = i1;
        return 1;
    }
    idx[0] = i0;
    idx[1] = i1;
    w[0] = (tu - times[i1]) / (times[i0] - times[i1]);
    w[1] = (tu - times[i0]) / (times[i1] - times[i0]);
    return 2;
}

// The double of a float, exactly: on the device the normal floats are
// widened on the integer pipes (sign, exponent rebiased, mantissa shifted;
// the conversion instruction runs on the FP64 pipe), the rest converted
DG_PT double widen(float f) {
#if defined(__CUDA_ARCH__)
    const unsigned int b = __float_as_uint(f);
    const unsigned int e = (b >> 23) & 0xFFu;
    if (e == 0u || e == 0xFFu) return (double)f;
    const unsigned long long sign = (unsigned long long)(b & 0x80000000u) << 32;
    return __longlong_as_double((long long)(sign | ((unsigned long long)(e + 896u) << 52) |
                                            ((unsigned long long)(b & 0x7FFFFFu) << 29)));
#else
    return (double)f;
#endif
}

// One field of the weather at flat node g, its snapshots summed in turn
// from zero (add_snapshot); values are [time][5][n_values] f32
DG_PT double weather_field(const float* values, int64_t n_values, int q, int64_t g,
                           const int idx[2], const double w[2], int len) {
    double s = 0.0;
    for (int j = 0; j < len; ++j)
        s += w[j] * widen(values[((int64_t)idx[j] * 5 + q) * n_values + g]);
    return s;
}

// crate::math::hypot (src/math.rs:202-245, musl's): √(x² + y²) from the
// squares split in two parts each (Dekker), so that the sum is exact enough
// for the square root; scaled by 2^±700 away from overflow and underflow
DG_PT double ref_hypot(double x, double y) {
    int64_t ux = fp::bits(x) & INT64_MAX, uy = fp::bits(y) & INT64_MAX;
    if (ux < uy) {
        const int64_t t = ux;
        ux = uy;
        uy = t;
    }
    const int64_t ex = ux >> 52, ey = uy >> 52;
    x = fp::from_bits(ux);
    y = fp::from_bits(uy);
    if (ey == 0x7ff) return y;
    if (ex == 0x7ff || uy == 0) return x;
    if (ex - ey > 64) return x + y;
    double z = 1.0;
    const double up = fp::from_bits(0x6bb0000000000000ll), down = fp::from_bits(0x1430000000000000ll);
    if (ex > 0x3ff + 510) {
        z = up;
        x *= down;
        y *= down;
    } else if (ey < 0x3ff - 450) {
        z = down;
        x *= up;
        y *= up;
    }
    // x² = hx + lx exactly: the reference splits x in two halves (Dekker's
    // product); a fused multiply-add gives the same exact low part in one
    // operation (the scaling above keeps the split's products in range)
    const double hx = x * x, hy = y * y;
    const double lx = fma(x, x, -hx), ly = fma(y, y, -hy);
    return z * vsqrt(ly + lx + hy + hx);
}

// DragCoefficient::compute (src/source/swe_2d/wind.rs:134-158) by its
// device code
DG_PT double drag_coefficient(int kind, double cd, double speed) {
    switch (kind) {
        case 0: return cd;
        case 1:
            return fp::le(speed, 11.0) ? 1.2e-3
                                       : (0.49 + 0.065 * (fp::lt(25.0, speed) ? 25.0 : speed)) * 1e-3;
        case 2: return (0.8 + 0.065 * speed) * 1e-3;
        case 3: return (0.61 + 0.063 * speed) * 1e-3;
        default: return fp::le(speed, 6.0) ? 1.1e-3 : (0.50 + 0.071 * speed) * 1e-3;
    }
}

// atmosphere_source (gridded_atmosphere.rs:161-196): (τ − h∇p)/ρ_water with
// τ = ρ_air C_d(|U|) |U| U from the ramped wind (u, v) and pressure gradient
// (px, py); nothing below h_min
DG_PT void atmosphere_source(double h, double u, double v, double px, double py, int drag,
                             double cd, double rho_air, double rho_water, double h_min,
                             double& su, double& sv) {
    su = 0.0;
    sv = 0.0;
    if (fp::lt(h, h_min)) return;
    const double speed = ref_hypot(u, v);
    const double stress = rho_air * drag_coefficient(drag, cd, speed) * speed;
    su = vdiv(stress * u - h * px, rho_water);
    sv = vdiv(stress * v - h * py, rho_water);
}

// inverse_barometer_level (gridded_atmosphere.rs:198-202): −ramp·p/(ρ g),
// g = 9.81 (the module's constant)
DG_PT double inverse_barometer_level(double p, double ramp, double rho_water) {
    return vdiv(-ramp * p, rho_water * 9.81);
}

}  // namespace DGSWE_NS
}  // namespace dgswe
