// Oracle — test infrastructure only. A CPU restatement of the pointwise
// physics of the reference's 2D split-form shallow-water kernel
// (EmilLindfors/dgcom), operation for operation, in double precision with
// every multiply and add separately rounded (built with -ffp-contract=off),
// correctly rounded sqrt and division, and the reference's selects. Only the
// tests, the smoke check and the bench's CPU-baseline leg use it; the
// product never links it.
//
// The reference writes this physics once, generic over `Lane`
// (src/types/lane.rs:1-150): a branch is a select, `max`/`min` keep the
// other operand on a tie or a NaN. Functions here that the reference writes
// on plain f64 use f64::max/min (NaN-dropping), written fmax_/fmin_.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <utility>

namespace oracle {

// Lane::max / Lane::min (src/types/lane.rs:60-75)
inline double lmax(double a, double b) { return a > b ? a : b; }
inline double lmin(double a, double b) { return a < b ? a : b; }
// f64::max / f64::min: a NaN operand gives the other
inline double fmax_(double a, double b) { return std::fmax(a, b); }
inline double fmin_(double a, double b) { return std::fmin(a, b); }

// SWEState2D (src/solver/state/swe_2d.rs)
struct State {
    double h = 0, hu = 0, hv = 0;
};
inline State operator+(State a, State b) { return {a.h + b.h, a.hu + b.hu, a.hv + b.hv}; }
inline State operator-(State a, State b) { return {a.h - b.h, a.hu - b.hu, a.hv - b.hv}; }
inline State operator-(State a) { return {-a.h, -a.hu, -a.hv}; }
inline State operator*(double s, State a) { return {s * a.h, s * a.hu, s * a.hv}; }

// SWENodeState2D (src/flux/swe_2d_entropy.rs:70-120)
struct Node {
    double h = 0, hu = 0, hv = 0, u = 0, v = 0, b = 0;
};
// SWESide2D (src/solver/rhs/swe_2d_split_form.rs:205-247)
struct Side {
    double h = 0, u = 0, v = 0, b = 0;
    double eta() const { return h + b; }
};
inline Side side_of(const Node& q) { return {q.h, q.u, q.v, q.b}; }

// node_velocity (src/flux/swe_2d_entropy.rs:106-116): one reciprocal of h,
// zero at h ≤ h_min
inline void node_velocity(double h, double hu, double hv, double h_min, double& u, double& v) {
    bool wet = h > h_min;
    double inv_h = 1.0 / h;
    u = wet ? hu * inv_h : 0.0;
    v = wet ? hv * inv_h : 0.0;
}

// SWENodeState2D::new (src/flux/swe_2d_entropy.rs:90-101)
inline Node make_node(State q, double b, double h_min) {
    Node n;
    n.h = q.h;
    n.hu = q.hu;
    n.hv = q.hv;
    node_velocity(q.h, q.hu, q.hv, h_min, n.u, n.v);
    n.b = b;
    return n;
}

// wintermeyer_flux_2d (src/flux/swe_2d_entropy.rs:140-160)
inline State wintermeyer_flux(const Node& l, const Node& r, double m0, double m1, double g) {
    const double half = 0.5;
    double mass = half * ((l.hu + r.hu) * m0 + (l.hv + r.hv) * m1);
    double pressure = (0.5 * g) * (l.h * r.h);
    double u_avg = half * (l.u + r.u);
    double v_avg = half * (l.v + r.v);
    return {mass, mass * u_avg + pressure * m0, mass * v_avg + pressure * m1};
}

// wintermeyer_bed_interface_term_2d (src/flux/swe_2d_entropy.rs:166-177)
inline State bed_interface_term(double h_int, double b_int, double b_ext, double n0, double n1,
                                double g) {
    double force = 0.5 * g * h_int * (b_ext - b_int);
    return {0.0, force * n0, force * n1};
}

// entropy_stable_dissipation_2d (src/flux/swe_2d_entropy.rs:182-205)
inline State entropy_stable_dissipation(const Node& qi, const Node& qe, double nx, double ny,
                                        double g) {
    double speed_int = std::fabs(qi.u * nx + qi.v * ny) + std::sqrt(g * fmax_(qi.h, 0.0));
    double speed_ext = std::fabs(qe.u * nx + qe.v * ny) + std::sqrt(g * fmax_(qe.h, 0.0));
    double scale = -0.5 * fmax_(speed_int, speed_ext);
    double jump_eta = (qe.h + qe.b) - (qi.h + qi.b);
    double h_avg = 0.5 * (qi.h + qe.h);
    double u_avg = 0.5 * (qi.u + qe.u);
    double v_avg = 0.5 * (qi.v + qe.v);
    return {scale * jump_eta, scale * (u_avg * jump_eta + h_avg * (qe.u - qi.u)),
            scale * (v_avg * jump_eta + h_avg * (qe.v - qi.v))};
}

// HllSide (src/flux/swe_2d.rs:229-265)
struct HllSide {
    double h, hun, hut, un, ut;
};

// HllSide::flux with half_g = ½g
inline State hll_side_flux(const HllSide& s, double half_g) {
    return {s.h * s.un, s.h * s.un * s.un + half_g * s.h * s.h, s.h * s.un * s.ut};
}

// einfeldt_speeds_2d (src/flux/swe_2d.rs:337-375)
inline void einfeldt_speeds(double h_l, double h_r, double sqrt_h_l, double sqrt_h_r, double un_l,
                            double un_r, double c_l, double c_r, double g, double h_min,
                            double& s_l, double& s_r) {
    bool roe = (sqrt_h_l + sqrt_h_r) > 1e-10;
    double h_roe = 0.5 * (h_l + h_r);
    double un_roe = roe ? (sqrt_h_l * un_l + sqrt_h_r * un_r) / (sqrt_h_l + sqrt_h_r) : 0.0;
    double c_roe = roe ? std::sqrt(g * h_roe) : 0.0;
    s_l = h_l > h_min ? lmin(un_l - c_l, un_roe - c_roe) : un_r - 2.0 * c_r;
    s_r = h_r > h_min ? lmax(un_r + c_r, un_roe + c_roe) : un_l + 2.0 * c_l;
}

// hll_flux_face_aligned (src/flux/swe_2d.rs:277-335)
inline State hll_flux_face_aligned(const HllSide& l, const HllSide& r, double g, double h_min) {
    double h_l = l.h, h_r = r.h;
    bool dry = (h_l <= h_min) && (h_r <= h_min);
    double sqrt_h_l = std::sqrt(lmax(h_l, 0.0));
    double sqrt_h_r = std::sqrt(lmax(h_r, 0.0));
    double sqrt_g = std::sqrt(g);
    double c_l = sqrt_g * sqrt_h_l, c_r = sqrt_g * sqrt_h_r;
    double s_l, s_r;
    einfeldt_speeds(h_l, h_r, sqrt_h_l, sqrt_h_r, l.un, r.un, c_l, c_r, g, h_min, s_l, s_r);
    double half_g = 0.5 * g;
    State f_l = hll_side_flux(l, half_g), f_r = hll_side_flux(r, half_g);
    double inv_ds = 1.0 / (s_r - s_l);
    double s_lr = s_l * s_r;
    State star{inv_ds * (s_r * f_l.h - s_l * f_r.h + s_lr * (h_r - h_l)),
               inv_ds * (s_r * f_l.hu - s_l * f_r.hu + s_lr * (r.hun - l.hun)),
               inv_ds * (s_r * f_l.hv - s_l * f_r.hv + s_lr * (r.hut - l.hut))};
    bool from_l = s_l >= 0.0, from_r = s_r <= 0.0;
    auto pick = [&](double fl, double fr, double st) {
        return dry ? 0.0 : (from_l ? fl : (from_r ? fr : st));
    };
    return {pick(f_l.h, f_r.h, star.h), pick(f_l.hu, f_r.hu, star.hu),
            pick(f_l.hv, f_r.hv, star.hv)};
}

// rotate_from_normal (src/flux/swe_2d.rs:38-44)
inline State rotate_from_normal(State f, double nx, double ny) {
    return {f.h, f.hu * nx - f.hv * ny, f.hu * ny + f.hv * nx};
}

// wall_ram_pressure (src/solver/rhs/swe_2d_split_form.rs:147-156)
inline double wall_ram_pressure(double h, double un, double sill, double g) {
    un = lmax(un, 0.0);
    double head = un * un * (0.5 / g);
    double ram = (1.0 - head / sill) * h * un * (2.0 * un + std::sqrt(g * h));
    return sill > head ? ram : 0.0;
}

// hydrostatic_hll (src/solver/rhs/swe_2d_split_form.rs:336-402): the flux
// as seen from side a and from side b along m (a unit normal or a
// contravariant vector)
inline void hydrostatic_hll(const Side& qa, const Side& qb, double m0, double m1, double g,
                            double h_min, State& fa, State& fb) {
    double norm = std::sqrt(m0 * m0 + m1 * m1);
    double inv_norm = 1.0 / norm;
    double nx = m0 * inv_norm, ny = m1 * inv_norm;
    double b_face = lmax(qa.b, qb.b);
    auto side = [&](const Side& q) {
        double h_star = lmax(q.h + q.b - b_face, 0.0);
        bool wet = q.h > h_min;
        double u = wet ? q.u : 0.0, v = wet ? q.v : 0.0;
        double un = u * nx + v * ny, ut = -u * ny + v * nx;
        double hun = h_star * un, hut = h_star * ut;
        bool star_wet = h_star > h_min;
        return HllSide{h_star, hun, hut, star_wet ? un : 0.0, star_wet ? ut : 0.0};
    };
    HllSide a = side(qa), b = side(qb);
    State rot = rotate_from_normal(hll_flux_face_aligned(a, b, g, h_min), nx, ny);
    State flux{norm * rot.h, norm * rot.hu, norm * rot.hv};
    bool hll_dry = (a.h <= h_min) && (b.h <= h_min);
    double h_star_a = hll_dry ? 0.0 : a.h, h_star_b = hll_dry ? 0.0 : b.h;
    double wall_a = 0.0, wall_b = 0.0;
    if (hll_dry) {
        auto wall = [&](const Side& q, double towards) {
            double un = towards * (q.u * nx + q.v * ny);
            double sill = b_face - (q.h + q.b);
            double ram = wall_ram_pressure(q.h, un, sill, g);
            return (hll_dry && q.h > h_min) ? ram : 0.0;
        };
        wall_a = wall(qa, 1.0);
        wall_b = wall(qb, -1.0);
    }
    double half_g = 0.5 * g;
    double dp_a = half_g * (qa.h * qa.h - h_star_a * h_star_a) + wall_a;
    double dp_b = half_g * (qb.h * qb.h - h_star_b * h_star_b) + wall_b;
    fa = {flux.h + 0.0, flux.hu + dp_a * m0, flux.hv + dp_a * m1};
    fb = {flux.h + 0.0, flux.hu + dp_b * m0, flux.hv + dp_b * m1};
}

// SlopeDistances (src/solver/rhs/swe_2d_split_form.rs:179-203)
struct SlopeDistances {
    double central, minus, plus;
};
inline SlopeDistances slope_distances(const double xi[3], double x_l, double x_r) {
    auto side = [](double face, double node) { return 1.0 / (face > 0.0 ? face : 0.5 * node); };
    return {1.0 / (xi[2] - xi[0]), side(xi[1] - x_l, xi[1] - xi[0]),
            side(x_r - xi[1], xi[2] - xi[1])};
}

// limited_slope (src/solver/rhs/swe_2d_split_form.rs:168-177)
inline double limited_slope(const double q[3], const SlopeDistances& inv) {
    double dm = q[1] - q[0], dp = q[2] - q[1];
    bool extremum = (dm * dp) <= 0.0;
    double central = (q[2] - q[0]) * inv.central;
    double bound = lmin(std::fabs(dm * inv.minus), std::fabs(dp * inv.plus));
    double sign = central < 0.0 ? -1.0 : 1.0;
    return extremum ? 0.0 : sign * lmin(std::fabs(central), bound);
}

// reconstruct_subcell (src/solver/rhs/swe_2d_split_form.rs:279-317)
inline void reconstruct_subcell(const Side nodes[3], const double xi[3], double x_l, double x_r,
                                double h_dry, Side& left, Side& right) {
    const Side& c = nodes[1];
    double eta[3] = {nodes[0].eta(), nodes[1].eta(), nodes[2].eta()};
    double h[3] = {nodes[0].h, nodes[1].h, nodes[2].h};
    double wet_surface = -std::numeric_limits<double>::infinity();
    for (int i = 0; i < 3; ++i) {
        bool higher = eta[i] > wet_surface;
        wet_surface = (h[i] >= h_dry && higher) ? eta[i] : wet_surface;
    }
    bool flooding = false;
    for (int i = 0; i < 3; ++i) flooding = flooding || (h[i] < h_dry && eta[i] < wet_surface);
    SlopeDistances inv = slope_distances(xi, x_l, x_r);
    double s_h = limited_slope(h, inv);
    double s_eta = flooding ? 0.0 : limited_slope(eta, inv);
    double us[3] = {nodes[0].u, nodes[1].u, nodes[2].u};
    double vs[3] = {nodes[0].v, nodes[1].v, nodes[2].v};
    double s_u = limited_slope(us, inv), s_v = limited_slope(vs, inv);
    auto at = [&](double x) {
        double d = x - xi[1];
        double hh = lmax(c.h + s_h * d, 0.0);
        return Side{hh, c.u + s_u * d, c.v + s_v * d, eta[1] + s_eta * d - hh};
    };
    left = at(x_l);
    right = at(x_r);
}

// cbrt of the Manning law (src/source/swe_2d/friction.rs:39-70): the
// reference's bit-pattern guess and three Halley steps; edge cases to cbrt
inline double manning_cbrt(double x) {
    if (!(x >= std::numeric_limits<double>::min() && std::isfinite(x))) return std::cbrt(x);
    uint64_t bits;
    std::memcpy(&bits, &x, 8);
    bits = bits / 3 + 0x2A9F7893782DA1CEull;
    double y;
    std::memcpy(&y, &bits, 8);
    for (int i = 0; i < 3; ++i) {
        double y3 = y * y * y;
        y += y * ((x - y3) / (2.0 * y3 + x));
    }
    return y;
}

// manning_rate (src/source/swe_2d/friction.rs:325-331)
inline double manning_rate(double g_n2, double h, double speed) {
    return g_n2 * speed / (manning_cbrt(h) * h);
}

// WetDryConfig (src/solver/algorithms/wetting_drying.rs:51-175)
struct WetDry {
    double h_dry = 1e-3, relaxation_time = 1.0, max_velocity = 20.0;

    // desingularized_velocity (wetting_drying.rs:115-130)
    void desingularized_velocity(double h, double hu, double hv, double& u, double& v) const {
        if (h <= 0.0) {
            u = v = 0.0;
            return;
        }
        double eps = h_dry;
        if (h >= eps) {
            double inv_h = 1.0 / h;
            u = hu * inv_h;
            v = hv * inv_h;
            return;
        }
        double r = h / eps;
        double factor = std::sqrt(2.0) * r / (eps * std::sqrt(1.0 + r * r * r * r));
        u = factor * hu;
        v = factor * hv;
    }

    // thin_layer_rate (wetting_drying.rs:135-146)
    double thin_layer_rate(double h) const {
        if (h >= h_dry) return 0.0;
        if (h <= 0.0) return std::numeric_limits<double>::infinity();
        double excess = h_dry / h - 1.0;
        return excess * excess / relaxation_time;
    }

    // correct_node (wetting_drying.rs:148-165)
    void correct_node(double h, double& hu, double& hv) const {
        if (h <= 0.0) {
            hu = hv = 0.0;
            return;
        }
        if (h < h_dry) {
            double u, v;
            desingularized_velocity(h, hu, hv, u, v);
            hu = h * u;
            hv = h * v;
        }
        double momentum = std::sqrt(hu * hu + hv * hv);
        if (momentum > max_velocity * h) {
            double scale = max_velocity * h / momentum;
            hu *= scale;
            hv *= scale;
        }
    }
};

// SWEState2D::velocity (src/solver/state/swe_2d.rs:54-61): desingularised
inline void state_velocity(State s, double h_min, double& u, double& v) {
    double h_reg = fmax_(s.h, h_min);
    double denom = s.h * s.h + h_reg * h_reg;
    double inv_denom = 1.0 / denom;
    double factor = 2.0 * s.h * inv_denom;
    u = s.hu * factor;
    v = s.hv * factor;
}

// SWEState2D::velocity_simple (src/solver/state/swe_2d.rs:67-75)
inline void velocity_simple(State s, double h_min, double& u, double& v) {
    if (s.h > h_min) {
        double h_inv = 1.0 / s.h;
        u = s.hu * h_inv;
        v = s.hv * h_inv;
    } else {
        u = v = 0.0;
    }
}

// characteristic_state (src/boundary/characteristic.rs:481-520)
inline State characteristic_state(State interior, double h_e, double un_e, double ut_e, double nx,
                                  double ny, double g, double h_min) {
    double h_i = fmax_(interior.h, 0.0);
    double un_i = 0.0, ut_i = 0.0;
    if (h_i > h_min) {
        double u = interior.hu / h_i, v = interior.hv / h_i;
        un_i = u * nx + v * ny;
        ut_i = -u * ny + v * nx;
    }
    double c_i = std::sqrt(g * h_i), c_e = std::sqrt(g * h_e);
    double w_out = un_i + 2.0 * c_i, w_in = un_e - 2.0 * c_e;
    bool wet_i = h_i > h_min, wet_e = h_e > h_min;
    double h_b, un_b;
    if (!wet_i && !wet_e) {
        h_b = 0.0;
        un_b = 0.0;
    } else if (wet_i && un_i >= c_i) {
        h_b = h_i;
        un_b = un_i;
    } else if (wet_e && un_e <= -c_e) {
        h_b = h_e;
        un_b = un_e;
    } else if (wet_i && !wet_e) {
        double c = fmax_(w_out / 3.0, 0.0);
        h_b = c * c / g;
        un_b = c;
    } else if (!wet_i && wet_e) {
        double c = fmax_(-w_in / 3.0, 0.0);
        h_b = c * c / g;
        un_b = -c;
    } else {
        double c = fmax_(0.25 * (w_out - w_in), 0.0);
        h_b = c * c / g;
        un_b = 0.5 * (w_out + w_in);
    }
    double ut_b = un_b > 0.0 ? ut_i : ut_e;
    double u = un_b * nx - ut_b * ny, v = un_b * ny + ut_b * nx;
    return {h_b, h_b * u, h_b * v};  // SWEState2D::from_primitives
}

// reflect_velocity (src/boundary/mod.rs:133-136)
inline void reflect_velocity(double u, double v, double nx, double ny, double& ur, double& vr) {
    double un = u * nx + v * ny;
    ur = u - 2.0 * un * nx;
    vr = v - 2.0 * un * ny;
}

// tidal_ramp (src/boundary/harmonic_tide.rs:24-32)
inline double tidal_ramp(double t, double duration) {
    if (!(duration > 0.0)) return 1.0;
    double tau = t / duration;
    tau = tau < 0.0 ? 0.0 : (tau > 1.0 ? 1.0 : tau);
    return tau * tau * (3.0 - 2.0 * tau);
}

// crate::math::hypot (src/math.rs:202-245): musl's hypot, the squares split
// in two parts each (Dekker) so that their sum is exact enough for the
// correctly rounded square root, scaled by 2^±700 near overflow/underflow
inline double ref_hypot(double x, double y) {
    auto square = [](double v, double& hi, double& lo) {
        const double split = 134217728.0 + 1.0;  // 2^27 + 1
        double vc = v * split;
        double vh = v - vc + vc;
        double vl = v - vh;
        hi = v * v;
        lo = vh * vh - hi + 2.0 * vh * vl + vl * vl;
    };
    auto from = [](uint64_t b) {
        double d;
        std::memcpy(&d, &b, sizeof d);
        return d;
    };
    auto to = [](double d) {
        uint64_t b;
        std::memcpy(&b, &d, sizeof b);
        return b;
    };
    uint64_t ux = to(x) & (UINT64_MAX >> 1), uy = to(y) & (UINT64_MAX >> 1);
    if (ux < uy) std::swap(ux, uy);
    int64_t ex = (int64_t)(ux >> 52), ey = (int64_t)(uy >> 52);
    x = from(ux);
    y = from(uy);
    if (ey == 0x7ff) return y;
    if (ex == 0x7ff || uy == 0) return x;
    if (ex - ey > 64) return x + y;
    double z = 1.0;
    if (ex > 0x3ff + 510) {
        z = from(0x6bb0000000000000ull);
        x *= from(0x1430000000000000ull);
        y *= from(0x1430000000000000ull);
    } else if (ey < 0x3ff - 450) {
        z = from(0x1430000000000000ull);
        x *= from(0x6bb0000000000000ull);
        y *= from(0x6bb0000000000000ull);
    }
    double hx, lx, hy, ly;
    square(x, hx, lx);
    square(y, hy, ly);
    return z * std::sqrt(ly + lx + hy + hx);
}

// DragCoefficient::compute (src/source/swe_2d/wind.rs:134-158), by its
// device code (DragCoefficient::from_device_code, wind.rs:118-128)
inline double drag_coefficient(int kind, double cd, double speed) {
    switch (kind) {
        case 0: return cd;
        case 1: return speed <= 11.0 ? 1.2e-3 : (0.49 + 0.065 * fmin_(speed, 25.0)) * 1e-3;
        case 2: return (0.8 + 0.065 * speed) * 1e-3;
        case 3: return (0.61 + 0.063 * speed) * 1e-3;
        default: return speed <= 6.0 ? 1.1e-3 : (0.50 + 0.071 * speed) * 1e-3;
    }
}

// atmosphere_source and wind_stress
// (src/source/swe_2d/gridded_atmosphere.rs:161-196): (τ − h ∇p)/ρ_water,
// τ = ρ_air C_d(|U|) |U| U, nothing below h_min
inline void atmosphere_source(double h, double u, double v, double px, double py, int drag,
                              double cd, double rho_air, double rho_water, double h_min,
                              double& su, double& sv) {
    su = 0.0;
    sv = 0.0;
    if (h < h_min) return;
    double speed = ref_hypot(u, v);
    double stress = rho_air * drag_coefficient(drag, cd, speed) * speed;
    double tau_x = stress * u, tau_y = stress * v;
    su = (tau_x - h * px) / rho_water;
    sv = (tau_y - h * py) / rho_water;
}

// inverse_barometer_level (gridded_atmosphere.rs:198-202), g = 9.81
inline double inverse_barometer_level(double p, double ramp, double rho_water) {
    return -ramp * p / (rho_water * 9.81);
}

}  // namespace oracle
