// Reverse (vector–Jacobian) forms of the point functions in point.cuh, for
// the discrete adjoint. Each *_rev function takes the forward inputs and the
// adjoints of the forward outputs, recomputes what it needs, and ADDS the
// adjoints of the inputs to its reference arguments. Branches (wet/dry
// tests, minima and maxima, the HLL wave-speed choices, limiter cases) are
// taken exactly as the forward takes them from the same inputs, so the
// result is the derivative of the branch the forward ran ("frozen"); at a
// depth of exactly zero the square root's infinite slope is taken as 0.
// Host and device both compile this header; the host for the
// finite-difference unit test of every function here.
#pragma once

#include "point.cuh"

namespace dgswe {
namespace DGSWE_NS {

// node_velocity: (u, v) = (hu, hv)/h where h > h_min, else 0
DG_PT void node_velocity_rev(double h, double hu, double hv, double h_min, double ub, double vb,
                             double& hb, double& hub, double& hvb) {
    if (!fp::gt(h, h_min)) return;
    const double inv = vrcp(h);
    const double u = hu * inv, v = hv * inv;
    hub += ub * inv;
    hvb += vb * inv;
    hb -= (ub * u + vb * v) * inv;
}

// One side of hll_aligned: depth, normal and tangential momentum, and the
// velocities
struct Side5 {
    double h, hun, hut, un, ut;
};

DG_PT F3 hll_aligned_s(const Side5& L, const Side5& R, double g, double sqrt_g, double half_g,
                       double h_min) {
    return hll_aligned(L.h, L.hun, L.hut, L.un, L.ut, R.h, R.hun, R.hut, R.un, R.ut, g, sqrt_g,
                       half_g, h_min);
}

DG_PT void hll_aligned_rev(const Side5& L, const Side5& R, double g, double sqrt_g,
                           double half_g, double h_min, const F3& Fb, Side5& Lb, Side5& Rb) {
    if (fp::le(L.h, h_min) && fp::le(R.h, h_min)) return;  // both dry: zero flux
    const double sh_l = vsqrt(fp::max0(L.h)), sh_r = vsqrt(fp::max0(R.h));
    const double c_l = sqrt_g * sh_l, c_r = sqrt_g * sh_r;
    const double sh_sum = sh_l + sh_r;
    const bool roe = fp::gt(sh_sum, 1e-10);
    const double h_roe = 0.5 * (L.h + R.h);
    const double un_roe = roe ? vdiv(sh_l * L.un + sh_r * R.un, sh_sum) : 0.0;
    const double c_roe = roe ? vsqrt(g * h_roe) : 0.0;
    const bool wl = fp::gt(L.h, h_min), wr = fp::gt(R.h, h_min);
    const double a1 = L.un - c_l, a2 = un_roe - c_roe;
    const bool min_first = fp::lt(a1, a2);
    const double s_l = wl ? (min_first ? a1 : a2) : R.un - 2.0 * c_r;
    const double b1 = R.un + c_r, b2 = un_roe + c_roe;
    const bool max_first = fp::gt(b1, b2);
    const double s_r = wr ? (max_first ? b1 : b2) : L.un + 2.0 * c_l;
    const double fl_h = L.h * L.un, fl_hu = L.h * L.un * L.un + half_g * L.h * L.h,
                 fl_hv = L.h * L.un * L.ut;
    const double fr_h = R.h * R.un, fr_hu = R.h * R.un * R.un + half_g * R.h * R.h,
                 fr_hv = R.h * R.un * R.ut;
    double flb_h = 0.0, flb_hu = 0.0, flb_hv = 0.0, frb_h = 0.0, frb_hu = 0.0, frb_hv = 0.0;
    double s_lb = 0.0, s_rb = 0.0;
    if (fp::ge0(s_l)) {
        flb_h = Fb.h;
        flb_hu = Fb.hu;
        flb_hv = Fb.hv;
    } else if (fp::le0(s_r)) {
        frb_h = Fb.h;
        frb_hu = Fb.hu;
        frb_hv = Fb.hv;
    } else {
        const double inv_ds = vrcp(s_r - s_l);
        const double s_lr = s_l * s_r;
        const double jh = R.h - L.h, jhu = R.hun - L.hun, jhv = R.hut - L.hut;
        const double nh = s_r * fl_h - s_l * fr_h + s_lr * jh;
        const double nhu = s_r * fl_hu - s_l * fr_hu + s_lr * jhu;
        const double nhv = s_r * fl_hv - s_l * fr_hv + s_lr * jhv;
        const double inv_dsb = Fb.h * nh + Fb.hu * nhu + Fb.hv * nhv;
        const double nbh = Fb.h * inv_ds, nbhu = Fb.hu * inv_ds, nbhv = Fb.hv * inv_ds;
        s_rb += nbh * fl_h + nbhu * fl_hu + nbhv * fl_hv;
        s_lb -= nbh * fr_h + nbhu * fr_hu + nbhv * fr_hv;
        flb_h = nbh * s_r;
        flb_hu = nbhu * s_r;
        flb_hv = nbhv * s_r;
        frb_h = -nbh * s_l;
        frb_hu = -nbhu * s_l;
        frb_hv = -nbhv * s_l;
        const double s_lrb = nbh * jh + nbhu * jhu + nbhv * jhv;
        Rb.h += nbh * s_lr;
        Lb.h -= nbh * s_lr;
        Rb.hun += nbhu * s_lr;
        Lb.hun -= nbhu * s_lr;
        Rb.hut += nbhv * s_lr;
        Lb.hut -= nbhv * s_lr;
        s_lb += s_lrb * s_r;
        s_rb += s_lrb * s_l;
        const double d = inv_dsb * inv_ds * inv_ds;  // d(1/x)/dx = −1/x²
        s_rb -= d;
        s_lb += d;
    }
    // the physical fluxes
    Lb.h += flb_h * L.un + flb_hu * (L.un * L.un + 2.0 * half_g * L.h) + flb_hv * L.un * L.ut;
    Lb.un += flb_h * L.h + flb_hu * 2.0 * L.h * L.un + flb_hv * L.h * L.ut;
    Lb.ut += flb_hv * L.h * L.un;
    Rb.h += frb_h * R.un + frb_hu * (R.un * R.un + 2.0 * half_g * R.h) + frb_hv * R.un * R.ut;
    Rb.un += frb_h * R.h + frb_hu * 2.0 * R.h * R.un + frb_hv * R.h * R.ut;
    Rb.ut += frb_hv * R.h * R.un;
    // Einfeldt speeds
    double c_lb = 0.0, c_rb = 0.0, un_roeb = 0.0, c_roeb = 0.0;
    if (wl) {
        if (min_first) {
            Lb.un += s_lb;
            c_lb -= s_lb;
        } else {
            un_roeb += s_lb;
            c_roeb -= s_lb;
        }
    } else {
        Rb.un += s_lb;
        c_rb -= 2.0 * s_lb;
    }
    if (wr) {
        if (max_first) {
            Rb.un += s_rb;
            c_rb += s_rb;
        } else {
            un_roeb += s_rb;
            c_roeb += s_rb;
        }
    } else {
        Lb.un += s_rb;
        c_lb += 2.0 * s_rb;
    }
    double sh_lb = sqrt_g * c_lb, sh_rb = sqrt_g * c_rb;
    if (roe) {
        const double q = un_roeb * vrcp(sh_sum);
        Lb.un += q * sh_l;
        Rb.un += q * sh_r;
        sh_lb += q * (L.un - un_roe);
        sh_rb += q * (R.un - un_roe);
        if (fp::gt0(c_roe)) {
            const double hb = c_roeb * g * 0.5 * vrcp(c_roe);
            Lb.h += 0.5 * hb;
            Rb.h += 0.5 * hb;
        }
    }
    if (fp::gt0(sh_l)) Lb.h += sh_lb * 0.5 * vrcp(sh_l);
    if (fp::gt0(sh_r)) Rb.h += sh_rb * 0.5 * vrcp(sh_r);
}

// wall_ram_pressure's reverse (swe_2d_split_form.rs:147-156)
DG_PT void wall_ram_rev(double h, double un, double sill, double g, double ramb, double& hb,
                        double& unb, double& sillb) {
    const double up = fp::max0(un);
    const double head = up * up * (0.5 / g);
    if (!fp::gt(sill, head)) return;
    const double c = sqrt(g * h);
    const double a = 1.0 - head / sill, p = h * up, q = 2.0 * up + c;
    const double ab = ramb * p * q, pb = ramb * a * q, qb = ramb * a * p;
    const double headb = -ab / sill;
    sillb += ab * head / (sill * sill);
    hb += pb * up;
    if (fp::gt0(c)) hb += qb * g * 0.5 / c;
    const double upb = pb * h + 2.0 * qb + headb * 2.0 * up * (0.5 / g);
    if (fp::gt0(un)) unb += upb;
}

// hydrostatic_hll's reverse: the adjoints of side a's and side b's fluxes
// (fa, fb as hydro_hll returns them, before any sign change)
DG_PT void hydro_hll_rev(const Sd& qa, const Sd& qb, double m0, double m1, double norm, double nx,
                         double ny, double g, double sqrt_g, double half_g, double h_min,
                         const F3& fab, const F3& fbb, Sd& qab, Sd& qbb) {
    const bool a_high = fp::gt(qa.b, qb.b);
    const double b_face = a_high ? qa.b : qb.b;
    const double ea = qa.h + qa.b - b_face, eb = qb.h + qb.b - b_face;
    const double hs_a = fp::max0(ea), hs_b = fp::max0(eb);
    const bool wet_a = fp::gt(qa.h, h_min), wet_b = fp::gt(qb.h, h_min);
    const double ua = wet_a ? qa.u : 0.0, va = wet_a ? qa.v : 0.0;
    const double ub = wet_b ? qb.u : 0.0, vb = wet_b ? qb.v : 0.0;
    const double un_a = ua * nx + va * ny, ut_a = -ua * ny + va * nx;
    const double un_b = ub * nx + vb * ny, ut_b = -ub * ny + vb * nx;
    const bool sw_a = fp::gt(hs_a, h_min), sw_b = fp::gt(hs_b, h_min);
    const Side5 L{hs_a, hs_a * un_a, hs_a * ut_a, sw_a ? un_a : 0.0, sw_a ? ut_a : 0.0};
    const Side5 R{hs_b, hs_b * un_b, hs_b * ut_b, sw_b ? un_b : 0.0, sw_b ? ut_b : 0.0};
    const bool hll_dry = fp::le(hs_a, h_min) && fp::le(hs_b, h_min);
    const double f_hb = fab.h + fbb.h, f_hub = fab.hu + fbb.hu, f_hvb = fab.hv + fbb.hv;
    const double dp_ab = fab.hu * m0 + fab.hv * m1, dp_bb = fbb.hu * m0 + fbb.hv * m1;
    double hs_ab = 0.0, hs_bb = 0.0, b_faceb = 0.0;
    // dp = ½g(h² − h*²) + wall ram pressure
    qab.h += dp_ab * 2.0 * half_g * qa.h;
    qbb.h += dp_bb * 2.0 * half_g * qb.h;
    if (!hll_dry) {
        hs_ab -= dp_ab * 2.0 * half_g * hs_a;
        hs_bb -= dp_bb * 2.0 * half_g * hs_b;
    } else {
        if (wet_a) {
            double hb = 0.0, unb = 0.0, sillb = 0.0;
            wall_ram_rev(qa.h, qa.u * nx + qa.v * ny, b_face - (qa.h + qa.b), g, dp_ab, hb, unb,
                         sillb);
            qab.h += hb - sillb;
            qab.b -= sillb;
            b_faceb += sillb;
            qab.u += unb * nx;
            qab.v += unb * ny;
        }
        if (wet_b) {
            double hb = 0.0, unb = 0.0, sillb = 0.0;
            wall_ram_rev(qb.h, -1.0 * (qb.u * nx + qb.v * ny), b_face - (qb.h + qb.b), g, dp_bb,
                         hb, unb, sillb);
            qbb.h += hb - sillb;
            qbb.b -= sillb;
            b_faceb += sillb;
            qbb.u -= unb * nx;
            qbb.v -= unb * ny;
        }
    }
    // rotation back, times |m|
    const F3 rb{norm * f_hb, norm * (f_hub * nx + f_hvb * ny), norm * (-f_hub * ny + f_hvb * nx)};
    Side5 Lb{}, Rb{};
    hll_aligned_rev(L, R, g, sqrt_g, half_g, h_min, rb, Lb, Rb);
    hs_ab += Lb.h + Lb.hun * un_a + Lb.hut * ut_a;
    hs_bb += Rb.h + Rb.hun * un_b + Rb.hut * ut_b;
    const double un_ab = Lb.hun * hs_a + (sw_a ? Lb.un : 0.0);
    const double ut_ab = Lb.hut * hs_a + (sw_a ? Lb.ut : 0.0);
    const double un_bb = Rb.hun * hs_b + (sw_b ? Rb.un : 0.0);
    const double ut_bb = Rb.hut * hs_b + (sw_b ? Rb.ut : 0.0);
    if (wet_a) {
        qab.u += un_ab * nx - ut_ab * ny;
        qab.v += un_ab * ny + ut_ab * nx;
    }
    if (wet_b) {
        qbb.u += un_bb * nx - ut_bb * ny;
        qbb.v += un_bb * ny + ut_bb * nx;
    }
    if (fp::gt0(ea)) {
        qab.h += hs_ab;
        qab.b += hs_ab;
        b_faceb -= hs_ab;
    }
    if (fp::gt0(eb)) {
        qbb.h += hs_bb;
        qbb.b += hs_bb;
        b_faceb -= hs_bb;
    }
    if (a_high)
        qab.b += b_faceb;
    else
        qbb.b += b_faceb;
}

// wflux(q, q, m)·: the flux F(q)·m of one state, reversed into q's depth,
// momentum and velocity adjoints
DG_PT void wflux_same_rev(const Q& q, double m0, double m1, double g, const F3& Fb, Q& qb) {
    const double mass = 0.5 * ((q.hu + q.hu) * m0 + (q.hv + q.hv) * m1);
    const double u_avg = 0.5 * (q.u + q.u), v_avg = 0.5 * (q.v + q.v);
    const double massb = Fb.h + Fb.hu * u_avg + Fb.hv * v_avg;
    const double pb = Fb.hu * m0 + Fb.hv * m1;  // pressure = ½g h²
    qb.u += Fb.hu * mass;
    qb.v += Fb.hv * mass;
    qb.h += pb * g * q.h;
    qb.hu += massb * m0;
    qb.hv += massb * m1;
}

// interior_velocity's reverse
DG_PT void interior_velocity_rev(const Q& qi, double h_min, double ub, double vb, Q& qib) {
    node_velocity_rev(qi.h, qi.hu, qi.hv, h_min, ub, vb, qib.h, qib.hu, qib.hv);
}

// wall_ghost's reverse: the adjoint of the ghost (h, hu, hv, u, v, b) into
// the interior node (its h and b) and the interior velocity (u, v)
DG_PT void wall_ghost_rev(const Q& qi, double u, double v, double nx, double ny, double wall_h_min,
                          double h_min, const Q& qe, const Q& qeb, Q& qib, double& ub,
                          double& vb) {
    double ghb = qeb.h, ghub = qeb.hu, ghvb = qeb.hv;
    node_velocity_rev(qe.h, qe.hu, qe.hv, h_min, qeb.u, qeb.v, ghb, ghub, ghvb);
    qib.h += ghb;
    qib.b += qeb.b;
    if (!fp::le(qi.h, wall_h_min)) {
        const double un = u * nx + v * ny;
        // ghu = h (u − 2 un nx), ghv = h (v − 2 un ny)
        qib.h += ghub * (u - 2.0 * un * nx) + ghvb * (v - 2.0 * un * ny);
        ub += ghub * qi.h;
        vb += ghvb * qi.h;
        const double unb = -2.0 * qi.h * (ghub * nx + ghvb * ny);
        ub += unb * nx;
        vb += unb * ny;
    }
}

// characteristic_state's reverse: the adjoints of the boundary state's h, hu,
// hv (its velocities reversed first into those) into the interior node, the
// interior velocity and the external elevation
DG_PT void characteristic_state_rev(const Q& qi, double u, double v, double eta, double nx,
                                    double ny, int elevation_only, double g, double h_min,
                                    const Q& qbb_in, Q& qib, double& ub_i, double& vb_i,
                                    double& etab) {
    const Q qb = characteristic_state(qi, u, v, eta, nx, ny, elevation_only, g, h_min);
    double h_bb = qbb_in.h, hu_bb = qbb_in.hu, hv_bb = qbb_in.hv;
    node_velocity_rev(qb.h, qb.hu, qb.hv, h_min, qbb_in.u, qbb_in.v, h_bb, hu_bb, hv_bb);
    // recompute the forward's pieces
    const double bathy = qi.b;
    const double e_arg = eta - bathy;
    const double h_e = fmax(e_arg, 0.0);
    double un_e = 0.0;
    const double neg_b = fmax(-bathy, 0.0);
    if (elevation_only == kIncomingWave) un_e = 2.0 * (sqrt(g * neg_b) - sqrt(g * h_e));
    const double ut_e = -u * ny + v * nx;
    const double h_i = fmax(qi.h, 0.0);
    double un_i = 0.0, ut_i = 0.0, ui = 0.0, vi = 0.0;
    const bool moving = h_i > h_min;
    if (moving) {
        ui = qi.hu / h_i;
        vi = qi.hv / h_i;
        un_i = ui * nx + vi * ny;
        ut_i = -ui * ny + vi * nx;
    }
    const double c_i = sqrt(g * h_i), c_e = sqrt(g * h_e);
    const double w_out = un_i + 2.0 * c_i, w_in = un_e - 2.0 * c_e;
    const bool wi = h_i > h_min, we = h_e > h_min;
    int branch;
    double h_b, un_b, cc = 0.0;
    if (!wi && !we) {
        branch = 0;
        h_b = 0.0;
        un_b = 0.0;
    } else if (wi && un_i >= c_i) {
        branch = 1;
        h_b = h_i;
        un_b = un_i;
    } else if (we && un_e <= -c_e) {
        branch = 2;
        h_b = h_e;
        un_b = un_e;
    } else if (wi && !we) {
        branch = 3;
        cc = fmax(w_out / 3.0, 0.0);
        h_b = cc * cc / g;
        un_b = cc;
    } else if (!wi && we) {
        branch = 4;
        cc = fmax(-w_in / 3.0, 0.0);
        h_b = cc * cc / g;
        un_b = -cc;
    } else {
        branch = 5;
        cc = fmax(0.25 * (w_out - w_in), 0.0);
        h_b = cc * cc / g;
        un_b = 0.5 * (w_out + w_in);
    }
    const bool t_in = un_b > 0.0;
    const double ut_b = t_in ? ut_i : ut_e;
    const double ubv = un_b * nx - ut_b * ny, vbv = un_b * ny + ut_b * nx;
    // qb.hu = h_b ub, qb.hv = h_b vb
    h_bb += hu_bb * ubv + hv_bb * vbv;
    const double ubvb = hu_bb * h_b, vbvb = hv_bb * h_b;
    double un_bb = ubvb * nx + vbvb * ny;
    const double ut_bb = -ubvb * ny + vbvb * nx;
    double ut_ib = 0.0, ut_eb = 0.0, un_ib = 0.0, un_eb = 0.0, h_ib = 0.0, h_eb = 0.0;
    double w_outb = 0.0, w_inb = 0.0;
    if (t_in)
        ut_ib += ut_bb;
    else
        ut_eb += ut_bb;
    switch (branch) {
        case 1:
            h_ib += h_bb;
            un_ib += un_bb;
            break;
        case 2:
            h_eb += h_bb;
            un_eb += un_bb;
            break;
        case 3: {
            const double ccb = h_bb * 2.0 * cc / g + un_bb;
            if (w_out / 3.0 > 0.0) w_outb += ccb / 3.0;
        } break;
        case 4: {
            const double ccb = h_bb * 2.0 * cc / g - un_bb;
            if (-w_in / 3.0 > 0.0) w_inb -= ccb / 3.0;
        } break;
        case 5: {
            const double ccb = h_bb * 2.0 * cc / g;
            if (0.25 * (w_out - w_in) > 0.0) {
                w_outb += 0.25 * ccb;
                w_inb -= 0.25 * ccb;
            }
            w_outb += 0.5 * un_bb;
            w_inb += 0.5 * un_bb;
        } break;
        default: break;
    }
    un_ib += w_outb;
    const double c_ib = 2.0 * w_outb;
    un_eb += w_inb;
    const double c_eb = -2.0 * w_inb;
    if (c_i > 0.0) h_ib += c_ib * g * 0.5 / c_i;
    if (c_e > 0.0) h_eb += c_eb * g * 0.5 / c_e;
    if (moving) {
        const double uib = un_ib * nx - ut_ib * ny, vib = un_ib * ny + ut_ib * nx;
        qib.hu += uib / h_i;
        qib.hv += vib / h_i;
        h_ib -= (uib * ui + vib * vi) / h_i;
    }
    if (qi.h > 0.0) qib.h += h_ib;
    ub_i -= ut_eb * ny;
    vb_i += ut_eb * nx;
    double bathyb = 0.0;
    if (elevation_only == kIncomingWave) {
        if (neg_b > 0.0) bathyb -= un_eb * 2.0 * g * 0.5 / sqrt(g * neg_b);
        if (h_e > 0.0) h_eb -= un_eb * 2.0 * g * 0.5 / sqrt(g * h_e);
    }
    if (e_arg > 0.0) {
        etab += h_eb;
        bathyb -= h_eb;
    }
    qib.b += bathyb;
    (void)qb;
}

// HarmonicTide::elevation's derivatives in each constituent's amplitude and
// phase at time t, times etab, added to grad[2i] and grad[2i+1]
DG_PT void tide_elevation_rev(const Condition& c, double t, double etab, double* grad) {
    double ramp = 1.0;
    if (fp::gt0(c.ramp)) {
        double tau = t / c.ramp;
        tau = fp::lt0(tau) ? 0.0 : (fp::gt(tau, 1.0) ? 1.0 : tau);
        ramp = tau * tau * (3.0 - 2.0 * tau);
    }
    for (int i = 0; i < c.n_constituents; ++i) {
        const Constituent& k = c.c[i];
        const double f = k.f + k.f_rate * t;
        const double u_deg = k.u_deg + k.u_rate_deg * t;
        const double offset = (k.v0_deg + u_deg) * (M_PI / 180.0);
        const double arg = k.omega * t + k.phase + offset;
        grad[2 * i] += etab * ramp * f * cos(arg);
        grad[2 * i + 1] -= etab * ramp * f * k.amplitude * sin(arg);
    }
}

// h^(-4/3) as manning_rate evaluates it (for its derivatives)
DG_PT double manning_z4(double h) {
#if DGSWE_FAST_PATH
    const int64_t b = fp::bits(h);
    double z = (b >= 0x3820000000000000ll && b < 0x47C0000000000000ll)
                   ? f64_of(rcbrtf(f32_seed(h)))
                   : 1.0 / cbrt(h);
    const double e = fma(-h, z * z * z, 1.0);
    z = fma(z * e, fma(e, 2.0 / 9.0, 1.0 / 3.0), z);
    const double z2 = z * z;
    return z2 * z2;
#else
    return 1.0 / (ref_cbrt(h) * h);
#endif
}

// desingularized_velocity / SWEState2D::velocity of the damping's input
// node, its reverse: (u, v) adjoints into the input's h, hu, hv, u, v
DG_PT void damp_velocity(const Physics& P, const DampIn& from, double& u, double& v) {
    if (P.has_wet_dry) {
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
            const double factor = 1.4142135623730951 * r / (P.h_dry * sqrt(1.0 + r * r * r * r));
            u = factor * from.hu;
            v = factor * from.hv;
        }
    } else {
        const double h_reg = lmax(from.h, P.h_min);
        const double inv_d = 1.0 / (from.h * from.h + h_reg * h_reg);
        const double factor = 2.0 * from.h * inv_d;
        u = from.hu * factor;
        v = from.hv * factor;
    }
}

// d/dh of the desingularising factor √2 r/(h_dry √(1 + r⁴)), r = h/h_dry
DG_PT double desing_factor_dh(double h, double h_dry) {
    const double r = h / h_dry, r4 = r * r * r * r;
    const double s = sqrt(1.0 + r4);
    return 1.4142135623730951 * (1.0 - r4) / (h_dry * h_dry * s * s * s);
}

DG_PT void damp_velocity_rev(const Physics& P, const DampIn& from, double ub, double vb,
                             DampIn& fromb) {
    if (P.has_wet_dry) {
        if (fp::le0(from.h)) return;
        if (fp::ge(from.h, P.h_dry)) {
            if (fp::gt(P.h_dry, P.h_min)) {
                fromb.u += ub;
                fromb.v += vb;
            } else {
                const double inv = 1.0 / from.h;
                const double u = from.hu * inv, v = from.hv * inv;
                fromb.hu += ub * inv;
                fromb.hv += vb * inv;
                fromb.h -= (ub * u + vb * v) * inv;
            }
        } else {
            const double r = from.h / P.h_dry;
            const double factor = 1.4142135623730951 * r / (P.h_dry * sqrt(1.0 + r * r * r * r));
            fromb.hu += ub * factor;
            fromb.hv += vb * factor;
            fromb.h += (ub * from.hu + vb * from.hv) * desing_factor_dh(from.h, P.h_dry);
        }
    } else {
        const bool reg = !fp::gt(from.h, P.h_min);  // lmax(h, h_min) took h_min
        const double h_reg = lmax(from.h, P.h_min);
        const double den = from.h * from.h + h_reg * h_reg;
        const double factor = 2.0 * from.h / den;
        fromb.hu += ub * factor;
        fromb.hv += vb * factor;
        const double fb = ub * from.hu + vb * from.hv;
        // factor = 2h/den, den = h² + h_reg², h_reg = h unless regularised
        const double dden = 2.0 * from.h + (reg ? 0.0 : 2.0 * h_reg);
        fromb.h += fb * (2.0 / den - 2.0 * from.h * dden / (den * den));
    }
}

// damp's reverse: h passes through unchanged (its adjoint is the caller's);
// hub_o, hvb_o are the adjoints of the damped momentum. Adds to the
// adjoints of the undamped h, hu, hv, of the input node and of g·n².
DG_PT void damp_rev(const Physics& P, double g_n2, double h, double hu, double hv,
                    const DampIn& from, double dt, double hub_o, double hvb_o, double& hb,
                    double& hub, double& hvb, DampIn& fromb, double& g_n2b) {
    if (fp::le0(h)) return;
    double rate = 0.0, u = 0.0, v = 0.0, speed = 0.0, z4 = 0.0, hm = 0.0;
    bool manning = false, hm_h = false;
    if (P.friction) {
        damp_velocity(P, from, u, v);
        speed = vsqrt(u * u + v * v);
        if (fp::gt0(speed)) {
            manning = true;
            hm_h = fp::gt(h, P.manning_h_min);
            hm = hm_h ? h : P.manning_h_min;
            z4 = manning_z4(hm);
            rate += g_n2 * speed * z4;  // manning_rate's value from the same h^(-4/3)
        }
    }
    const bool thin = P.has_wet_dry && fp::lt(h, P.h_dry);
    const double excess = thin ? P.h_dry / h - 1.0 : 0.0;
    if (thin) rate += excess * excess / P.relaxation_time;
    const double factor = vrcp(1.0 + dt * rate);
    hub += factor * hub_o;
    hvb += factor * hvb_o;
    const double factorb = hu * hub_o + hv * hvb_o;
    const double rateb = -factorb * factor * factor * dt;
    if (thin) hb += rateb * 2.0 * excess * (-P.h_dry / (h * h)) / P.relaxation_time;
    if (manning) {
        g_n2b += rateb * speed * z4;
        const double speedb = rateb * g_n2 * z4;
        if (hm_h) hb += rateb * g_n2 * speed * z4 * (-4.0 / 3.0) * vrcp(hm);
        const double inv = vrcp(speed);
        damp_velocity_rev(P, from, speedb * u * inv, speedb * v * inv, fromb);
    }
}

// correct_node's reverse: adjoints of the corrected h, hu, hv into the
// uncorrected ones
DG_PT void correct_node_rev(const Physics& P, double h, double hu, double hv, double hb_o,
                            double hub_o, double hvb_o, double& hb, double& hub, double& hvb) {
    hb += hb_o;
    if (fp::le0(h)) return;  // momentum zeroed
    double hu1 = hu, hv1 = hv, factor = 0.0;
    const bool desing = fp::lt(h, P.h_dry);
    if (desing) {
        const double r = h / P.h_dry;
        factor = 1.4142135623730951 * r / (P.h_dry * sqrt(1.0 + r * r * r * r));
        hu1 = h * (factor * hu);
        hv1 = h * (factor * hv);
    }
    double hu1b = hub_o, hv1b = hvb_o;
    // the cap, with the forward's exponent pre-test
    const int e_h = (int)((fp::bits(h) >> 52) & 0x7FF);
    const int e_u = (int)((fp::bits(P.max_velocity) >> 52) & 0x7FF);
    const int e_hu = (int)((fp::bits(hu1) >> 52) & 0x7FF), e_hv = (int)((fp::bits(hv1) >> 52) & 0x7FF);
    const bool skip = e_h >= 1 && e_u >= 1 && (e_hu > e_hv ? e_hu : e_hv) + 1025 <= e_h + e_u;
    if (!skip) {
        const double m2 = hu1 * hu1 + hv1 * hv1;
        const double cap = P.max_velocity * h;
        if (fp::gt(m2, 0.99 * (cap * cap))) {
            const double m = sqrt(m2);
            if (fp::gt(m, cap)) {
                const double scale = cap / m;
                const double dot = hub_o * hu1 + hvb_o * hv1;
                const double k = -cap / (m * m * m);
                hu1b = hub_o * scale + dot * k * hu1;
                hv1b = hvb_o * scale + dot * k * hv1;
                hb += dot * P.max_velocity / m;
            }
        }
    }
    if (desing) {
        const double hf = h * factor;
        hub += hu1b * hf;
        hvb += hv1b * hf;
        const double dfh = factor + h * desing_factor_dh(h, P.h_dry);
        hb += (hu1b * hu + hv1b * hv) * dfh;
    } else {
        hub += hu1b;
        hvb += hv1b;
    }
}

// limited_slope with its partials in q0, q1, q2 (the branch it took)
DG_PT double limited_slope_d(double q0, double q1, double q2, double ic, double im, double ip,
                             double& d0, double& d1, double& d2) {
    d0 = d1 = d2 = 0.0;
    const double dm = q1 - q0, dp = q2 - q1;
    if (fp::le0(dm * dp)) return 0.0;
    const double central = (q2 - q0) * ic;
    const double a = fabs(dm * im), b = fabs(dp * ip);
    const bool use_a = fp::bits(a) < fp::bits(b);  // min_nn(a, b) took a
    const double bound = use_a ? a : b;
    const double sign = fp::lt0(central) ? -1.0 : 1.0;
    const double ac = fabs(central);
    if (fp::bits(ac) < fp::bits(bound)) {  // min_nn(|central|, bound) took |central|
        d2 = ic;
        d0 = -ic;
        return sign * ac;
    }
    if (use_a) {
        d1 = sign * (fp::lt0(dm * im) ? -1.0 : 1.0) * im;
        d0 = -d1;
        return sign * a;
    }
    d2 = sign * (fp::lt0(dp * ip) ? -1.0 : 1.0) * ip;
    d1 = -d2;
    return sign * b;
}

// reconstruct_subcell's reverse: the adjoints of the left and right face
// states into the three nodes
DG_PT void reconstruct_rev(const Sd& m, const Sd& c, const Sd& p, double x0, double x1, double x2,
                           double xl, double xr, double h_dry, const Sd& lb, const Sd& rb, Sd& mb,
                           Sd& cb, Sd& pb) {
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
    double hd[3], ed[3], ud[3], vd[3];
    const double s_h = limited_slope_d(m.h, c.h, p.h, ic, im, ip, hd[0], hd[1], hd[2]);
    if (flooding) ed[0] = ed[1] = ed[2] = 0.0;
    else limited_slope_d(e0, e1, e2, ic, im, ip, ed[0], ed[1], ed[2]);
    limited_slope_d(m.u, c.u, p.u, ic, im, ip, ud[0], ud[1], ud[2]);
    limited_slope_d(m.v, c.v, p.v, ic, im, ip, vd[0], vd[1], vd[2]);
    double s_hb = 0.0, s_eb = 0.0, s_ub = 0.0, s_vb = 0.0, e1b = 0.0;
    for (int side = 0; side < 2; ++side) {
        const double d = side == 0 ? xl - x1 : xr - x1;
        const Sd& fb = side == 0 ? lb : rb;
        // face = {hh, c.u + s_u d, c.v + s_v d, e1 + s_eta d − hh}, hh = max0(c.h + s_h d)
        const double hhb = fb.h - fb.b;
        e1b += fb.b;
        s_eb += fb.b * d;
        cb.u += fb.u;
        s_ub += fb.u * d;
        cb.v += fb.v;
        s_vb += fb.v * d;
        if (fp::gt0(c.h + s_h * d)) {
            cb.h += hhb;
            s_hb += hhb * d;
        }
    }
    mb.h += s_hb * hd[0];
    cb.h += s_hb * hd[1];
    pb.h += s_hb * hd[2];
    const double e0b = s_eb * ed[0], e2b = s_eb * ed[2];
    e1b += s_eb * ed[1];
    mb.h += e0b;
    mb.b += e0b;
    cb.h += e1b;
    cb.b += e1b;
    pb.h += e2b;
    pb.b += e2b;
    mb.u += s_ub * ud[0];
    cb.u += s_ub * ud[1];
    pb.u += s_ub * ud[2];
    mb.v += s_vb * vd[0];
    cb.v += s_vb * vd[1];
    pb.v += s_vb * vd[2];
}

}  // namespace DGSWE_NS
}  // namespace dgswe
