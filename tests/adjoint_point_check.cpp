// Finite-difference check of the reverse point functions
// (dgcom_gb300/csrc/adjoint_point.cuh) against their forward functions
// (point.cuh), built for the host with the EXACT arithmetic.
//
// For each function F and random inputs x, output weights w and direction
// d: the adjoint's x̄·d must equal w·(F(x+εd) − F(x−εd))/(2ε). A sample
// whose two central differences (ε and ε/4) disagree crossed a branch and
// is skipped; each function must pass at least half its samples, all of
// them to the tolerance. Prints one line per function; exits 1 on failure.
#define DGSWE_FAST 0
#define DGSWE_NS exact
#include <cmath>
#include <cstdio>
#include <functional>
#include <utility>
#include <random>
#include <vector>

#include "adjoint_point.cuh"

using namespace dgswe;
using namespace dgswe::exact;
using Vec = std::vector<double>;
using Fwd = std::function<Vec(const Vec&)>;
using Rev = std::function<Vec(const Vec&, const Vec&)>;

static std::mt19937_64 rng(20261204);
static double uni(double a, double b) { return std::uniform_real_distribution<double>(a, b)(rng); }

static double dot(const Vec& a, const Vec& b) {
    double s = 0.0;
    for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
    return s;
}

struct Result {
    int passed = 0, skipped = 0, failed = 0;
    double worst = 0.0;
};

// one sample: true = pass, false = fail; skipped counted in r
// `tie` (i, j): direction components i and j equal, for inputs that are
// equal where a min or max of them has a kink (coincident beds)
static void sample(const char* name, const Fwd& f, const Rev& rv, const Vec& x, Result& r,
                   double tol = 2e-6, std::pair<int, int> tie = {-1, -1}) {
    const Vec y = f(x);
    Vec w(y.size()), d(x.size());
    for (auto& v : w) v = uni(-1.0, 1.0);
    for (size_t i = 0; i < x.size(); ++i) d[i] = uni(-1.0, 1.0) * (std::fabs(x[i]) + 1e-3);
    if (tie.first >= 0) d[tie.second] = d[tie.first];
    auto fd = [&](double eps) {
        Vec xp = x, xm = x;
        for (size_t i = 0; i < x.size(); ++i) {
            xp[i] += eps * d[i];
            xm[i] -= eps * d[i];
        }
        return (dot(w, f(xp)) - dot(w, f(xm))) / (2.0 * eps);
    };
    const double e1 = 1e-6, g1 = fd(e1), g2 = fd(e1 / 4.0);
    const double scale = std::fabs(g1) + std::fabs(g2) + 1e-12;
    if (std::fabs(g1 - g2) > 1e-5 * scale) {
        r.skipped += 1;
        return;
    }
    const double adj = dot(rv(x, w), d);
    const double err = std::fabs(adj - g2) / (std::fabs(g2) + std::fabs(adj) + 1e-10);
    r.worst = std::fmax(r.worst, err);
    if (err <= tol) {
        r.passed += 1;
    } else {
        r.failed += 1;
        if (r.failed <= 3) {
            std::printf("  %s: adjoint %.12e fd %.12e (rel %.2e) x =", name, adj, g2, err);
            for (double v : x) std::printf(" %.6g", v);
            std::printf("\n");
        }
    }
}

static bool report(const char* name, const Result& r) {
    const int total = r.passed + r.skipped + r.failed;
    const bool ok = r.failed == 0 && r.passed * 2 >= total;
    std::printf("%-28s %s passed %d skipped %d failed %d worst %.2e\n", name, ok ? "ok  " : "FAIL",
                r.passed, r.skipped, r.failed, r.worst);
    return ok;
}

static Physics physics(bool wet_dry, int friction) {
    Physics P{};
    P.g = 9.81;
    P.h_min = 1e-6;
    P.sqrt_g = std::sqrt(P.g);
    P.half_g = 0.5 * P.g;
    P.two_g = 2.0 * P.g;
    P.has_wet_dry = wet_dry ? 1 : 0;
    P.h_dry = 1e-3;
    P.relaxation_time = 1.0;
    P.max_velocity = 20.0;
    P.friction = friction;
    P.manning_h_min = 1e-3;
    return P;
}

int main() {
    bool ok = true;
    const double g = 9.81, sg = std::sqrt(g), hg = 0.5 * g, h_min = 1e-6;

    {  // node_velocity
        Result r;
        Fwd f = [&](const Vec& x) {
            double u, v;
            node_velocity(x[0], x[1], x[2], h_min, u, v);
            return Vec{u, v};
        };
        Rev rv = [&](const Vec& x, const Vec& w) {
            Vec b(3, 0.0);
            node_velocity_rev(x[0], x[1], x[2], h_min, w[0], w[1], b[0], b[1], b[2]);
            return b;
        };
        for (int i = 0; i < 300; ++i) sample("node_velocity", f, rv, {uni(1e-4, 30), uni(-5, 5), uni(-5, 5)}, r);
        ok &= report("node_velocity", r);
    }
    {  // hll_aligned over its regimes
        Result r;
        Fwd f = [&](const Vec& x) {
            const F3 o = hll_aligned_s({x[0], x[1], x[2], x[3], x[4]}, {x[5], x[6], x[7], x[8], x[9]},
                                       g, sg, hg, h_min);
            return Vec{o.h, o.hu, o.hv};
        };
        Rev rv = [&](const Vec& x, const Vec& w) {
            Side5 lb{}, rb{};
            hll_aligned_rev({x[0], x[1], x[2], x[3], x[4]}, {x[5], x[6], x[7], x[8], x[9]}, g, sg,
                            hg, h_min, F3{w[0], w[1], w[2]}, lb, rb);
            return Vec{lb.h, lb.hun, lb.hut, lb.un, lb.ut, rb.h, rb.hun, rb.hut, rb.un, rb.ut};
        };
        for (int i = 0; i < 2000; ++i) {
            const int regime = i % 5;
            double hl = uni(0.5, 20), hr = uni(0.5, 20), ul = uni(-2, 2), ur = uni(-2, 2);
            if (regime == 1) ul = ur = uni(15, 30);    // supersonic to the right: from the left
            if (regime == 2) ul = ur = -uni(15, 30);   // from the right
            if (regime == 3) hl = uni(0.0, 5e-7);      // dry left side
            if (regime == 4) hr = uni(0.0, 5e-7);      // dry right side
            const double tl = uni(-1, 1), tr = uni(-1, 1);
            sample("hll_aligned", f, rv, {hl, hl * ul, hl * tl, ul, tl, hr, hr * ur, hr * tr, ur, tr}, r);
        }
        ok &= report("hll_aligned", r);
    }
    {  // hydro_hll: continuous and stepped beds, wall ram pressure
        Result r;
        const double nx0 = 0.6, ny0 = 0.8, norm = 37.0;
        Fwd f = [&](const Vec& x) {
            F3 fa, fb;
            hydro_hll(Sd{x[0], x[1], x[2], x[3]}, Sd{x[4], x[5], x[6], x[7]}, norm * nx0, norm * ny0,
                      norm, nx0, ny0, g, sg, hg, h_min, fa, fb);
            return Vec{fa.h, fa.hu, fa.hv, fb.h, fb.hu, fb.hv};
        };
        Rev rv = [&](const Vec& x, const Vec& w) {
            Sd ab{}, bb{};
            hydro_hll_rev(Sd{x[0], x[1], x[2], x[3]}, Sd{x[4], x[5], x[6], x[7]}, norm * nx0,
                          norm * ny0, norm, nx0, ny0, g, sg, hg, h_min, F3{w[0], w[1], w[2]},
                          F3{w[3], w[4], w[5]}, ab, bb);
            return Vec{ab.h, ab.u, ab.v, ab.b, bb.h, bb.u, bb.v, bb.b};
        };
        for (int i = 0; i < 2000; ++i) {
            const int regime = i % 4;
            double ha = uni(0.5, 20), hb = uni(0.5, 20), ba = uni(-20, 0), bb = uni(-20, 0);
            if (regime == 1) bb = ba;                         // continuous bed
            if (regime == 2) { bb = ba + uni(0.5, 3.0); hb = uni(1e-9, 5e-7); ha = uni(0.1, 0.4); }  // shore
            if (regime == 3) { bb = ba + ha + uni(0.2, 1.0); hb = 0.0; }  // wall: a's surface below b's bed
            sample("hydro_hll", f, rv,
                   {ha, uni(-2, 2), uni(-2, 2), ba, hb, uni(-2, 2), uni(-2, 2), bb}, r, 2e-6,
                   regime == 1 ? std::pair<int, int>{3, 7} : std::pair<int, int>{-1, -1});
        }
        ok &= report("hydro_hll", r);
    }
    {  // the wall boundary flux: mirror ghost, then hydro_hll (unit normal, as the
       // face kernel passes it)
        Result r;
        const double nx0 = -0.28, ny0 = 0.96, norm = 1.0;
        auto flux = [&](const Vec& x) {
            Q qi{x[0], x[1], x[2], 0, 0, x[3]};
            node_velocity(qi.h, qi.hu, qi.hv, h_min, qi.u, qi.v);
            double u, v;
            interior_velocity(qi, h_min, u, v);
            const Q qe = wall_ghost(qi, u, v, norm * nx0, norm * ny0, 1e-4, h_min);
            F3 fs, dummy;
            hydro_hll(side(qi), side(qe), norm * nx0, norm * ny0, norm, nx0, ny0, g, sg, hg, h_min,
                      fs, dummy);
            return Vec{fs.h, fs.hu, fs.hv};
        };
        Rev rv = [&](const Vec& x, const Vec& w) {
            Q qi{x[0], x[1], x[2], 0, 0, x[3]};
            node_velocity(qi.h, qi.hu, qi.hv, h_min, qi.u, qi.v);
            double u, v;
            interior_velocity(qi, h_min, u, v);
            const Q qe = wall_ghost(qi, u, v, norm * nx0, norm * ny0, 1e-4, h_min);
            Sd sib{}, seb{};
            hydro_hll_rev(side(qi), side(qe), norm * nx0, norm * ny0, norm, nx0, ny0, g, sg, hg,
                          h_min, F3{w[0], w[1], w[2]}, F3{0, 0, 0}, sib, seb);
            Q qib{sib.h, 0, 0, 0, 0, sib.b};
            Q qeb{seb.h, 0, 0, seb.u, seb.v, seb.b};
            double ub = 0.0, vb = 0.0;
            wall_ghost_rev(qi, u, v, norm * nx0, norm * ny0, 1e-4, h_min, qe, qeb, qib, ub, vb);
            // qi's own node velocity and the interior velocity are the same function
            ub += sib.u;
            vb += sib.v;
            interior_velocity_rev(qi, h_min, ub, vb, qib);
            return Vec{qib.h, qib.hu, qib.hv, qib.b};
        };
        for (int i = 0; i < 600; ++i) {
            const double h = uni(0.1, 20);
            sample("wall_flux", flux, rv, {h, h * uni(-2, 2), h * uni(-2, 2), uni(-20, 0)}, r);
        }
        ok &= report("wall_flux", r);
    }
    {  // the characteristic open boundary flux F(q_b)·n with its elevation
        for (int eo = 0; eo < 2; ++eo) {
            Result r;
            const double nx0 = -1.0, ny0 = 0.0, norm = 1.0;
            auto state = [&](const Vec& x, Q& qi, double& u, double& v) {
                qi = Q{x[0], x[1], x[2], 0, 0, x[3]};
                interior_velocity(qi, h_min, u, v);
            };
            Fwd f = [&](const Vec& x) {
                Q qi;
                double u, v;
                state(x, qi, u, v);
                const Q qb = characteristic_state(qi, u, v, x[4], norm * nx0, norm * ny0, eo, g, h_min);
                const F3 fs = wflux(qb, qb, norm * nx0, norm * ny0, g);
                return Vec{fs.h, fs.hu, fs.hv};
            };
            Rev rv = [&](const Vec& x, const Vec& w) {
                Q qi;
                double u, v;
                state(x, qi, u, v);
                const Q qb = characteristic_state(qi, u, v, x[4], norm * nx0, norm * ny0, eo, g, h_min);
                Q qbb{};
                wflux_same_rev(qb, norm * nx0, norm * ny0, g, F3{w[0], w[1], w[2]}, qbb);
                Q qib{};
                double ub = 0.0, vb = 0.0, etab = 0.0;
                characteristic_state_rev(qi, u, v, x[4], norm * nx0, norm * ny0, eo, g, h_min, qbb,
                                         qib, ub, vb, etab);
                interior_velocity_rev(qi, h_min, ub, vb, qib);
                return Vec{qib.h, qib.hu, qib.hv, qib.b, etab};
            };
            for (int i = 0; i < 1500; ++i) {
                const int regime = i % 3;
                double h = uni(0.5, 25), un = uni(-1.5, 1.5), b = -uni(1, 25), eta = uni(-1, 1);
                if (regime == 1) un = -uni(20, 40);  // supercritical inflow
                if (regime == 2) un = uni(20, 40);   // supercritical outflow
                sample(eo ? "characteristic_wave" : "characteristic_rest", f, rv,
                       {h, -h * un, h * uni(-1, 1), b, eta}, r);
            }
            ok &= report(eo ? "characteristic_wave" : "characteristic_rest", r);
        }
    }
    {  // damping, with and without the wet/dry layer, Manning uniform or per node
        for (int wd = 0; wd < 2; ++wd) {
            Result r;
            const Physics P = physics(wd == 1, 1);
            const double dt = 0.37;
            auto from_of = [&](const Vec& x) {
                DampIn fr{x[3], x[4], x[5], 0, 0};
                node_velocity(fr.h, fr.hu, fr.hv, P.h_min, fr.u, fr.v);
                return fr;
            };
            Fwd f = [&](const Vec& x) {
                double hu = x[1], hv = x[2];
                damp(P, x[6], x[0], hu, hv, from_of(x), dt);
                return Vec{hu, hv};
            };
            Rev rv = [&](const Vec& x, const Vec& w) {
                const DampIn fr = from_of(x);
                double hb = 0, hub = 0, hvb = 0, gb = 0;
                DampIn frb{};
                damp_rev(P, x[6], x[0], x[1], x[2], fr, dt, w[0], w[1], hb, hub, hvb, frb, gb);
                node_velocity_rev(fr.h, fr.hu, fr.hv, P.h_min, frb.u, frb.v, frb.h, frb.hu, frb.hv);
                return Vec{hb, hub, hvb, frb.h, frb.hu, frb.hv, gb};
            };
            for (int i = 0; i < 1500; ++i) {
                const int regime = i % 3;
                double h = uni(0.01, 20), fh = uni(0.01, 20);
                if (regime == 1 && wd) { h = uni(2e-4, 9e-4); fh = uni(2e-4, 9e-4); }  // thin layer
                if (regime == 2) h = uni(1e-4, 9e-4);  // below Manning's depth floor
                sample(wd ? "damp_wet_dry" : "damp", f, rv,
                       {h, h * uni(-2, 2), h * uni(-2, 2), fh, fh * uni(-2, 2), fh * uni(-2, 2),
                        9.81 * 0.025 * 0.025 * uni(0.5, 2.0)}, r);
            }
            ok &= report(wd ? "damp_wet_dry" : "damp", r);
        }
    }
    {  // correct_node: desingularisation and the velocity cap
        Result r;
        const Physics P = physics(true, 1);
        Fwd f = [&](const Vec& x) {
            double hu = x[1], hv = x[2];
            correct_node(P, x[0], hu, hv);
            return Vec{x[0], hu, hv};
        };
        Rev rv = [&](const Vec& x, const Vec& w) {
            double hb = 0, hub = 0, hvb = 0;
            correct_node_rev(P, x[0], x[1], x[2], w[0], w[1], w[2], hb, hub, hvb);
            return Vec{hb, hub, hvb};
        };
        for (int i = 0; i < 1500; ++i) {
            const int regime = i % 3;
            double h = uni(0.01, 10), s = uni(-3, 3);
            if (regime == 1) h = uni(1e-4, 9e-4);
            if (regime == 2) s = uni(25, 60) * (i % 2 ? 1 : -1);  // above the cap
            sample("correct_node", f, rv, {h, h * s, h * uni(-3, 3)}, r);
        }
        ok &= report("correct_node", r);
    }
    {  // subcell reconstruction
        Result r;
        const double x0 = -1.3, x1 = -0.6, x2 = 0.2, xl = -0.9, xr = -0.3, h_dry = 1e-3;
        auto unpack = [](const Vec& x, int o) { return Sd{x[o], x[o + 1], x[o + 2], x[o + 3]}; };
        Fwd f = [&](const Vec& x) {
            Sd l, rr;
            reconstruct(unpack(x, 0), unpack(x, 4), unpack(x, 8), x0, x1, x2, xl, xr, h_dry, l, rr);
            return Vec{l.h, l.u, l.v, l.b, rr.h, rr.u, rr.v, rr.b};
        };
        Rev rv = [&](const Vec& x, const Vec& w) {
            Sd mb{}, cb{}, pb{};
            reconstruct_rev(unpack(x, 0), unpack(x, 4), unpack(x, 8), x0, x1, x2, xl, xr, h_dry,
                            Sd{w[0], w[1], w[2], w[3]}, Sd{w[4], w[5], w[6], w[7]}, mb, cb, pb);
            return Vec{mb.h, mb.u, mb.v, mb.b, cb.h, cb.u, cb.v, cb.b, pb.h, pb.u, pb.v, pb.b};
        };
        for (int i = 0; i < 3000; ++i) {
            Vec x;
            for (int k = 0; k < 3; ++k) {
                const double h = (i % 4 == 0 && k == 2) ? uni(0, 5e-4) : uni(0.01, 3);
                x.insert(x.end(), {h, uni(-2, 2), uni(-2, 2), uni(-3, 0)});
            }
            sample("reconstruct", f, rv, x, r);
        }
        ok &= report("reconstruct", r);
    }
    {  // the tide's amplitude and phase
        Result r;
        Condition c{};
        c.n_constituents = 2;
        c.ramp = 3600.0;
        c.mean = 0.1;
        const double t = 2000.0;
        Fwd f = [&](const Vec& x) {
            Condition cc = c;
            for (int i = 0; i < 2; ++i)
                cc.c[i] = {x[2 * i], 2 * M_PI / (44712.0 + 3000.0 * i), x[2 * i + 1], 1.02, 1e-9,
                           3.0, 1e-7, 40.0};
            return Vec{tide_elevation(cc, t)};
        };
        Rev rv = [&](const Vec& x, const Vec& w) {
            Condition cc = c;
            for (int i = 0; i < 2; ++i)
                cc.c[i] = {x[2 * i], 2 * M_PI / (44712.0 + 3000.0 * i), x[2 * i + 1], 1.02, 1e-9,
                           3.0, 1e-7, 40.0};
            Vec gr(4, 0.0);
            tide_elevation_rev(cc, t, w[0], gr.data());
            return gr;
        };
        for (int i = 0; i < 300; ++i) sample("tide", f, rv, {uni(0.2, 2), uni(-3, 3), uni(0.1, 1), uni(-3, 3)}, r);
        ok &= report("tide", r);
    }
    std::printf(ok ? "all ok\n" : "FAILED\n");
    return ok ? 0 : 1;
}
