// Host-side pieces shared by one mesh's handle (api.cu) and the ensemble
// (ensemble.cu): form checks, the SSP schemes' tables, the dt parameters and
// the device physics constants of a form.
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/dgswe.h"
#include "device.hpp"
#include "setup.hpp"

namespace dgswe {

// SspScheme::stages (src/time/integrator.rs:239-263): (start, input, beta, c)
inline int scheme_table(int scheme, double st[4][4]) {
    if (scheme == DGSWE_SSP_RK43) {
        const double t[4][4] = {{1.0, 0.0, 0.5, 0.0},
                                {0.0, 1.0, 0.5, 0.5},
                                {2.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0, 1.0},
                                {0.0, 1.0, 0.5, 0.5}};
        std::memcpy(st, t, sizeof t);
        return 4;
    }
    const double t[3][4] = {{1.0, 0.0, 1.0, 0.0}, {0.75, 0.25, 0.25, 1.0},
                            {1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0, 0.5}};
    std::memcpy(st, t, sizeof t);
    return 3;
}

// PositivityBound::new (src/solver/rhs/swe_2d.rs:2194-2212) with the linear
// limits of linear_cfl_swe_2d / linear_cfl_subcells_swe_2d (swe_2d.rs:1263-1300)
inline DtParams dt_params(const dgswe_form& f, double cfl, int scheme) {
    DtParams d{};
    d.cfl = cfl;
    d.positivity = f.positivity_h_dry > 0.0 ? 1 : 0;
    const int order = f.order;
    const double n = (double)order;
    const double ssp = scheme == DGSWE_SSP_RK43 ? 2.0 : 1.0;
    const double bound = ssp * ((2.0 * n + 1.0) / (2.0 * n * (n + 1.0)));
    static const double lin3[4] = {1.6, 1.04, 0.73, 0.56}, lin43[4] = {2.2, 1.51, 1.15, 0.93};
    static const double sub3[4] = {0.94, 0.65, 0.47, 0.36}, sub43[4] = {1.5, 1.1, 0.97, 0.75};
    const double lin = scheme == DGSWE_SSP_RK43 ? lin43[order - 1] : lin3[order - 1];
    const double sub = scheme == DGSWE_SSP_RK43 ? sub43[order - 1] : sub3[order - 1];
    d.bound_cfl = bound;
    d.max_cfl = std::fmax(bound, 0.9 * lin);
    d.max_cfl_subcells = std::fmax(bound, 0.9 * sub);
    d.shallow = 100.0 * f.positivity_h_dry;
    return d;
}

inline int check_form(const dgswe_form* f, std::string& why) {
    if (!f) return why = "form is NULL", DGSWE_ERR_INVALID;
    if (f->abi_version != DGSWE_ABI_VERSION) return why = "ABI version mismatch", DGSWE_ERR_INVALID;
    if (f->order < 1 || f->order > 4) return why = "order must be 1..4", DGSWE_ERR_UNSUPPORTED;
    if (f->n_elements <= 0 || f->n_vertices <= 0 || !f->vertices || !f->elements)
        return why = "the mesh is empty", DGSWE_ERR_INVALID;
    if (f->n_elements >= (1ll << 40)) return why = "too many elements", DGSWE_ERR_INVALID;
    if (f->n_periodic < 0 || (f->n_periodic > 0 && !f->periodic))
        return why = "periodic pairs without data", DGSWE_ERR_INVALID;
    if (f->formulation < DGSWE_WET_DRY || f->formulation > DGSWE_ENTROPY_CONSERVATIVE)
        return why = "unknown formulation", DGSWE_ERR_UNSUPPORTED;
    if (!(f->g > 0.0) || !(f->h_min >= 0.0)) return why = "g and h_min", DGSWE_ERR_INVALID;
    if (f->friction < DGSWE_FRICTION_NONE || f->friction > DGSWE_FRICTION_MANNING_NODES)
        return why = "unknown friction law", DGSWE_ERR_UNSUPPORTED;
    if (f->friction == DGSWE_FRICTION_MANNING_NODES && !f->manning_n_nodes)
        return why = "per-node Manning without data", DGSWE_ERR_INVALID;
    if (f->has_wet_dry && !(f->wet_dry_h_dry > 0.0 && f->wet_dry_relaxation_time > 0.0))
        return why = "the wet/dry depth and relaxation time must be positive", DGSWE_ERR_INVALID;
    if (f->relaxation) {
        const dgswe_relaxation& r = *f->relaxation;
        const dgswe_parent_series* p = r.parent;
        if (!p || p->n_slots <= 0 || p->n_times <= 0 || !p->times || !p->values ||
            !p->slot_of_node || !r.weight || !(r.rate >= 0.0) || !(r.wet_depth >= 0.0))
            return why = "a relaxation band without its data", DGSWE_ERR_INVALID;
        if (p->n_slots >= (1ll << 31) || p->n_times >= (1ll << 31))
            return why = "a relaxation band too large", DGSWE_ERR_INVALID;
        for (int64_t i = 1; i < p->n_times; ++i)
            if (!(p->times[i] > p->times[i - 1]))
                return why = "parent snapshot times must increase", DGSWE_ERR_INVALID;
    }
    if (f->atmosphere) {
        const dgswe_atmosphere& a = *f->atmosphere;
        if (a.n_times <= 0 || !a.times || !a.values)
            return why = "an atmosphere without its snapshots", DGSWE_ERR_INVALID;
        if (a.n_times >= (1ll << 31)) return why = "too many weather snapshots", DGSWE_ERR_INVALID;
        for (int64_t i = 1; i < a.n_times; ++i)
            if (!(a.times[i] > a.times[i - 1]))
                return why = "weather snapshot times must increase", DGSWE_ERR_INVALID;
        if (a.drag < DGSWE_DRAG_CONSTANT || a.drag > DGSWE_DRAG_YELLAND_TAYLOR)
            return why = "unknown drag coefficient", DGSWE_ERR_UNSUPPORTED;
        if (!(a.rho_water > 0.0) || !(a.rho_air >= 0.0) || !std::isfinite(a.epoch_unix))
            return why = "the atmosphere's densities and epoch", DGSWE_ERR_INVALID;
    }
    if (f->n_boundaries < 0 || f->n_boundaries > kMaxConditions ||
        (f->n_boundaries > 0 && !f->boundaries))
        return why = "boundary conditions", DGSWE_ERR_INVALID;
    for (int b = 0; b < f->n_boundaries; ++b) {
        const dgswe_boundary& c = f->boundaries[b];
        if (c.kind != DGSWE_BC_WALL && c.kind != DGSWE_BC_CHARACTERISTIC &&
            c.kind != DGSWE_BC_NODE_TIDES && c.kind != DGSWE_BC_PARENT)
            return why = "a boundary condition without a device form", DGSWE_ERR_UNSUPPORTED;
        if (c.raise && c.kind == DGSWE_BC_WALL)
            return why = "a wall raised by the inverse barometer", DGSWE_ERR_INVALID;
        if (c.raise && !f->atmosphere)
            return why = "an inverse-barometer raise without an atmosphere", DGSWE_ERR_INVALID;
        if (c.raise && !std::isfinite(c.raise_factor))
            return why = "the raise factor", DGSWE_ERR_INVALID;
        if (c.kind == DGSWE_BC_PARENT) {
            const dgswe_parent_series* p = c.parent;
            if (!p || p->n_slots <= 0 || p->n_times <= 0 || !p->positions || !p->times ||
                !p->values)
                return why = "a parent series without its data", DGSWE_ERR_INVALID;
            if (p->n_slots >= (1ll << 31) || p->n_times >= (1ll << 31))
                return why = "a parent series too large", DGSWE_ERR_INVALID;
            for (int64_t i = 1; i < p->n_times; ++i)
                if (!(p->times[i] > p->times[i - 1]))
                    return why = "parent snapshot times must increase", DGSWE_ERR_INVALID;
            if (p->velocity && p->max_transport_ratio > 0.0 && p->max_transport_ratio < 1.0)
                return why = "a transport ratio limit below 1", DGSWE_ERR_INVALID;
            bool any = p->on_boundary == nullptr;
            for (int64_t q = 0; !any && q < p->n_slots; ++q) any = p->on_boundary[q] != 0;
            if (!any) return why = "a parent series without boundary slots", DGSWE_ERR_INVALID;
            continue;
        }
        if (c.kind == DGSWE_BC_NODE_TIDES) {
            const dgswe_node_tides* t = c.node_tides;
            if (!t || t->n_constituents < 0 || t->n_constituents > 256 || t->n_slots <= 0 ||
                !t->positions || !t->coefficients ||
                (t->n_constituents > 0 && (!t->omega || !t->f_rate)))
                return why = "per-node tides without their data", DGSWE_ERR_INVALID;
            if (t->n_slots >= (1ll << 31)) return why = "too many tide slots", DGSWE_ERR_INVALID;
            if (t->velocity && t->max_transport_ratio > 0.0 && t->max_transport_ratio < 1.0)
                return why = "a transport ratio limit below 1", DGSWE_ERR_INVALID;
            continue;
        }
        if (c.n_constituents < 0 || c.n_constituents > kMaxConstituents ||
            (c.n_constituents > 0 && !c.constituents))
            return why = "tide constituents", DGSWE_ERR_INVALID;
        for (int i = 0; i < c.n_constituents; ++i)
            if (!(c.constituents[i].period > 0.0)) return why = "a tide period", DGSWE_ERR_INVALID;
    }
    if (f->numerics != DGSWE_NUMERICS_FAST && f->numerics != DGSWE_NUMERICS_EXACT)
        return why = "unknown numerics", DGSWE_ERR_INVALID;
    return DGSWE_OK;
}

// A boundary condition's device form; TidalConstituent::angular_frequency
// (src/boundary/tidal.rs:40-43) for each constituent
inline Condition make_condition(const dgswe_boundary& in) {
    Condition c{};
    c.kind = in.kind;
    c.elevation_only = in.elevation_only;
    c.wall_h_min = in.wall_h_min;
    c.mean = in.mean_elevation;
    c.ramp = in.ramp_duration;
    c.raise = in.kind != DGSWE_BC_WALL && in.raise ? 1 : 0;
    c.raise_factor = c.raise ? in.raise_factor : 0.0;
    if (in.kind == DGSWE_BC_NODE_TIDES) {
        // the tables' offsets are the handle's (nt_omega0, nt_slot0, nt_coef0)
        const dgswe_node_tides& t = *in.node_tides;
        c.ramp = t.ramp_duration;
        c.nt_n = t.n_constituents;
        c.nt_velocity = t.velocity ? 1 : 0;
        c.nt_use_mean = t.use_mean && t.mean ? 1 : 0;
        c.nt_max_ratio = t.max_transport_ratio;
        return c;
    }
    if (in.kind == DGSWE_BC_PARENT) {
        // the tables' offsets are the handle's (nt_slot0, pt_time0, pt_val0)
        const dgswe_parent_series& p = *in.parent;
        c.ramp = p.ramp_duration;
        c.nt_velocity = p.velocity ? 1 : 0;
        c.nt_max_ratio = p.max_transport_ratio;
        c.pt_n_times = (int)p.n_times;
        c.pt_cubic = p.cubic ? 1 : 0;
        c.pt_reference_level = p.reference_level;
        return c;
    }
    c.n_constituents = in.n_constituents;
    for (int i = 0; i < in.n_constituents; ++i) {
        const dgswe_tide_constituent& k = in.constituents[i];
        c.c[i] = {k.amplitude, 2.0 * M_PI / k.period, k.phase, k.f,
                  k.f_rate,    k.u_deg,                k.u_rate_deg, k.v0_deg};
    }
    return c;
}

// The device physics of a form, without its boundary conditions, and the
// subcell bounds of its operators
inline void fill_physics(const dgswe_form& f, const Operators& ops, bool coriolis_field,
                         Physics& P, StageExtra& X) {
    P.order = ops.order;  // the operators' order (an ensemble group's, not member 0's)
    P.n1 = ops.n1;
    P.nn = ops.nn;
    P.formulation = f.formulation;
    P.g = f.g;
    P.h_min = f.h_min;
    P.sqrt_g = std::sqrt(f.g);  // correctly rounded, as the device's sqrt
    P.half_g = 0.5 * f.g;
    P.two_g = 2.0 * f.g;
    P.subcell_depth = f.subcell_depth;
    P.subcell_h_dry = f.subcell_h_dry;
    P.has_bed = f.bathymetry ? 1 : 0;
    P.has_wet_dry = f.has_wet_dry ? 1 : 0;
    P.h_dry = f.wet_dry_h_dry;
    P.relaxation_time = f.wet_dry_relaxation_time;
    P.max_velocity = f.wet_dry_max_velocity;
    P.friction = f.friction;
    P.g_n2 = f.friction_g * f.manning_n * f.manning_n;
    P.manning_h_min = f.manning_h_min;
    P.has_coriolis = f.has_coriolis ? 1 : 0;
    P.coriolis_field = coriolis_field ? 1 : 0;
    P.f0 = f.coriolis_f0;
    for (int i = 0; i < ops.n1; ++i) {
        P.x[i] = ops.x[i];
        P.w[i] = ops.w[i];
    }
    for (int i = 0; i < ops.n1 * ops.n1; ++i) P.d[i] = ops.d[i];
    for (int face = 0; face < 4; ++face)
        for (int fi = 0; fi < ops.n1; ++fi) P.face_node[face][fi] = ops.face_node[face][fi];
    // subcell bounds as the reference sums them (swe_2d_split_form.rs:968-990)
    double x_left = -1.0;
    for (int a = 0; a < ops.n1; ++a) {
        const double x_right = x_left + ops.w[a];
        X.xl[a] = x_left;
        X.xr[a] = x_right;
        X.inv_w[a] = 1.0 / ops.w[a];
        x_left = x_right;
    }
}

// The owned pairs of a schedule as the device reads them (a, c, dir, pa, pc)
inline std::vector<int8_t> owned_table(const PairSchedule& sched) {
    std::vector<int8_t> owned;
    for (const PairSlot& p : sched.owned) {
        owned.push_back(p.a);
        owned.push_back(p.c);
        owned.push_back(p.dir);
        owned.push_back(p.pa);
        owned.push_back(p.pc);
    }
    return owned;
}

// Per owned pair slot, its two nodes' accumulation coefficients and their
// halves: [slot][coef of a, coef of c, coef of a / 2, coef of c / 2] (the
// adjoint's pair path, which forms both products at the owner)
inline std::vector<double> pair_coef_table(const PairSchedule& sched) {
    const int na = 2 * (sched.n1 - 1);
    std::vector<double> pc(sched.owned.size() * 4, 0.0);
    for (int i = 0; i < sched.nn; ++i)
        for (int q = 0; q < na; ++q) {
            const int sl = sched.accum_slot[(size_t)i * na + q];
            const int side = sched.owned[sl].a == i ? 0 : 1;
            const double c = sched.accum_coef[(size_t)i * na + q];
            pc[(size_t)sl * 4 + side] = c;
            pc[(size_t)sl * 4 + 2 + side] = 0.5 * c;
        }
    return pc;
}

// The ready lists of a state uploaded in `chunks` element chunks of
// ⌈K/chunks⌉ (dgswe_step_host): an element's dt pass reads its nodes and its
// face neighbours' face nodes, so it is ready with the last of their chunks;
// an interior edge with the later of its two elements' chunks; a boundary
// face with its element's. Each list in index order; off[c]..off[c+1] is
// chunk c's part. nb[k][f]: the neighbour across face f, −1 on the boundary;
// edge_left/right and bface: element·4 + face.
struct ReadyLists {
    std::vector<int32_t> elems, edges, bfaces;
    std::vector<int64_t> elem_off, edge_off, bface_off;  // chunks + 1 each
};

inline ReadyLists ready_lists(int64_t K, int chunks, const std::vector<std::array<int64_t, 4>>& nb,
                              const std::vector<int64_t>& edge_left,
                              const std::vector<int64_t>& edge_right,
                              const std::vector<int64_t>& bface) {
    const int64_t per = std::max<int64_t>(1, (K + chunks - 1) / chunks);
    auto chunk = [&](int64_t k) { return (int)(k / per); };
    std::vector<std::vector<int32_t>> el(chunks), ed(chunks), bf(chunks);
    for (int64_t k = 0; k < K; ++k) {
        int c = chunk(k);
        for (int f = 0; f < 4; ++f)
            if (nb[k][f] >= 0) c = std::max(c, chunk(nb[k][f]));
        el[c].push_back((int32_t)k);
    }
    for (size_t e = 0; e < edge_left.size(); ++e)
        ed[std::max(chunk(edge_left[e] >> 2), chunk(edge_right[e] >> 2))].push_back((int32_t)e);
    for (size_t b = 0; b < bface.size(); ++b) bf[chunk(bface[b] >> 2)].push_back((int32_t)b);
    ReadyLists r;
    auto flatten = [&](std::vector<std::vector<int32_t>>& parts, std::vector<int32_t>& all,
                       std::vector<int64_t>& off) {
        off.assign(chunks + 1, 0);
        for (int c = 0; c < chunks; ++c) {
            off[c] = (int64_t)all.size();
            all.insert(all.end(), parts[c].begin(), parts[c].end());
        }
        off[chunks] = (int64_t)all.size();
    };
    flatten(el, r.elems, r.elem_off);
    flatten(ed, r.edges, r.edge_off);
    flatten(bf, r.bfaces, r.bface_off);
    return r;
}

}  // namespace dgswe
