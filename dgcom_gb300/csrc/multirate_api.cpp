// The level planner's C entry points (host only, no device): a form's mesh,
// the planner of multirate.cpp on it, and its plan for given element steps.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/dgswe.h"
#include "host_common.hpp"
#include "multirate.hpp"
#include "setup.hpp"

struct dgswe_planner {
    dgswe::MultiratePlanner* p = nullptr;
    int n_stages = 0;
    int64_t K = 0;
    ~dgswe_planner() { delete p; }
};

extern "C" {

int dgswe_planner_create(const dgswe_form* form, int32_t max_levels, int32_t scheme,
                         dgswe_planner** out) {
    if (!out) return DGSWE_ERR_INVALID;
    *out = nullptr;
    std::string why;
    if (int s = dgswe::check_form(form, why)) return s;
    if (max_levels < 0 || max_levels > DGSWE_MAX_LEVELS) return DGSWE_ERR_INVALID;
    if (scheme != DGSWE_SSP_RK3 && scheme != DGSWE_SSP_RK43) return DGSWE_ERR_INVALID;
    dgswe::Operators ops(form->order);
    dgswe::Topology topo;
    if (!dgswe::build_topology(*form, topo).empty()) return DGSWE_ERR_INVALID;
    std::vector<std::array<int64_t, 4>> nb((size_t)topo.n_elements);
    std::vector<std::array<int8_t, 4>> nb_face((size_t)topo.n_elements);
    for (int64_t k = 0; k < topo.n_elements; ++k)
        for (int f = 0; f < 4; ++f) {
            nb[k][f] = topo.link[k][f].element;
            nb_face[k][f] = (int8_t)topo.link[k][f].face;
        }
    auto* pl = new dgswe_planner();
    pl->n_stages = scheme == DGSWE_SSP_RK43 ? 4 : 3;
    pl->K = topo.n_elements;
    pl->p = new dgswe::MultiratePlanner(std::move(nb), std::move(nb_face), ops.face_node, ops.n1,
                                        max_levels, pl->n_stages);
    *out = pl;
    return DGSWE_OK;
}

void dgswe_planner_destroy(dgswe_planner* planner) { delete planner; }

int dgswe_planner_assign(dgswe_planner* planner, const double* element_dt,
                         const uint8_t* line_local, double dt_cap, double landing,
                         dgswe_plan_result* result, uint8_t* levels, uint8_t* rates,
                         int32_t* order) {
    if (!planner || !element_dt) return DGSWE_ERR_INVALID;
    dgswe::MultiratePlanner& p = *planner->p;
    const double dt = p.assign(element_dt, line_local, dt_cap, landing);
    const int64_t K = planner->K;
    if (result) {
        result->dt = dt;
        result->stable_step = p.stable_step();
        result->finest = p.finest();
        result->evaluations = p.evaluations_per_step();
        result->level_evaluations = p.level_evaluations_per_step();
        result->inverse_dt_sum = p.inverse_dt_sum();
    }
    if (levels) std::copy(p.level().begin(), p.level().end(), levels);
    for (int s = 0; s < planner->n_stages; ++s) {
        if (rates) std::copy(p.rate(s).begin(), p.rate(s).end(), rates + s * K);
    }
    for (int j = 0; j <= planner->n_stages; ++j)
        if (order) std::copy(p.order(j).begin(), p.order(j).end(), order + j * K);
    return DGSWE_OK;
}

int dgswe_planner_spread(dgswe_planner* planner, uint8_t* levels, int32_t limit,
                         const uint8_t* line_local, uint8_t* rates) {
    if (!planner || !levels) return DGSWE_ERR_INVALID;
    dgswe::MultiratePlanner& p = *planner->p;
    const int64_t K = planner->K;
    const int nn = p.nn();
    std::vector<uint8_t> level(levels, levels + K);
    if (limit) {
        p.limit_level_jumps(level);
        std::copy(level.begin(), level.end(), levels);
    }
    std::vector<uint8_t> from, to, rate;
    if (line_local) {
        from.assign((size_t)K * nn, 0);
        for (int64_t k = 0; k < K; ++k)
            std::fill(from.begin() + k * nn, from.begin() + (k + 1) * nn, level[k]);
    }
    std::vector<uint8_t> prev = level;
    for (int s = 0; s < planner->n_stages; ++s) {
        if (line_local) {
            p.spread_lines(line_local, from, to, rate);
            std::swap(from, to);
        } else {
            p.spread_faces(prev, rate);
            prev = rate;
        }
        if (rates) std::copy(rate.begin(), rate.end(), rates + s * K);
    }
    return DGSWE_OK;
}

}  // extern "C"
