// dgswe_run with local time stepping: Simulation::run_with_callback's loop
// (src/simulation/runner.rs:347-478) on a Multirate integrator, as the
// reference's device backend runs it (gpu/src/swe2d.rs:4403-4660): per
// coarse step the element steps and depth flags come to the host, the
// planner (multirate.cpp) assigns levels and rates and orders the passes,
// and the device runs MultirateStepper::schedule (src/time/multirate.rs:
// 1249-1283): for every finest substep each stage over the elements whose
// rate reaches the substep's depth, with the faces they read, then the end
// of the substeps that end there.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/dgswe.h"
#include "device.hpp"
#include "handle.hpp"
#include "host_common.hpp"
#include "kernel_set.hpp"
#include "multirate.hpp"

using namespace dgswe;
using namespace dgswe::host;

namespace {

const double kLineLocalHeadroom = 1.0;       // LINE_LOCAL_HEADROOM (src/physics/builder.rs:148)
const double kSubcellCapDepthFactor = 100.0; // SUBCELL_CAP_DEPTH_FACTOR (src/solver/rhs/swe_2d.rs:2185)
const double kLandingSlack = 1e-9;

template <class T>
int dev_alloc(dgswe_handle* h, size_t n, T** out) {
    void* p = nullptr;
    CK(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)));
    h->allocations.push_back(p);
    *out = (T*)p;
    return DGSWE_OK;
}

// The planner for `levels` and the scheme's stages, and the device plan
int prepare(dgswe_handle* h, int levels, int n_stages) {
    if (!h->planner || h->planner_levels != levels || h->planner_stages != n_stages) {
        delete h->planner;
        h->planner = new MultiratePlanner(h->nb, h->nb_face, h->ops->face_node, h->n1, levels,
                                          n_stages);
        h->planner_levels = levels;
        h->planner_stages = n_stages;
        h->plan_uploaded = 0;
        h->dplan.memo_valid = false;
    }
    if (!h->ev_lts[0]) {
        CK(cudaEventCreate(&h->ev_lts[0]));
        CK(cudaEventCreate(&h->ev_lts[1]));
    }
    if (!h->d_level) {
        const size_t K = (size_t)h->K, E = h->h_edge_left.size(), B = h->h_bface.size();
        if (int s = dev_alloc(h, K, &h->d_level)) return s;
        if (int s = dev_alloc(h, kPlanStages * K, &h->d_rate)) return s;
        if (int s = dev_alloc(h, K, &h->d_flags)) return s;
        if (int s = dev_alloc(h, (kPlanStages + 1) * K, &h->d_order)) return s;
        if (int s = dev_alloc(h, kPlanStages * E, &h->d_edges)) return s;
        if (int s = dev_alloc(h, kPlanStages * B, &h->d_bfaces)) return s;
    }
    return DGSWE_OK;
}

// The planner's levels, rates and pass orders to the device, if new
int upload_plan(dgswe_handle* h, int n_stages) {
    MultiratePlanner& pl = *h->planner;
    if (h->plan_uploaded == pl.version()) return DGSWE_OK;
    h->dplan.memo_valid = false;  // the device planner's kept plan is overwritten
    pl.edge_lists(h->h_edge_left, h->h_edge_right, h->h_bface);
    const size_t K = (size_t)h->K, E = h->h_edge_left.size(), B = h->h_bface.size();
    cudaStream_t st = h->stream;
    CK(cudaMemcpyAsync(h->d_level, pl.level().data(), K, cudaMemcpyHostToDevice, st));
    for (int s = 0; s < n_stages; ++s) {
        CK(cudaMemcpyAsync(h->d_rate + s * K, pl.rate(s).data(), K, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(h->d_order + s * K, pl.order(s).data(), K * sizeof(int32_t),
                           cudaMemcpyHostToDevice, st));
        if (E)
            CK(cudaMemcpyAsync(h->d_edges + s * E, pl.edge_order(s).data(), E * sizeof(int32_t),
                               cudaMemcpyHostToDevice, st));
        if (B)
            CK(cudaMemcpyAsync(h->d_bfaces + s * B, pl.bface_order(s).data(), B * sizeof(int32_t),
                               cudaMemcpyHostToDevice, st));
    }
    CK(cudaMemcpyAsync(h->d_order + n_stages * K, pl.order(n_stages).data(), K * sizeof(int32_t),
                       cudaMemcpyHostToDevice, st));
    // the host vectors are read by the copies: wait before the planner changes them
    CK(cudaStreamSynchronize(st));
    h->plan_uploaded = pl.version();
    return DGSWE_OK;
}

// One coarse step of dt from t (MultirateStepper::schedule + step)
void coarse_step(dgswe_handle* h, const double (*sc)[4], int n, double t, double dt) {
    const MultiratePlanner& pl = *h->planner;
    const int L = pl.finest();
    const size_t K = (size_t)h->K, E = h->h_edge_left.size(), B = h->h_bface.size();
    const DevBuf& state = h->buf[DGSWE_STATE].view;
    const DevBuf& last = h->buf[n].view;
    const DevBuf& acc = h->buf[n + 1].view;
    cudaStream_t st = h->stream;
    for (int64_t p = 0; p < (int64_t)1 << L; ++p) {
        const int d = MultiratePlanner::depth(p, L);
        for (int s = 0; s < n; ++s) {
            LtsPass lp;
            lp.n = pl.count(s, d);
            if (lp.n == 0) continue;
            lp.list = h->d_order + s * K;
            lp.edges = h->d_edges + s * E;
            lp.n_edges = pl.edge_count(s, d);
            lp.bfaces = h->d_bfaces + s * B;
            lp.n_bfaces = pl.bface_count(s, d);
            lp.level = h->d_level;
            lp.rate = h->d_rate + s * K;
            lp.t = t;
            lp.dt = dt;
            lp.finest = L;
            lp.substep = (int)p;
            lp.depth = d;
            lp.last = s + 1 == n;
            lp.start = sc[s][0];
            lp.input = sc[s][1];
            lp.beta = sc[s][2];
            lp.c = sc[s][3];
            const DevBuf& in = s == 0 ? state : h->buf[s].view;
            const DevBuf& out = s + 1 < n ? h->buf[s + 1].view : last;
            h->ks->face_listed(h->n1, h->T, h->P, in, h->fb_h, h->fb_hu, h->fb_hv, h->ctl, lp, st);
            h->ks->stage_listed(h->n1, h->T, h->P, h->X, in, state, out, acc, h->fb_h, h->fb_hu,
                                h->fb_hv, h->ctl, lp.last ? kModeAccumulate : kModePost, lp, st);
        }
        // the substeps ending here
        LtsPass fin;
        const int next = MultiratePlanner::depth(p + 1, L);
        fin.list = h->d_order + n * K;
        fin.n = pl.count(n, next);
        h->ks->finish_listed(h->n1, h->T, h->P, acc, state, h->ctl, fin, st);
    }
}

}  // namespace

namespace dgswe {
namespace host {

int run_multirate(dgswe_handle* h, const dgswe_run_config* run, dgswe_callback callback,
                  void* user, dgswe_report* report) {
    std::memset(report, 0, sizeof(*report));
    std::snprintf(report->device, sizeof report->device, "%s", h->device_name.c_str());
    CK(cudaSetDevice(h->device));
    const auto wall0 = std::chrono::steady_clock::now();
    double sc[4][4];
    const int n = scheme_table(run->scheme, sc);
    for (int b = 1; b <= n + 1; ++b)
        if (int s = ensure_buffer(h, b)) return s;
    if (int s = prepare(h, run->levels, n)) return s;
    MultiratePlanner& pl = *h->planner;
    cudaStream_t st = h->stream;
    const int64_t K = h->K;

    // the device clock's flags only (the host keeps the time): clips carry on
    StepCtl& c = *h->h_ctl;
    long long clips0 = 0;
    CK(cudaMemcpy(&clips0, &h->ctl->clips, sizeof clips0, cudaMemcpyDeviceToHost));
    std::memset(&c, 0, sizeof c);
    c.clips = clips0;
    c.always = 1;
    c.active = 1;
    c.dt_bits = 0x7FF0000000000000ull;
    CK(cudaMemcpyAsync(h->ctl, &c, sizeof c, cudaMemcpyHostToDevice, st));
    h->ks->velocity(h->buf[DGSWE_STATE].view, h->n_values, h->P.h_min, st);
    // the stage values, the last stage's and the sums start as the state
    // (MultirateStepper::step, src/time/multirate.rs:1287-1293)
    for (int b = 1; b <= n + 1; ++b)
        CK(cudaMemcpyAsync(h->buf[b].base, h->buf[DGSWE_STATE].base,
                           5 * (size_t)h->n_values * sizeof(double), cudaMemcpyDeviceToDevice, st));
    if (int s = sync(h)) return s;

    const dgswe_form& f = h->form;
    const DtParams D = dt_params(f, run->cfl, run->scheme);
    const bool lines = f.has_line_local != 0 && h->n1 >= 2;
    const double d0 = !lines ? INFINITY
                             : (std::isinf(f.line_local_depth) && f.line_local_depth < 0.0
                                    ? -INFINITY
                                    : f.line_local_depth + kLineLocalHeadroom);
    const bool bounded = f.positivity_h_dry > 0.0;
    const double d1 = bounded ? kSubcellCapDepthFactor * f.positivity_h_dry : INFINITY;
    const double d2 = bounded ? f.positivity_h_dry : INFINITY;
    std::vector<double> hh, hu, hv;

    double t = run->t_start;
    int64_t n_steps = 0;
    double dt_min_used = INFINITY, dt_max_used = 0.0;
    const bool has_interval = run->interval > 0.0;
    unsigned long long callbacks_done = 0;
    auto next_callback = [&](unsigned long long k) {
        return run->t_start + (double)(k + 1) * run->interval;
    };
    auto call = [&](double time) -> int {
        if (!callback) return DGSWE_OK;
        hh.resize(h->n_values);
        hu.resize(h->n_values);
        hv.resize(h->n_values);
        if (int s = dgswe_download(h, DGSWE_STATE, hh.data(), hu.data(), hv.data(), h->n_values))
            return s;
        callback(user, time, hh.data(), hu.data(), hv.data(), h->n_values);
        return DGSWE_OK;
    };
    dgswe_multirate_stats& stats = h->mr_stats;
    std::memset(&stats, 0, sizeof stats);
    auto finish = [&](int status, const char* msg) {
        long long clips = 0;
        cudaMemcpy(&clips, &h->ctl->clips, sizeof clips, cudaMemcpyDeviceToHost);
        report->success = status == DGSWE_OK;
        report->final_time = t;
        report->n_steps = n_steps;
        report->dt_min_used = dt_min_used;
        report->dt_max_used = dt_max_used;
        report->negative_depth_clips = clips;
        report->wall_time =
            std::chrono::duration<double>(std::chrono::steady_clock::now() - wall0).count();
        std::snprintf(report->message, sizeof report->message, "%s", msg);
        if (status != DGSWE_OK) h->error = msg;
        return status;
    };
    if (int s = call(t)) return s;
    char msg[256];
    while (t < run->t_end) {
        if (run->max_steps > 0 && n_steps >= run->max_steps) {
            std::snprintf(msg, sizeof msg, "Maximum step limit (%lld) reached",
                          (long long)run->max_steps);
            return finish(DGSWE_ERR_MAX_STEPS, msg);
        }
        if (run->stop && *run->stop) {
            std::snprintf(msg, sizeof msg, "Stopped at t = %.1f s", t);
            return finish(DGSWE_ERR_STOPPED, msg);
        }
        const double target =
            has_interval ? std::fmin(next_callback(callbacks_done), run->t_end) : run->t_end;
        // the element steps and depth flags of the coarse step's start
        const DevBuf& q = h->buf[DGSWE_STATE].view;
        h->ks->dt(h->n1, h->T, h->P, q, D, h->dt_el, h->ctl, &h->ctl->always, st);
        h->ks->depth_flags(q.h, K, h->nn, d0, d1, d2, h->d_flags, st);
        // the plan, made on the device from the element steps and flags
        // (multirate_plan.cu): the coarse step's levels, rates and pass
        // orders stay there, its counts come to the host
        const auto plan0 = std::chrono::steady_clock::now();
        const uint64_t version0 = pl.version();
        double fitted = 0.0, dt = 0.0;
        if (int s = device_plan(h, n, lines, bounded, run->dt_max, target - t, fitted, dt))
            return s;
        if (run->dt_max > 0.0) dt = std::fmin(dt, run->dt_max);
        if (run->dt_min > 0.0 && dt < run->dt_min) {
            std::snprintf(msg, sizeof msg, "Time step (%.2e) below minimum (%.2e)", dt,
                          run->dt_min);
            return finish(DGSWE_ERR_DT_MIN, msg);
        }
        dt_min_used = std::fmin(dt_min_used, dt);
        dt_max_used = std::fmax(dt_max_used, dt);
        dt = std::fmin(dt, fitted);
        const bool landed = t + dt * (1.0 + kLandingSlack) >= target;
        if (landed) dt = target - t;
        stats.plans += pl.version() != version0 ? 1 : 0;
        stats.plan_seconds +=
            std::chrono::duration<double>(std::chrono::steady_clock::now() - plan0).count();
        CK(cudaEventRecord(h->ev_lts[0], st));
        coarse_step(h, sc, n, t, dt);
        CK(cudaEventRecord(h->ev_lts[1], st));
        // MultirateStepper::count_step (src/time/multirate.rs:1319-1331)
        stats.steps += 1;
        stats.element_evaluations += pl.evaluations_per_step();
        stats.global_evaluations += (int64_t)n * K * ((int64_t)1 << pl.finest());
        stats.finest_level = std::max(stats.finest_level, pl.finest());
        stats.model_seconds += dt;
        stats.ideal_evaluations += (double)n * pl.inverse_dt_sum() * dt;
        stats.level_evaluations += (double)pl.level_evaluations_per_step();
        stats.line_local_elements += pl.n_line_local();
        t = landed ? target : t + dt;
        n_steps += 1;
        int nonfinite = 0;
        CK(cudaMemcpyAsync(&nonfinite, &h->ctl->nonfinite, sizeof nonfinite,
                           cudaMemcpyDeviceToHost, st));
        if (int s = sync(h)) return s;
        float pass_ms = 0.0f;
        CK(cudaEventElapsedTime(&pass_ms, h->ev_lts[0], h->ev_lts[1]));
        stats.device_seconds += 1e-3 * pass_ms;
        if (nonfinite) {
            std::snprintf(msg, sizeof msg, "The state is not finite at t = %.1f s: it has blown up",
                          t);
            return finish(DGSWE_ERR_NONFINITE, msg);
        }
        if (has_interval) {
            if (t >= next_callback(callbacks_done)) {
                if (int s = call(t)) return s;
                callbacks_done += 1;
            }
        } else {
            if (int s = call(t)) return s;
        }
    }
    return finish(DGSWE_OK, "");
}

}  // namespace host
}  // namespace dgswe

extern "C" {

int dgswe_begin_coarse_step(dgswe_handle* h, int32_t n_stages, const uint8_t* levels,
                            const uint8_t* rates) {
    if (!h) return DGSWE_ERR_INVALID;
    if ((n_stages != 3 && n_stages != 4) || !levels || !rates)
        return fail(h, DGSWE_ERR_INVALID, "begin_coarse_step: %d stages", n_stages);
    int finest = 0;
    for (int64_t k = 0; k < h->K; ++k) finest = std::max(finest, (int)levels[k]);
    if (finest > kMaxLevels)
        return fail(h, DGSWE_ERR_INVALID, "begin_coarse_step: level %d above %d", finest,
                    kMaxLevels);
    // a stage's rate lies between the element's level and the finest
    // (MultirateStepper::rates)
    for (int64_t k = 0; k < h->K; ++k) {
        for (int s = 0; s < n_stages; ++s)
            if (rates[s * h->K + k] < levels[k] || rates[s * h->K + k] > finest)
                return fail(h, DGSWE_ERR_INVALID,
                            "begin_coarse_step: element %lld's stage %d rate %d (level %d)",
                            (long long)k, s, rates[s * h->K + k], levels[k]);
    }
    CK(cudaSetDevice(h->device));
    if (int s = prepare(h, kMaxLevels, n_stages)) return s;
    h->planner->set_plan(levels, rates);
    return upload_plan(h, n_stages);
}

int dgswe_stage_where(dgswe_handle* h, const dgswe_multirate_stage* p) {
    if (!h) return DGSWE_ERR_INVALID;
    if (!h->planner || h->plan_uploaded != h->planner->version())
        return fail(h, DGSWE_ERR_INVALID, "stage_where: no coarse step begun");
    const MultiratePlanner& pl = *h->planner;
    const int n = h->planner_stages;
    if (!p || p->stage < 0 || p->stage >= n || p->finest != pl.finest() || p->depth < 0 ||
        p->depth > p->finest || p->substep < 0 || p->substep >= (1 << p->finest))
        return fail(h, DGSWE_ERR_INVALID, "stage_where: stage %d, finest %d, depth %d",
                    p ? p->stage : -1, p ? p->finest : -1, p ? p->depth : -1);
    for (int id : {p->base, p->input_buffer, p->out})
        if (id < 0 || id >= DGSWE_N_BUFFERS)
            return fail(h, DGSWE_ERR_INVALID, "stage_where: buffer %d", id);
    if (p->last && (p->acc < 0 || p->acc >= DGSWE_N_BUFFERS))
        return fail(h, DGSWE_ERR_INVALID, "stage_where: accumulation buffer %d", p->acc);
    if (p->out == p->input_buffer)
        return fail(h, DGSWE_ERR_INVALID, "stage_where: out must differ from input");
    CK(cudaSetDevice(h->device));
    for (int id : {p->base, p->input_buffer, p->out, p->last ? p->acc : p->out})
        if (int s = ensure_buffer(h, id)) return s;
    const size_t K = (size_t)h->K, E = h->h_edge_left.size(), B = h->h_bface.size();
    LtsPass lp;
    lp.n = pl.count(p->stage, p->depth);
    lp.list = h->d_order + p->stage * K;
    lp.edges = h->d_edges + p->stage * E;
    lp.n_edges = pl.edge_count(p->stage, p->depth);
    lp.bfaces = h->d_bfaces + p->stage * B;
    lp.n_bfaces = pl.bface_count(p->stage, p->depth);
    lp.level = h->d_level;
    lp.rate = h->d_rate + p->stage * K;
    lp.t = p->t;
    lp.dt = p->dt;
    lp.finest = p->finest;
    lp.substep = p->substep;
    lp.depth = p->depth;
    lp.last = p->last ? 1 : 0;
    lp.start = p->start;
    lp.input = p->input;
    lp.beta = p->beta;
    lp.c = p->c;
    if (lp.n > 0) {
        const DevBuf& in = h->buf[p->input_buffer].view;
        h->ks->face_listed(h->n1, h->T, h->P, in, h->fb_h, h->fb_hu, h->fb_hv, h->ctl, lp,
                           h->stream);
        h->ks->stage_listed(h->n1, h->T, h->P, h->X, in, h->buf[p->base].view,
                            h->buf[p->out].view, h->buf[p->last ? p->acc : p->out].view, h->fb_h,
                            h->fb_hu, h->fb_hv, h->ctl, lp.last ? kModeAccumulate : kModePost, lp,
                            h->stream);
    }
    CK(cudaGetLastError());
    return sync(h);
}

int dgswe_finish_where(dgswe_handle* h, int32_t acc, int32_t depth) {
    if (!h) return DGSWE_ERR_INVALID;
    if (!h->planner || h->plan_uploaded != h->planner->version())
        return fail(h, DGSWE_ERR_INVALID, "finish_where: no coarse step begun");
    const MultiratePlanner& pl = *h->planner;
    if (acc <= DGSWE_STATE || acc >= DGSWE_N_BUFFERS || depth < 0 || depth > pl.finest())
        return fail(h, DGSWE_ERR_INVALID, "finish_where: buffer %d, depth %d", acc, depth);
    CK(cudaSetDevice(h->device));
    if (int s = ensure_buffer(h, acc)) return s;
    LtsPass fin;
    fin.list = h->d_order + h->planner_stages * (size_t)h->K;
    fin.n = pl.count(h->planner_stages, depth);
    h->ks->finish_listed(h->n1, h->T, h->P, h->buf[acc].view, h->buf[DGSWE_STATE].view, h->ctl,
                         fin, h->stream);
    CK(cudaGetLastError());
    return sync(h);
}

int dgswe_depth_flags(dgswe_handle* h, int32_t buffer, double d0, double d1, double d2,
                      uint8_t* flags) {
    if (!h) return DGSWE_ERR_INVALID;
    if (buffer < 0 || buffer >= DGSWE_N_BUFFERS || !flags)
        return fail(h, DGSWE_ERR_INVALID, "depth_flags: buffer %d", buffer);
    CK(cudaSetDevice(h->device));
    if (int s = ensure_buffer(h, buffer)) return s;
    if (int s = prepare(h, h->planner ? h->planner_levels : kMaxLevels,
                        h->planner ? h->planner_stages : 3))
        return s;
    h->ks->depth_flags(h->buf[buffer].view.h, h->K, h->nn, d0, d1, d2, h->d_flags, h->stream);
    CK(cudaMemcpyAsync(flags, h->d_flags, (size_t)h->K, cudaMemcpyDeviceToHost, h->stream));
    return sync(h);
}

}  // extern "C"

extern "C" int dgswe_multirate_stats_get(const dgswe_handle* h, dgswe_multirate_stats* out) {
    if (!h || !out) return DGSWE_ERR_INVALID;
    *out = h->mr_stats;
    return DGSWE_OK;
}
