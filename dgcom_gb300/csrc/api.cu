// The C ABI (include/dgswe.h): a handle owns the device copy of a
// dgswe_form's physics, the solution buffers, the face-flux buffer and the
// step control block, and runs host-driven calls (one stage, one step, the
// RHS, the element steps) or a device-driven run whose steps are one CUDA
// graph each, the clock kept on the device.

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstddef>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/dgswe.h"
#include "device.hpp"
#include "handle.hpp"
#include "host_common.hpp"
#include "kernel_set.hpp"
#include "setup.hpp"

using namespace dgswe;

namespace dgswe {
namespace host {

int fail(dgswe_handle* h, int status, const char* fmt, ...) {
    char msg[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(msg, sizeof msg, fmt, ap);
    va_end(ap);
    if (h) h->error = msg;
    return status;
}


template <class T>
int upload_vec(dgswe_handle* h, const std::vector<T>& v, const T** out) {
    *out = nullptr;
    if (v.empty()) return DGSWE_OK;
    void* p = nullptr;
    CK(cudaMalloc(&p, v.size() * sizeof(T)));
    h->allocations.push_back(p);
    CK(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    *out = (const T*)p;
    return DGSWE_OK;
}

int ensure_buffer(dgswe_handle* h, int id) {
    DeviceBuffer& b = h->buf[id];
    if (b.base) return DGSWE_OK;
    void* p = nullptr;
    size_t n = (size_t)h->n_values;
    CK(cudaMalloc(&p, 5 * n * sizeof(double)));
    h->allocations.push_back(p);
    CK(cudaMemset(p, 0, 5 * n * sizeof(double)));
    b.base = (double*)p;
    b.view = {b.base, b.base + n, b.base + 2 * n, b.base + 3 * n, b.base + 4 * n};
    return DGSWE_OK;
}

bool valid_buffer(int id) { return id >= 0 && id < DGSWE_N_BUFFERS; }

int sync(dgswe_handle* h) {
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaGetLastError());
    return DGSWE_OK;
}

// Launch one stage: the face pass then the element stage
void launch_stage(dgswe_handle* h, int in, int base, int out, int acc, int slot, int mode,
                  int check_finite, const int* active) {
    h->ks->face(h->n1, h->T, h->P, h->buf[in].view, h->fb_h, h->fb_hu, h->fb_hv, h->ctl, slot,
                active, h->stream);
    h->ks->stage(h->n1, h->T, h->P, h->X, h->buf[in].view, h->buf[base].view, h->buf[out].view,
                 h->buf[acc].view, h->fb_h, h->fb_hu, h->fb_hv, h->ctl, slot, mode, check_finite,
                 active, h->stream);
}

int write_host_args(dgswe_handle* h, const StageArgs& a) {
    h->h_ctl->stage[kHostSlot] = a;
    CK(cudaMemcpyAsync(&h->ctl->stage[kHostSlot], &h->h_ctl->stage[kHostSlot], sizeof(StageArgs),
                       cudaMemcpyHostToDevice, h->stream));
    return DGSWE_OK;
}

const int* always(dgswe_handle* h) { return &h->ctl->always; }

// The device clock of a run from run->t_start towards `target`
int begin_run(dgswe_handle* h, const dgswe_run_config* run, double target) {
    double st[4][4];
    const int n_stages = scheme_table(run->scheme, st);
    StepCtl& c = *h->h_ctl;
    long long clips0 = 0;
    CK(cudaMemcpy(&clips0, &h->ctl->clips, sizeof clips0, cudaMemcpyDeviceToHost));
    std::memset(&c, 0, sizeof c);
    c.t = run->t_start;
    c.t_end = run->t_end;
    c.target = target;
    c.dt_max = run->dt_max;
    c.dt_min = run->dt_min;
    c.cfl = run->cfl;
    c.dt_min_used = INFINITY;
    c.dt_max_used = 0.0;
    c.dt_bits = 0x7FF0000000000000ull;
    c.max_steps = run->max_steps > 0 ? run->max_steps : 0;
    c.clips = clips0;
    c.always = 1;
    c.scheme_stages = n_stages;
    for (int s = 0; s < n_stages; ++s) {
        c.st_start[s] = st[s][0];
        c.st_input[s] = st[s][1];
        c.st_beta[s] = st[s][2];
        c.st_c[s] = st[s][3];
    }
    CK(cudaMemcpyAsync(h->ctl, &c, sizeof c, cudaMemcpyHostToDevice, h->stream));
    h->ks->velocity(h->buf[DGSWE_STATE].view, h->n_values, h->P.h_min, h->stream);
    return sync(h);
}

int ensure_dt_stream(dgswe_handle* h) {
    if (h->dt_stream) return DGSWE_OK;
    // the highest priority: the block scheduler starts the dt pass's blocks
    // before the face pass's, so the stage pass waiting for both is not
    // left waiting for the dt pass's tail
    int least = 0, greatest = 0;
    CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    CK(cudaStreamCreateWithPriority(&h->dt_stream, cudaStreamNonBlocking, greatest));
    CK(cudaEventCreateWithFlags(&h->dt_fork, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&h->dt_join, cudaEventDisableTiming));
    return DGSWE_OK;
}

// A step's dt pass and fit on the dt stream beside its first stage's face
// pass on the handle's stream: both read the step's start state; the face
// pass is held by the FP64 pipe and the dt pass by memory, so the one hides
// the other. The first stage's time comes from step_begin, so the face pass
// needs nothing from the fit. The stage pass that follows waits for both.
int dt_beside_first_face(dgswe_handle* h, const DtParams& D, const int* active) {
    CK(cudaEventRecord(h->dt_fork, h->stream));
    CK(cudaStreamWaitEvent(h->dt_stream, h->dt_fork, 0));
    h->ks->dt(h->n1, h->T, h->P, h->buf[DGSWE_STATE].view, D, nullptr, h->ctl, active,
              h->dt_stream);
    h->ks->step_dt(h->ctl, 1, h->dt_stream);
    CK(cudaEventRecord(h->dt_join, h->dt_stream));
    h->ks->face(h->n1, h->T, h->P, h->buf[DGSWE_STATE].view, h->fb_h, h->fb_hu, h->fb_hv, h->ctl,
                0, active, h->stream);
    CK(cudaStreamWaitEvent(h->stream, h->dt_join, 0));
    return DGSWE_OK;
}

int run_device_step_graph(dgswe_handle* h, int scheme, double cfl) {
    if (h->step_graph && h->graph_scheme == scheme && h->graph_cfl == cfl) return DGSWE_OK;
    if (h->step_graph) {
        cudaGraphExecDestroy(h->step_graph);
        h->step_graph = nullptr;
    }
    double st[4][4];
    const int n = scheme_table(scheme, st);
    for (int b = 1; b < n; ++b)
        if (int s = ensure_buffer(h, b)) return s;
    const DtParams D = dt_params(h->form, cfl, scheme);
    if (int s = ensure_dt_stream(h)) return s;
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    const int* active = &h->ctl->active;
    h->ks->step_begin(h->ctl, 1, h->stream);
    if (int s = dt_beside_first_face(h, D, active)) {
        cudaStreamEndCapture(h->stream, &graph);
        if (graph) cudaGraphDestroy(graph);
        return s;
    }
    for (int s = 0; s < n; ++s) {
        const int in = s == 0 ? DGSWE_STATE : s;
        const int out = s + 1 < n ? s + 1 : DGSWE_STATE;
        if (s == 0)  // its face pass ran beside the dt pass
            h->ks->stage(h->n1, h->T, h->P, h->X, h->buf[in].view, h->buf[DGSWE_STATE].view,
                         h->buf[out].view, h->buf[DGSWE_STATE].view, h->fb_h, h->fb_hu, h->fb_hv,
                         h->ctl, s, kModePost, s + 1 == n, active, h->stream);
        else
            launch_stage(h, in, DGSWE_STATE, out, DGSWE_STATE, s, kModePost, s + 1 == n, active);
    }
    h->ks->step_end(h->ctl, 1, h->stream);
    cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
    if (e != cudaSuccess) return fail(h, DGSWE_ERR_CUDA, "stream capture: %s", cudaGetErrorString(e));
    // the kernel nodes keep the priority of the stream they were captured on
    e = cudaGraphInstantiate(&h->step_graph, graph, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail(h, DGSWE_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
    h->graph_scheme = scheme;
    h->graph_cfl = cfl;
    return DGSWE_OK;
}

}  // namespace host
}  // namespace dgswe

using namespace dgswe::host;

extern "C" {

uint32_t dgswe_abi_version(void) { return DGSWE_ABI_VERSION; }

int dgswe_check_form(const dgswe_form* f, dgswe_form_info* info, char* message,
                     size_t message_size) {
    auto say = [&](int status, const std::string& why) {
        if (message && message_size > 0) std::snprintf(message, message_size, "%s", why.c_str());
        return status;
    };
    std::string why;
    if (int s = check_form(f, why)) return say(s, why);
    Operators ops(f->order);
    Topology topo;
    std::string err = build_topology(*f, topo);
    if (!err.empty()) return say(DGSWE_ERR_INVALID, err);
    std::vector<int32_t> tags, cond_index;
    for (int b = 0; b < f->n_boundaries; ++b) {
        tags.push_back(f->boundaries[b].tag);
        cond_index.push_back(b);
    }
    Tables t;
    err = build_tables(*f, ops, topo, tags, cond_index, t);
    if (!err.empty()) return say(DGSWE_ERR_INVALID, err);
    if (info) {
        std::memset(info, 0, sizeof(*info));
        info->n_elements = f->n_elements;
        info->n_interior_edges = (int64_t)t.edge_left.size();
        info->n_boundary_faces = (int64_t)t.bface.size();
        for (int64_t k = 0; k < topo.n_elements; ++k)
            for (int face = 0; face < 4; ++face) {
                const Link& L = topo.link[k][face];
                if (L.element >= 0 && L.left && !L.shared) info->n_periodic_edges += 1;
            }
        double min_j = INFINITY, area = 0.0;
        for (int64_t k = 0; k < topo.n_elements; ++k) {
            info->n_affine += t.affine[k];
            area += 1.0 / t.inv_area[k];
            for (int i = 0; i < ops.nn; ++i) min_j = std::fmin(min_j, 1.0 / t.jinv[k * ops.nn + i]);
        }
        info->min_jacobian = min_j;
        info->area = area;
        double sum = 0.0;
        for (const auto* v : {&t.bed, &t.jinv, &t.pair_hm, &t.gdb, &t.contra, &t.lift_scale,
                              &t.outer_dist, &t.mass, &t.inv_area, &t.weight_ratio, &t.dtm_own,
                              &t.dtm_face, &t.edge_geo, &t.bface_geo})
            for (double x : *v) sum += x;
        info->table_checksum = sum;
    }
    return say(DGSWE_OK, "");
}

const char* dgswe_status_string(int status) {
    switch (status) {
        case DGSWE_OK: return "ok";
        case DGSWE_ERR_INVALID: return "invalid input";
        case DGSWE_ERR_CUDA: return "CUDA error";
        case DGSWE_ERR_NONFINITE: return "the state is not finite";
        case DGSWE_ERR_DT_MIN: return "time step below the minimum";
        case DGSWE_ERR_MAX_STEPS: return "step limit reached";
        case DGSWE_ERR_STOPPED: return "stopped";
        case DGSWE_ERR_UNSUPPORTED: return "unsupported physics";
        case DGSWE_ERR_NO_DEVICE: return "no CUDA device";
        default: return "unknown status";
    }
}

const char* dgswe_last_error(const dgswe_handle* h) { return h ? h->error.c_str() : ""; }

int64_t dgswe_n_values(const dgswe_handle* h) { return h ? h->n_values : 0; }

int64_t dgswe_negative_depth_clips(const dgswe_handle* h) {
    if (!h) return 0;
    long long clips = 0;
    if (cudaMemcpy(&clips, &h->ctl->clips, sizeof clips, cudaMemcpyDeviceToHost) != cudaSuccess)
        return -1;
    return clips;
}

}  // extern "C"

namespace {

// Boundary data per node (DGSWE_BC_NODE_TIDES, DGSWE_BC_PARENT): the
// conditions' constituents and constants, or snapshot times and series,
// back to back, and every boundary face node's slot: the one slot_of_node
// gives its flat node, else the nearest forced node (BoundaryTides::slot_of,
// src/boundary/tidal_atlas.rs:1026-1045; OceanModelState::slot_of,
// src/boundary/ocean_nesting.rs:543-562)
bool per_node(const dgswe_boundary& b) {
    return b.kind == DGSWE_BC_NODE_TIDES || b.kind == DGSWE_BC_PARENT;
}

int boundary_node_tables(dgswe_handle* h, const dgswe_form& f, const Operators& ops,
                     const Topology& topo, const Tables& t) {
    bool any = false;
    for (int b = 0; b < f.n_boundaries; ++b) any = any || per_node(f.boundaries[b]);
    if (!any) return DGSWE_OK;
    std::vector<double> omega, frate, coef, mean, depth, ptimes;
    std::vector<float> pvalues;
    std::vector<int64_t> slot0(f.n_boundaries, 0);
    for (int b = 0; b < f.n_boundaries; ++b) {
        if (f.boundaries[b].kind == DGSWE_BC_PARENT) {
            const dgswe_parent_series& ps = *f.boundaries[b].parent;
            Condition& c = h->P.cond[b];
            c.nt_slot0 = slot0[b] = (int64_t)depth.size();
            c.pt_time0 = (int64_t)ptimes.size();
            c.pt_val0 = (int64_t)pvalues.size();
            ptimes.insert(ptimes.end(), ps.times, ps.times + ps.n_times);
            pvalues.insert(pvalues.end(), ps.values, ps.values + (size_t)ps.n_slots * ps.n_times * 3);
            for (int64_t q = 0; q < ps.n_slots; ++q) {
                mean.push_back(0.0);
                depth.push_back(ps.parent_depth ? ps.parent_depth[q] : NAN);
            }
            continue;
        }
        if (f.boundaries[b].kind != DGSWE_BC_NODE_TIDES) continue;
        const dgswe_node_tides& nt = *f.boundaries[b].node_tides;
        Condition& c = h->P.cond[b];
        c.nt_omega0 = (int)omega.size();
        c.nt_slot0 = slot0[b] = (int64_t)mean.size();
        c.nt_coef0 = (int64_t)coef.size();
        omega.insert(omega.end(), nt.omega, nt.omega + nt.n_constituents);
        frate.insert(frate.end(), nt.f_rate, nt.f_rate + nt.n_constituents);
        coef.insert(coef.end(), nt.coefficients,
                    nt.coefficients + (size_t)nt.n_slots * nt.n_constituents * 6);
        for (int64_t q = 0; q < nt.n_slots; ++q) {
            mean.push_back(nt.mean ? nt.mean[q] : 0.0);
            depth.push_back(nt.source_depth ? nt.source_depth[q] : 0.0);
        }
    }
    const int n1 = ops.n1, nn = ops.nn;
    std::vector<int32_t> slot(t.bface.size() * n1, -1);
    for (size_t bf = 0; bf < t.bface.size(); ++bf) {
        const int ci = t.bface_cond[bf];
        if (ci < 0 || ci >= f.n_boundaries || !per_node(f.boundaries[ci])) continue;
        const dgswe_boundary& bc = f.boundaries[ci];
        const bool parent = bc.kind == DGSWE_BC_PARENT;
        const int64_t n_slots = parent ? bc.parent->n_slots : bc.node_tides->n_slots;
        const double* positions = parent ? bc.parent->positions : bc.node_tides->positions;
        const uint32_t* slot_of_node = parent ? bc.parent->slot_of_node : bc.node_tides->slot_of_node;
        const uint8_t* on_boundary = parent ? bc.parent->on_boundary : nullptr;
        const int64_t k = t.bface[bf] >> 2;
        const int face = (int)(t.bface[bf] & 3);
        for (int fi = 0; fi < n1; ++fi) {
            const int node = ops.face_node[face][fi];
            int64_t q = -1;
            if (slot_of_node) {
                const uint32_t v = slot_of_node[k * nn + node];
                if (v != 0xFFFFFFFFu) {
                    if ((int64_t)v >= n_slots)
                        return fail(h, DGSWE_ERR_INVALID, "a boundary slot beyond n_slots");
                    q = v;
                }
            }
            if (q < 0) {  // the nearest forced node (Mesh2D::reference_to_physical)
                const std::array<double, 8>& c = topo.corners[k];
                const double r = ops.r[node], sv = ops.s[node];
                const double n0 = (1 - r) * (1 - sv) / 4, n1b = (1 + r) * (1 - sv) / 4,
                             n2 = (1 + r) * (1 + sv) / 4, n3 = (1 - r) * (1 + sv) / 4;
                const double x = n0 * c[0] + n1b * c[2] + n2 * c[4] + n3 * c[6];
                const double y = n0 * c[1] + n1b * c[3] + n2 * c[5] + n3 * c[7];
                double best = INFINITY;
                for (int64_t p = 0; p < n_slots; ++p) {
                    if (on_boundary && !on_boundary[p]) continue;
                    const double d = std::hypot(positions[2 * p] - x, positions[2 * p + 1] - y);
                    if (d < best) {
                        best = d;
                        q = p;
                    }
                }
            }
            slot[bf * n1 + fi] = (int32_t)(slot0[ci] + q);
        }
    }
    DevTables& T = h->T;
    int s = DGSWE_OK;
    if ((s = upload_vec(h, slot, &T.bface_slot))) return s;
    if ((s = upload_vec(h, omega, &T.nt_omega))) return s;
    if ((s = upload_vec(h, frate, &T.nt_frate))) return s;
    if ((s = upload_vec(h, coef, &T.nt_coef))) return s;
    if ((s = upload_vec(h, mean, &T.nt_mean))) return s;
    if ((s = upload_vec(h, depth, &T.nt_depth))) return s;
    if ((s = upload_vec(h, ptimes, &T.pt_times))) return s;
    if ((s = upload_vec(h, pvalues, &T.pt_values))) return s;
    // the parents' time ranges, for the runs' checks
    if (f.relaxation && f.relaxation->parent->n_times > 1) {
        const dgswe_parent_series& ps = *f.relaxation->parent;
        h->parent_range = {std::max(h->parent_range.first, ps.times[0]),
                           std::min(h->parent_range.second, ps.times[ps.n_times - 1])};
    }
    for (int b = 0; b < f.n_boundaries; ++b)
        if (f.boundaries[b].kind == DGSWE_BC_PARENT) {
            const dgswe_parent_series& ps = *f.boundaries[b].parent;
            if (ps.n_times > 1)
                h->parent_range = {std::max(h->parent_range.first, ps.times[0]),
                                   std::min(h->parent_range.second, ps.times[ps.n_times - 1])};
        }
    return DGSWE_OK;
}

// The nesting relaxation band: the nodes whose slot has a positive weight,
// the parent's series, and the per-node source buffer
int relaxation_tables(dgswe_handle* h, const dgswe_form& f) {
    if (!f.relaxation) return DGSWE_OK;
    const dgswe_relaxation& r = *f.relaxation;
    const dgswe_parent_series& ps = *r.parent;
    std::vector<int64_t> node;
    std::vector<int32_t> slot;
    for (int64_t g = 0; g < h->n_values; ++g) {
        const uint32_t q = ps.slot_of_node[g];
        if (q == 0xFFFFFFFFu) continue;
        if ((int64_t)q >= ps.n_slots)
            return fail(h, DGSWE_ERR_INVALID, "a relaxation slot beyond n_slots");
        if (!(r.weight[q] > 0.0)) continue;
        node.push_back(g);
        slot.push_back((int32_t)q);
    }
    DevTables& T = h->T;
    T.rx_n = (int64_t)node.size();
    if (T.rx_n == 0) return DGSWE_OK;
    std::vector<double> weight(r.weight, r.weight + ps.n_slots);
    std::vector<double> depth(ps.n_slots, NAN);
    if (ps.parent_depth) depth.assign(ps.parent_depth, ps.parent_depth + ps.n_slots);
    std::vector<double> times(ps.times, ps.times + ps.n_times);
    std::vector<float> values(ps.values, ps.values + (size_t)ps.n_slots * ps.n_times * 3);
    int s = DGSWE_OK;
    if ((s = upload_vec(h, node, &T.rx_node))) return s;
    if ((s = upload_vec(h, slot, &T.rx_slot))) return s;
    if ((s = upload_vec(h, weight, &T.rx_weight))) return s;
    if ((s = upload_vec(h, depth, &T.rx_depth))) return s;
    if ((s = upload_vec(h, times, &T.rx_times))) return s;
    if ((s = upload_vec(h, values, &T.rx_values))) return s;
    T.rx_n_times = (int)ps.n_times;
    T.rx_cubic = ps.cubic ? 1 : 0;
    T.rx_velocity = ps.velocity ? 1 : 0;
    T.rx_momentum_only = r.momentum_only ? 1 : 0;
    T.rx_ref_level = ps.reference_level;
    T.rx_max_ratio = ps.max_transport_ratio;
    T.rx_ramp = ps.ramp_duration;
    T.rx_rate = r.rate;
    T.rx_wet = r.wet_depth;
    void* p = nullptr;
    CK(cudaMalloc(&p, 3 * (size_t)h->n_values * sizeof(double)));
    h->allocations.push_back(p);
    CK(cudaMemset(p, 0, 3 * (size_t)h->n_values * sizeof(double)));
    T.rx_src = (double*)p;
    return DGSWE_OK;
}

// The weather: its snapshots regridded onto the nodes, in SoA per time
// ([time][5][K·nn]) so that a warp's nodes read each field contiguously,
// and the per-node source buffer it writes (shared with the relaxation
// band's)
int atmosphere_tables(dgswe_handle* h, const dgswe_form& f) {
    if (!f.atmosphere) return DGSWE_OK;
    const dgswe_atmosphere& a = *f.atmosphere;
    DevTables& T = h->T;
    const int64_t n = h->n_values;
    std::vector<float> values((size_t)a.n_times * 5 * n);
    for (int64_t t = 0; t < a.n_times; ++t)
        for (int64_t g = 0; g < n; ++g)
            for (int q = 0; q < 5; ++q)
                values[((size_t)t * 5 + q) * n + g] = a.values[((size_t)t * n + g) * 5 + q];
    std::vector<double> times(a.times, a.times + a.n_times);
    int s = DGSWE_OK;
    if ((s = upload_vec(h, times, &T.at_times))) return s;
    if ((s = upload_vec(h, values, &T.at_values))) return s;
    T.at_n_times = (int)a.n_times;
    T.at_source = a.source ? 1 : 0;
    T.at_wind = a.wind ? 1 : 0;
    T.at_pressure = a.pressure ? 1 : 0;
    T.at_level = a.level ? 1 : 0;
    T.at_drag = a.drag;
    T.at_cd = a.drag_cd;
    T.at_rho_air = a.rho_air;
    T.at_rho_water = a.rho_water;
    T.at_h_min = a.h_min;
    T.at_ramp = a.ramp_duration;
    T.at_epoch = a.epoch_unix;
    // the runs' times must lie within the snapshots' (the reference panics
    // outside them)
    if (a.n_times > 1)
        h->parent_range = {std::max(h->parent_range.first, a.times[0] - a.epoch_unix),
                           std::min(h->parent_range.second, a.times[a.n_times - 1] - a.epoch_unix)};
    if (T.at_source && !T.rx_src) {
        void* p = nullptr;
        CK(cudaMalloc(&p, 3 * (size_t)n * sizeof(double)));
        h->allocations.push_back(p);
        CK(cudaMemset(p, 0, 3 * (size_t)n * sizeof(double)));
        T.rx_src = (double*)p;
    }
    return DGSWE_OK;
}

int create_impl(dgswe_handle* h, const dgswe_form* f, int device) {
    auto bail = [](int s) { return s; };
    h->device = device;
    h->form = *f;
    CK(cudaSetDevice(device));
    cudaDeviceProp prop{};
    CK(cudaGetDeviceProperties(&prop, device));
    h->device_name = prop.name;
    CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    h->ks = f->numerics == DGSWE_NUMERICS_EXACT ? kernels_exact() : kernels_fast();
    h->ops = new Operators(f->order);
    const Operators& ops = *h->ops;
    h->n1 = ops.n1;
    h->nn = ops.nn;
    h->K = f->n_elements;
    h->n_values = h->K * ops.nn;

    Topology topo;
    std::string err = build_topology(*f, topo);
    if (!err.empty()) return bail(fail(h, DGSWE_ERR_INVALID, "%s", err.c_str()));
    std::vector<int32_t> tags, cond_index;
    for (int b = 0; b < f->n_boundaries; ++b) {
        tags.push_back(f->boundaries[b].tag);
        cond_index.push_back(b);
    }
    Tables t;
    err = build_tables(*f, ops, topo, tags, cond_index, t);
    if (!err.empty()) return bail(fail(h, DGSWE_ERR_INVALID, "%s", err.c_str()));
    // what the multirate planner reads: the face neighbours and the edges
    h->nb.resize(h->K);
    h->nb_face.resize(h->K);
    for (int64_t k = 0; k < h->K; ++k)
        for (int face = 0; face < 4; ++face) {
            h->nb[k][face] = topo.link[k][face].element;
            h->nb_face[k][face] = (int8_t)topo.link[k][face].face;
        }
    h->h_edge_left = t.edge_left;
    h->h_edge_right = t.edge_right;
    h->h_bface = t.bface;
    PairSchedule sched(ops);
    std::vector<int8_t> owned;
    for (const PairSlot& p : sched.owned) {
        owned.push_back(p.a);
        owned.push_back(p.c);
        owned.push_back(p.dir);
        owned.push_back(p.pa);
        owned.push_back(p.pc);
    }

    DevTables& T = h->T;
    T.K = h->K;
    T.n_edges = (int64_t)t.edge_left.size();
    T.n_bfaces = (int64_t)t.bface.size();
    int s = DGSWE_OK;
#define UP(field, vec)                          \
    if ((s = upload_vec(h, vec, &T.field)) != 0) \
        return bail(s);
    UP(bed, t.bed);
    UP(jinv, t.jinv);
    UP(pair_hm, t.pair_hm);
    UP(gdb, t.gdb);
    UP(contra, t.contra);
    UP(lift_scale, t.lift_scale);
    UP(outer_dist, t.outer_dist);
    UP(fcor, t.fcor);
    UP(g_n2, t.g_n2);
    UP(mass, t.mass);
    UP(inv_area, t.inv_area);
    UP(weight_ratio, t.weight_ratio);
    UP(dtm_own, t.dtm_own);
    UP(dtm_face, t.dtm_face);
    UP(dtm32_own, t.dtm32_own);
    UP(dtm32_face, t.dtm32_face);
    UP(edge_geo, t.edge_geo);
    UP(bface_geo, t.bface_geo);
    UP(outer_idx, t.outer_idx);
    UP(nb_face_node, t.nb_face_node);
    UP(edge_left, t.edge_left);
    UP(edge_right, t.edge_right);
    UP(bface, t.bface);
    UP(bface_cond, t.bface_cond);
    UP(affine, t.affine);
    UP(sched_owned, owned);
    UP(sched_slot, sched.accum_slot);
    UP(sched_coef, sched.accum_coef);
    std::vector<double> hcoef(sched.accum_coef.size());
    for (size_t q = 0; q < hcoef.size(); ++q) hcoef[q] = 0.5 * sched.accum_coef[q];
    UP(sched_hcoef, hcoef);
    UP(pair_coef, pair_coef_table(sched));
#undef UP

    fill_physics(*f, ops, !t.fcor.empty(), h->P, h->X);
    h->P.n_conditions = f->n_boundaries;
    for (int b = 0; b < f->n_boundaries; ++b) h->P.cond[b] = make_condition(f->boundaries[b]);
    if ((s = boundary_node_tables(h, *f, ops, topo, t))) return bail(s);
    if ((s = relaxation_tables(h, *f))) return bail(s);
    if ((s = atmosphere_tables(h, *f))) return bail(s);

    // buffers, faces, control
    if ((s = ensure_buffer(h, DGSWE_STATE))) return bail(s);
    const size_t nf = (size_t)h->K * 4 * ops.n1;
    void* p = nullptr;
    CK(cudaMalloc(&p, 3 * nf * sizeof(double)));
    h->allocations.push_back(p);
    CK(cudaMemset(p, 0, 3 * nf * sizeof(double)));
    h->fb_h = (double*)p;
    h->fb_hu = h->fb_h + nf;
    h->fb_hv = h->fb_hu + nf;
    CK(cudaMalloc(&p, (size_t)h->K * sizeof(double)));
    h->allocations.push_back(p);
    h->dt_el = (double*)p;
    CK(cudaMalloc(&p, sizeof(StepCtl)));
    h->allocations.push_back(p);
    h->ctl = (StepCtl*)p;
    CK(cudaMallocHost(&p, sizeof(StepCtl)));
    h->h_ctl = (StepCtl*)p;
    std::memset(h->h_ctl, 0, sizeof(StepCtl));
    h->h_ctl->always = 1;
    h->h_ctl->active = 1;
    CK(cudaMemcpy(h->ctl, h->h_ctl, sizeof(StepCtl), cudaMemcpyHostToDevice));
    h->form.vertices = nullptr;
    h->form.elements = nullptr;
    h->form.periodic = nullptr;
    h->form.face_tags = nullptr;
    h->form.bathymetry = nullptr;
    h->form.manning_n_nodes = nullptr;
    h->form.boundaries = nullptr;
    h->form.relaxation = nullptr;
    h->form.atmosphere = nullptr;
    return DGSWE_OK;
}

}  // namespace

extern "C" {

int dgswe_create(const dgswe_form* f, int device, dgswe_handle** out) {
    if (!out) return DGSWE_ERR_INVALID;
    *out = nullptr;
    std::string why;
    dgswe_handle* h = new dgswe_handle();
    int s = check_form(f, why);
    if (s == DGSWE_OK) {
        int count = 0;
        if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0 || device < 0 ||
            device >= count) {
            s = DGSWE_ERR_NO_DEVICE;
            why = "no CUDA device " + std::to_string(device);
        }
    }
    if (s == DGSWE_OK) {
        s = create_impl(h, f, device);
    } else {
        h->error = why;
    }
    // On failure the handle is still returned, so that dgswe_last_error can
    // tell why; the caller destroys it
    *out = h;
    return s;
}

void dgswe_destroy(dgswe_handle* h) {
    if (!h) return;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    delete h;
}

int dgswe_upload(dgswe_handle* h, int32_t buffer, const double* hh, const double* hu,
                 const double* hv, int64_t n) {
    if (!h) return DGSWE_ERR_INVALID;
    if (!valid_buffer(buffer) || n != h->n_values || !hh || !hu || !hv)
        return fail(h, DGSWE_ERR_INVALID, "upload: buffer %d, %lld values (expected %lld)", buffer,
                    (long long)n, (long long)h->n_values);
    CK(cudaSetDevice(h->device));
    if (int s = ensure_buffer(h, buffer)) return s;
    const DevBuf& b = h->buf[buffer].view;
    const size_t bytes = (size_t)n * sizeof(double);
    CK(cudaMemcpyAsync(b.h, hh, bytes, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(b.hu, hu, bytes, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(b.hv, hv, bytes, cudaMemcpyHostToDevice, h->stream));
    h->ks->velocity(b, n, h->P.h_min, h->stream);
    return sync(h);
}

int dgswe_download(dgswe_handle* h, int32_t buffer, double* hh, double* hu, double* hv,
                   int64_t n) {
    if (!h) return DGSWE_ERR_INVALID;
    if (!valid_buffer(buffer) || n != h->n_values || !hh || !hu || !hv)
        return fail(h, DGSWE_ERR_INVALID, "download: buffer %d, %lld values (expected %lld)",
                    buffer, (long long)n, (long long)h->n_values);
    CK(cudaSetDevice(h->device));
    if (int s = ensure_buffer(h, buffer)) return s;
    const DevBuf& b = h->buf[buffer].view;
    const size_t bytes = (size_t)n * sizeof(double);
    CK(cudaMemcpyAsync(hh, b.h, bytes, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(hu, b.hu, bytes, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(hv, b.hv, bytes, cudaMemcpyDeviceToHost, h->stream));
    return sync(h);
}

int dgswe_compute_rhs(dgswe_handle* h, int32_t input, double time, double* out_h, double* out_hu,
                      double* out_hv, int64_t n) {
    if (!h) return DGSWE_ERR_INVALID;
    if (!valid_buffer(input) || n != h->n_values || !out_h || !out_hu || !out_hv)
        return fail(h, DGSWE_ERR_INVALID, "compute_rhs: buffer %d, %lld values", input,
                    (long long)n);
    if (!(time >= h->parent_range.first && time <= h->parent_range.second))
        return fail(h, DGSWE_ERR_INVALID, "compute_rhs: t = %g leaves the forcing's snapshots", time);
    CK(cudaSetDevice(h->device));
    if (int s = ensure_buffer(h, input)) return s;
    if (int s = ensure_buffer(h, kRhsBuffer)) return s;
    if (int s = write_host_args(h, StageArgs{time, 0.0, 0.0, 1.0, 1.0, 0.0})) return s;
    launch_stage(h, input, input, kRhsBuffer, kRhsBuffer, kHostSlot, kModeRhsOnly, 0, always(h));
    CK(cudaGetLastError());
    const DevBuf& b = h->buf[kRhsBuffer].view;
    const size_t bytes = (size_t)n * sizeof(double);
    CK(cudaMemcpyAsync(out_h, b.h, bytes, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(out_hu, b.hu, bytes, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(out_hv, b.hv, bytes, cudaMemcpyDeviceToHost, h->stream));
    return sync(h);
}

int dgswe_compute_rhs_mass_fluxes(dgswe_handle* h, int32_t input, double time, double* out_h,
                                  double* out_hu, double* out_hv, int64_t n, double* face_mass,
                                  int64_t n_face, double* subcell_mass, int64_t n_sub) {
    if (!h) return DGSWE_ERR_INVALID;
    const int64_t face_len = h->K * 4 * h->n1, sub_len = h->K * 2 * h->n1 * (h->n1 - 1);
    if (!valid_buffer(input) || n != h->n_values || !out_h || !out_hu || !out_hv ||
        (face_mass && n_face != face_len) || (subcell_mass && n_sub != sub_len))
        return fail(h, DGSWE_ERR_INVALID,
                    "compute_rhs_mass_fluxes: buffer %d, %lld values, %lld face and %lld subcell "
                    "fluxes (expected %lld, %lld, %lld)",
                    input, (long long)n, (long long)n_face, (long long)n_sub,
                    (long long)h->n_values, (long long)face_len, (long long)sub_len);
    if (!(time >= h->parent_range.first && time <= h->parent_range.second))
        return fail(h, DGSWE_ERR_INVALID,
                    "compute_rhs_mass_fluxes: t = %g leaves the forcing's snapshots", time);
    CK(cudaSetDevice(h->device));
    if (int s = ensure_buffer(h, input)) return s;
    if (int s = ensure_buffer(h, kRhsBuffer)) return s;
    if (subcell_mass && !h->sub_mass) {
        void* p = nullptr;
        CK(cudaMalloc(&p, (size_t)sub_len * sizeof(double)));
        h->allocations.push_back(p);
        h->sub_mass = (double*)p;
    }
    if (int s = write_host_args(h, StageArgs{time, 0.0, 0.0, 1.0, 1.0, 0.0})) return s;
    StageExtra X = h->X;
    X.subcell_mass = subcell_mass ? h->sub_mass : nullptr;
    const DevBuf& in = h->buf[input].view;
    const DevBuf& rhs = h->buf[kRhsBuffer].view;
    h->ks->face(h->n1, h->T, h->P, in, h->fb_h, h->fb_hu, h->fb_hv, h->ctl, kHostSlot, always(h),
                h->stream);
    h->ks->stage(h->n1, h->T, h->P, X, in, in, rhs, rhs, h->fb_h, h->fb_hu, h->fb_hv, h->ctl,
                 kHostSlot, kModeRhsOnly, 0, always(h), h->stream);
    CK(cudaGetLastError());
    const size_t bytes = (size_t)n * sizeof(double);
    CK(cudaMemcpyAsync(out_h, rhs.h, bytes, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(out_hu, rhs.hu, bytes, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(out_hv, rhs.hv, bytes, cudaMemcpyDeviceToHost, h->stream));
    // the face-flux buffer is the reference's face_mass layout already:
    // [(k·4 + face)·n1 + fi], F*_h along the element's outward unit normal
    if (face_mass)
        CK(cudaMemcpyAsync(face_mass, h->fb_h, (size_t)face_len * sizeof(double),
                           cudaMemcpyDeviceToHost, h->stream));
    if (subcell_mass)
        CK(cudaMemcpyAsync(subcell_mass, h->sub_mass, (size_t)sub_len * sizeof(double),
                           cudaMemcpyDeviceToHost, h->stream));
    return sync(h);
}

int dgswe_autotune(dgswe_handle* h, int32_t repeats, int32_t force_face, int32_t force_stage,
                   dgswe_tuning* out) {
    if (!h) return DGSWE_ERR_INVALID;
    if (!out || repeats < 1 || force_stage > 2 ||
        (force_face >= 0 && force_face != 64 && force_face != 128 && force_face != 256))
        return fail(h, DGSWE_ERR_INVALID, "autotune: repeats %d, face %d, stage %d", repeats,
                    force_face, force_stage);
    CK(cudaSetDevice(h->device));
    if (int s = ensure_buffer(h, DGSWE_STATE)) return s;
    if (int s = ensure_buffer(h, kRhsBuffer)) return s;
    if (int s = write_host_args(h, StageArgs{0.0, 0.0, 0.0, 1.0, 1.0, 0.0})) return s;
    std::memset(out, 0, sizeof *out);
    const DevBuf& in = h->buf[DGSWE_STATE].view;
    const DevBuf& rhs = h->buf[kRhsBuffer].view;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    auto timed = [&](auto&& launch, double& ms) -> int {
        launch();  // warm
        CK(cudaEventRecord(e0, h->stream));
        for (int r = 0; r < repeats; ++r) launch();
        CK(cudaEventRecord(e1, h->stream));
        CK(cudaEventSynchronize(e1));
        float t = 0.0f;
        CK(cudaEventElapsedTime(&t, e0, e1));
        ms = (double)t / repeats;
        return DGSWE_OK;
    };
    auto face = [&]() {
        h->ks->face(h->n1, h->T, h->P, in, h->fb_h, h->fb_hu, h->fb_hv, h->ctl, kHostSlot,
                    always(h), h->stream);
    };
    auto stage = [&]() {
        h->ks->stage(h->n1, h->T, h->P, h->X, in, in, rhs, rhs, h->fb_h, h->fb_hu, h->fb_hv,
                     h->ctl, kHostSlot, kModeRhsOnly, 0, always(h), h->stream);
    };
    int status = DGSWE_OK;
    static const int kFace[3] = {64, 128, 256};
    if (force_face >= 0) {
        h->P.face_threads = force_face;
    } else {
        int best = 2;
        for (int c = 0; c < 3 && status == DGSWE_OK; ++c) {
            h->P.face_threads = kFace[c];
            status = timed(face, out->face_ms[c]);
            if (out->face_ms[c] < out->face_ms[best]) best = c;
        }
        h->P.face_threads = kFace[best];
    }
    if (status == DGSWE_OK) face();  // the stage reads its fluxes
    if (force_stage >= 0) {
        h->P.stage_shape = force_stage;
    } else {
        int best = 0;
        for (int c = 0; c < 3 && status == DGSWE_OK; ++c) {
            h->P.stage_shape = c;
            status = timed(stage, out->stage_ms[c]);
            if (out->stage_ms[c] < out->stage_ms[best]) best = c;
        }
        h->P.stage_shape = best;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (status != DGSWE_OK) return status;
    CK(cudaGetLastError());
    out->face_threads = h->P.face_threads;
    const int per = h->P.stage_shape == 1 ? 64 : 128;
    out->stage_threads = std::max(1, per / h->nn) * h->nn;
    // the step graph holds the old shapes in its launches
    if (h->step_graph) {
        cudaGraphExecDestroy(h->step_graph);
        h->step_graph = nullptr;
    }
    return sync(h);
}

int dgswe_stage(dgswe_handle* h, const dgswe_stage_plan* plan) {
    if (!h) return DGSWE_ERR_INVALID;
    if (!plan || !valid_buffer(plan->base) || !valid_buffer(plan->input) ||
        !valid_buffer(plan->out) || (plan->accumulate && !valid_buffer(plan->acc)))
        return fail(h, DGSWE_ERR_INVALID, "stage: invalid plan or buffer ids");
    if (plan->out == plan->input)
        return fail(h, DGSWE_ERR_INVALID, "stage: out must differ from input");
    if (!(plan->time >= h->parent_range.first && plan->time <= h->parent_range.second))
        return fail(h, DGSWE_ERR_INVALID, "stage: t = %g leaves the forcing's snapshots",
                    plan->time);
    CK(cudaSetDevice(h->device));
    for (int id : {plan->base, plan->input, plan->out})
        if (int s = ensure_buffer(h, id)) return s;
    const int acc = plan->accumulate ? plan->acc : plan->out;
    if (int s = ensure_buffer(h, acc)) return s;
    if (int s = write_host_args(h, StageArgs{plan->time, plan->a, plan->b, plan->c, plan->w,
                                             plan->keep}))
        return s;
    launch_stage(h, plan->input, plan->base, plan->out, acc, kHostSlot,
                 plan->accumulate ? kModeAccumulate : kModePost, 0, always(h));
    if (plan->accumulate) {
        h->ks->velocity(h->buf[plan->out].view, h->n_values, h->P.h_min, h->stream);
        h->ks->velocity(h->buf[acc].view, h->n_values, h->P.h_min, h->stream);
    }
    CK(cudaGetLastError());
    return sync(h);
}

int dgswe_finish(dgswe_handle* h, int32_t acc) {
    if (!h) return DGSWE_ERR_INVALID;
    if (!valid_buffer(acc) || acc == DGSWE_STATE)
        return fail(h, DGSWE_ERR_INVALID, "finish: invalid accumulation buffer %d", acc);
    CK(cudaSetDevice(h->device));
    if (int s = ensure_buffer(h, acc)) return s;
    h->ks->finish(h->n1, h->T, h->P, h->buf[acc].view, h->buf[DGSWE_STATE].view, h->ctl,
                  h->stream);
    CK(cudaGetLastError());
    return sync(h);
}

int dgswe_implicit_damping(dgswe_handle* h, int32_t stage, int32_t from, double dt) {
    if (!h) return DGSWE_ERR_INVALID;
    if (!valid_buffer(stage) || !valid_buffer(from) || !(dt >= 0.0) || !std::isfinite(dt))
        return fail(h, DGSWE_ERR_INVALID, "implicit_damping: buffers %d, %d, dt %g", stage, from,
                    dt);
    // ImplicitDamping2D::is_active: neither friction nor the thin layer, no change
    if (!h->P.friction && !h->P.has_wet_dry) return DGSWE_OK;
    CK(cudaSetDevice(h->device));
    if (int s = ensure_buffer(h, stage)) return s;
    if (int s = ensure_buffer(h, from)) return s;
    h->ks->implicit_damping(h->T, h->P, h->buf[stage].view, h->buf[from].view, dt, h->n_values,
                            h->stream);
    CK(cudaGetLastError());
    return sync(h);
}

int dgswe_post_process(dgswe_handle* h, int32_t buffer) {
    if (!h) return DGSWE_ERR_INVALID;
    if (!valid_buffer(buffer))
        return fail(h, DGSWE_ERR_INVALID, "post_process: invalid buffer %d", buffer);
    CK(cudaSetDevice(h->device));
    if (int s = ensure_buffer(h, buffer)) return s;
    // the end of a substep with the buffer as both its sum and its state:
    // each node read before it is written, the limiter's element sums from
    // shared memory
    h->ks->finish(h->n1, h->T, h->P, h->buf[buffer].view, h->buf[buffer].view, h->ctl,
                  h->stream);
    CK(cudaGetLastError());
    return sync(h);
}

int dgswe_element_dt(dgswe_handle* h, double cfl, int32_t scheme, double* dt_elements,
                     double* dt_min) {
    if (!h) return DGSWE_ERR_INVALID;
    if (!(cfl > 0.0) || (scheme != DGSWE_SSP_RK3 && scheme != DGSWE_SSP_RK43))
        return fail(h, DGSWE_ERR_INVALID, "element_dt: cfl %g, scheme %d", cfl, scheme);
    CK(cudaSetDevice(h->device));
    const unsigned long long inf_bits = 0x7FF0000000000000ull;
    CK(cudaMemcpyAsync(&h->ctl->dt_bits, &inf_bits, sizeof inf_bits, cudaMemcpyHostToDevice,
                       h->stream));
    const DtParams D = dt_params(h->form, cfl, scheme);
    h->ks->dt(h->n1, h->T, h->P, h->buf[DGSWE_STATE].view, D, h->dt_el, h->ctl, always(h),
              h->stream);
    CK(cudaGetLastError());
    unsigned long long bits = 0;
    CK(cudaMemcpyAsync(&bits, &h->ctl->dt_bits, sizeof bits, cudaMemcpyDeviceToHost, h->stream));
    if (dt_elements)
        CK(cudaMemcpyAsync(dt_elements, h->dt_el, (size_t)h->K * sizeof(double),
                           cudaMemcpyDeviceToHost, h->stream));
    if (int s = sync(h)) return s;
    if (dt_min) std::memcpy(dt_min, &bits, sizeof(double));
    return DGSWE_OK;
}

int dgswe_step(dgswe_handle* h, int32_t scheme, double t, double dt) {
    if (!h) return DGSWE_ERR_INVALID;
    if (scheme != DGSWE_SSP_RK3 && scheme != DGSWE_SSP_RK43)
        return fail(h, DGSWE_ERR_INVALID, "step: scheme %d", scheme);
    if (!(t >= h->parent_range.first && t + dt <= h->parent_range.second))
        return fail(h, DGSWE_ERR_INVALID, "step: (%g, %g) leaves the forcing's snapshots", t, t + dt);
    CK(cudaSetDevice(h->device));
    double st[4][4];
    const int n = scheme_table(scheme, st);
    for (int b = 1; b < n; ++b)
        if (int s = ensure_buffer(h, b)) return s;
    // element_stage with one level (src/time/multirate.rs:169-200)
    for (int s = 0; s < n; ++s)
        h->h_ctl->stage[s] = StageArgs{t + st[s][3] * dt, st[s][0], st[s][1], st[s][2] * dt, 1.0, 0.0};
    CK(cudaMemcpyAsync(&h->ctl->stage[0], &h->h_ctl->stage[0], n * sizeof(StageArgs),
                       cudaMemcpyHostToDevice, h->stream));
    for (int s = 0; s < n; ++s) {
        const int in = s == 0 ? DGSWE_STATE : s;
        const int out = s + 1 < n ? s + 1 : DGSWE_STATE;
        launch_stage(h, in, DGSWE_STATE, out, DGSWE_STATE, s, kModePost, 0, always(h));
    }
    CK(cudaGetLastError());
    return sync(h);
}

namespace {

// The ready lists of dgswe_step_host's upload chunks (ready_lists,
// host_common.hpp), on the device
int build_ready_lists(dgswe_handle* h) {
    if (h->ready_built) return DGSWE_OK;
    const ReadyLists r = ready_lists(h->K, kHostChunks, h->nb, h->h_edge_left, h->h_edge_right,
                                     h->h_bface);
    std::copy(r.elem_off.begin(), r.elem_off.end(), h->ready_elem_off);
    std::copy(r.edge_off.begin(), r.edge_off.end(), h->ready_edge_off);
    std::copy(r.bface_off.begin(), r.bface_off.end(), h->ready_bface_off);
    if (int s = upload_vec(h, r.elems, &h->ready_elems)) return s;
    if (int s = upload_vec(h, r.edges, &h->ready_edges)) return s;
    if (int s = upload_vec(h, r.bfaces, &h->ready_bfaces)) return s;
    h->ready_built = true;
    return DGSWE_OK;
}

}  // namespace

int dgswe_step_host(dgswe_handle* h, int32_t scheme, double t, double cfl, double dt_max,
                    double* hh, double* hu, double* hv, int64_t n, double* dt_out) {
    if (!h) return DGSWE_ERR_INVALID;
    if (scheme != DGSWE_SSP_RK3 && scheme != DGSWE_SSP_RK43)
        return fail(h, DGSWE_ERR_INVALID, "step_host: scheme %d", scheme);
    if (n != h->n_values || !hh || !hu || !hv || !(cfl > 0.0) || !(dt_max >= 0.0))
        return fail(h, DGSWE_ERR_INVALID,
                    "step_host: %lld values (expected %lld), NULL arrays, cfl %g or dt_max %g",
                    (long long)n, (long long)h->n_values, cfl, dt_max);
    if (!(t >= h->parent_range.first && t < h->parent_range.second))
        return fail(h, DGSWE_ERR_INVALID, "step_host: t = %g leaves the forcing's snapshots", t);
    CK(cudaSetDevice(h->device));
    double st[4][4];
    const int n_st = scheme_table(scheme, st);
    for (int b = 1; b < n_st; ++b)
        if (int s = ensure_buffer(h, b)) return s;
    if (!h->copy_stream) {
        CK(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
        for (cudaEvent_t& e : h->chunk_done)
            CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    // one step of the device clock from t; it lands on the end of any
    // forcing series' snapshots rather than leave them. The running clip
    // count stays on the device: the record is written around it
    {
        StepCtl& c = *h->h_ctl;
        std::memset(&c, 0, sizeof c);
        c.t = t;
        c.t_end = h->parent_range.second;
        c.target = h->parent_range.second;
        c.dt_max = dt_max;
        c.cfl = cfl;
        c.dt_min_used = INFINITY;
        c.dt_bits = 0x7FF0000000000000ull;
        c.always = 1;
        c.scheme_stages = n_st;
        for (int s = 0; s < n_st; ++s) {
            c.st_start[s] = st[s][0];
            c.st_input[s] = st[s][1];
            c.st_beta[s] = st[s][2];
            c.st_c[s] = st[s][3];
        }
        const size_t at = offsetof(StepCtl, clips), past = at + sizeof c.clips;
        CK(cudaMemcpyAsync(h->ctl, &c, at, cudaMemcpyHostToDevice, h->stream));
        CK(cudaMemcpyAsync((char*)h->ctl + past, (const char*)&c + past, sizeof c - past,
                           cudaMemcpyHostToDevice, h->stream));
    }
    // the state in element chunks on the copy stream; as each chunk
    // arrives, its node velocities, and the dt pass and the first stage's
    // face fluxes of whatever reads nothing later
    if (int s = build_ready_lists(h)) return s;
    const DevBuf& q = h->buf[DGSWE_STATE].view;
    const int* active = &h->ctl->active;
    const DtParams D = dt_params(h->form, cfl, scheme);
    const int64_t per = (h->K + kHostChunks - 1) / kHostChunks;
    h->ks->step_begin(h->ctl, 1, h->stream);  // the dt reset, the first stage's time
    CK(cudaEventRecord(h->chunk_done[0], h->stream));  // after the work queued before
    CK(cudaStreamWaitEvent(h->copy_stream, h->chunk_done[0], 0));
    for (int c = 0; c < kHostChunks; ++c) {
        const int64_t k0 = std::min<int64_t>(h->K, c * per), k1 = std::min<int64_t>(h->K, k0 + per);
        if (k1 > k0) {
            const size_t off = (size_t)k0 * h->nn, cnt = (size_t)(k1 - k0) * h->nn;
            const size_t len = cnt * sizeof(double);
            CK(cudaMemcpyAsync(q.h + off, hh + off, len, cudaMemcpyHostToDevice, h->copy_stream));
            CK(cudaMemcpyAsync(q.hu + off, hu + off, len, cudaMemcpyHostToDevice,
                               h->copy_stream));
            CK(cudaMemcpyAsync(q.hv + off, hv + off, len, cudaMemcpyHostToDevice,
                               h->copy_stream));
            CK(cudaEventRecord(h->chunk_done[c], h->copy_stream));
            CK(cudaStreamWaitEvent(h->stream, h->chunk_done[c], 0));
            const DevBuf part{q.h + off, q.hu + off, q.hv + off, q.u + off, q.v + off};
            h->ks->velocity(part, (int64_t)cnt, h->P.h_min, h->stream);
        }
        const int64_t e0 = h->ready_elem_off[c], e1 = h->ready_elem_off[c + 1];
        h->ks->dt_listed(h->n1, h->T, h->P, q, D, nullptr, h->ctl, active, h->ready_elems + e0,
                         e1 - e0, h->stream);
        const int64_t f0 = h->ready_edge_off[c], f1 = h->ready_edge_off[c + 1];
        const int64_t b0 = h->ready_bface_off[c], b1 = h->ready_bface_off[c + 1];
        h->ks->face_ready(h->n1, h->T, h->P, q, h->fb_h, h->fb_hu, h->fb_hv, h->ctl, 0, active,
                          h->ready_edges + f0, f1 - f0, h->ready_bfaces + b0, b1 - b0, h->stream);
    }
    h->ks->node_sources(h->T, h->P, q, h->ctl, 0, h->stream);
    h->ks->step_dt(h->ctl, 1, h->stream);
    for (int s = 0; s + 1 < n_st; ++s) {
        const int in = s == 0 ? DGSWE_STATE : s;
        if (s == 0)  // its face fluxes came with the upload
            h->ks->stage(h->n1, h->T, h->P, h->X, h->buf[in].view, q, h->buf[s + 1].view, q,
                         h->fb_h, h->fb_hu, h->fb_hv, h->ctl, s, kModePost, 0, active, h->stream);
        else
            launch_stage(h, in, DGSWE_STATE, s + 1, DGSWE_STATE, s, kModePost, 0, active);
    }
    // the last stage in element chunks, each copied back while the next runs
    const int last = n_st - 1;
    const DevBuf& in = h->buf[last].view;
    h->ks->face(h->n1, h->T, h->P, in, h->fb_h, h->fb_hu, h->fb_hv, h->ctl, last, active,
                h->stream);
    for (int c = 0; c < kHostChunks; ++c) {
        const int64_t k0 = c * per, k1 = std::min<int64_t>(h->K, k0 + per);
        if (k1 <= k0) break;
        StageExtra X = h->X;
        X.k_first = k0;
        X.k_last = k1;
        h->ks->stage(h->n1, h->T, h->P, X, in, q, q, q, h->fb_h, h->fb_hu, h->fb_hv, h->ctl, last,
                     kModePost, 1, active, h->stream);
        CK(cudaEventRecord(h->chunk_done[c], h->stream));
        CK(cudaStreamWaitEvent(h->copy_stream, h->chunk_done[c], 0));
        const size_t off = (size_t)k0 * h->nn, len = (size_t)(k1 - k0) * h->nn * sizeof(double);
        CK(cudaMemcpyAsync(hh + off, q.h + off, len, cudaMemcpyDeviceToHost, h->copy_stream));
        CK(cudaMemcpyAsync(hu + off, q.hu + off, len, cudaMemcpyDeviceToHost, h->copy_stream));
        CK(cudaMemcpyAsync(hv + off, q.hv + off, len, cudaMemcpyDeviceToHost, h->copy_stream));
    }
    h->ks->step_end(h->ctl, 1, h->stream);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(h->h_ctl, h->ctl, sizeof(StepCtl), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->copy_stream));
    if (int s = sync(h)) return s;
    const StepCtl& c = *h->h_ctl;
    if (dt_out) *dt_out = c.dt;
    if (c.failure || c.nonfinite || !c.active)
        return fail(h, DGSWE_ERR_NONFINITE, "step_host: the step did not complete (%d%s)",
                    c.failure, c.nonfinite ? ", a non-finite state" : "");
    return DGSWE_OK;
}

int dgswe_run(dgswe_handle* h, const dgswe_run_config* run, dgswe_callback callback, void* user,
              dgswe_report* report) {
    if (!h) return DGSWE_ERR_INVALID;
    if (!run || !report) return fail(h, DGSWE_ERR_INVALID, "run: NULL config or report");
    if (!(run->cfl > 0.0) || (run->scheme != DGSWE_SSP_RK3 && run->scheme != DGSWE_SSP_RK43) ||
        !(run->t_end >= run->t_start))
        return fail(h, DGSWE_ERR_INVALID, "run: cfl %g, scheme %d, span (%g, %g)", run->cfl,
                    run->scheme, run->t_start, run->t_end);
    if (run->levels < 0 || run->levels > DGSWE_MAX_LEVELS)
        return fail(h, DGSWE_ERR_INVALID, "run: %d levels of local time stepping (0..%d)",
                    run->levels, DGSWE_MAX_LEVELS);
    if (!(run->t_start >= h->parent_range.first && run->t_end <= h->parent_range.second))
        return fail(h, DGSWE_ERR_INVALID,
                    "run: the span (%g, %g) leaves the forcing's snapshots (%g, %g)", run->t_start,
                    run->t_end, h->parent_range.first, h->parent_range.second);
    if (run->levels > 0) return run_multirate(h, run, callback, user, report);
    std::memset(report, 0, sizeof(*report));
    std::snprintf(report->device, sizeof report->device, "%s", h->device_name.c_str());
    CK(cudaSetDevice(h->device));
    const auto wall0 = std::chrono::steady_clock::now();
    if (int s = run_device_step_graph(h, run->scheme, run->cfl)) return s;
    // host copies for the callbacks
    std::vector<double> hh, hu, hv;
    const bool has_interval = run->interval > 0.0;
    auto next_callback = [&](unsigned long long k) {
        return run->t_start + (double)(k + 1) * run->interval;
    };
    unsigned long long callbacks_done = 0;
    auto call = [&](double t) -> int {
        if (!callback) return DGSWE_OK;
        hh.resize(h->n_values);
        hu.resize(h->n_values);
        hv.resize(h->n_values);
        if (int s = dgswe_download(h, DGSWE_STATE, hh.data(), hu.data(), hv.data(), h->n_values))
            return s;
        callback(user, t, hh.data(), hu.data(), hv.data(), h->n_values);
        return DGSWE_OK;
    };

    StepCtl& c = *h->h_ctl;
    const double first_target = has_interval ? std::fmin(next_callback(0), run->t_end) : run->t_end;
    if (int s = begin_run(h, run, first_target)) return s;

    auto finish = [&](int status, const char* msg) {
        report->success = status == DGSWE_OK;
        report->final_time = c.t;
        report->n_steps = c.steps;
        report->dt_min_used = c.dt_min_used;
        report->dt_max_used = c.dt_max_used;
        report->negative_depth_clips = c.clips;
        report->wall_time =
            std::chrono::duration<double>(std::chrono::steady_clock::now() - wall0).count();
        std::snprintf(report->message, sizeof report->message, "%s", msg);
        if (status != DGSWE_OK) h->error = msg;
        return status;
    };
    if (int s = call(c.t)) return s;
    // steps launched between host checks: one when the host acts after
    // every step (callbacks every step, a stop flag); with no host action
    // due, many. The device's step_begin stops at the target, the step
    // limit or a failure, so graphs launched past that point do nothing.
    const int chunk = run->stop || (callback && !has_interval) ? 1 : (has_interval ? 4 : 64);
    char msg[256];
    while (c.t < run->t_end) {
        if (run->stop && *run->stop) {
            std::snprintf(msg, sizeof msg, "Stopped at t = %.1f s", c.t);
            return finish(DGSWE_ERR_STOPPED, msg);
        }
        for (int i = 0; i < chunk; ++i) CK(cudaGraphLaunch(h->step_graph, h->stream));
        CK(cudaMemcpyAsync(&c, h->ctl, sizeof c, cudaMemcpyDeviceToHost, h->stream));
        if (int s = sync(h)) return s;
        if (c.failure == 3) {
            std::snprintf(msg, sizeof msg, "The state is not finite at t = %.1f s: it has blown up",
                          c.t);
            return finish(DGSWE_ERR_NONFINITE, msg);
        }
        if (c.failure == 4) {
            std::snprintf(msg, sizeof msg, "Time step (%.2e) below minimum (%.2e)", c.dt,
                          run->dt_min);
            return finish(DGSWE_ERR_DT_MIN, msg);
        }
        if (c.failure == 5) {
            std::snprintf(msg, sizeof msg, "Maximum step limit (%lld) reached",
                          (long long)run->max_steps);
            return finish(DGSWE_ERR_MAX_STEPS, msg);
        }
        if (has_interval) {
            if (c.t >= next_callback(callbacks_done)) {
                if (int s = call(c.t)) return s;
                callbacks_done += 1;
                c.target = std::fmin(next_callback(callbacks_done), run->t_end);
                CK(cudaMemcpyAsync(&h->ctl->target, &c.target, sizeof c.target,
                                   cudaMemcpyHostToDevice, h->stream));
                if (int s = sync(h)) return s;
            }
        } else {
            if (int s = call(c.t)) return s;
        }
    }
    return finish(DGSWE_OK, "");
}

int dgswe_profile_steps(dgswe_handle* h, const dgswe_run_config* run, int64_t n_steps,
                        dgswe_profile* out) {
    if (!h) return DGSWE_ERR_INVALID;
    if (!run || !out || n_steps <= 0 || !(run->cfl > 0.0) ||
        (run->scheme != DGSWE_SSP_RK3 && run->scheme != DGSWE_SSP_RK43))
        return fail(h, DGSWE_ERR_INVALID, "profile_steps: invalid arguments");
    CK(cudaSetDevice(h->device));
    std::memset(out, 0, sizeof(*out));
    double st[4][4];
    const int n = scheme_table(run->scheme, st);
    for (int b = 1; b < n; ++b)
        if (int s = ensure_buffer(h, b)) return s;
    if (int s = begin_run(h, run, INFINITY)) return s;
    if (int s = ensure_dt_stream(h)) return s;
    const DtParams D = dt_params(h->form, run->cfl, run->scheme);
    const int* active = &h->ctl->active;
    // per step, as the step graph runs it: begin; the dt pass and the fit on
    // the dt stream beside the first face pass; then the first stage pass and
    // n − 1 × (face, stage); end. Events: before begin, after begin (the
    // fork), after dt and after the fit (dt stream), after the first face
    // pass, after the join, after each later pass → 5 + 2n per step
    const int per_step = 5 + 2 * n;
    std::vector<cudaEvent_t> ev((size_t)n_steps * per_step + 1);
    for (auto& e : ev) CK(cudaEventCreate(&e));
    auto cleanup = [&]() {
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
    };
    size_t q = 0;
    for (int64_t step = 0; step < n_steps; ++step) {
        CK(cudaEventRecord(ev[q++], h->stream));
        h->ks->step_begin(h->ctl, 1, h->stream);
        cudaEvent_t fork = ev[q++], dt_done = ev[q++], fit_done = ev[q++];
        CK(cudaEventRecord(fork, h->stream));
        CK(cudaStreamWaitEvent(h->dt_stream, fork, 0));
        h->ks->dt(h->n1, h->T, h->P, h->buf[DGSWE_STATE].view, D, nullptr, h->ctl, active,
                  h->dt_stream);
        CK(cudaEventRecord(dt_done, h->dt_stream));
        h->ks->step_dt(h->ctl, 1, h->dt_stream);
        CK(cudaEventRecord(fit_done, h->dt_stream));
        h->ks->face(h->n1, h->T, h->P, h->buf[DGSWE_STATE].view, h->fb_h, h->fb_hu, h->fb_hv,
                    h->ctl, 0, active, h->stream);
        CK(cudaEventRecord(ev[q++], h->stream));
        CK(cudaStreamWaitEvent(h->stream, fit_done, 0));
        CK(cudaEventRecord(ev[q++], h->stream));
        for (int s = 0; s < n; ++s) {
            const int in = s == 0 ? DGSWE_STATE : s;
            const int o = s + 1 < n ? s + 1 : DGSWE_STATE;
            if (s > 0) {
                h->ks->face(h->n1, h->T, h->P, h->buf[in].view, h->fb_h, h->fb_hu, h->fb_hv,
                            h->ctl, s, active, h->stream);
                CK(cudaEventRecord(ev[q++], h->stream));
            }
            h->ks->stage(h->n1, h->T, h->P, h->X, h->buf[in].view, h->buf[DGSWE_STATE].view,
                         h->buf[o].view, h->buf[DGSWE_STATE].view, h->fb_h, h->fb_hu, h->fb_hv,
                         h->ctl, s, kModePost, s + 1 == n, active, h->stream);
            CK(cudaEventRecord(ev[q++], h->stream));
        }
        h->ks->step_end(h->ctl, 1, h->stream);
    }
    const size_t last = q;
    CK(cudaEventRecord(ev[q++], h->stream));
    CK(cudaGetLastError());
    if (int s = sync(h)) {
        cleanup();
        return s;
    }
    auto ms = [&](size_t a, size_t b) {
        float v = 0.0f;
        cudaEventElapsedTime(&v, ev[a], ev[b]);
        return (double)v;
    };
    // the parts: the first face pass and the dt pass overlap, so the parts
    // sum to more than the step; total_ms is the step's own time
    q = 0;
    for (int64_t step = 0; step < n_steps; ++step) {
        const size_t s0 = q;
        out->control_ms += ms(s0, s0 + 1);      // begin
        out->dt_ms += ms(s0 + 1, s0 + 2);       // from the fork
        out->control_ms += ms(s0 + 2, s0 + 3);  // fit
        out->face_ms += ms(s0 + 1, s0 + 4);     // the first face pass, from the fork
        size_t e = s0 + 5;                      // after the join
        out->stage_ms += ms(e, e + 1);
        e += 1;
        for (int s = 1; s < n; ++s) {
            out->face_ms += ms(e, e + 1);
            out->stage_ms += ms(e + 1, e + 2);
            e += 2;
        }
        q = e + 1;  // the next step's first event (or the last)
        out->control_ms += ms(e, q);  // end
    }
    out->total_ms = ms(0, last);
    out->steps = n_steps;
    out->face_launches = n_steps * n;
    out->stage_launches = n_steps * n;
    out->dt_launches = n_steps;
    out->control_launches = n_steps * 3;
    StepCtl c{};
    CK(cudaMemcpy(&c, h->ctl, sizeof c, cudaMemcpyDeviceToHost));
    out->t_final = c.t;
    cleanup();
    if (c.failure) return fail(h, DGSWE_ERR_NONFINITE, "profile_steps: the run failed (%d)", c.failure);
    return DGSWE_OK;
}

// ---------------------------------------------------------------------------
// dgswe_compute_rhs_noalloc: the RHS with the library's own scratch array,
// for callers that cannot allocate device memory while they step.

namespace {

// The working memory of dgswe_compute_rhs_noalloc: 64 MiB, 256-byte aligned.
// In host code this name stands for the array, not for its device address;
// that comes from cudaGetSymbolAddress with the device current, looked up
// by a handle's first call and kept on the handle (a handle lives in one
// context, so the address it keeps cannot outlive the module it names).
constexpr size_t kNoAllocBytes = size_t(64) << 20;
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocBytes / sizeof(double)];

}  // namespace

int dgswe_compute_rhs_noalloc(dgswe_handle* h, const double* hh, const double* hu,
                              const double* hv, double time, double* out_h, double* out_hu,
                              double* out_hv, int64_t n) {
    if (!h) return DGSWE_ERR_INVALID;
    if (n != h->n_values || !hh || !hu || !hv || !out_h || !out_hu || !out_hv)
        return fail(h, DGSWE_ERR_INVALID, "compute_rhs_noalloc: %lld values (expected %lld), or a NULL pointer",
                    (long long)n, (long long)h->n_values);
    if (!(time >= h->parent_range.first && time <= h->parent_range.second))
        return fail(h, DGSWE_ERR_INVALID, "compute_rhs_noalloc: t = %g leaves the forcing's snapshots",
                    time);
    // face fluxes (3 × n_elements·4·(N+1)) and node velocities (2 × n)
    const size_t nf = (size_t)h->K * 4 * h->n1;
    const size_t need = (3 * nf + 2 * (size_t)n) * sizeof(double);
    if (need > kNoAllocBytes)
        return fail(h, DGSWE_ERR_INVALID,
                    "compute_rhs_noalloc: the mesh needs %zu bytes of working memory, more than "
                    "the %zu-byte array holds (use dgswe_compute_rhs)",
                    need, kNoAllocBytes);
    CK(cudaSetDevice(h->device));
    if (!h->noalloc_scratch) {
        void* p = nullptr;
        CK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        h->noalloc_scratch = (double*)p;
    }
    double* fb_h = h->noalloc_scratch;
    double* fb_hu = fb_h + nf;
    double* fb_hv = fb_hu + nf;
    DevBuf in{const_cast<double*>(hh), const_cast<double*>(hu), const_cast<double*>(hv),
              fb_hv + nf, fb_hv + nf + n};
    DevBuf out{out_h, out_hu, out_hv, nullptr, nullptr};
    if (int s = write_host_args(h, StageArgs{time, 0.0, 0.0, 1.0, 1.0, 0.0})) return s;
    h->ks->velocity(in, n, h->P.h_min, h->stream);
    h->ks->face(h->n1, h->T, h->P, in, fb_h, fb_hu, fb_hv, h->ctl, kHostSlot, always(h),
                h->stream);
    h->ks->stage(h->n1, h->T, h->P, h->X, in, in, out, out, fb_h, fb_hu, fb_hv, h->ctl, kHostSlot,
                 kModeRhsOnly, 0, always(h), h->stream);
    CK(cudaGetLastError());
    return sync(h);
}

}  // extern "C"
