// The ensemble driver: independent runs on meshes of uneven sizes and mixed
// polynomial order, advanced together (no reference counterpart; the
// reference runs one case per `CaseDevice::run_2d` call, src/case/run.rs:179-212).
//
// Layout in HBM: the members of one order are concatenated into one set of
// the single-mesh tables (element, node and face-slot arrays back to back,
// indices shifted by the member's offsets), with each element's member in
// elem_member and the members' boundary conditions in one device array.
// Each member keeps its own StepCtl (clock, dt, stage weights, clips and
// failure), so the members take their own time steps. The stage, face and
// dt kernels are the single-mesh kernels: a kernel reads the StepCtl of the
// element's member. One captured graph advances every member by one step:
// step_begin over all members, each order group's dt pass, step_dt, then per
// stage each group's face and stage passes, the groups on two streams.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/dgswe.h"
#include "device.hpp"
#include "ensemble_internal.hpp"
#include "host_common.hpp"
#include "kernel_set.hpp"
#include "setup.hpp"

using namespace dgswe;
using namespace dgswe::host;

namespace {

int fail(dgswe_ensemble* h, int status, const char* fmt, ...) {
    char msg[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(msg, sizeof msg, fmt, ap);
    va_end(ap);
    if (h) h->error = msg;
    return status;
}

#define CK(call)                                                                             \
    do {                                                                                     \
        cudaError_t err_ = (call);                                                           \
        if (err_ != cudaSuccess)                                                             \
            return fail(h, DGSWE_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(err_)); \
    } while (0)

template <class T>
int device_array(dgswe_ensemble* h, size_t n, T** out) {
    *out = nullptr;
    if (n == 0) return DGSWE_OK;
    void* p = nullptr;
    CK(cudaMalloc(&p, n * sizeof(T)));
    h->allocations.push_back(p);
    *out = (T*)p;
    return DGSWE_OK;
}

// The physics that must agree across members (everything but the mesh, the
// bathymetry, Manning's coefficient and the boundary data)
bool same_physics(const dgswe_form& a, const dgswe_form& b) {
    return a.g == b.g && a.h_min == b.h_min && a.formulation == b.formulation &&
           a.subcell_depth == b.subcell_depth && a.subcell_h_dry == b.subcell_h_dry &&
           a.has_wet_dry == b.has_wet_dry && a.wet_dry_h_dry == b.wet_dry_h_dry &&
           a.wet_dry_relaxation_time == b.wet_dry_relaxation_time &&
           a.wet_dry_max_velocity == b.wet_dry_max_velocity &&
           a.positivity_h_dry == b.positivity_h_dry &&
           (a.friction == DGSWE_FRICTION_NONE) == (b.friction == DGSWE_FRICTION_NONE) &&
           a.friction_g == b.friction_g && a.manning_h_min == b.manning_h_min &&
           a.has_coriolis == b.has_coriolis && a.coriolis_f0 == b.coriolis_f0 &&
           a.coriolis_beta == b.coriolis_beta && a.coriolis_y0 == b.coriolis_y0 &&
           a.numerics == b.numerics && (a.bathymetry != nullptr) == (b.bathymetry != nullptr);
}

template <class T>
void append(std::vector<T>& dst, const std::vector<T>& src) {
    dst.insert(dst.end(), src.begin(), src.end());
}

int upload_into(dgswe_ensemble* h, const void* src, size_t bytes, void* dst) {
    if (bytes == 0) return DGSWE_OK;
    CK(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
    return DGSWE_OK;
}

// Build one order group from its members' tables: concatenate, shift the
// indices, upload.
int build_group(dgswe_ensemble* h, Group& G, std::vector<Tables>& tabs,
                const std::vector<int>& cond_base, const dgswe_form* forms) {
    const Operators& ops = *G.ops;
    const int nn = ops.nn, n1 = ops.n1;
    const bool friction = forms[G.members[0]].friction != DGSWE_FRICTION_NONE;
    const bool fcor = !tabs[0].fcor.empty();
    Tables all;
    std::vector<int32_t> elem_member;
    int64_t k0 = 0;
    for (size_t q = 0; q < G.members.size(); ++q) {
        const int m = G.members[q];
        Tables& t = tabs[q];
        const dgswe_form& f = forms[m];
        const int64_t n0 = k0 * nn;
        for (auto& x : t.outer_idx)
            if (x >= 0) x += n0;
        for (auto& x : t.nb_face_node)
            if (x >= 0) x += n0;
        for (auto& x : t.edge_left) x += 4 * k0;
        for (auto& x : t.edge_right) x += 4 * k0;
        for (auto& x : t.bface) x += 4 * k0;
        for (auto& x : t.bface_cond) x += cond_base[m];
        if (friction && t.g_n2.empty())  // a uniform coefficient as a per-node field
            t.g_n2.assign((size_t)t.K * nn, f.friction_g * f.manning_n * f.manning_n);
        if (fcor != !t.fcor.empty())
            return fail(h, DGSWE_ERR_INVALID, "members differ in their Coriolis field");
        append(all.bed, t.bed);
        append(all.jinv, t.jinv);
        append(all.pair_hm, t.pair_hm);
        append(all.gdb, t.gdb);
        append(all.contra, t.contra);
        append(all.affine, t.affine);
        append(all.lift_scale, t.lift_scale);
        append(all.outer_idx, t.outer_idx);
        append(all.outer_dist, t.outer_dist);
        append(all.fcor, t.fcor);
        append(all.g_n2, t.g_n2);
        append(all.mass, t.mass);
        append(all.inv_area, t.inv_area);
        append(all.weight_ratio, t.weight_ratio);
        append(all.dtm_own, t.dtm_own);
        append(all.dtm_face, t.dtm_face);
        append(all.dtm32_own, t.dtm32_own);
        append(all.dtm32_face, t.dtm32_face);
        append(all.nb_face_node, t.nb_face_node);
        append(all.edge_left, t.edge_left);
        append(all.edge_right, t.edge_right);
        append(all.edge_geo, t.edge_geo);
        append(all.bface, t.bface);
        append(all.bface_cond, t.bface_cond);
        append(all.bface_geo, t.bface_geo);
        elem_member.insert(elem_member.end(), (size_t)t.K, m);
        Member& mm = h->members[m];
        mm.group = (int)(&G - h->groups.data());
        mm.k0 = k0;
        mm.K = t.K;
        mm.node0 = k0 * nn;
        mm.n_values = t.K * nn;
        k0 += t.K;
        t = Tables();  // release as we go
    }
    G.K = k0;
    G.n_values = k0 * nn;
    DevTables& T = G.T;
    T.K = G.K;
    T.n_edges = (int64_t)all.edge_left.size();
    T.n_bfaces = (int64_t)all.bface.size();
    int s = DGSWE_OK;
#define UP(field, vec)                                                                \
    do {                                                                              \
        using E = std::remove_const_t<std::remove_pointer_t<decltype(T.field)>>;      \
        E* p = nullptr;                                                               \
        if ((s = device_array(h, vec.size(), &p))) return s;                          \
        if ((s = upload_into(h, vec.data(), vec.size() * sizeof(E), p))) return s;    \
        T.field = p;                                                                  \
    } while (0)
    UP(bed, all.bed);
    UP(jinv, all.jinv);
    UP(pair_hm, all.pair_hm);
    UP(gdb, all.gdb);
    UP(contra, all.contra);
    UP(lift_scale, all.lift_scale);
    UP(outer_dist, all.outer_dist);
    UP(fcor, all.fcor);
    UP(g_n2, all.g_n2);
    UP(mass, all.mass);
    UP(inv_area, all.inv_area);
    UP(weight_ratio, all.weight_ratio);
    UP(dtm_own, all.dtm_own);
    UP(dtm_face, all.dtm_face);
    UP(dtm32_own, all.dtm32_own);
    UP(dtm32_face, all.dtm32_face);
    UP(edge_geo, all.edge_geo);
    UP(bface_geo, all.bface_geo);
    UP(outer_idx, all.outer_idx);
    UP(nb_face_node, all.nb_face_node);
    UP(edge_left, all.edge_left);
    UP(edge_right, all.edge_right);
    UP(bface, all.bface);
    UP(bface_cond, all.bface_cond);
    UP(affine, all.affine);
    UP(elem_member, elem_member);
    PairSchedule sched(ops);
    const std::vector<int8_t> owned = owned_table(sched);
    UP(sched_owned, owned);
    UP(sched_slot, sched.accum_slot);
    UP(sched_coef, sched.accum_coef);
    std::vector<double> hcoef(sched.accum_coef.size());
    for (size_t q = 0; q < hcoef.size(); ++q) hcoef[q] = 0.5 * sched.accum_coef[q];
    UP(sched_hcoef, hcoef);
    UP(pair_coef, pair_coef_table(sched));
#undef UP
    fill_physics(h->form0, ops, fcor, G.P, G.X);
    G.P.has_bed = h->form0.bathymetry ? 1 : 0;
    G.P.friction = friction ? DGSWE_FRICTION_MANNING_NODES : DGSWE_FRICTION_NONE;
    G.P.n_conditions = 0;  // the conditions are in T.cond
    // state and stage buffers, face fluxes
    for (int b = 0; b < kEnsBuffers; ++b) {
        double* p = nullptr;
        if ((s = device_array(h, 5 * (size_t)G.n_values, &p))) return s;
        CK(cudaMemset(p, 0, 5 * (size_t)G.n_values * sizeof(double)));
        const size_t n = (size_t)G.n_values;
        G.buf_base[b] = p;
        G.buf[b] = {p, p + n, p + 2 * n, p + 3 * n, p + 4 * n};
    }
    const size_t nf = (size_t)G.K * 4 * n1;
    double* fb = nullptr;
    if ((s = device_array(h, 3 * nf, &fb))) return s;
    CK(cudaMemset(fb, 0, 3 * nf * sizeof(double)));
    G.fb_h = fb;
    G.fb_hu = fb + nf;
    G.fb_hv = fb + 2 * nf;
    return DGSWE_OK;
}

int create_impl(dgswe_ensemble* h, const dgswe_form* forms, int n, int device) {
    h->device = device;
    h->n_members = n;
    CK(cudaSetDevice(device));
    cudaDeviceProp prop{};
    CK(cudaGetDeviceProperties(&prop, device));
    h->device_name = prop.name;
    CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&h->fork, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&h->join, cudaEventDisableTiming));
    CK(cudaEventCreate(&h->t0));
    CK(cudaEventCreate(&h->t1));
    h->form0 = forms[0];
    h->ks = forms[0].numerics == DGSWE_NUMERICS_EXACT ? kernels_exact() : kernels_fast();
    h->members.assign(n, Member{});
    // members' boundary conditions, back to back
    std::vector<int> cond_base(n, 0);
    std::vector<Condition> conds;
    for (int m = 0; m < n; ++m) {
        if (forms[m].relaxation)
            return fail(h, DGSWE_ERR_UNSUPPORTED,
                        "member %d: a nesting relaxation band runs on a single mesh", m);
        if (forms[m].atmosphere)
            return fail(h, DGSWE_ERR_UNSUPPORTED, "member %d: the weather runs on a single mesh",
                        m);
        cond_base[m] = (int)conds.size();
        for (int b = 0; b < forms[m].n_boundaries; ++b) {
            if (forms[m].boundaries[b].kind == DGSWE_BC_NODE_TIDES ||
                forms[m].boundaries[b].kind == DGSWE_BC_PARENT)
                return fail(h, DGSWE_ERR_UNSUPPORTED,
                            "member %d: boundary data per node runs on a single mesh", m);
            conds.push_back(make_condition(forms[m].boundaries[b]));
        }
    }
    h->cond_base = cond_base;
    // order groups, members in the caller's order within each
    for (int order = 1; order <= 4; ++order) {
        std::vector<int> ms;
        for (int m = 0; m < n; ++m)
            if (forms[m].order == order) ms.push_back(m);
        if (ms.empty()) continue;
        h->groups.emplace_back();
        Group& G = h->groups.back();
        G.ops = new Operators(order);
        G.n1 = G.ops->n1;
        G.nn = G.ops->nn;
        G.members = ms;
    }
    for (Group& G : h->groups) {
        std::vector<Tables> tabs(G.members.size());
        std::vector<std::string> errs(G.members.size());
#pragma omp parallel for schedule(dynamic, 1)
        for (int64_t q = 0; q < (int64_t)G.members.size(); ++q) {
            const dgswe_form& f = forms[G.members[q]];
            Topology topo;
            std::string err = build_topology(f, topo);
            if (err.empty()) {
                std::vector<int32_t> tags, cond_index;
                for (int b = 0; b < f.n_boundaries; ++b) {
                    tags.push_back(f.boundaries[b].tag);
                    cond_index.push_back(b);
                }
                err = build_tables(f, *G.ops, topo, tags, cond_index, tabs[q]);
            }
            errs[q] = err;
        }
        for (size_t q = 0; q < errs.size(); ++q)
            if (!errs[q].empty())
                return fail(h, DGSWE_ERR_INVALID, "member %d: %s", G.members[q], errs[q].c_str());
        if (int s = build_group(h, G, tabs, cond_base, forms)) return s;
    }
    Condition* d_cond = nullptr;
    if (int s = device_array(h, conds.size(), &d_cond)) return s;
    if (int s = upload_into(h, conds.data(), conds.size() * sizeof(Condition), d_cond)) return s;
    for (Group& G : h->groups) G.T.cond = d_cond;
    if (int s = device_array(h, (size_t)n, &h->ctl)) return s;
    void* p = nullptr;
    CK(cudaMallocHost(&p, (size_t)n * sizeof(StepCtl)));
    h->h_ctl = (StepCtl*)p;
    std::memset(h->h_ctl, 0, (size_t)n * sizeof(StepCtl));
    for (int m = 0; m < n; ++m) {
        h->h_ctl[m].always = 1;
        h->h_ctl[m].active = 1;
    }
    CK(cudaMemcpy(h->ctl, h->h_ctl, (size_t)n * sizeof(StepCtl), cudaMemcpyHostToDevice));
    if (int s = device_array(h, 1, &h->always)) return s;
    const int one = 1;
    CK(cudaMemcpy(h->always, &one, sizeof one, cudaMemcpyHostToDevice));
    h->form0.vertices = nullptr;
    h->form0.elements = nullptr;
    h->form0.periodic = nullptr;
    h->form0.face_tags = nullptr;
    h->form0.manning_n_nodes = nullptr;
    h->form0.boundaries = nullptr;
    return DGSWE_OK;
}

// Every member's clock from run->t_start (NaN: from the member's own time,
// where its previous run ended), and the node velocities
int begin_run(dgswe_ensemble* h, const dgswe_run_config* run, int64_t steps) {
    double st[4][4];
    const int n_stages = scheme_table(run->scheme, st);
    for (int m = 0; m < h->n_members; ++m) {
        StepCtl& c = h->h_ctl[m];
        const double t_own = c.t;  // the mirror holds the device's state after each run
        const long long clips = c.clips;
        std::memset(&c, 0, sizeof c);
        c.t = std::isnan(run->t_start) ? t_own : run->t_start;
        c.clips = clips;
        c.t_end = INFINITY;
        c.target = INFINITY;
        c.dt_max = run->dt_max;
        c.dt_min = run->dt_min;
        c.cfl = run->cfl;
        c.dt_min_used = INFINITY;
        c.dt_max_used = 0.0;
        c.dt_bits = 0x7FF0000000000000ull;
        c.max_steps = steps;
        c.always = 1;
        c.active = 1;
        c.scheme_stages = n_stages;
        for (int s = 0; s < n_stages; ++s) {
            c.st_start[s] = st[s][0];
            c.st_input[s] = st[s][1];
            c.st_beta[s] = st[s][2];
            c.st_c[s] = st[s][3];
        }
    }
    CK(cudaMemcpyAsync(h->ctl, h->h_ctl, (size_t)h->n_members * sizeof(StepCtl),
                       cudaMemcpyHostToDevice, h->stream));
    for (Group& G : h->groups) h->ks->velocity(G.buf[DGSWE_STATE], G.n_values, G.P.h_min, h->stream);
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaGetLastError());
    return DGSWE_OK;
}

// One step of every member, captured once per (scheme, cfl)
int step_graph(dgswe_ensemble* h, int scheme, double cfl) {
    if (h->graph && h->graph_scheme == scheme && h->graph_cfl == cfl) return DGSWE_OK;
    if (h->graph) {
        cudaGraphExecDestroy(h->graph);
        h->graph = nullptr;
    }
    double st[4][4];
    const int n = scheme_table(scheme, st);
    const int* on = h->always;
    cudaStream_t main = h->stream;
    auto stream_of = [&](size_t g) { return g % 2 == 0 ? main : h->side; };
    auto fork = [&]() -> cudaError_t {
        cudaError_t e = cudaEventRecord(h->fork, main);
        return e != cudaSuccess ? e : cudaStreamWaitEvent(h->side, h->fork, 0);
    };
    auto join = [&]() -> cudaError_t {
        cudaError_t e = cudaEventRecord(h->join, h->side);
        return e != cudaSuccess ? e : cudaStreamWaitEvent(main, h->join, 0);
    };
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(main, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaSuccess;
    h->ks->step_begin(h->ctl, h->n_members, main);
    if (e == cudaSuccess) e = fork();
    for (size_t g = 0; g < h->groups.size(); ++g) {
        Group& G = h->groups[g];
        dgswe_form fg = h->form0;  // the positivity bound's limits of the group's order
        fg.order = G.ops->order;
        const DtParams Dg = dt_params(fg, cfl, scheme);
        h->ks->dt(G.n1, G.T, G.P, G.buf[DGSWE_STATE], Dg, nullptr, h->ctl, on, stream_of(g));
    }
    if (e == cudaSuccess) e = join();
    h->ks->step_dt(h->ctl, h->n_members, main);
    for (int s = 0; s < n; ++s) {
        const int in = s == 0 ? DGSWE_STATE : s;
        const int out = s + 1 < n ? s + 1 : DGSWE_STATE;
        if (e == cudaSuccess) e = fork();
        for (size_t g = 0; g < h->groups.size(); ++g) {
            Group& G = h->groups[g];
            cudaStream_t sg = stream_of(g);
            h->ks->face(G.n1, G.T, G.P, G.buf[in], G.fb_h, G.fb_hu, G.fb_hv, h->ctl, s, on, sg);
            h->ks->stage(G.n1, G.T, G.P, G.X, G.buf[in], G.buf[DGSWE_STATE], G.buf[out],
                         G.buf[DGSWE_STATE], G.fb_h, G.fb_hu, G.fb_hv, h->ctl, s, kModePost,
                         s + 1 == n, on, sg);
        }
        if (e == cudaSuccess) e = join();
    }
    h->ks->step_end(h->ctl, h->n_members, main);
    cudaError_t e2 = cudaStreamEndCapture(main, &graph);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return fail(h, DGSWE_ERR_CUDA, "stream capture: %s",
                    cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    e = cudaGraphInstantiate(&h->graph, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail(h, DGSWE_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
    h->graph_scheme = scheme;
    h->graph_cfl = cfl;
    return DGSWE_OK;
}

bool valid_member(const dgswe_ensemble* h, int m) { return h && m >= 0 && m < h->n_members; }

}  // namespace

extern "C" {

int dgswe_ensemble_create(const dgswe_form* forms, int n_members, int device,
                          dgswe_ensemble** out) {
    if (!out) return DGSWE_ERR_INVALID;
    *out = nullptr;
    auto* h = new dgswe_ensemble();
    *out = h;
    if (!forms || n_members <= 0) return fail(h, DGSWE_ERR_INVALID, "no members");
    for (int m = 0; m < n_members; ++m) {
        std::string why;
        if (int s = check_form(&forms[m], why)) return fail(h, s, "member %d: %s", m, why.c_str());
        if (!same_physics(forms[0], forms[m]))
            return fail(h, DGSWE_ERR_INVALID,
                        "member %d: the physics options differ from member 0's", m);
    }
    int n_dev = 0;
    if (cudaGetDeviceCount(&n_dev) != cudaSuccess || n_dev == 0)
        return fail(h, DGSWE_ERR_NO_DEVICE, "no CUDA device");
    if (device < 0 || device >= n_dev) return fail(h, DGSWE_ERR_INVALID, "no device %d", device);
    return create_impl(h, forms, n_members, device);
}

void dgswe_ensemble_destroy(dgswe_ensemble* h) { delete h; }

const char* dgswe_ensemble_last_error(const dgswe_ensemble* h) {
    return h ? h->error.c_str() : "";
}

int dgswe_ensemble_n_members(const dgswe_ensemble* h) { return h ? h->n_members : 0; }

int64_t dgswe_ensemble_n_values(const dgswe_ensemble* h, int member) {
    return valid_member(h, member) ? h->members[member].n_values : 0;
}

int dgswe_ensemble_upload(dgswe_ensemble* h, int member, const double* hh, const double* hu,
                          const double* hv, int64_t n) {
    if (!valid_member(h, member)) return fail(h, DGSWE_ERR_INVALID, "no member %d", member);
    const Member& m = h->members[member];
    if (n != m.n_values || !hh || !hu || !hv)
        return fail(h, DGSWE_ERR_INVALID, "member %d holds %lld values", member,
                    (long long)m.n_values);
    CK(cudaSetDevice(h->device));
    const DevBuf& b = h->groups[m.group].buf[DGSWE_STATE];
    CK(cudaMemcpyAsync(b.h + m.node0, hh, n * sizeof(double), cudaMemcpyDefault, h->stream));
    CK(cudaMemcpyAsync(b.hu + m.node0, hu, n * sizeof(double), cudaMemcpyDefault, h->stream));
    CK(cudaMemcpyAsync(b.hv + m.node0, hv, n * sizeof(double), cudaMemcpyDefault, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return DGSWE_OK;
}

int dgswe_ensemble_download(dgswe_ensemble* h, int member, double* hh, double* hu, double* hv,
                            int64_t n) {
    if (!valid_member(h, member)) return fail(h, DGSWE_ERR_INVALID, "no member %d", member);
    const Member& m = h->members[member];
    if (n != m.n_values || !hh || !hu || !hv)
        return fail(h, DGSWE_ERR_INVALID, "member %d holds %lld values", member,
                    (long long)m.n_values);
    CK(cudaSetDevice(h->device));
    const DevBuf& b = h->groups[m.group].buf[DGSWE_STATE];
    CK(cudaMemcpyAsync(hh, b.h + m.node0, n * sizeof(double), cudaMemcpyDefault, h->stream));
    CK(cudaMemcpyAsync(hu, b.hu + m.node0, n * sizeof(double), cudaMemcpyDefault, h->stream));
    CK(cudaMemcpyAsync(hv, b.hv + m.node0, n * sizeof(double), cudaMemcpyDefault, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return DGSWE_OK;
}

int dgswe_ensemble_run(dgswe_ensemble* h, const dgswe_run_config* run, int64_t steps,
                       dgswe_report* reports, dgswe_profile* profile) {
    if (!h) return DGSWE_ERR_INVALID;
    if (!run || steps < 0) return fail(h, DGSWE_ERR_INVALID, "run configuration");
    if (run->scheme != DGSWE_SSP_RK3 && run->scheme != DGSWE_SSP_RK43)
        return fail(h, DGSWE_ERR_UNSUPPORTED, "unknown SSP scheme");
    if (!(run->cfl > 0.0)) return fail(h, DGSWE_ERR_INVALID, "cfl must be positive");
    CK(cudaSetDevice(h->device));
    if (int s = begin_run(h, run, steps)) return s;
    if (int s = step_graph(h, run->scheme, run->cfl)) return s;
    const auto wall0 = std::chrono::steady_clock::now();
    CK(cudaEventRecord(h->t0, h->stream));
    for (int64_t i = 0; i < steps; ++i) CK(cudaGraphLaunch(h->graph, h->stream));
    CK(cudaEventRecord(h->t1, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaGetLastError());
    const double wall =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - wall0).count();
    float ms = 0.0f;
    CK(cudaEventElapsedTime(&ms, h->t0, h->t1));
    CK(cudaMemcpy(h->h_ctl, h->ctl, (size_t)h->n_members * sizeof(StepCtl),
                  cudaMemcpyDeviceToHost));
    int status = DGSWE_OK;
    for (int m = 0; m < h->n_members; ++m) {
        const StepCtl& c = h->h_ctl[m];
        // a member that used its steps stops with the step-limit flag: that is success here
        const int failure = c.failure == DGSWE_ERR_MAX_STEPS ? 0 : c.failure;
        if (failure && status == DGSWE_OK) status = failure;
        if (!reports) continue;
        dgswe_report& r = reports[m];
        std::memset(&r, 0, sizeof r);
        r.success = failure == 0;
        r.final_time = c.t;
        r.n_steps = c.steps;
        r.dt_min_used = c.dt_min_used;
        r.dt_max_used = c.dt_max_used;
        r.wall_time = wall;
        r.negative_depth_clips = c.clips;
        if (failure) std::snprintf(r.message, sizeof r.message, "%s", dgswe_status_string(failure));
        std::snprintf(r.device, sizeof r.device, "%s", h->device_name.c_str());
    }
    if (profile) {
        std::memset(profile, 0, sizeof(*profile));
        profile->steps = steps;
        profile->total_ms = ms;
        profile->control_launches = 3 * steps;
        profile->dt_launches = (int64_t)h->groups.size() * steps;
        profile->face_launches = (int64_t)h->groups.size() * h->h_ctl[0].scheme_stages * steps;
        profile->stage_launches = profile->face_launches;
        double t_max = 0.0;
        for (int m = 0; m < h->n_members; ++m) t_max = std::fmax(t_max, h->h_ctl[m].t);
        profile->t_final = t_max;
    }
    if (status != DGSWE_OK) fail(h, status, "%s", dgswe_status_string(status));
    return status;
}

}  // extern "C"
