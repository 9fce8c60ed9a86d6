// The discrete adjoint of a WetDry SSP-RK3 run (no reference counterpart:
// the reference has no adjoint). J = Σ over the steps n = 1..N and the
// stations s of (η_s(q_n) − η_obs[n][s])², η = h + B interpolated in the
// station's element. Reverse mode gives ∂J/∂ of the initial state, the bed
// elevation B per node, Manning's n per node and each boundary condition's
// tide constituents (amplitude, phase), for the steps the forward took:
// the time steps and every branch (wet/dry tests, limiter, HLL wave speeds)
// are the forward's.
//
// It runs on one mesh (a dgswe handle) or on an ensemble of members of one
// order (the ensemble's concatenated tables; each member its own time steps,
// stations and J): the same kernels, with each element reading its member's
// step control.
//
// Storage: the reverse of a step needs its start state, its stage inputs
// and what each stage's reverse keeps (the combination and the damped
// momentum). When all N step-start states fit in the memory budget, the
// forward sweep keeps them all and the reverse recomputes each step's
// stages once. Otherwise the forward keeps every s-th state (checkpoints)
// and the reverse replays each segment of s steps from its checkpoint
// before reversing it:
//  - full segments, when the budget holds them: the replay keeps every
//    step's stage inputs with their node velocities and the kept values
//    (10 states a step), so each step is computed once in the reverse
//    sweep;
//  - else step-start segments: the replay keeps the s step-start states and
//    each step's stages are computed again as it is reversed (twice in all).
// s is the caller's checkpoint interval, or the one the budget allows with
// the least memory.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/dgswe.h"
#include "device.hpp"
#include "ensemble_internal.hpp"
#include "handle.hpp"
#include "host_common.hpp"
#include "kernel_set.hpp"
#include "setup.hpp"

using namespace dgswe;
using namespace dgswe::host;

static_assert(DGSWE_MAX_CONSTITUENTS == kMaxConstituents, "constituent table size");

namespace {

// What the adjoint drives: the tables, physics, buffers and step control of
// one mesh or of one order group of an ensemble
struct Target {
    int device = 0;
    cudaStream_t stream = nullptr;
    const KernelSet* ks = nullptr;
    DevTables* T = nullptr;
    const Physics* P = nullptr;
    const StageExtra* X = nullptr;
    StepCtl* ctl = nullptr;
    int n_members = 1;
    double *fb_h = nullptr, *fb_hu = nullptr, *fb_hv = nullptr;
    DevBuf state{};
    int64_t K = 0, nv = 0;
    int n1 = 0, nn = 0, order = 0;
    dgswe_form form0{};
    std::vector<int64_t> k0, nvals;   // per member: first element, values
    std::vector<int> cond0, ncond;    // per member: first condition, count
    int n_cond = 0;
    // the parameters a calibration changes between sweeps: the tide
    // constituents (in Physics::cond of one mesh, or the ensemble's device
    // table) and g·n² per node (null: a uniform coefficient)
    Physics* cond_host = nullptr;
    Condition* cond_dev = nullptr;
    double* g_n2 = nullptr;
};

}  // namespace

struct dgswe_adjoint {
    dgswe_handle* h = nullptr;       // one mesh
    dgswe_ensemble* ens = nullptr;   // or an ensemble
    Target tg;
    std::string error;
    dgswe_adjoint_config cfg{};
    std::vector<double> stations;    // [n][2]
    std::vector<int32_t> st_member;
    std::vector<int64_t> st_elem;    // global element
    std::vector<double> st_w;        // [n][nn]
    std::vector<double> manning_n;   // n per node, concatenated
    double friction_g = 0.0;
    std::vector<double> J_member;
    // device
    std::vector<void*> allocations;
    int64_t* d_node0 = nullptr;
    double* d_w = nullptr;
    StageArgs* d_args = nullptr;  // [n_steps][n_members][3] the forward's stage weights
    double* d_eta = nullptr;      // [n_steps][n_stations]
    double* d_obs = nullptr;      // [n_steps][n_stations]
    double* d_ckpt = nullptr;     // stored step-start states, 3·nv doubles each
    double* d_seg = nullptr;      // a segment's step-start states, or full steps (stride > 1)
    int64_t stride = 1, n_ckpt = 0;
    bool full = false;            // full segments: per step q, S1, S2 (3 fields), keep (3 × 5)
    DevBuf S[4]{};  // the step's stage inputs and last output
    DevBuf Kp[3]{}; // kept combination and damped momentum of each stage
    double *lam[3] = {}, *lam_t[3] = {}, *lam_b[3] = {};
    // the current reverse sweep sums λ of the bed (its caller asked for it)
    bool want_bed = true;
    AdjStage A{};
    bool forward_done = false;
    dgswe_adjoint_stats stats{};
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    // the stage adjoint's subcell pass runs on its own stream beside the
    // wet pass, forked from and joined to the target's stream
    cudaStream_t sub_stream = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;

    ~dgswe_adjoint() {
        if (h || ens) {
            cudaSetDevice(tg.device);
            for (void* p : allocations) cudaFree(p);
            if (e0) cudaEventDestroy(e0);
            if (e1) cudaEventDestroy(e1);
            if (fork) cudaEventDestroy(fork);
            if (join) cudaEventDestroy(join);
            if (sub_stream) cudaStreamDestroy(sub_stream);
        }
        if (h) dgswe_destroy(h);
        if (ens) dgswe_ensemble_destroy(ens);
    }
};

namespace {

int afail(dgswe_adjoint* a, int status, const char* fmt, ...) {
    char msg[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(msg, sizeof msg, fmt, ap);
    va_end(ap);
    if (a) a->error = msg;
    return status;
}

#define ACK(call)                                                                              \
    do {                                                                                       \
        cudaError_t err_ = (call);                                                             \
        if (err_ != cudaSuccess)                                                               \
            return afail(a, DGSWE_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(err_)); \
    } while (0)

template <class T>
int dalloc(dgswe_adjoint* a, size_t n, T** out) {
    *out = nullptr;
    if (n == 0) return DGSWE_OK;
    void* p = nullptr;
    ACK(cudaMalloc(&p, n * sizeof(T)));
    a->allocations.push_back(p);
    ACK(cudaMemset(p, 0, n * sizeof(T)));
    *out = (T*)p;
    return DGSWE_OK;
}

int devbuf(dgswe_adjoint* a, int64_t n, DevBuf& b) {
    double* p = nullptr;
    if (int s = dalloc(a, 5 * (size_t)n, &p)) return s;
    b = {p, p + n, p + 2 * n, p + 3 * n, p + 4 * n};
    return DGSWE_OK;
}

// (r, s) of (x, y) in a bilinear quad by Newton from its centre; false if
// outside (with a small tolerance)
bool locate(const double* c, double x, double y, double& r, double& s) {
    r = 0.0;
    s = 0.0;
    for (int it = 0; it < 30; ++it) {
        const double n0 = (1 - r) * (1 - s) / 4, n1 = (1 + r) * (1 - s) / 4, n2 = (1 + r) * (1 + s) / 4,
                     n3 = (1 - r) * (1 + s) / 4;
        const double fx = n0 * c[0] + n1 * c[2] + n2 * c[4] + n3 * c[6] - x;
        const double fy = n0 * c[1] + n1 * c[3] + n2 * c[5] + n3 * c[7] - y;
        const double xr = (-(1 - s) * c[0] + (1 - s) * c[2] + (1 + s) * c[4] - (1 + s) * c[6]) / 4;
        const double xs = (-(1 - r) * c[0] - (1 + r) * c[2] + (1 + r) * c[4] + (1 - r) * c[6]) / 4;
        const double yr = (-(1 - s) * c[1] + (1 - s) * c[3] + (1 + s) * c[5] - (1 + s) * c[7]) / 4;
        const double ys = (-(1 - r) * c[1] - (1 + r) * c[3] + (1 + r) * c[5] + (1 - r) * c[7]) / 4;
        const double det = xr * ys - xs * yr;
        if (det == 0.0) return false;
        const double dr = (ys * fx - xs * fy) / det, ds = (-yr * fx + xr * fy) / det;
        r -= dr;
        s -= ds;
        if (std::fabs(dr) + std::fabs(ds) < 1e-14) break;
    }
    const double tol = 1e-9;
    return std::fabs(r) <= 1.0 + tol && std::fabs(s) <= 1.0 + tol;
}

double lagrange(const std::vector<double>& x, int a, double r) {
    double l = 1.0;
    for (size_t m = 0; m < x.size(); ++m)
        if ((int)m != a) l *= (r - x[m]) / (x[a] - x[m]);
    return l;
}

// the element of a form holding (x, y), and the point's reference coordinates
int64_t find_element(const dgswe_form& f, double x, double y, double& r, double& s) {
    for (int64_t k = 0; k < f.n_elements; ++k) {
        double c[8];
        for (int v = 0; v < 4; ++v) {
            const int64_t vi = f.elements[k * 4 + v];
            c[2 * v] = f.vertices[vi * 2];
            c[2 * v + 1] = f.vertices[vi * 2 + 1];
        }
        const double xmin = std::min({c[0], c[2], c[4], c[6]}), xmax = std::max({c[0], c[2], c[4], c[6]});
        const double ymin = std::min({c[1], c[3], c[5], c[7]}), ymax = std::max({c[1], c[3], c[5], c[7]});
        if (x < xmin - 1e-9 * (1 + std::fabs(xmin)) || x > xmax + 1e-9 * (1 + std::fabs(xmax)) ||
            y < ymin - 1e-9 * (1 + std::fabs(ymin)) || y > ymax + 1e-9 * (1 + std::fabs(ymax)))
            continue;
        if (locate(c, x, y, r, s)) return k;
    }
    return -1;
}

// copy (h, hu, hv) between a DevBuf and 3n packed doubles
int pack(dgswe_adjoint* a, double* dst, const DevBuf& src, int64_t n, cudaStream_t st) {
    const size_t bytes = (size_t)n * sizeof(double);
    ACK(cudaMemcpyAsync(dst, src.h, bytes, cudaMemcpyDeviceToDevice, st));
    ACK(cudaMemcpyAsync(dst + n, src.hu, bytes, cudaMemcpyDeviceToDevice, st));
    ACK(cudaMemcpyAsync(dst + 2 * n, src.hv, bytes, cudaMemcpyDeviceToDevice, st));
    return DGSWE_OK;
}
int unpack(dgswe_adjoint* a, const DevBuf& dst, const double* src, int64_t n, cudaStream_t st) {
    const size_t bytes = (size_t)n * sizeof(double);
    ACK(cudaMemcpyAsync(dst.h, src, bytes, cudaMemcpyDeviceToDevice, st));
    ACK(cudaMemcpyAsync(dst.hu, src + n, bytes, cudaMemcpyDeviceToDevice, st));
    ACK(cudaMemcpyAsync(dst.hv, src + 2 * n, bytes, cudaMemcpyDeviceToDevice, st));
    return DGSWE_OK;
}

// the stage weights of step n into every member's StepCtl, or back
int args_to_ctl(dgswe_adjoint* a, int64_t n) {
    const Target& t = a->tg;
    ACK(cudaMemcpy2DAsync(t.ctl[0].stage, sizeof(StepCtl), a->d_args + 3 * n * t.n_members,
                          3 * sizeof(StageArgs), 3 * sizeof(StageArgs), t.n_members,
                          cudaMemcpyDeviceToDevice, t.stream));
    return DGSWE_OK;
}
int ctl_to_args(dgswe_adjoint* a, int64_t n) {
    const Target& t = a->tg;
    ACK(cudaMemcpy2DAsync(a->d_args + 3 * n * t.n_members, 3 * sizeof(StageArgs), t.ctl[0].stage,
                          sizeof(StepCtl), 3 * sizeof(StageArgs), t.n_members,
                          cudaMemcpyDeviceToDevice, t.stream));
    return DGSWE_OK;
}

// One forward step of the state in `q` (velocities current), with the
// stage weights already in every member's StepCtl; S[1], S[2] take the
// intermediate stages, the result lands in q
void forward_step(dgswe_adjoint* a, const DevBuf& q) {
    const Target& t = a->tg;
    const int* on = &t.ctl[0].always;
    const DevBuf* ins[3] = {&q, &a->S[1], &a->S[2]};
    const DevBuf* outs[3] = {&a->S[1], &a->S[2], &q};
    for (int s = 0; s < 3; ++s) {
        t.ks->face(t.n1, *t.T, *t.P, *ins[s], t.fb_h, t.fb_hu, t.fb_hv, t.ctl, s, on, t.stream);
        t.ks->stage(t.n1, *t.T, *t.P, *t.X, *ins[s], q, *outs[s], q, t.fb_h, t.fb_hu, t.fb_hv,
                    t.ctl, s, kModePost, s == 2, on, t.stream);
    }
}

// The three stages of a step reversed, the stage inputs in[0..2] and what
// they keep keep[0..2]: λ of each stage's input from λ of its output, then
// λ of the step's start state (the first stage's input plus the three
// stages' base terms) into lam
int reverse_stages(dgswe_adjoint* a, const DevBuf* in, const DevBuf* keep) {
    const Target& t = a->tg;
    const int64_t nv = t.nv;
    cudaStream_t st = t.stream;
    // the three stage inputs' subcell elements
    ACK(cudaMemsetAsync(a->A.sub_count, 0, 3 * sizeof(unsigned long long), st));
    t.ks->subcell_list(*t.T, *t.P, in[0].h, in[1].h, in[2].h, a->A, t.nn, st);
    for (int s = 2; s >= 0; --s) {
        AdjStage As = a->A;
        double** lo = s == 2 ? a->lam : a->lam_t;
        As.lo_h = lo[0];
        As.lo_hu = lo[1];
        As.lo_hv = lo[2];
        if (!a->want_bed) As.lbed = nullptr;  // λ of the bed neither summed nor written
        // the subcell pass beside the wet pass; the face adjoint after both
        ACK(cudaEventRecord(a->fork, st));
        ACK(cudaStreamWaitEvent(a->sub_stream, a->fork, 0));
        t.ks->stage_adjoint(t.n1, *t.T, *t.P, *t.X, in[s], keep[s], As, t.ctl, s, 1,
                            a->sub_stream);
        ACK(cudaEventRecord(a->join, a->sub_stream));
        t.ks->stage_adjoint(t.n1, *t.T, *t.P, *t.X, in[s], keep[s], As, t.ctl, s, 0, st);
        ACK(cudaStreamWaitEvent(st, a->join, 0));
        t.ks->face_adjoint(t.n1, *t.T, *t.P, in[s], As, t.ctl, s, st);
        // the first stage's input is the step's start: its λ, with the base
        // terms, into lam
        double** out = s == 0 ? a->lam : a->lam_t;
        t.ks->adjoint_combine(in[s], As, out[0], out[1], out[2], s == 0 ? a->lam_b : nullptr, nv,
                              t.P->h_min, st);
    }
    return DGSWE_OK;
}

// Everything after the target exists: stations, the bed slope's transpose,
// buffers, checkpoints
int setup(dgswe_adjoint* a, const dgswe_form* forms, const dgswe_adjoint_config* cfg) {
    Target& t = a->tg;
    const int nn = t.nn, n1 = t.n1;
    const int64_t nv = t.nv;
    Operators ops(t.order);
    // stations: element (global) and Lagrange weights
    for (int s = 0; s < cfg->n_stations; ++s) {
        const int m = a->st_member[s];
        double r = 0, q = 0;
        const int64_t k = find_element(forms[m], a->stations[2 * s], a->stations[2 * s + 1], r, q);
        if (k < 0) return afail(a, DGSWE_ERR_INVALID, "station %d is outside member %d's mesh", s, m);
        a->st_elem.push_back(t.k0[m] + k);
        for (int i = 0; i < nn; ++i)
            a->st_w.push_back(lagrange(ops.x, i % n1, r) * lagrange(ops.x, i / n1, q));
    }
    // Manning's n per node, for ∂J/∂n = ∂J/∂(g n²)·2 g n
    a->friction_g = forms[0].friction_g;
    a->manning_n.assign((size_t)nv, 0.0);
    for (int m = 0; m < t.n_members; ++m) {
        const dgswe_form& f = forms[m];
        double* o = &a->manning_n[(size_t)t.k0[m] * nn];
        for (int64_t i = 0; i < t.nvals[m]; ++i)
            o[i] = f.friction == DGSWE_FRICTION_MANNING_NODES ? f.manning_n_nodes[i]
                   : f.friction == DGSWE_FRICTION_MANNING       ? f.manning_n
                                                                : 0.0;
    }
    ACK(cudaSetDevice(t.device));
    ACK(cudaEventCreate(&a->e0));
    ACK(cudaEventCreate(&a->e1));
    ACK(cudaEventCreateWithFlags(&a->fork, cudaEventDisableTiming));
    ACK(cudaEventCreateWithFlags(&a->join, cudaEventDisableTiming));
    // the highest priority: the few subcell blocks, each long, start first
    int least = 0, greatest = 0;
    ACK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    ACK(cudaStreamCreateWithPriority(&a->sub_stream, cudaStreamNonBlocking, greatest));
    const int64_t nf = t.K * 4 * n1;
    // the bed slope's transpose: for node c, each line partner i's
    // ∂(g∇B)_i/∂B_c = g·D[pos_i][pos_c]·w(i, c), with w the forward's metric
    // weight (i's own on an affine element, else the mean of i's and c's)
    if (t.P->has_bed) {
        std::vector<double> contra(4 * (size_t)nv), gt(4 * (size_t)n1 * nv);
        std::vector<uint8_t> aff((size_t)t.K);
        ACK(cudaMemcpy(contra.data(), t.T->contra, contra.size() * sizeof(double), cudaMemcpyDeviceToHost));
        ACK(cudaMemcpy(aff.data(), t.T->affine, aff.size(), cudaMemcpyDeviceToHost));
        const double g = forms[0].g;
#pragma omp parallel for schedule(static)
        for (int64_t k = 0; k < t.K; ++k)
            for (int c = 0; c < nn; ++c)
                for (int dir = 0; dir < 2; ++dir) {
                    const int line = dir == 0 ? c / n1 : c % n1;
                    const int pc = dir == 0 ? c % n1 : c / n1;
                    const double* mc = &contra[(k * nn + c) * 4 + 2 * dir];
                    for (int pa = 0; pa < n1; ++pa) {
                        const int i = dir == 0 ? line * n1 + pa : pa * n1 + line;
                        const double* mi = &contra[(k * nn + i) * 4 + 2 * dir];
                        const double wx = aff[k] ? mi[0] : 0.5 * (mi[0] + mc[0]);
                        const double wy = aff[k] ? mi[1] : 0.5 * (mi[1] + mc[1]);
                        const double gd = g * ops.d[pa * n1 + pc];
                        double* o = &gt[(((k * nn + c) * 2 + dir) * n1 + pa) * 2];
                        o[0] = gd * wx;
                        o[1] = gd * wy;
                    }
                }
        double* d_gt = nullptr;
        if (int s = dalloc(a, gt.size(), &d_gt)) return s;
        ACK(cudaMemcpy(d_gt, gt.data(), gt.size() * sizeof(double), cudaMemcpyHostToDevice));
        t.T->gdb_t = d_gt;
    }
    const int n_st = cfg->n_stations;
    std::vector<int64_t> node0(n_st);
    for (int s = 0; s < n_st; ++s) node0[s] = a->st_elem[s] * nn;
    int s = DGSWE_OK;
    if ((s = dalloc(a, (size_t)n_st, &a->d_node0))) return s;
    if ((s = dalloc(a, a->st_w.size(), &a->d_w))) return s;
    if (n_st) {
        ACK(cudaMemcpy(a->d_node0, node0.data(), n_st * sizeof(int64_t), cudaMemcpyHostToDevice));
        ACK(cudaMemcpy(a->d_w, a->st_w.data(), a->st_w.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
    const int64_t N = cfg->n_steps;
    if ((s = dalloc(a, 3 * (size_t)N * t.n_members, &a->d_args))) return s;
    if ((s = dalloc(a, (size_t)N * n_st, &a->d_eta))) return s;
    if ((s = dalloc(a, (size_t)N * n_st, &a->d_obs))) return s;
    for (int b = 0; b < 4; ++b)
        if ((s = devbuf(a, nv, a->S[b]))) return s;
    for (int b = 0; b < 3; ++b)
        if ((s = devbuf(a, nv, a->Kp[b]))) return s;
    for (int c = 0; c < 3; ++c) {
        if ((s = dalloc(a, (size_t)nv, &a->lam[c]))) return s;
        if ((s = dalloc(a, (size_t)nv, &a->lam_t[c]))) return s;
        if ((s = dalloc(a, (size_t)nv, &a->lam_b[c]))) return s;
    }
    AdjStage& A = a->A;
    double* p = nullptr;
    if ((s = dalloc(a, 5 * (size_t)nv, &p))) return s;
    A.li_h = p;
    A.li_hu = p + nv;
    A.li_hv = p + 2 * nv;
    A.li_u = p + 3 * nv;
    A.li_v = p + 4 * nv;
    if ((s = dalloc(a, 5 * (size_t)nv, &p))) return s;
    A.lx_h = p;
    A.lx_hu = p + nv;
    A.lx_hv = p + 2 * nv;
    A.lx_u = p + 3 * nv;
    A.lx_v = p + 4 * nv;
    if ((s = dalloc(a, 3 * (size_t)nf, &p))) return s;
    A.lf_h = p;
    A.lf_hu = p + nf;
    A.lf_hv = p + 2 * nf;
    if ((s = dalloc(a, (size_t)nv, &A.lbed))) return s;
    if ((s = dalloc(a, (size_t)nv, &A.lgn2))) return s;
    if ((s = dalloc(a, (size_t)std::max(1, t.n_cond) * 2 * kMaxConstituents, &A.ltide))) return s;
    if ((s = dalloc(a, 3 * (size_t)std::max<int64_t>(1, t.T->K), &A.sub_list))) return s;
    if ((s = dalloc(a, 3, &A.sub_count))) return s;
    A.lb_h = a->lam_b[0];
    A.lb_hu = a->lam_b[1];
    A.lb_hv = a->lam_b[2];
    // checkpoints: every step-start state if the budget allows, else every
    // stride-th and one segment
    const double sb = 3.0 * (double)nv * sizeof(double);
    double budget = cfg->memory_budget;
    if (!(budget > 0.0)) {
        size_t free_b = 0, total = 0;
        ACK(cudaMemGetInfo(&free_b, &total));
        budget = std::max(0.0, (double)free_b - 2.0 * (1ull << 30));
    }
    // states held: checkpoints, and the segment (10 states a step when full)
    auto held = [&](int64_t st, bool full) {
        return (double)((N + st - 1) / st + (st > 1 ? (full ? 10 : 1) * st : 0)) * sb;
    };
    int64_t stride = 0;
    bool full = false;
    if (cfg->checkpoint_every > 0) {
        stride = std::min<int64_t>(cfg->checkpoint_every, N);
        if (stride > 1 && held(stride, true) <= budget) full = true;
        else if (held(stride, false) > budget)
            return afail(a, DGSWE_ERR_INVALID,
                         "checkpoints every %lld steps need %.3g B, over the budget of %.3g B",
                         (long long)stride, held(stride, false), budget);
    } else if (held(1, false) <= budget) {
        stride = 1;
    } else {
        double least = INFINITY;
        for (int64_t st = 2; st <= N; ++st)  // full segments with the least memory
            if (held(st, true) <= budget && held(st, true) < least) {
                least = held(st, true);
                stride = st;
                full = true;
            }
        for (int64_t st = 2; stride == 0 && st <= N; ++st)
            if (held(st, false) <= budget) stride = st;
        if (stride == 0)
            return afail(a, DGSWE_ERR_INVALID,
                         "the memory budget (%.3g B) holds fewer than 2·√N states of %.3g B", budget,
                         sb);
    }
    a->stride = stride;
    a->full = full;
    a->n_ckpt = (N + stride - 1) / stride;
    if ((s = dalloc(a, 3 * (size_t)nv * a->n_ckpt, &a->d_ckpt))) return s;
    if (stride > 1 && (s = dalloc(a, (full ? 30 : 3) * (size_t)nv * stride, &a->d_seg))) return s;
    a->stats.stride = stride;
    a->stats.full_segments = full ? 1 : 0;
    a->stats.stored_states = a->n_ckpt + (stride > 1 ? (full ? 10 : 1) * stride : 0);
    a->stats.stored_bytes = (double)a->stats.stored_states * sb;
    return DGSWE_OK;
}

int check_config(dgswe_adjoint* a, const dgswe_form* forms, int n, const dgswe_adjoint_config* cfg) {
    if (!cfg) return afail(a, DGSWE_ERR_INVALID, "no configuration");
    for (int m = 0; m < n; ++m) {
        std::string why;
        if (int s = check_form(&forms[m], why)) return afail(a, s, "member %d: %s", m, why.c_str());
        if (forms[m].formulation != DGSWE_WET_DRY)
            return afail(a, DGSWE_ERR_UNSUPPORTED, "the adjoint covers the WetDry formulation");
        if (forms[m].order != forms[0].order)
            return afail(a, DGSWE_ERR_UNSUPPORTED, "an adjoint ensemble has members of one order");
        if (forms[m].relaxation)
            return afail(a, DGSWE_ERR_UNSUPPORTED, "the adjoint covers no relaxation band");
        if (forms[m].atmosphere)
            return afail(a, DGSWE_ERR_UNSUPPORTED, "the adjoint covers no weather forcing");
        for (int b = 0; b < forms[m].n_boundaries; ++b)
            if (forms[m].boundaries[b].kind == DGSWE_BC_NODE_TIDES ||
                forms[m].boundaries[b].kind == DGSWE_BC_PARENT)
                return afail(a, DGSWE_ERR_UNSUPPORTED,
                             "the adjoint covers walls and uniform tides, not data per node");
    }
    if (cfg->scheme != DGSWE_SSP_RK3)
        return afail(a, DGSWE_ERR_UNSUPPORTED, "the adjoint covers SSP-RK3");
    if (cfg->n_steps <= 0 || cfg->n_stations < 0 || (cfg->n_stations > 0 && !cfg->stations))
        return afail(a, DGSWE_ERR_INVALID, "steps and stations");
    a->cfg = *cfg;
    a->stations.assign(cfg->stations, cfg->stations + 2 * (size_t)cfg->n_stations);
    a->cfg.stations = nullptr;
    a->st_member.assign((size_t)cfg->n_stations, 0);
    if (cfg->station_member) {
        for (int s = 0; s < cfg->n_stations; ++s) {
            if (cfg->station_member[s] < 0 || cfg->station_member[s] >= n)
                return afail(a, DGSWE_ERR_INVALID, "station %d's member", s);
            a->st_member[s] = cfg->station_member[s];
        }
    }
    a->cfg.station_member = nullptr;
    return DGSWE_OK;
}

}  // namespace

extern "C" {

int dgswe_adjoint_create(const dgswe_form* f, int device, const dgswe_adjoint_config* cfg,
                         dgswe_adjoint** out) {
    if (!out) return DGSWE_ERR_INVALID;
    auto* a = new dgswe_adjoint();
    *out = a;
    if (int s = check_config(a, f, 1, cfg)) return s;
    dgswe_handle* hd = nullptr;
    const int st = dgswe_create(f, device, &hd);
    a->h = hd;
    if (st != DGSWE_OK) return afail(a, st, "%s", hd ? dgswe_last_error(hd) : "create failed");
    dgswe_handle* h = hd;
    Target& t = a->tg;
    t.device = h->device;
    t.stream = h->stream;
    t.ks = h->ks;
    t.T = &h->T;
    t.P = &h->P;
    t.X = &h->X;
    t.ctl = h->ctl;
    t.n_members = 1;
    t.fb_h = h->fb_h;
    t.fb_hu = h->fb_hu;
    t.fb_hv = h->fb_hv;
    t.state = h->buf[DGSWE_STATE].view;
    t.K = h->K;
    t.nv = h->n_values;
    t.n1 = h->n1;
    t.nn = h->nn;
    t.order = f->order;
    t.form0 = h->form;
    t.k0 = {0};
    t.nvals = {h->n_values};
    t.cond0 = {0};
    t.ncond = {f->n_boundaries};
    t.n_cond = f->n_boundaries;
    t.cond_host = &h->P;
    t.g_n2 = const_cast<double*>(h->T.g_n2);
    return setup(a, f, cfg);
}

int dgswe_adjoint_create_ensemble(const dgswe_form* forms, int n_members, int device,
                                  const dgswe_adjoint_config* cfg, dgswe_adjoint** out) {
    if (!out) return DGSWE_ERR_INVALID;
    auto* a = new dgswe_adjoint();
    *out = a;
    if (!forms || n_members <= 0) return afail(a, DGSWE_ERR_INVALID, "no members");
    if (int s = check_config(a, forms, n_members, cfg)) return s;
    dgswe_ensemble* e = nullptr;
    const int st = dgswe_ensemble_create(forms, n_members, device, &e);
    a->ens = e;
    if (st != DGSWE_OK)
        return afail(a, st, "%s", e ? dgswe_ensemble_last_error(e) : "ensemble create failed");
    if (e->groups.size() != 1) return afail(a, DGSWE_ERR_UNSUPPORTED, "one order per ensemble");
    Group& G = e->groups[0];
    Target& t = a->tg;
    t.device = e->device;
    t.stream = e->stream;
    t.ks = e->ks;
    t.T = &G.T;
    t.P = &G.P;
    t.X = &G.X;
    t.ctl = e->ctl;
    t.n_members = n_members;
    t.fb_h = G.fb_h;
    t.fb_hu = G.fb_hu;
    t.fb_hv = G.fb_hv;
    t.state = G.buf[DGSWE_STATE];
    t.K = G.K;
    t.nv = G.n_values;
    t.n1 = G.n1;
    t.nn = G.nn;
    t.order = forms[0].order;
    t.form0 = e->form0;
    t.form0.order = forms[0].order;
    for (int m = 0; m < n_members; ++m) {
        t.k0.push_back(e->members[m].k0);
        t.nvals.push_back(e->members[m].n_values);
        t.cond0.push_back(e->cond_base[m]);
        t.ncond.push_back(forms[m].n_boundaries);
        t.n_cond += forms[m].n_boundaries;
    }
    t.cond_dev = const_cast<Condition*>(G.T.cond);
    t.g_n2 = const_cast<double*>(G.T.g_n2);
    return setup(a, forms, cfg);
}

void dgswe_adjoint_destroy(dgswe_adjoint* a) { delete a; }

const char* dgswe_adjoint_last_error(const dgswe_adjoint* a) { return a ? a->error.c_str() : ""; }

int64_t dgswe_adjoint_n_values(const dgswe_adjoint* a) { return a ? a->tg.nv : 0; }

int64_t dgswe_adjoint_member_offset(const dgswe_adjoint* a, int member) {
    if (!a || member < 0 || member >= a->tg.n_members) return -1;
    return a->tg.k0[member] * a->tg.nn;
}

int dgswe_adjoint_stations(const dgswe_adjoint* a, int64_t* element, double* weights) {
    if (!a || (!a->h && !a->ens)) return DGSWE_ERR_INVALID;
    if (element) std::copy(a->st_elem.begin(), a->st_elem.end(), element);
    if (weights) std::copy(a->st_w.begin(), a->st_w.end(), weights);
    return DGSWE_OK;
}

int dgswe_adjoint_forward(dgswe_adjoint* a, const double* h0, const double* hu0, const double* hv0,
                          const double* dts, const double* eta_obs, double* eta_out,
                          double* dts_out, double* J) {
    if (!a || (!a->h && !a->ens)) return DGSWE_ERR_INVALID;
    if (!h0 || !hu0 || !hv0) return afail(a, DGSWE_ERR_INVALID, "no initial state");
    Target& t = a->tg;
    ACK(cudaSetDevice(t.device));
    const int64_t nv = t.nv, N = a->cfg.n_steps;
    const int n_st = a->cfg.n_stations, nn = t.nn, M = t.n_members;
    cudaStream_t st = t.stream;
    const size_t bv = (size_t)nv * sizeof(double);
    ACK(cudaMemcpyAsync(t.state.h, h0, bv, cudaMemcpyDefault, st));
    ACK(cudaMemcpyAsync(t.state.hu, hu0, bv, cudaMemcpyDefault, st));
    ACK(cudaMemcpyAsync(t.state.hv, hv0, bv, cudaMemcpyDefault, st));
    if (n_st)
        ACK(eta_obs ? cudaMemcpyAsync(a->d_obs, eta_obs, (size_t)N * n_st * sizeof(double),
                                      cudaMemcpyDefault, st)
                    : cudaMemsetAsync(a->d_obs, 0, (size_t)N * n_st * sizeof(double), st));
    // every member's clock (CFL steps), or the given steps' stage weights
    double sc[4][4];
    const int n_stages = scheme_table(DGSWE_SSP_RK3, sc);
    const double cfl = a->cfg.cfl > 0.0 ? a->cfg.cfl : 0.5;
    std::vector<StepCtl> c0((size_t)M);
    for (int m = 0; m < M; ++m) {
        StepCtl& c = c0[m];
        std::memset(&c, 0, sizeof c);
        c.t = a->cfg.t_start;
        c.t_end = INFINITY;
        c.target = INFINITY;
        c.cfl = cfl;
        c.dt_min_used = INFINITY;
        c.dt_bits = 0x7FF0000000000000ull;
        c.always = 1;
        c.active = 1;
        c.scheme_stages = n_stages;
        for (int s = 0; s < n_stages; ++s) {
            c.st_start[s] = sc[s][0];
            c.st_input[s] = sc[s][1];
            c.st_beta[s] = sc[s][2];
            c.st_c[s] = sc[s][3];
        }
    }
    ACK(cudaMemcpyAsync(t.ctl, c0.data(), c0.size() * sizeof(StepCtl), cudaMemcpyHostToDevice, st));
    t.ks->velocity(t.state, nv, t.P->h_min, st);
    if (dts) {  // dts[n][m]
        std::vector<StageArgs> args(3 * (size_t)N * M);
        for (int m = 0; m < M; ++m) {
            double tm = a->cfg.t_start;
            for (int64_t n = 0; n < N; ++n) {
                const double dt = dts[n * M + m];
                for (int s = 0; s < 3; ++s)
                    args[(n * M + m) * 3 + s] =
                        StageArgs{tm + sc[s][3] * dt, sc[s][0], sc[s][1], sc[s][2] * dt, 1.0, 0.0};
                tm += dt;
            }
        }
        ACK(cudaMemcpyAsync(a->d_args, args.data(), args.size() * sizeof(StageArgs),
                            cudaMemcpyHostToDevice, st));
        ACK(cudaStreamSynchronize(st));  // `args` is pageable and goes out of scope
    }
    const DtParams D = dt_params(t.form0, cfl, DGSWE_SSP_RK3);
    DevBuf q = t.state;
    const auto wall0 = std::chrono::steady_clock::now();
    ACK(cudaEventRecord(a->e0, st));
    for (int64_t n = 0; n < N; ++n) {
        if (n % a->stride == 0)
            if (int s = pack(a, a->d_ckpt + (n / a->stride) * 3 * nv, q, nv, st)) return s;
        if (dts) {
            if (int s = args_to_ctl(a, n)) return s;
        } else {
            t.ks->step_begin(t.ctl, M, st);
            t.ks->dt(t.n1, *t.T, *t.P, q, D, nullptr, t.ctl, &t.ctl[0].always, st);
            t.ks->step_dt(t.ctl, M, st);
            if (int s = ctl_to_args(a, n)) return s;
        }
        forward_step(a, q);
        if (!dts) t.ks->step_end(t.ctl, M, st);
        t.ks->station_eval(q.h, t.T->bed, a->d_node0, a->d_w, n_st, nn, a->d_eta + n * n_st, st);
    }
    ACK(cudaEventRecord(a->e1, st));
    ACK(cudaStreamSynchronize(st));
    ACK(cudaGetLastError());
    float ms = 0.0f;
    ACK(cudaEventElapsedTime(&ms, a->e0, a->e1));
    a->stats.forward_ms = ms;
    a->stats.forward_wall_s =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - wall0).count();
    ACK(cudaMemcpy(c0.data(), t.ctl, c0.size() * sizeof(StepCtl), cudaMemcpyDeviceToHost));
    for (int m = 0; m < M; ++m)
        if (c0[m].nonfinite)
            return afail(a, DGSWE_ERR_NONFINITE, "member %d's forward state is not finite", m);
    std::vector<double> eta((size_t)N * n_st), obs((size_t)N * n_st, 0.0);
    if (n_st) {
        ACK(cudaMemcpy(eta.data(), a->d_eta, eta.size() * sizeof(double), cudaMemcpyDeviceToHost));
        if (eta_obs) std::copy(eta_obs, eta_obs + obs.size(), obs.begin());
    }
    a->J_member.assign((size_t)M, 0.0);
    double j = 0.0;
    for (int64_t n = 0; n < N; ++n)
        for (int s = 0; s < n_st; ++s) {
            const size_t i = (size_t)n * n_st + s;
            const double r = (eta[i] - obs[i]) * (eta[i] - obs[i]);
            j += r;
            a->J_member[a->st_member[s]] += r;
        }
    a->stats.J = j;
    if (J) *J = j;
    if (eta_out) std::copy(eta.begin(), eta.end(), eta_out);
    if (dts_out) {
        std::vector<StageArgs> args(3 * (size_t)N * M);
        ACK(cudaMemcpy(args.data(), a->d_args, args.size() * sizeof(StageArgs), cudaMemcpyDeviceToHost));
        for (int64_t n = 0; n < N; ++n)
            for (int m = 0; m < M; ++m) dts_out[n * M + m] = args[(n * M + m) * 3].c / sc[0][2];
    }
    a->forward_done = true;
    return DGSWE_OK;
}

int dgswe_adjoint_member_misfit(const dgswe_adjoint* a, double* J) {
    if (!a || !J || !a->forward_done) return DGSWE_ERR_INVALID;
    std::copy(a->J_member.begin(), a->J_member.end(), J);
    return DGSWE_OK;
}

int dgswe_adjoint_reverse(dgswe_adjoint* a, double* grad_h0, double* grad_hu0, double* grad_hv0,
                          double* grad_bed, double* grad_manning, double* grad_tide) {
    if (!a || (!a->h && !a->ens)) return DGSWE_ERR_INVALID;
    if (!a->forward_done) return afail(a, DGSWE_ERR_INVALID, "run dgswe_adjoint_forward first");
    Target& t = a->tg;
    ACK(cudaSetDevice(t.device));
    const int64_t nv = t.nv, N = a->cfg.n_steps;
    const int n_st = a->cfg.n_stations, nn = t.nn;
    cudaStream_t st = t.stream;
    const size_t bv = (size_t)nv * sizeof(double);
    for (int c = 0; c < 3; ++c) {
        ACK(cudaMemsetAsync(a->lam[c], 0, bv, st));
        ACK(cudaMemsetAsync(a->lam_b[c], 0, bv, st));
    }
    AdjStage& A = a->A;
    a->want_bed = grad_bed != nullptr;
    ACK(cudaMemsetAsync(A.lx_h, 0, 5 * bv, st));
    ACK(cudaMemsetAsync(A.lbed, 0, bv, st));
    ACK(cudaMemsetAsync(A.lgn2, 0, bv, st));
    ACK(cudaMemsetAsync(A.ltide, 0,
                        (size_t)std::max(1, t.n_cond) * 2 * kMaxConstituents * sizeof(double), st));
    const int* on = &t.ctl[0].always;
    const auto wall0 = std::chrono::steady_clock::now();
    ACK(cudaEventRecord(a->e0, st));
    int64_t recomputed = 0;
    DevBuf& q = a->S[0];
    // a full segment's step n: its start state and the inputs of stages 1
    // and 2 (h, hu, hv and their node velocities, 5 fields each) and what the
    // three stages keep (5 fields each), written there by the replay itself
    const size_t slot = 30 * (size_t)nv;
    auto view = [&](int64_t n, int64_t c0, int b) {
        double* p = a->d_seg + (n - c0) * slot + 5 * (size_t)b * nv;
        return DevBuf{p, p + nv, p + 2 * nv, p + 3 * nv, p + 4 * nv};
    };
    auto keep_view = [&](int64_t n, int64_t c0, int s) {
        double* p = a->d_seg + (n - c0) * slot + (15 + 5 * (size_t)s) * nv;
        return DevBuf{p, p + nv, p + 2 * nv, p + 3 * nv, p + 4 * nv};
    };
    for (int64_t c0 = (a->n_ckpt - 1) * a->stride; c0 >= 0; c0 -= a->stride) {
        const int64_t c1 = std::min(c0 + a->stride, N);
        const double* ck = a->d_ckpt + (c0 / a->stride) * 3 * nv;
        if (a->full) {
            // the segment replayed once into its storage, every step's
            // reverse data kept; the last step's result is not needed
            {
                const DevBuf q0 = view(c0, c0, 0);
                if (int s = unpack(a, q0, ck, nv, st)) return s;
                t.ks->velocity(q0, nv, t.P->h_min, st);
            }
            for (int64_t n = c0; n < c1; ++n) {
                if (int s = args_to_ctl(a, n)) return s;
                const DevBuf in[3] = {view(n, c0, 0), view(n, c0, 1), view(n, c0, 2)};
                // stage 2 writes the next step's start; each stage writes its
                // output's node velocities beside it
                const DevBuf out[3] = {in[1], in[2], n + 1 < c1 ? view(n + 1, c0, 0) : a->S[3]};
                for (int s = 0; s < 3; ++s) {
                    t.ks->face(t.n1, *t.T, *t.P, in[s], t.fb_h, t.fb_hu, t.fb_hv, t.ctl, s, on,
                               st);
                    t.ks->stage_keep(t.n1, *t.T, *t.P, *t.X, in[s], in[0], out[s], t.fb_h, t.fb_hu,
                                     t.fb_hv, t.ctl, s, 0, keep_view(n, c0, s), st);
                }
                recomputed += 1;
            }
            for (int64_t n = c1 - 1; n >= c0; --n) {
                t.ks->station_seed(a->d_eta + n * n_st, a->d_obs + n * n_st, a->d_node0, a->d_w,
                                   n_st, nn, a->lam[0],
                                   t.P->has_bed && a->want_bed ? A.lbed : nullptr, st);
                const DevBuf in[3] = {view(n, c0, 0), view(n, c0, 1), view(n, c0, 2)};
                const DevBuf keep[3] = {keep_view(n, c0, 0), keep_view(n, c0, 1),
                                        keep_view(n, c0, 2)};
                if (int s = args_to_ctl(a, n)) return s;
                if (int s = reverse_stages(a, in, keep)) return s;
            }
            if (c0 == 0) break;
            continue;
        }
        if (a->stride > 1) {  // the segment's step-start states, recomputed from its checkpoint
            if (int s = unpack(a, q, ck, nv, st)) return s;
            t.ks->velocity(q, nv, t.P->h_min, st);
            for (int64_t n = c0; n < c1; ++n) {
                if (int s = pack(a, a->d_seg + (n - c0) * 3 * nv, q, nv, st)) return s;
                if (n + 1 == c1) break;  // the last step is recomputed below
                if (int s = args_to_ctl(a, n)) return s;
                forward_step(a, q);
                recomputed += 1;
            }
        }
        for (int64_t n = c1 - 1; n >= c0; --n) {
            // J's dependence on q_{n+1}
            t.ks->station_seed(a->d_eta + n * n_st, a->d_obs + n * n_st, a->d_node0, a->d_w, n_st,
                               nn, a->lam[0],
                               t.P->has_bed && a->want_bed ? A.lbed : nullptr, st);
            // the step's start state and its stages, recomputed with what the reverse keeps
            const double* q0 = a->stride > 1 ? a->d_seg + (n - c0) * 3 * nv : ck;
            if (int s = unpack(a, q, q0, nv, st)) return s;
            t.ks->velocity(q, nv, t.P->h_min, st);
            if (int s = args_to_ctl(a, n)) return s;
            for (int s = 0; s < 3; ++s) {
                t.ks->face(t.n1, *t.T, *t.P, a->S[s], t.fb_h, t.fb_hu, t.fb_hv, t.ctl, s, on, st);
                t.ks->stage_keep(t.n1, *t.T, *t.P, *t.X, a->S[s], q, a->S[s + 1], t.fb_h, t.fb_hu,
                                 t.fb_hv, t.ctl, s, 0, a->Kp[s], st);
            }
            if (int s = reverse_stages(a, a->S, a->Kp)) return s;
            recomputed += 1;
        }
        if (c0 == 0) break;
    }
    ACK(cudaEventRecord(a->e1, st));
    ACK(cudaStreamSynchronize(st));
    ACK(cudaGetLastError());
    float ms = 0.0f;
    ACK(cudaEventElapsedTime(&ms, a->e0, a->e1));
    a->stats.reverse_ms = ms;
    a->stats.reverse_wall_s =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - wall0).count();
    a->stats.recomputed_steps = recomputed;
    if (grad_h0) ACK(cudaMemcpy(grad_h0, a->lam[0], bv, cudaMemcpyDeviceToHost));
    if (grad_hu0) ACK(cudaMemcpy(grad_hu0, a->lam[1], bv, cudaMemcpyDeviceToHost));
    if (grad_hv0) ACK(cudaMemcpy(grad_hv0, a->lam[2], bv, cudaMemcpyDeviceToHost));
    if (grad_bed) ACK(cudaMemcpy(grad_bed, A.lbed, bv, cudaMemcpyDeviceToHost));
    if (grad_manning) {
        ACK(cudaMemcpy(grad_manning, A.lgn2, bv, cudaMemcpyDeviceToHost));
        for (int64_t i = 0; i < nv; ++i) grad_manning[i] *= 2.0 * a->friction_g * a->manning_n[i];
    }
    if (grad_tide && t.n_cond > 0)
        ACK(cudaMemcpy(grad_tide, A.ltide, (size_t)t.n_cond * 2 * kMaxConstituents * sizeof(double),
                       cudaMemcpyDeviceToHost));
    return DGSWE_OK;
}

int dgswe_adjoint_set_parameters(dgswe_adjoint* a, const double* manning_n, const double* tide) {
    if (!a || (!a->h && !a->ens)) return DGSWE_ERR_INVALID;
    Target& t = a->tg;
    ACK(cudaSetDevice(t.device));
    if (manning_n) {
        if (!t.g_n2)
            return afail(a, DGSWE_ERR_UNSUPPORTED,
                         "Manning's n per node needs a per-node friction field (DGSWE_FRICTION_MANNING_NODES)");
        std::vector<double> gn2((size_t)t.nv);
        for (int64_t i = 0; i < t.nv; ++i) {
            if (!(manning_n[i] >= 0.0) || !std::isfinite(manning_n[i]))
                return afail(a, DGSWE_ERR_INVALID, "Manning's n at node %lld", (long long)i);
            gn2[i] = a->friction_g * manning_n[i] * manning_n[i];
        }
        ACK(cudaMemcpy(t.g_n2, gn2.data(), gn2.size() * sizeof(double), cudaMemcpyHostToDevice));
        a->manning_n.assign(manning_n, manning_n + t.nv);
    }
    if (tide && t.n_cond > 0) {
        std::vector<Condition> c((size_t)t.n_cond);
        if (t.cond_dev)
            ACK(cudaMemcpy(c.data(), t.cond_dev, c.size() * sizeof(Condition), cudaMemcpyDeviceToHost));
        else
            std::copy(t.cond_host->cond, t.cond_host->cond + t.n_cond, c.begin());
        for (int ci = 0; ci < t.n_cond; ++ci)
            for (int i = 0; i < c[ci].n_constituents; ++i) {
                const double amp = tide[((size_t)ci * kMaxConstituents + i) * 2];
                const double ph = tide[((size_t)ci * kMaxConstituents + i) * 2 + 1];
                if (!std::isfinite(amp) || !std::isfinite(ph))
                    return afail(a, DGSWE_ERR_INVALID, "condition %d constituent %d", ci, i);
                c[ci].c[i].amplitude = amp;
                c[ci].c[i].phase = ph;
            }
        if (t.cond_dev)
            ACK(cudaMemcpy(t.cond_dev, c.data(), c.size() * sizeof(Condition), cudaMemcpyHostToDevice));
        else
            std::copy(c.begin(), c.end(), t.cond_host->cond);
    }
    a->forward_done = false;
    return DGSWE_OK;
}

int dgswe_adjoint_get_stats(const dgswe_adjoint* a, dgswe_adjoint_stats* out) {
    if (!a || !out) return DGSWE_ERR_INVALID;
    *out = a->stats;
    return DGSWE_OK;
}

}  // extern "C"
