// The discrete adjoint of a WetDry SSP-RK3 run (no reference counterpart:
// the reference has no adjoint). J = Σ over the steps n = 1..N and the
// stations s of (η_s(q_n) − η_obs[n][s])², η = h + B interpolated in the
// station's element. Reverse mode gives ∂J/∂ of the initial state, the bed
// elevation B per node, Manning's n per node and each boundary condition's
// tide constituents (amplitude, phase), for the steps the forward took:
// the time steps and every branch (wet/dry tests, limiter, HLL wave speeds)
// are the forward's.
//
// Storage: the state at the start of each step (h, hu, hv) is what the
// reverse sweep needs; within a step the three stages are recomputed. When
// all N states fit in the memory budget, the forward sweep keeps them all;
// otherwise it keeps every s-th one, and the reverse sweep recomputes each
// segment of s steps once from its checkpoint, into a segment buffer,
// before reversing it (two-level checkpointing, s the smallest stride the
// budget allows).
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
#include "handle.hpp"
#include "host_common.hpp"
#include "kernel_set.hpp"
#include "setup.hpp"

using namespace dgswe;
using namespace dgswe::host;

static_assert(DGSWE_MAX_CONSTITUENTS == kMaxConstituents, "constituent table size");

struct dgswe_adjoint {
    dgswe_handle* h = nullptr;  // the forward: tables, state buffer, step control
    std::string error;
    dgswe_adjoint_config cfg{};
    std::vector<double> stations;  // [n][2]
    std::vector<int64_t> st_elem;
    std::vector<double> st_w;      // [n][nn]
    std::vector<double> manning_n; // n per node (for ∂J/∂n)
    double friction_g = 0.0;
    int n_cond = 0;
    // device
    std::vector<void*> allocations;
    int64_t* d_node0 = nullptr;
    double* d_w = nullptr;
    StageArgs* d_args = nullptr;  // [n_steps][3] the forward's stage weights
    double* d_eta = nullptr;      // [n_steps][n_stations]
    double* d_obs = nullptr;      // [n_steps][n_stations] or null
    double* d_ckpt = nullptr;     // stored step-start states, 3·nv doubles each
    double* d_seg = nullptr;      // a segment's step-start states (stride > 1)
    int64_t stride = 1, n_ckpt = 0;
    DevBuf S[4]{};  // the step's stage inputs and last output
    DevBuf Kp[3]{}; // kept combination and damped momentum of each stage
    double *lam[3] = {}, *lam_t[3] = {}, *lam_b[3] = {};
    AdjStage A{};
    bool forward_done = false;
    dgswe_adjoint_stats stats{};
    cudaEvent_t e0 = nullptr, e1 = nullptr;

    ~dgswe_adjoint() {
        if (h) {
            cudaSetDevice(h->device);
            for (void* p : allocations) cudaFree(p);
            if (e0) cudaEventDestroy(e0);
            if (e1) cudaEventDestroy(e1);
            dgswe_destroy(h);
        }
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

__global__ void sum_clear_kernel(double* out, const double* a, double* b, int64_t n) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n) return;
    out[g] = a[g] + b[g];
    b[g] = 0.0;
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

// One forward step of the state in `q` (velocities current), with the
// stage weights already in ctl->stage[0..2]; the state buffers S[1], S[2]
// take the intermediate stages, the result lands in q
void forward_step(dgswe_adjoint* a, const DevBuf& q, cudaStream_t st) {
    dgswe_handle* h = a->h;
    const int* on = &h->ctl->always;
    const DevBuf* ins[3] = {&q, &a->S[1], &a->S[2]};
    const DevBuf* outs[3] = {&a->S[1], &a->S[2], &q};
    for (int s = 0; s < 3; ++s) {
        h->ks->face(h->n1, h->T, h->P, *ins[s], h->fb_h, h->fb_hu, h->fb_hv, h->ctl, s, on, st);
        h->ks->stage(h->n1, h->T, h->P, h->X, *ins[s], q, *outs[s], q, h->fb_h, h->fb_hu, h->fb_hv,
                     h->ctl, s, kModePost, s == 2, on, st);
    }
}

}  // namespace

extern "C" {

int dgswe_adjoint_create(const dgswe_form* f, int device, const dgswe_adjoint_config* cfg,
                         dgswe_adjoint** out) {
    if (!out) return DGSWE_ERR_INVALID;
    auto* a = new dgswe_adjoint();
    *out = a;
    if (!cfg) return afail(a, DGSWE_ERR_INVALID, "no configuration");
    std::string why;
    if (int s = check_form(f, why)) return afail(a, s, "%s", why.c_str());
    if (f->formulation != DGSWE_WET_DRY)
        return afail(a, DGSWE_ERR_UNSUPPORTED, "the adjoint covers the WetDry formulation");
    if (cfg->scheme != DGSWE_SSP_RK3)
        return afail(a, DGSWE_ERR_UNSUPPORTED, "the adjoint covers SSP-RK3");
    if (cfg->n_steps <= 0 || cfg->n_stations < 0 || (cfg->n_stations > 0 && !cfg->stations))
        return afail(a, DGSWE_ERR_INVALID, "steps and stations");
    a->cfg = *cfg;
    a->stations.assign(cfg->stations, cfg->stations + 2 * (size_t)cfg->n_stations);
    a->cfg.stations = nullptr;
    // stations: element and Lagrange weights
    Operators ops(f->order);
    const int nn = ops.nn;
    for (int s = 0; s < cfg->n_stations; ++s) {
        const double x = a->stations[2 * s], y = a->stations[2 * s + 1];
        int64_t found = -1;
        double r = 0, q = 0;
        for (int64_t k = 0; k < f->n_elements && found < 0; ++k) {
            double c[8];
            for (int v = 0; v < 4; ++v) {
                const int64_t vi = f->elements[k * 4 + v];
                c[2 * v] = f->vertices[vi * 2];
                c[2 * v + 1] = f->vertices[vi * 2 + 1];
            }
            const double xmin = std::min({c[0], c[2], c[4], c[6]}), xmax = std::max({c[0], c[2], c[4], c[6]});
            const double ymin = std::min({c[1], c[3], c[5], c[7]}), ymax = std::max({c[1], c[3], c[5], c[7]});
            if (x < xmin - 1e-9 * (1 + std::fabs(xmin)) || x > xmax + 1e-9 * (1 + std::fabs(xmax)) ||
                y < ymin - 1e-9 * (1 + std::fabs(ymin)) || y > ymax + 1e-9 * (1 + std::fabs(ymax)))
                continue;
            if (locate(c, x, y, r, q)) found = k;
        }
        if (found < 0) return afail(a, DGSWE_ERR_INVALID, "station %d is outside the mesh", s);
        a->st_elem.push_back(found);
        for (int i = 0; i < nn; ++i)
            a->st_w.push_back(lagrange(ops.x, i % ops.n1, r) * lagrange(ops.x, i / ops.n1, q));
    }
    // Manning's n per node, for ∂J/∂n = ∂J/∂(g n²)·2 g n
    const int64_t nv = f->n_elements * nn;
    a->friction_g = f->friction_g;
    if (f->friction == DGSWE_FRICTION_MANNING_NODES)
        a->manning_n.assign(f->manning_n_nodes, f->manning_n_nodes + nv);
    else
        a->manning_n.assign(nv, f->friction == DGSWE_FRICTION_MANNING ? f->manning_n : 0.0);
    a->n_cond = f->n_boundaries;
    dgswe_handle* hd = nullptr;
    const int st = dgswe_create(f, device, &hd);
    a->h = hd;
    if (st != DGSWE_OK)
        return afail(a, st, "%s", hd ? dgswe_last_error(hd) : "create failed");
    dgswe_handle* h = hd;
    ACK(cudaSetDevice(h->device));
    ACK(cudaEventCreate(&a->e0));
    ACK(cudaEventCreate(&a->e1));
    const int64_t nf = h->K * 4 * h->n1;
    // the bed slope's transpose: for node c, each line partner i's
    // ∂(g∇B)_i/∂B_c = g·D[pos_i][pos_c]·w(i, c), with w the forward's metric
    // weight (i's own on an affine element, else the mean of i's and c's)
    if (h->P.has_bed) {
        const int n1 = ops.n1;
        std::vector<double> contra(4 * (size_t)nv), gt(4 * (size_t)n1 * nv);
        std::vector<uint8_t> aff((size_t)h->K);
        ACK(cudaMemcpy(contra.data(), h->T.contra, contra.size() * sizeof(double), cudaMemcpyDeviceToHost));
        ACK(cudaMemcpy(aff.data(), h->T.affine, aff.size(), cudaMemcpyDeviceToHost));
#pragma omp parallel for schedule(static)
        for (int64_t k = 0; k < h->K; ++k)
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
                        const double gd = f->g * ops.d[pa * n1 + pc];
                        double* o = &gt[(((k * nn + c) * 2 + dir) * n1 + pa) * 2];
                        o[0] = gd * wx;
                        o[1] = gd * wy;
                    }
                }
        double* d_gt = nullptr;
        if (int s = dalloc(a, gt.size(), &d_gt)) return s;
        ACK(cudaMemcpy(d_gt, gt.data(), gt.size() * sizeof(double), cudaMemcpyHostToDevice));
        h->T.gdb_t = d_gt;
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
    if ((s = dalloc(a, 3 * (size_t)N, &a->d_args))) return s;
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
    if ((s = dalloc(a, (size_t)std::max(1, a->n_cond) * 2 * kMaxConstituents, &A.ltide))) return s;
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
    int64_t stride = 1;
    if ((double)N * sb > budget) {
        stride = 0;
        for (int64_t t = 2; t <= N; ++t)
            if ((double)((N + t - 1) / t + t) * sb <= budget) {
                stride = t;
                break;
            }
        if (stride == 0)
            return afail(a, DGSWE_ERR_INVALID,
                         "the memory budget (%.3g B) holds fewer than 2·√N states of %.3g B", budget,
                         sb);
    }
    a->stride = stride;
    a->n_ckpt = (N + stride - 1) / stride;
    if ((s = dalloc(a, 3 * (size_t)nv * a->n_ckpt, &a->d_ckpt))) return s;
    if (stride > 1 && (s = dalloc(a, 3 * (size_t)nv * stride, &a->d_seg))) return s;
    a->stats.stride = stride;
    a->stats.stored_states = a->n_ckpt + (stride > 1 ? stride : 0);
    a->stats.stored_bytes = (double)a->stats.stored_states * sb;
    return DGSWE_OK;
}

void dgswe_adjoint_destroy(dgswe_adjoint* a) { delete a; }

const char* dgswe_adjoint_last_error(const dgswe_adjoint* a) { return a ? a->error.c_str() : ""; }

int64_t dgswe_adjoint_n_values(const dgswe_adjoint* a) { return a && a->h ? a->h->n_values : 0; }

int dgswe_adjoint_stations(const dgswe_adjoint* a, int64_t* element, double* weights) {
    if (!a || !a->h) return DGSWE_ERR_INVALID;
    const size_t n = a->st_elem.size();
    if (element) std::copy(a->st_elem.begin(), a->st_elem.end(), element);
    if (weights) std::copy(a->st_w.begin(), a->st_w.end(), weights);
    (void)n;
    return DGSWE_OK;
}

int dgswe_adjoint_forward(dgswe_adjoint* a, const double* h0, const double* hu0, const double* hv0,
                          const double* dts, const double* eta_obs, double* eta_out,
                          double* dts_out, double* J) {
    if (!a || !a->h) return DGSWE_ERR_INVALID;
    dgswe_handle* h = a->h;
    ACK(cudaSetDevice(h->device));
    const int64_t nv = h->n_values, N = a->cfg.n_steps;
    const int n_st = a->cfg.n_stations, nn = h->nn;
    cudaStream_t st = h->stream;
    if (int s = dgswe_upload(h, DGSWE_STATE, h0, hu0, hv0, nv)) return afail(a, s, "%s", h->error.c_str());
    if (n_st)
        ACK(eta_obs ? cudaMemcpy(a->d_obs, eta_obs, (size_t)N * n_st * sizeof(double), cudaMemcpyHostToDevice)
                    : cudaMemset(a->d_obs, 0, (size_t)N * n_st * sizeof(double)));
    // the run's clock (CFL steps) or the given steps' stage weights
    dgswe_run_config run{};
    run.scheme = DGSWE_SSP_RK3;
    run.cfl = a->cfg.cfl > 0.0 ? a->cfg.cfl : 0.5;
    run.t_start = a->cfg.t_start;
    run.t_end = INFINITY;
    if (int s = begin_run(h, &run, INFINITY)) return afail(a, s, "%s", h->error.c_str());
    double sc[4][4];
    scheme_table(DGSWE_SSP_RK3, sc);
    if (dts) {
        std::vector<StageArgs> args(3 * (size_t)N);
        double t = a->cfg.t_start;
        for (int64_t n = 0; n < N; ++n) {
            for (int s = 0; s < 3; ++s)
                args[3 * n + s] = StageArgs{t + sc[s][3] * dts[n], sc[s][0], sc[s][1],
                                            sc[s][2] * dts[n], 1.0, 0.0};
            t += dts[n];
        }
        ACK(cudaMemcpy(a->d_args, args.data(), args.size() * sizeof(StageArgs), cudaMemcpyHostToDevice));
    }
    const DtParams D = dt_params(h->form, run.cfl, DGSWE_SSP_RK3);
    DevBuf q = h->buf[DGSWE_STATE].view;
    const auto wall0 = std::chrono::steady_clock::now();
    ACK(cudaEventRecord(a->e0, st));
    for (int64_t n = 0; n < N; ++n) {
        if (n % a->stride == 0)
            if (int s = pack(a, a->d_ckpt + (n / a->stride) * 3 * nv, q, nv, st)) return s;
        if (dts) {
            ACK(cudaMemcpyAsync(h->ctl->stage, a->d_args + 3 * n, 3 * sizeof(StageArgs),
                                cudaMemcpyDeviceToDevice, st));
        } else {
            h->ks->step_begin(h->ctl, 1, st);
            h->ks->dt(h->n1, h->T, h->P, q, D, nullptr, h->ctl, &h->ctl->active, st);
            h->ks->step_dt(h->ctl, 1, st);
            ACK(cudaMemcpyAsync(a->d_args + 3 * n, h->ctl->stage, 3 * sizeof(StageArgs),
                                cudaMemcpyDeviceToDevice, st));
        }
        forward_step(a, q, st);
        if (!dts) h->ks->step_end(h->ctl, 1, st);
        h->ks->station_eval(q.h, h->T.bed, a->d_node0, a->d_w, n_st, nn, a->d_eta + n * n_st, st);
    }
    ACK(cudaEventRecord(a->e1, st));
    ACK(cudaStreamSynchronize(st));
    ACK(cudaGetLastError());
    float ms = 0.0f;
    ACK(cudaEventElapsedTime(&ms, a->e0, a->e1));
    a->stats.forward_ms = ms;
    a->stats.forward_wall_s =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - wall0).count();
    StepCtl c{};
    ACK(cudaMemcpy(&c, h->ctl, sizeof c, cudaMemcpyDeviceToHost));
    if (c.nonfinite) return afail(a, DGSWE_ERR_NONFINITE, "the forward state is not finite");
    std::vector<double> eta((size_t)N * n_st), obs((size_t)N * n_st, 0.0);
    if (n_st) {
        ACK(cudaMemcpy(eta.data(), a->d_eta, eta.size() * sizeof(double), cudaMemcpyDeviceToHost));
        if (eta_obs) std::copy(eta_obs, eta_obs + obs.size(), obs.begin());
    }
    double j = 0.0;
    for (size_t m = 0; m < eta.size(); ++m) j += (eta[m] - obs[m]) * (eta[m] - obs[m]);
    a->stats.J = j;
    if (J) *J = j;
    if (eta_out) std::copy(eta.begin(), eta.end(), eta_out);
    if (dts_out) {
        std::vector<StageArgs> args(3 * (size_t)N);
        ACK(cudaMemcpy(args.data(), a->d_args, args.size() * sizeof(StageArgs), cudaMemcpyDeviceToHost));
        for (int64_t n = 0; n < N; ++n) dts_out[n] = args[3 * n].c / sc[0][2];
    }
    a->forward_done = true;
    return DGSWE_OK;
}

int dgswe_adjoint_reverse(dgswe_adjoint* a, double* grad_h0, double* grad_hu0, double* grad_hv0,
                          double* grad_bed, double* grad_manning, double* grad_tide) {
    if (!a || !a->h) return DGSWE_ERR_INVALID;
    if (!a->forward_done) return afail(a, DGSWE_ERR_INVALID, "run dgswe_adjoint_forward first");
    dgswe_handle* h = a->h;
    ACK(cudaSetDevice(h->device));
    const int64_t nv = h->n_values, N = a->cfg.n_steps, nf = h->K * 4 * h->n1;
    const int n_st = a->cfg.n_stations, nn = h->nn;
    cudaStream_t st = h->stream;
    const size_t bv = (size_t)nv * sizeof(double);
    for (int c = 0; c < 3; ++c) {
        ACK(cudaMemsetAsync(a->lam[c], 0, bv, st));
        ACK(cudaMemsetAsync(a->lam_b[c], 0, bv, st));
    }
    AdjStage& A = a->A;
    ACK(cudaMemsetAsync(A.lx_h, 0, 5 * bv, st));
    ACK(cudaMemsetAsync(A.lbed, 0, bv, st));
    ACK(cudaMemsetAsync(A.lgn2, 0, bv, st));
    ACK(cudaMemsetAsync(A.ltide, 0, (size_t)std::max(1, a->n_cond) * 2 * kMaxConstituents * sizeof(double), st));
    (void)nf;
    const int* on = &h->ctl->always;
    const auto wall0 = std::chrono::steady_clock::now();
    ACK(cudaEventRecord(a->e0, st));
    int64_t recomputed = 0;
    DevBuf& q = a->S[0];
    for (int64_t c0 = (a->n_ckpt - 1) * a->stride; c0 >= 0; c0 -= a->stride) {
        const int64_t c1 = std::min(c0 + a->stride, N);
        const double* ck = a->d_ckpt + (c0 / a->stride) * 3 * nv;
        if (a->stride > 1) {  // the segment's step-start states, recomputed from its checkpoint
            if (int s = unpack(a, q, ck, nv, st)) return s;
            h->ks->velocity(q, nv, h->P.h_min, st);
            for (int64_t n = c0; n < c1; ++n) {
                if (int s = pack(a, a->d_seg + (n - c0) * 3 * nv, q, nv, st)) return s;
                if (n + 1 == c1) break;  // the last step is recomputed below
                ACK(cudaMemcpyAsync(h->ctl->stage, a->d_args + 3 * n, 3 * sizeof(StageArgs),
                                    cudaMemcpyDeviceToDevice, st));
                forward_step(a, q, st);
                recomputed += 1;
            }
        }
        for (int64_t n = c1 - 1; n >= c0; --n) {
            // J's dependence on q_{n+1}
            h->ks->station_seed(a->d_eta + n * n_st, a->d_obs + n * n_st, a->d_node0, a->d_w, n_st,
                                nn, a->lam[0], h->P.has_bed ? A.lbed : nullptr, st);
            // the step's start state and its stages, recomputed with what the reverse keeps
            const double* q0 = a->stride > 1 ? a->d_seg + (n - c0) * 3 * nv : ck;
            if (int s = unpack(a, q, q0, nv, st)) return s;
            h->ks->velocity(q, nv, h->P.h_min, st);
            ACK(cudaMemcpyAsync(h->ctl->stage, a->d_args + 3 * n, 3 * sizeof(StageArgs),
                                cudaMemcpyDeviceToDevice, st));
            for (int s = 0; s < 3; ++s) {
                h->ks->face(h->n1, h->T, h->P, a->S[s], h->fb_h, h->fb_hu, h->fb_hv, h->ctl, s, on, st);
                h->ks->stage_keep(h->n1, h->T, h->P, h->X, a->S[s], q, a->S[s + 1], h->fb_h,
                                  h->fb_hu, h->fb_hv, h->ctl, s, 0, a->Kp[s], st);
            }
            // the stages reversed: λ of each stage's input from λ of its output
            for (int s = 2; s >= 0; --s) {
                AdjStage As = A;
                double** lo = s == 2 ? a->lam : a->lam_t;
                As.lo_h = lo[0];
                As.lo_hu = lo[1];
                As.lo_hv = lo[2];
                h->ks->stage_adjoint(h->n1, h->T, h->P, h->X, a->S[s], a->Kp[s], As, h->ctl, s, st);
                h->ks->face_adjoint(h->n1, h->T, h->P, a->S[s], As, h->ctl, s, st);
                h->ks->adjoint_combine(a->S[s], As, a->lam_t[0], a->lam_t[1], a->lam_t[2], nv,
                                       h->P.h_min, st);
            }
            // λ of q_n: the first stage's input plus the three stages' base terms
            for (int c = 0; c < 3; ++c)
                sum_clear_kernel<<<(unsigned)((nv + 255) / 256), 256, 0, st>>>(a->lam[c], a->lam_t[c],
                                                                               a->lam_b[c], nv);
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
    if (grad_tide && a->n_cond > 0)
        ACK(cudaMemcpy(grad_tide, A.ltide, (size_t)a->n_cond * 2 * kMaxConstituents * sizeof(double),
                       cudaMemcpyDeviceToHost));
    return DGSWE_OK;
}

int dgswe_adjoint_get_stats(const dgswe_adjoint* a, dgswe_adjoint_stats* out) {
    if (!a || !out) return DGSWE_ERR_INVALID;
    *out = a->stats;
    return DGSWE_OK;
}

}  // extern "C"
