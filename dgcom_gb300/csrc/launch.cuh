// Launchers of one numerics variant (included after kernels.cuh by
// kernels_fast.cu and kernels_exact.cu): the order N is a template
// parameter of the kernels and a run-time value of the handle.
#pragma once

#include "kernel_set.hpp"

namespace dgswe {
namespace DGSWE_NS {

// The node sources of a stage, before its stage kernel reads them: the
// weather's, then the relaxation band's
template <bool LISTED>
static void relax(const DevTables& T, const Physics& P, const DevBuf& in, const StepCtl* ctl,
                  int slot, const LtsPass& lp, cudaStream_t s) {
    if (T.at_source && T.rx_src) {
        const int64_t n = (LISTED ? lp.n : T.K) * P.nn;
        if (n > 0)
            atmos_kernel<LISTED><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(T, P, in, ctl, slot,
                                                                            lp);
    }
    if (T.rx_n == 0 || !T.rx_src) return;
    relax_kernel<LISTED><<<(unsigned)((T.rx_n + 255) / 256), 256, 0, s>>>(T, P, in, ctl, slot, lp);
}

template <int N1>
static void face_n(const DevTables& T, const Physics& P, const DevBuf& in, double* fh, double* fhu,
                   double* fhv, const StepCtl* ctl, int slot, const int* active, cudaStream_t s) {
    relax<false>(T, P, in, ctl, slot, LtsPass{}, s);
    const int64_t items = (T.n_edges + T.n_bfaces) * N1;
    if (items == 0) return;
    const int threads = P.face_threads > 0 && P.face_threads <= 256 ? P.face_threads : 256;
    const unsigned blocks = (unsigned)((items + threads - 1) / threads);
    face_kernel<N1, false><<<blocks, threads, 0, s>>>(T, P, in, fh, fhu, fhv, ctl, slot, active,
                                                      LtsPass{});
}

template <int N1>
static void face_listed_n(const DevTables& T, const Physics& P, const DevBuf& in, double* fh,
                          double* fhu, double* fhv, StepCtl* ctl, const LtsPass& lp,
                          cudaStream_t s) {
    relax<true>(T, P, in, ctl, 0, lp, s);
    const int64_t items = (lp.n_edges + lp.n_bfaces) * N1;
    if (items == 0) return;
    const int threads = P.face_threads > 0 && P.face_threads <= 256 ? P.face_threads : 256;
    const unsigned blocks = (unsigned)((items + threads - 1) / threads);
    face_kernel<N1, true><<<blocks, threads, 0, s>>>(T, P, in, fh, fhu, fhv, ctl, 0, &ctl->always,
                                                     lp);
}

template <int N1>
static void stage_n(const DevTables& T, const Physics& P, const StageExtra& X, const DevBuf& in,
                    const DevBuf& base, const DevBuf& out, const DevBuf& acc, const double* fh,
                    const double* fhu, const double* fhv, StepCtl* ctl, int slot, int mode,
                    int check_finite, const int* active, const DevBuf& keep, cudaStream_t s) {
    // the pass's elements: all, or the chunk [k_first, k_last) of X
    const int64_t k1 = X.k_last < T.K ? X.k_last : T.K;
    const int64_t count = k1 - X.k_first;
    if (count <= 0) return;
    if (P.stage_shape == 1) {
        using C1 = Cfg<N1, 1>;
        const unsigned blocks = (unsigned)((count + C1::EPB - 1) / C1::EPB);
        stage_kernel<N1, false, 1><<<blocks, C1::THREADS, 0, s>>>(
            T, P, X, in, base, out, acc, fh, fhu, fhv, ctl, slot, mode, check_finite, active, keep,
            LtsPass{});
        return;
    }
    if (P.stage_shape == 2) {
        using C2 = Cfg<N1, 2>;
        const unsigned blocks = (unsigned)((count + C2::EPB - 1) / C2::EPB);
        stage_kernel<N1, false, 2><<<blocks, C2::THREADS, 0, s>>>(
            T, P, X, in, base, out, acc, fh, fhu, fhv, ctl, slot, mode, check_finite, active, keep,
            LtsPass{});
        return;
    }
    using C = Cfg<N1>;
    const unsigned blocks = (unsigned)((count + C::EPB - 1) / C::EPB);
    stage_kernel<N1, false><<<blocks, C::THREADS, 0, s>>>(T, P, X, in, base, out, acc, fh, fhu, fhv,
                                                          ctl, slot, mode, check_finite, active,
                                                          keep, LtsPass{});
}

template <int N1>
static void stage_listed_n(const DevTables& T, const Physics& P, const StageExtra& X,
                           const DevBuf& in, const DevBuf& base, const DevBuf& out,
                           const DevBuf& acc, const double* fh, const double* fhu,
                           const double* fhv, StepCtl* ctl, int mode, const LtsPass& lp,
                           cudaStream_t s) {
    using C = Cfg<N1>;
    if (lp.n == 0) return;
    const unsigned blocks = (unsigned)((lp.n + C::EPB - 1) / C::EPB);
    stage_kernel<N1, true><<<blocks, C::THREADS, 0, s>>>(T, P, X, in, base, out, acc, fh, fhu, fhv,
                                                         ctl, 0, mode, 0, &ctl->always, DevBuf{},
                                                         lp);
}

template <int N1>
static void finish_n(const DevTables& T, const Physics& P, const DevBuf& acc, const DevBuf& state,
                     StepCtl* ctl, cudaStream_t s) {
    using C = Cfg<N1>;
    const unsigned blocks = (unsigned)((T.K + C::EPB - 1) / C::EPB);
    finish_kernel<N1, false><<<blocks, C::THREADS, 0, s>>>(T, P, acc, state, ctl, LtsPass{});
}

template <int N1>
static void finish_listed_n(const DevTables& T, const Physics& P, const DevBuf& acc,
                            const DevBuf& state, StepCtl* ctl, const LtsPass& lp, cudaStream_t s) {
    using C = Cfg<N1>;
    if (lp.n == 0) return;
    const unsigned blocks = (unsigned)((lp.n + C::EPB - 1) / C::EPB);
    finish_kernel<N1, true><<<blocks, C::THREADS, 0, s>>>(T, P, acc, state, ctl, lp);
}

template <int N1>
static void dt_n(const DevTables& T, const Physics& P, const DevBuf& q, const DtParams& D,
                 double* dt_el, StepCtl* ctl, const int* active, cudaStream_t s) {
    using C = DtCfg<N1>;
    const unsigned blocks = (unsigned)((T.K + C::EPB - 1) / C::EPB);
    dt_kernel<N1, false><<<blocks, C::THREADS, 0, s>>>(T, P, q, D, dt_el, ctl, active, nullptr, 0);
}

template <int N1>
static void dt_listed_n(const DevTables& T, const Physics& P, const DevBuf& q, const DtParams& D,
                        double* dt_el, StepCtl* ctl, const int* active, const int32_t* list,
                        int64_t n, cudaStream_t s) {
    using C = DtCfg<N1>;
    if (n <= 0) return;
    const unsigned blocks = (unsigned)((n + C::EPB - 1) / C::EPB);
    dt_kernel<N1, true><<<blocks, C::THREADS, 0, s>>>(T, P, q, D, dt_el, ctl, active, list, n);
}

// The face fluxes of the listed interior edges and boundary faces of a
// global stage (no node sources: node_sources launches those)
template <int N1>
static void face_ready_n(const DevTables& T, const Physics& P, const DevBuf& in, double* fh,
                         double* fhu, double* fhv, const StepCtl* ctl, int slot,
                         const int* active, const int32_t* edges, int64_t n_edges,
                         const int32_t* bfaces, int64_t n_bfaces, cudaStream_t s) {
    const int64_t items = (n_edges + n_bfaces) * N1;
    if (items <= 0) return;
    LtsPass lp{};  // no levels: the boundary faces at the stage's time
    lp.edges = edges;
    lp.n_edges = n_edges;
    lp.bfaces = bfaces;
    lp.n_bfaces = n_bfaces;
    const int threads = P.face_threads > 0 && P.face_threads <= 256 ? P.face_threads : 256;
    const unsigned blocks = (unsigned)((items + threads - 1) / threads);
    face_kernel<N1, true><<<blocks, threads, 0, s>>>(T, P, in, fh, fhu, fhv, ctl, slot, active,
                                                     lp);
}

#define DGSWE_BY_ORDER(fn, ...)            \
    switch (n1) {                          \
        case 2: fn<2>(__VA_ARGS__); break; \
        case 3: fn<3>(__VA_ARGS__); break; \
        case 4: fn<4>(__VA_ARGS__); break; \
        default: fn<5>(__VA_ARGS__); break; \
    }

static void face(int n1, const DevTables& T, const Physics& P, const DevBuf& in, double* fh,
                 double* fhu, double* fhv, const StepCtl* ctl, int slot, const int* active,
                 cudaStream_t s) {
    DGSWE_BY_ORDER(face_n, T, P, in, fh, fhu, fhv, ctl, slot, active, s);
}

static void face_ready(int n1, const DevTables& T, const Physics& P, const DevBuf& in, double* fh,
                       double* fhu, double* fhv, const StepCtl* ctl, int slot, const int* active,
                       const int32_t* edges, int64_t n_edges, const int32_t* bfaces,
                       int64_t n_bfaces, cudaStream_t s) {
    DGSWE_BY_ORDER(face_ready_n, T, P, in, fh, fhu, fhv, ctl, slot, active, edges, n_edges, bfaces,
                   n_bfaces, s);
}

static void node_sources(const DevTables& T, const Physics& P, const DevBuf& in,
                         const StepCtl* ctl, int slot, cudaStream_t s) {
    relax<false>(T, P, in, ctl, slot, LtsPass{}, s);
}

static void dt_listed(int n1, const DevTables& T, const Physics& P, const DevBuf& q,
                      const DtParams& D, double* dt_el, StepCtl* ctl, const int* active,
                      const int32_t* list, int64_t n, cudaStream_t s) {
    DGSWE_BY_ORDER(dt_listed_n, T, P, q, D, dt_el, ctl, active, list, n, s);
}

static void stage(int n1, const DevTables& T, const Physics& P, const StageExtra& X,
                  const DevBuf& in, const DevBuf& base, const DevBuf& out, const DevBuf& acc,
                  const double* fh, const double* fhu, const double* fhv, StepCtl* ctl, int slot,
                  int mode, int check_finite, const int* active, cudaStream_t s) {
    DGSWE_BY_ORDER(stage_n, T, P, X, in, base, out, acc, fh, fhu, fhv, ctl, slot, mode,
                   check_finite, active, DevBuf{}, s);
}

static void stage_keep(int n1, const DevTables& T, const Physics& P, const StageExtra& X,
                       const DevBuf& in, const DevBuf& base, const DevBuf& out, const double* fh,
                       const double* fhu, const double* fhv, StepCtl* ctl, int slot,
                       int check_finite, const DevBuf& keep, cudaStream_t s) {
    DGSWE_BY_ORDER(stage_n, T, P, X, in, base, out, base, fh, fhu, fhv, ctl, slot, kPost,
                   check_finite, &ctl->always, keep, s);
}

static void finish(int n1, const DevTables& T, const Physics& P, const DevBuf& acc,
                   const DevBuf& state, StepCtl* ctl, cudaStream_t s) {
    DGSWE_BY_ORDER(finish_n, T, P, acc, state, ctl, s);
}

static void dt(int n1, const DevTables& T, const Physics& P, const DevBuf& q, const DtParams& D,
               double* dt_el, StepCtl* ctl, const int* active, cudaStream_t s) {
    DGSWE_BY_ORDER(dt_n, T, P, q, D, dt_el, ctl, active, s);
}

static void face_listed(int n1, const DevTables& T, const Physics& P, const DevBuf& in,
                        double* fh, double* fhu, double* fhv, StepCtl* ctl, const LtsPass& lp,
                        cudaStream_t s) {
    DGSWE_BY_ORDER(face_listed_n, T, P, in, fh, fhu, fhv, ctl, lp, s);
}

static void stage_listed(int n1, const DevTables& T, const Physics& P, const StageExtra& X,
                         const DevBuf& in, const DevBuf& base, const DevBuf& out,
                         const DevBuf& acc, const double* fh, const double* fhu, const double* fhv,
                         StepCtl* ctl, int mode, const LtsPass& lp, cudaStream_t s) {
    DGSWE_BY_ORDER(stage_listed_n, T, P, X, in, base, out, acc, fh, fhu, fhv, ctl, mode, lp, s);
}

static void finish_listed(int n1, const DevTables& T, const Physics& P, const DevBuf& acc,
                          const DevBuf& state, StepCtl* ctl, const LtsPass& lp, cudaStream_t s) {
    DGSWE_BY_ORDER(finish_listed_n, T, P, acc, state, ctl, lp, s);
}

template <int N1>
static void stage_adjoint_n(const DevTables& T, const Physics& P, const StageExtra& X,
                            const DevBuf& in, const DevBuf& keep, const AdjStage& A,
                            const StepCtl* ctl, int slot, int subcells, cudaStream_t s) {
    if (T.K == 0) return;
    if (!subcells) {
        using CW = AdjCfg<N1, kAdjWet>;
        stage_adjoint_kernel<N1, kAdjWet><<<(unsigned)((T.K + CW::EPB - 1) / CW::EPB),
                                            CW::THREADS, 0, s>>>(T, P, X, in, keep, A, ctl, slot);
    } else {
        // sized for every element; the blocks past the list's end leave at once
        using CS = AdjCfg<N1, kAdjSub>;
        stage_adjoint_kernel<N1, kAdjSub><<<(unsigned)((T.K + CS::EPB - 1) / CS::EPB),
                                            CS::THREADS, 0, s>>>(T, P, X, in, keep, A, ctl, slot);
    }
}

template <int N1>
static void face_adjoint_n(const DevTables& T, const Physics& P, const DevBuf& in,
                           const AdjStage& A, const StepCtl* ctl, int slot, cudaStream_t s) {
    const int64_t items = (T.n_edges + T.n_bfaces) * N1;
    if (items == 0) return;
    face_adjoint_kernel<N1><<<(unsigned)((items + 255) / 256), 256, 0, s>>>(T, P, in, A, ctl, slot);
}

static void stage_adjoint(int n1, const DevTables& T, const Physics& P, const StageExtra& X,
                          const DevBuf& in, const DevBuf& keep, const AdjStage& A,
                          const StepCtl* ctl, int slot, int subcells, cudaStream_t s) {
    DGSWE_BY_ORDER(stage_adjoint_n, T, P, X, in, keep, A, ctl, slot, subcells, s);
}

static void face_adjoint(int n1, const DevTables& T, const Physics& P, const DevBuf& in,
                         const AdjStage& A, const StepCtl* ctl, int slot, cudaStream_t s) {
    DGSWE_BY_ORDER(face_adjoint_n, T, P, in, A, ctl, slot, s);
}

#undef DGSWE_BY_ORDER

static void adjoint_combine(const DevBuf& in, const AdjStage& A, double* out_h, double* out_hu,
                            double* out_hv, double* const* base, int64_t n, double h_min,
                            cudaStream_t s) {
    if (n == 0) return;
    adjoint_combine_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
        in, A, out_h, out_hu, out_hv, base ? base[0] : nullptr, base ? base[1] : nullptr,
        base ? base[2] : nullptr, n, h_min);
}

static void subcell_list(const DevTables& T, const Physics& P, const double* h0, const double* h1,
                         const double* h2, const AdjStage& A, int nn, cudaStream_t s) {
    if (T.K == 0) return;
    subcell_list_kernel<<<(unsigned)((T.K + 255) / 256), 256, 0, s>>>(T, P, h0, h1, h2, A, nn);
}

static void station_eval(const double* h, const double* bed, const int64_t* node0, const double* w,
                         int n_stations, int nn, double* eta, cudaStream_t s) {
    if (n_stations == 0) return;
    station_eval_kernel<<<(n_stations + 127) / 128, 128, 0, s>>>(h, bed, node0, w, n_stations, nn,
                                                                  eta);
}

static void station_seed(const double* eta, const double* obs, const int64_t* node0,
                         const double* w, int n_stations, int nn, double* lh, double* lbed,
                         cudaStream_t s) {
    const int n = n_stations * nn;
    if (n == 0) return;
    station_seed_kernel<<<(n + 127) / 128, 128, 0, s>>>(eta, obs, node0, w, n_stations, nn, lh,
                                                         lbed);
}

static void depth_flags(const double* h, int64_t K, int nn, double d0, double d1, double d2,
                        uint8_t* flags, cudaStream_t s) {
    if (K == 0) return;
    depth_flags_kernel<<<(unsigned)((K + 255) / 256), 256, 0, s>>>(h, K, nn, d0, d1, d2, flags);
}

static void implicit_damping(const DevTables& T, const Physics& P, const DevBuf& stage,
                             const DevBuf& from, double dt, int64_t n, cudaStream_t s) {
    if (n == 0) return;
    damping_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(T, P, stage, from, dt, n);
}

static void velocity(const DevBuf& b, int64_t n, double h_min, cudaStream_t s) {
    if (n == 0) return;
    velocity_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(b, n, h_min);
}

// one thread per member's StepCtl
static unsigned member_blocks(int n) { return (unsigned)((n + 127) / 128); }
static void begin(StepCtl* c, int n, cudaStream_t s) {
    step_begin<<<member_blocks(n), 128, 0, s>>>(c, n);
}
static void dt_fit(StepCtl* c, int n, cudaStream_t s) {
    step_dt<<<member_blocks(n), 128, 0, s>>>(c, n);
}
static void end(StepCtl* c, int n, cudaStream_t s) {
    step_end<<<member_blocks(n), 128, 0, s>>>(c, n);
}

static const KernelSet kSet = {face,          stage,         finish,          dt,
                                velocity,      stage_keep,    stage_adjoint,   face_adjoint,
                                adjoint_combine, station_eval, station_seed,   begin,
                                dt_fit,        end,           face_listed,     stage_listed,
                                finish_listed, depth_flags,    subcell_list,
                                implicit_damping, face_ready,  node_sources,
                                dt_listed};

}  // namespace DGSWE_NS
}  // namespace dgswe
