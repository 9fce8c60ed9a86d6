// The sm_103a kernels of the FP64 2D shallow-water split-form stage.
//
// This file is compiled twice (kernels_fast.cu, kernels_exact.cu) into two
// namespaces: DGSWE_FAST = 1 lets the compiler contract multiply-adds into
// FMA (-fmad=true) and evaluates the Manning rate without divisions; 0 keeps
// every multiply and add separately rounded (-fmad=false) and follows the
// reference's arithmetic, its cube root included. Both are FP64 throughout.
//
// Kernels of one stage (one RK stage of every element):
//  - face_kernel: the numerical flux F* of every interior edge node once,
//    from the edge's left side with that side's normal (the reference's
//    edge_fluxes, src/solver/rhs/swe_2d_split_form.rs:580-616), and of every
//    boundary face node (wall or characteristic open boundary), stored per
//    element face node as each side sees it;
//  - stage_kernel<N1>: per element, the split-form volume term (flux
//    differencing on wet elements, subcell finite volumes on elements with a
//    node shallower than the subcell depth), the face fluxes lifted by each
//    face node's sJ·LIFT (a multiply-add in the stage, not a multiply in
//    the face pass), 1/J,
//    Coriolis, the Shu–Osher combination, the point-implicit damping and the
//    wet/dry correction or the accumulation (the reference's fused
//    stage_where, src/physics/builder.rs:652-737), and the node velocities
//    the next stage reads.
// Per step: dt_kernel<N1> (element steps, atomic minimum) and three
// one-thread kernels that run the step's clock on the device, so that a
// whole step is one CUDA graph.
//
// The volume and surface terms use the summation-by-parts identity of the
// GLL operators: at a line end the volume term's 2·D₀₀·F(q)·Ja and the
// surface term's LIFT·sJ·F(q)·n are equal and opposite (2D₀₀ = −1/w₀,
// LIFT = 1/w₀ on the face node, sJ·n = −Ja), so neither is evaluated: the
// interior diagonal of D is zero, and what remains is the pair fluxes and
// −LIFT·sJ·F*. The same holds for the subcells' end fluxes. The result
// differs from the reference's by rounding only.

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "device.hpp"
#include "fp64_bits.hpp"
#include "point.cuh"

namespace dgswe {
namespace DGSWE_NS {

enum StageMode { kRhsOnly = 0, kPost = 1, kAccumulate = 2 };

__device__ __forceinline__ Q load_q(const DevBuf& in, const DevTables& T, const Physics& P,
                                    int64_t g) {
    Q q;
    q.h = in.h[g];
    q.hu = in.hu[g];
    q.hv = in.hv[g];
    q.u = in.u[g];
    q.v = in.v[g];
    q.b = P.has_bed ? T.bed[g] : 0.0;
    return q;
}

// An element's stage in a multirate pass (element_stage,
// src/time/multirate.rs:169-200), every operation rounded on its own as the
// reference's are (no contraction): its substep's start time and step, the
// Shu–Osher weights, and for the last stage the weight of its sum (the mean
// of the substep's 2^(rate − level) blocks, restarted where the substep
// starts). dt/2^level and 1/2^(rate − level) are exact.
__device__ __forceinline__ StageArgs lts_stage(const LtsPass& p, int64_t k) {
    const int l = p.level[k];
    const double inv_2l = __longlong_as_double((long long)(1023 - l) << 52);  // 2^-l
    const double dt_l = __dmul_rn(p.dt, inv_2l);
    const long long q = (long long)p.substep >> (p.finest - l);
    const double t_k = __dadd_rn(p.t, __dmul_rn((double)q, dt_l));
    StageArgs a;
    a.time = __dadd_rn(t_k, __dmul_rn(p.c, dt_l));
    a.a = p.start;
    a.b = p.input;
    a.c = __dmul_rn(p.beta, dt_l);
    a.w = 1.0;
    a.keep = 0.0;
    if (p.last) {
        const int blocks = p.rate[k] - l;
        a.w = __longlong_as_double((long long)(1023 - blocks) << 52);  // 1/2^(rate − level)
        a.keep = l >= p.depth ? 0.0 : 1.0;
    }
    return a;
}

// The interface flux of the other split forms (EntropyStable / EntropyConservative):
// F#·n (+ dissipation) with the bed interface term per side
// (src/solver/rhs/swe_2d_split_form.rs:639-650, src/flux/swe_2d_entropy.rs:166-205)
__device__ void entropy_surface(const Q& qa, const Q& qb, double nx, double ny, const Physics& P,
                                F3& fa, F3& fb) {
    const double g = P.g;
    F3 s = wflux(qa, qb, nx, ny, g);
    if (P.formulation == kEntropyStable) {
        const double sp_i = fabs(qa.u * nx + qa.v * ny) + sqrt(g * fmax(qa.h, 0.0));
        const double sp_e = fabs(qb.u * nx + qb.v * ny) + sqrt(g * fmax(qb.h, 0.0));
        const double scale = -0.5 * fmax(sp_i, sp_e);
        const double jump = (qb.h + qb.b) - (qa.h + qa.b);
        const double h_avg = 0.5 * (qa.h + qb.h), u_avg = 0.5 * (qa.u + qb.u),
                     v_avg = 0.5 * (qa.v + qb.v);
        s.h = s.h + scale * jump;
        s.hu = s.hu + scale * (u_avg * jump + h_avg * (qb.u - qa.u));
        s.hv = s.hv + scale * (v_avg * jump + h_avg * (qb.v - qa.v));
    }
    const double fa_b = 0.5 * g * qa.h * (qb.b - qa.b);
    const double fb_b = 0.5 * g * qb.h * (qa.b - qb.b);
    fa = {s.h + 0.0, s.hu + fa_b * nx, s.hv + fa_b * ny};
    fb = {-s.h + 0.0, -s.hu + fb_b * (-nx), -s.hv + fb_b * (-ny)};
}

// The nesting relaxation band's source at the stage's input, per band node
// (NestingRelaxation2D::add_element and relaxation_source,
// src/boundary/ocean_nesting.rs:955-1030), into T.rx_src at its element's
// stage time (in a multirate pass, the element's own)
template <bool LISTED>
__global__ void __launch_bounds__(256) relax_kernel(DevTables T, Physics P, DevBuf in,
                                                    const StepCtl* ctl, int slot, LtsPass lp) {
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= T.rx_n) return;
    const int64_t g = T.rx_node[b];
    const int64_t k = g / P.nn;
    const int32_t s = T.rx_slot[b];
    const int64_t nv = T.K * P.nn;
    double sh = 0.0, shu = 0.0, shv = 0.0;
    const double h = in.h[g], w = T.rx_weight[s];
    if (fp::gt0(w) && !fp::lt(h, T.rx_wet)) {
        const int member = T.elem_member ? T.elem_member[k] : 0;
        const double t = LISTED ? lts_stage(lp, k).time : ctl[member].stage[slot].time;
        const double bed = P.has_bed ? T.bed[g] : 0.0;
        double eta, u, v;
        bool has_uv;
        parent_state_at(T.rx_times, T.rx_n_times, T.rx_cubic, T.rx_values + (int64_t)s * T.rx_n_times * 3,
                        t, T.rx_ramp, T.rx_ref_level, T.rx_velocity, T.rx_max_ratio, T.rx_depth[s],
                        bed, eta, u, v, has_uv);
        const double hp = eta - bed;
        if (!fp::lt(hp, T.rx_wet)) {
            const double gamma = w * T.rx_rate;
            const double hu = in.hu[g], hv = in.hv[g];
            if (!has_uv) {
                u = hu / h;
                v = hv / h;
            }
            const double dh = T.rx_momentum_only ? 0.0 : hp - h;
            const double depth = T.rx_momentum_only ? h : hp;
            sh = gamma * dh;
            shu = gamma * (depth * u - hu);
            shv = gamma * (depth * v - hv);
        }
    }
    if (T.at_source) {  // added to the weather's source of this pass
        T.rx_src[g] += sh;
        T.rx_src[nv + g] += shu;
        T.rx_src[2 * nv + g] += shv;
    } else {
        T.rx_src[g] = sh;
        T.rx_src[nv + g] = shu;
        T.rx_src[2 * nv + g] = shv;
    }
}

// The weather's momentum source at the stage's input
// (GriddedAtmosphere2D::add_element, src/source/swe_2d/gridded_atmosphere.rs:698-729),
// per node of every element (LISTED: of the pass's elements) at its
// element's stage time, into T.rx_src; the relaxation band's kernel,
// launched after it, adds the band's
template <bool LISTED>
__global__ void __launch_bounds__(256) atmos_kernel(DevTables T, Physics P, DevBuf in,
                                                    const StepCtl* ctl, int slot, LtsPass lp) {
    // one stage time for every node of a global stage: its time weights and
    // ramp once per block, in shared memory
    __shared__ int s_idx[2], s_len;
    __shared__ double s_w[2], s_ramp;
    if (!LISTED) {
        if (threadIdx.x == 0) {
            const double t = ctl[0].stage[slot].time;
            int idx[2];
            double w[2];
            s_len = weather_weights(T.at_times, T.at_n_times, T.at_epoch + t, idx, w);
            s_idx[0] = idx[0];
            s_idx[1] = idx[1];
            s_w[0] = w[0];
            s_w[1] = w[1];
            s_ramp = tidal_ramp(t, T.at_ramp);
        }
        __syncthreads();
    }
    const int64_t item = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (item >= (LISTED ? lp.n : T.K) * P.nn) return;
    const int64_t e = item / P.nn;
    const int64_t k = LISTED ? (int64_t)lp.list[e] : e;
    const int64_t g = k * P.nn + item % P.nn;
    const int64_t nv = T.K * P.nn;
    double su = 0.0, sv = 0.0;
    const double h = in.h[g];
    if (!fp::lt(h, T.at_h_min)) {
        int idx[2];
        double w[2];
        int len;
        double ramp;
        if (LISTED) {
            const double t = lts_stage(lp, k).time;
            len = weather_weights(T.at_times, T.at_n_times, T.at_epoch + t, idx, w);
            ramp = tidal_ramp(t, T.at_ramp);
        } else {
            len = s_len;
            idx[0] = s_idx[0];
            idx[1] = s_idx[1];
            w[0] = s_w[0];
            w[1] = s_w[1];
            ramp = s_ramp;
        }
        const double rw = T.at_wind ? ramp : 0.0, rp = T.at_pressure ? ramp : 0.0;
        const double u = weather_field(T.at_values, nv, 0, g, idx, w, len);
        const double v = weather_field(T.at_values, nv, 1, g, idx, w, len);
        const double px = weather_field(T.at_values, nv, 2, g, idx, w, len);
        const double py = weather_field(T.at_values, nv, 3, g, idx, w, len);
        atmosphere_source(h, rw * u, rw * v, rp * px, rp * py, T.at_drag, T.at_cd, T.at_rho_air,
                          T.at_rho_water, T.at_h_min, su, sv);
    }
    if (T.rx_n > 0) T.rx_src[g] = 0.0;
    T.rx_src[nv + g] = su;
    T.rx_src[2 * nv + g] = sv;
}

// The weather's inverse-barometer level at flat node g and simulation time
// t (GriddedAtmosphere2D's BoundaryLevel by node index,
// gridded_atmosphere.rs:873-895), 0 unless the level is the pressure's
__device__ __forceinline__ double weather_level(const DevTables& T, const Physics& P, int64_t g,
                                                double t) {
    if (!T.at_level) return 0.0;
    int idx[2];
    double w[2];
    const int len = weather_weights(T.at_times, T.at_n_times, T.at_epoch + t, idx, w);
    const double p = weather_field(T.at_values, T.K * P.nn, 4, g, idx, w, len);
    return inverse_barometer_level(p, tidal_ramp(t, T.at_ramp), T.at_rho_water);
}

// LISTED: a multirate pass's faces (lp's edge and boundary-face lists),
// each boundary face at its element's stage time
template <int N1, bool LISTED>
__global__ void __launch_bounds__(256) face_kernel(DevTables T, Physics P, DevBuf in, double* fb_h,
                                                   double* fb_hu, double* fb_hv,
                                                   const StepCtl* ctl, int slot,
                                                   const int* active, LtsPass lp) {
    if (!*active) return;
    const int64_t item = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n_int = (LISTED ? lp.n_edges : T.n_edges) * N1;
    if (item >= n_int + (LISTED ? lp.n_bfaces : T.n_bfaces) * N1) return;
    constexpr int NN = N1 * N1;
    const double g = P.g, h_min = P.h_min, sqrt_g = P.sqrt_g, half_g = P.half_g;
    if (item < n_int) {
        const int64_t e = LISTED ? (int64_t)lp.edges[item / N1] : item / N1;
        const int fi = (int)(item % N1);
        const int64_t L = T.edge_left[e], R = T.edge_right[e];
        const int64_t kl = L >> 2, kr = R >> 2;
        const int fl = (int)(L & 3), fr = (int)(R & 3);
        const int rfi = N1 - 1 - fi;
        const int nl = P.face_node[fl][fi], nr = P.face_node[fr][rfi];
        const Q ql = load_q(in, T, P, kl * NN + nl), qr = load_q(in, T, P, kr * NN + nr);
        const double* geo = &T.edge_geo[e * 5];
        F3 fa, fbb;
        if (P.formulation == kWetDry) {
            hydro_hll(side(ql), side(qr), geo[0], geo[1], geo[2], geo[3], geo[4], g, sqrt_g, half_g,
                      h_min, fa, fbb);
            fbb = {-fbb.h, -fbb.hu, -fbb.hv};
        } else {
            entropy_surface(ql, qr, geo[0], geo[1], P, fa, fbb);
        }
        const int64_t sl = (L * N1) + fi, sr = (R * N1) + rfi;
        fb_h[sl] = fa.h;
        fb_hu[sl] = fa.hu;
        fb_hv[sl] = fa.hv;
        fb_h[sr] = fbb.h;
        fb_hu[sr] = fbb.hu;
        fb_hv[sr] = fbb.hv;
        return;
    }
    // boundary face node (src/solver/rhs/swe_2d_split_form.rs:1090-1123)
    const int64_t bfi = LISTED ? (int64_t)lp.bfaces[(item - n_int) / N1] : (item - n_int) / N1;
    const int fi = (int)((item - n_int) % N1);
    const int64_t B = T.bface[bfi];
    const int64_t k = B >> 2;
    const int face = (int)(B & 3);
    const int node = P.face_node[face][fi];
    const Q qi = load_q(in, T, P, k * NN + node);
    const double* geo = &T.bface_geo[bfi * 5];
    const double nx = geo[0], ny = geo[1];
    const Condition& c = T.cond ? T.cond[T.bface_cond[bfi]] : P.cond[T.bface_cond[bfi]];
    F3 fs;
    double u, v;
    interior_velocity(qi, h_min, u, v);
    if (c.kind == kBcWall) {
        const Q qe = wall_ghost(qi, u, v, nx, ny, c.wall_h_min, h_min);
        F3 fdummy;
        if (P.formulation == kWetDry)
            hydro_hll(side(qi), side(qe), nx, ny, geo[2], geo[3], geo[4], g, sqrt_g, half_g, h_min,
                      fs, fdummy);
        else
            entropy_surface(qi, qe, nx, ny, P, fs, fdummy);
    } else {
        // CharacteristicOBC, flux F(q_b)·n: a uniform harmonic tide, or the
        // tide per boundary node (characteristic_boundary_state,
        // src/boundary/characteristic.rs:411-437)
        const int member = T.elem_member ? T.elem_member[k] : 0;
        // a multirate pass: the element's own stage time; a listed global
        // pass (no levels): the stage's
        const double t =
            (LISTED && lp.level) ? lts_stage(lp, k).time : ctl[member].stage[slot].time;
        Q qb;
        if (c.kind == kBcNodeTides || c.kind == kBcParent) {
            const int64_t s = T.bface_slot[bfi * N1 + fi];
            double eta, ue, ve;
            bool has_uv;
            if (c.kind == kBcNodeTides)
                node_tide_state(T.nt_omega + c.nt_omega0, T.nt_frate + c.nt_omega0,
                                T.nt_coef + c.nt_coef0 + (s - c.nt_slot0) * c.nt_n * 6, c.nt_n, t,
                                c.ramp, c.nt_use_mean ? T.nt_mean[s] : 0.0, c.nt_velocity,
                                c.nt_max_ratio, T.nt_depth[s], qi.b, eta, ue, ve, has_uv);
            else
                parent_state_at(T.pt_times + c.pt_time0, c.pt_n_times, c.pt_cubic,
                                T.pt_values + c.pt_val0 + (s - c.nt_slot0) * c.pt_n_times * 3, t,
                                c.ramp, c.pt_reference_level, c.nt_velocity, c.nt_max_ratio,
                                T.nt_depth[s], qi.b, eta, ue, ve, has_uv);
            if (c.raise) eta += c.raise_factor * weather_level(T, P, k * NN + node, t);
            const double h_e = fmax(eta - qi.b, 0.0);
            double un_e = 0.0, ut_e;
            if (has_uv) {
                un_e = ue * nx + ve * ny;
                ut_e = -ue * ny + ve * nx;
            } else {
                if (c.elevation_only == kIncomingWave)
                    un_e = 2.0 * (sqrt(g * fmax(-qi.b, 0.0)) - sqrt(g * h_e));
                ut_e = -u * ny + v * nx;
            }
            qb = characteristic_state_ext(qi, h_e, un_e, ut_e, nx, ny, g, h_min);
        } else {
            double eta = tide_elevation(c, t);
            if (c.raise) eta += c.raise_factor * weather_level(T, P, k * NN + node, t);
            qb = characteristic_state(qi, u, v, eta, nx, ny, c.elevation_only, g, h_min);
        }
        fs = wflux(qb, qb, nx, ny, g);
    }
    const int64_t sl = B * N1 + fi;
    fb_h[sl] = fs.h;
    fb_hu[sl] = fs.hu;
    fb_hv[sl] = fs.hv;
}

// ---------------------------------------------------------------------------
// the stage kernel

// SHAPE 0: ⌊128/NN⌋ elements a block; SHAPE 1: ⌊64/NN⌋ elements a block
// at twice the blocks per SM (the same registers and warps per SM); SHAPE 2:
// ⌊128/NN⌋ elements a block at 6 blocks per SM (80 registers at N1 = 4,
// with a few spilled). The launch shapes dgswe_autotune chooses between.
template <int N1, int SHAPE = 0>
struct Cfg {
    static constexpr int NN = N1 * N1;
    static constexpr int NP = N1 - 1;      // pairs a node owns
    static constexpr int NA = 2 * (N1 - 1);  // pairs a node is in
    static constexpr int PER = SHAPE == 1 ? 64 : 128;
    static constexpr int EPB = (PER / NN) > 0 ? (PER / NN) : 1;
    static constexpr int THREADS = EPB * NN;
    // stage_kernel blocks per SM: 5 caps it at ≤ 102 registers (96 at
    // N1 = 4, no spills) for 20 warps per SM; it is bound by the FP64 pipe
    // and waits on it, so more warps keep it busier (measured 5 % faster
    // on the 1 M-quad N = 3 case than 4 blocks)
    static constexpr int MIN_BLOCKS = SHAPE == 0 ? 5 : (SHAPE == 1 ? 10 : 6);
    static constexpr int PAIR_DOUBLES = NN * NP * 3;
    static constexpr int FACE_DOUBLES = 2 * NN * 8;           // reconstructed faces
    static constexpr int NSUB = 2 * N1 * (N1 - 1);            // subcell interfaces
    static constexpr int IFL_DOUBLES = NSUB * 6;               // their fluxes
    static constexpr int X = PAIR_DOUBLES > FACE_DOUBLES + IFL_DOUBLES ? PAIR_DOUBLES
                                                                       : FACE_DOUBLES + IFL_DOUBLES;
};

__device__ __forceinline__ int line_node(int n1, int dir, int line, int pos) {
    return dir == 0 ? line * n1 + pos : pos * n1 + line;
}

// The subcell interface directions of one line (src/solver/rhs/subcells.rs:63-92)
template <int N1>
__device__ void telescoped(const Physics& P, const double (&m0)[N1], const double (&m1)[N1],
                           bool affine, double (&i0)[N1 + 1], double (&i1)[N1 + 1]) {
    if (affine) {
#pragma unroll
        for (int a = 0; a <= N1; ++a) {
            i0[a] = m0[0];
            i1[a] = m1[0];
        }
        return;
    }
    i0[0] = m0[0];
    i1[0] = m1[0];
    double s0 = 0.0, s1 = 0.0;
#pragma unroll
    for (int a = 0; a < N1 - 1; ++a) {
#pragma unroll
        for (int c = 0; c < N1; ++c) {
            if (c == a) continue;
            const double q2 = 2.0 * P.w[a] * P.d[a * N1 + c];
            s0 += q2 * 0.5 * (m0[a] + m0[c]);
            s1 += q2 * 0.5 * (m1[a] + m1[c]);
        }
        i0[a + 1] = s0;
        i1[a + 1] = s1;
    }
    i0[N1] = m0[N1 - 1];
    i1[N1] = m1[N1 - 1];
}

template <int N1>
__device__ __forceinline__ void line_metric(const DevTables& T, int64_t k, int dir, int line,
                                            double (&m0)[N1], double (&m1)[N1]) {
    constexpr int NN = N1 * N1;
#pragma unroll
    for (int p = 0; p < N1; ++p) {
        const int64_t g = k * NN + line_node(N1, dir, line, p);
        m0[p] = T.contra[g * 4 + 2 * dir];
        m1[p] = T.contra[g * 4 + 2 * dir + 1];
    }
}

// LISTED: a multirate pass over lp's elements, each with its own stage
template <int N1, bool LISTED, int SHAPE = 0>
__global__ void __launch_bounds__(Cfg<N1, SHAPE>::THREADS, Cfg<N1, SHAPE>::MIN_BLOCKS)
    stage_kernel(DevTables T, Physics P, StageExtra X, DevBuf in, DevBuf base, DevBuf out,
                 DevBuf acc, const double* __restrict__ fb_h, const double* __restrict__ fb_hu,
                 const double* __restrict__ fb_hv, StepCtl* ctl, int slot, int mode,
                 int check_finite, const int* active, DevBuf keep, LtsPass lp) {
    using C = Cfg<N1, SHAPE>;
    constexpr int NN = C::NN, NP = C::NP, NA = C::NA, EPB = C::EPB;
    __shared__ double s_q[EPB][7][NN];  // h, hu, hv, u, v, b, 2g·h
    __shared__ double s_x[EPB][C::X];
    __shared__ int s_flag[EPB][3];
    __shared__ double s_red[EPB][5];

    if (!*active) return;
    const int tid = threadIdx.x;
    const int e = tid / NN, i = tid % NN;
    int64_t k = (int64_t)blockIdx.x * EPB + e;
    if (LISTED) k = k < lp.n ? (int64_t)lp.list[k] : T.K;
    else k += X.k_first;
    const int64_t k_end = (LISTED || X.k_last > T.K) ? T.K : X.k_last;
    // the element's member (its StepCtl); an ensemble member that has
    // stopped keeps its state: its elements take no part
    StepCtl* const cm = ctl + ((T.elem_member && k < k_end) ? T.elem_member[k] : 0);
    const bool valid = k < k_end && (!T.elem_member || cm->active);
    const int64_t gi = k * NN + i;
    const int a = i % N1, j = i / N1;
    const double g = P.g, h_min = P.h_min, sqrt_g = P.sqrt_g, half_g = P.half_g;

    if (i == 0) {
        s_flag[e][0] = 0;
        s_flag[e][1] = 0;
        s_flag[e][2] = 0;
    }
    double h = 0, hu = 0, hv = 0, u = 0, v = 0, b = 0;
    if (valid) {
        h = in.h[gi];
        hu = in.hu[gi];
        hv = in.hv[gi];
        u = in.u[gi];
        v = in.v[gi];
        b = P.has_bed ? T.bed[gi] : 0.0;
    }
    s_q[e][0][i] = h;
    s_q[e][1][i] = hu;
    s_q[e][2][i] = hv;
    s_q[e][3][i] = u;
    s_q[e][4][i] = v;
    s_q[e][5][i] = b;
    s_q[e][6][i] = P.two_g * h;  // the pairs' pressure 2g·h_a·h_c takes one multiply
    __syncthreads();
    if (valid && P.formulation == kWetDry && fp::lt(h, P.subcell_depth)) {
        atomicOr(&s_flag[e][0], 1);
        if (!fp::nz(h)) atomicAdd(&s_flag[e][2], 1);
    }
    __syncthreads();
    const bool sub = s_flag[e][0] != 0;
    // A subcell element without water at any node (every h = ±0, so every
    // u = v = 0): its reconstructed subcell faces are dry, so the interface
    // fluxes, pressure and bed terms are all ±0, and it skips the subcell
    // phases (they read only h, u, v and the bed)
    const bool dry = s_flag[e][2] == NN;
    double rh = 0.0, rhu = 0.0, rhv = 0.0;
    const bool affine = valid ? T.affine[k] != 0 : true;

    auto node_side = [&](int n) {
        return Sd{s_q[e][0][n], s_q[e][3][n], s_q[e][4][n], s_q[e][5][n]};
    };
    double* faces = &s_x[e][0];                      // [dir][line][pos][8]
    double* ifl = &s_x[e][C::FACE_DOUBLES];          // [dir][line][pos][6]

    // ---- phase A: pair fluxes, or the subcells' reconstructed faces ----
    if (valid && !sub) {
#pragma unroll
        for (int q = 0; q < NP; ++q) {
            const int8_t* own = &T.sched_owned[(i * NP + q) * 5];
            const int na = own[0], nc = own[1];
            const double hm0 = T.pair_hm[(gi * NP + q) * 2];
            const double hm1 = T.pair_hm[(gi * NP + q) * 2 + 1];
            const double hc = s_q[e][0][nc];
            // ½·F#(q_a, q_c)·{{Ja}} scaled: mass, 2·F_hu, 2·F_hv
            const double mass = (s_q[e][1][na] + s_q[e][1][nc]) * hm0 +
                                (s_q[e][2][na] + s_q[e][2][nc]) * hm1;
            const double gp2 = s_q[e][6][na] * hc;
            const double g_hu = mass * (s_q[e][3][na] + s_q[e][3][nc]) + gp2 * hm0;
            const double g_hv = mass * (s_q[e][4][na] + s_q[e][4][nc]) + gp2 * hm1;
            double* slot_f = &s_x[e][(i * NP + q) * 3];
            slot_f[0] = mass;
            slot_f[1] = g_hu;
            slot_f[2] = g_hv;
        }
    } else if (valid && sub && !dry) {
        // subcell faces of this node's subcell on its r-line and s-line
#pragma unroll
        for (int dir = 0; dir < 2; ++dir) {
            const int line = dir == 0 ? j : a;
            const int pos = dir == 0 ? a : j;
            const Sd q = node_side(i);
            Sd l{}, r{};
            double x_l = 0.0, x_r = 0.0;
            bool have_l = true, have_r = true;
            if (pos > 0) {
                l = node_side(line_node(N1, dir, line, pos - 1));
                x_l = P.x[pos - 1];
            } else {
                // r-lines end on faces 3 (reversed) and 1; s-lines on 0 and 2 (reversed)
                const int face = dir == 0 ? 3 : 0;
                const int fi = dir == 0 ? N1 - 1 - line : line;
                const int64_t o = (k * 4 + face) * N1 + fi;
                const int64_t og = T.outer_idx[o];
                have_l = og >= 0;
                if (have_l) {
                    l = Sd{in.h[og], in.u[og], in.v[og], P.has_bed ? T.bed[og] : 0.0};
                    x_l = -1.0 - T.outer_dist[o];
                }
            }
            if (pos + 1 < N1) {
                r = node_side(line_node(N1, dir, line, pos + 1));
                x_r = P.x[pos + 1];
            } else {
                const int face = dir == 0 ? 1 : 2;
                const int fi = dir == 0 ? line : N1 - 1 - line;
                const int64_t o = (k * 4 + face) * N1 + fi;
                const int64_t og = T.outer_idx[o];
                have_r = og >= 0;
                if (have_r) {
                    r = Sd{in.h[og], in.u[og], in.v[og], P.has_bed ? T.bed[og] : 0.0};
                    x_r = 1.0 + T.outer_dist[o];
                }
            }
            Sd fl = q, fr = q;
            if (have_l && have_r)
                reconstruct(l, q, r, x_l, P.x[pos], x_r, X.xl[pos], X.xr[pos], P.subcell_h_dry,
                            fl, fr);
            double* f = &faces[((dir * N1 + line) * N1 + pos) * 8];
            f[0] = fl.h;
            f[1] = fl.u;
            f[2] = fl.v;
            f[3] = fl.b;
            f[4] = fr.h;
            f[5] = fr.u;
            f[6] = fr.v;
            f[7] = fr.b;
        }
    }
    __syncthreads();

    // ---- phase B: sum the pairs; or the subcell interface fluxes ----
    if (valid && !sub) {
#pragma unroll
        for (int q = 0; q < NA; ++q) {
            const int slot_id = T.sched_slot[i * NA + q];
            const double coef = T.sched_coef[i * NA + q];
            const double hcoef = T.sched_hcoef[i * NA + q];  // coef / 2
            const double* f = &s_x[e][slot_id * 3];
            rh -= coef * f[0];
            rhu -= hcoef * f[1];
            rhv -= hcoef * f[2];
        }
        if (P.has_bed) {
            rhu -= h * T.gdb[gi * 2];
            rhv -= h * T.gdb[gi * 2 + 1];
        }
        if (X.subcell_mass)  // no subcells: NaN (compute_rhs_swe_2d_mass_fluxes_into)
            for (int q = i; q < C::NSUB; q += NN)
                X.subcell_mass[k * C::NSUB + q] = fp::from_bits(0x7FF8000000000000ll);
    } else if (valid && sub && dry) {
        if (X.subcell_mass)  // the dry element's interface fluxes are ±0
            for (int q = i; q < C::NSUB; q += NN) X.subcell_mass[k * C::NSUB + q] = 0.0;
    } else if (valid && sub && !dry) {
#pragma unroll
        for (int dir = 0; dir < 2; ++dir) {
            const int line = dir == 0 ? j : a;
            const int pos = dir == 0 ? a : j;
            if (pos + 1 >= N1) continue;
            double m0[N1], m1[N1], i0[N1 + 1], i1[N1 + 1];
            line_metric<N1>(T, k, dir, line, m0, m1);
            telescoped<N1>(P, m0, m1, affine, i0, i1);
            const double mx = i0[pos + 1], my = i1[pos + 1];
            const double norm = vsqrt(mx * mx + my * my);
            const double inv = vrcp(norm);
            const double* fa_ = &faces[((dir * N1 + line) * N1 + pos) * 8 + 4];   // right face of pos
            const double* fb_ = &faces[((dir * N1 + line) * N1 + pos + 1) * 8];   // left face of pos+1
            F3 fa, fb;
            hydro_hll(Sd{fa_[0], fa_[1], fa_[2], fa_[3]}, Sd{fb_[0], fb_[1], fb_[2], fb_[3]}, mx, my,
                      norm, mx * inv, my * inv, g, sqrt_g, half_g, h_min, fa, fb);
            double* o = &ifl[((dir * N1 + line) * (N1 - 1) + pos) * 6];
            if (X.subcell_mass)  // subcell_slot (src/solver/rhs/subcells.rs:37-42)
                X.subcell_mass[k * C::NSUB + (dir * N1 + line) * (N1 - 1) + pos] = fa.h;
            o[0] = fa.h;
            o[1] = fa.hu;
            o[2] = fa.hv;
            o[3] = fb.h;
            o[4] = fb.hu;
            o[5] = fb.hv;
        }
    }
    __syncthreads();

    // ---- phase C: the subcells' fluxes and bed terms at this node ----
    if (valid && sub && !dry) {
#pragma unroll
        for (int dir = 0; dir < 2; ++dir) {
            const int line = dir == 0 ? j : a;
            const int pos = dir == 0 ? a : j;
            const double iw = X.inv_w[pos];
            if (pos + 1 < N1) {
                const double* o = &ifl[((dir * N1 + line) * (N1 - 1) + pos) * 6];
                rh -= iw * o[0];
                rhu -= iw * o[1];
                rhv -= iw * o[2];
            }
            if (pos > 0) {
                const double* o = &ifl[((dir * N1 + line) * (N1 - 1) + pos - 1) * 6];
                rh += iw * o[3];
                rhu += iw * o[4];
                rhv += iw * o[5];
            }
            const double* f = &faces[((dir * N1 + line) * N1 + pos) * 8];
            const double lh = f[0], lb = f[3], rhh = f[4], rb = f[7];
            const double w_a = P.w[pos];
#if DGSWE_FAST
            (void)w_a;
            const double bed = -0.5 * g * (lh + rhh) * (rb - lb) * iw;  // iw = 1/w_a
#else
            const double bed = -0.5 * g * (lh + rhh) * (rb - lb) / w_a;
#endif
            double m0[N1], m1[N1];
            line_metric<N1>(T, k, dir, line, m0, m1);
            double fx, fy;
            if (affine) {
                fx = bed * m0[0];
                fy = bed * m1[0];
            } else {
                double i0[N1 + 1], i1[N1 + 1];
                telescoped<N1>(P, m0, m1, false, i0, i1);
                const double ml0 = i0[pos], ml1 = i1[pos], mr0 = i0[pos + 1], mr1 = i1[pos + 1];
                const double metric =
#if DGSWE_FAST
                    0.25 * g * ((rhh + h) * (b - rb) + (lh + h) * (b - lb)) * iw;
#else
                    0.25 * g * ((rhh + h) * (b - rb) + (lh + h) * (b - lb)) / w_a;
#endif
                fx = bed * 0.5 * (ml0 + mr0) + metric * (mr0 - ml0);
                fy = bed * 0.5 * (ml1 + mr1) + metric * (mr1 - ml1);
            }
            rhu += fx;
            rhv += fy;
        }
    }

    // ---- surface: −LIFT·sJ·F* of the node's faces ----
    // A node lies on at most one s-face (0 or 2) and one r-face (1 or 3).
    // Every lane takes two slots in face order, a missing one as zero, so
    // the warp's FP64 instructions run on all lanes instead of once per
    // face with only that face's nodes active. Subtracting +0 is exact.
    if (valid) {
        int f_a = j == 0 ? 0 : (j == N1 - 1 ? 2 : -1);
        int f_b = a == N1 - 1 ? 1 : (a == 0 ? 3 : -1);
        if (f_a == 2 && f_b == 1) {  // the reference's face order
            f_a = 1;
            f_b = 2;
        }
        const int64_t fbase = k * 4 * N1;
        auto slot = [&](int f) -> int64_t {
            const int fi = f == 0 ? a : (f == 1 ? j : (f == 2 ? N1 - 1 - a : N1 - 1 - j));
            return fbase + f * N1 + fi;
        };
        double c_a = 0.0, h_a = 0.0, hu_a = 0.0, hv_a = 0.0;
        double c_b = 0.0, h_b = 0.0, hu_b = 0.0, hv_b = 0.0;
        if (f_a >= 0) {
            const int64_t s_a = slot(f_a);
            c_a = T.lift_scale[s_a];
            h_a = fb_h[s_a];
            hu_a = fb_hu[s_a];
            hv_a = fb_hv[s_a];
        }
        if (f_b >= 0) {
            const int64_t s_b = slot(f_b);
            c_b = T.lift_scale[s_b];
            h_b = fb_h[s_b];
            hu_b = fb_hu[s_b];
            hv_b = fb_hv[s_b];
        }
        rh -= c_a * h_a;
        rhu -= c_a * hu_a;
        rhv -= c_a * hv_a;
        rh -= c_b * h_b;
        rhu -= c_b * hu_b;
        rhv -= c_b * hv_b;
    }

    // ---- 1/J and the sources ----
    double Fh = 0.0, Fhu = 0.0, Fhv = 0.0;
    if (valid) {
        const double jinv = T.jinv[gi];
        Fh = jinv * rh;
        Fhu = jinv * rhu;
        Fhv = jinv * rhv;
        if (P.has_coriolis) {
            const double f = P.coriolis_field ? T.fcor[gi] : P.f0;
            Fhu += f * hv;
            Fhv += -f * hu;
        }
        if (T.rx_src) {  // the nesting relaxation band (0 off the band)
            const int64_t nv = T.K * NN;
            Fh += T.rx_src[gi];
            Fhu += T.rx_src[nv + gi];
            Fhv += T.rx_src[2 * nv + gi];
        }
        if (mode == kRhsOnly) {
            out.h[gi] = Fh;
            out.hu[gi] = Fhu;
            out.hv[gi] = Fhv;
        }
    }
    if (mode == kRhsOnly) return;  // uniform: no barrier follows for this mode

    // ---- stage combination and damping ----
    const StageArgs sa = LISTED ? (valid ? lts_stage(lp, k) : StageArgs{}) : cm->stage[slot];
    double vh = 0.0, vhu = 0.0, vhv = 0.0;
    if (valid) {
        if (fp::nz(sa.a)) {
            vh = sa.a * base.h[gi];
            vhu = sa.a * base.hu[gi];
            vhv = sa.a * base.hv[gi];
        }
        if (fp::nz(sa.b)) {
            vh += sa.b * h;
            vhu += sa.b * hu;
            vhv += sa.b * hv;
        }
        if (fp::nz(sa.c)) {
            vh += sa.c * Fh;
            vhu += sa.c * Fhu;
            vhv += sa.c * Fhv;
        }
        // for the adjoint: the combination, then the damped momentum
        if (keep.h) {
            keep.h[gi] = vh;
            keep.hu[gi] = vhu;
            keep.hv[gi] = vhv;
        }
        if (P.friction || P.has_wet_dry) {
            const double g_n2 = P.friction == 2 ? T.g_n2[gi] : P.g_n2;
            damp(P, g_n2, vh, vhu, vhv, DampIn{h, hu, hv, u, v}, sa.c);
        }
        if (keep.h) {
            keep.u[gi] = vhu;
            keep.v[gi] = vhv;
        }
    }

    if (mode == kAccumulate) {
        if (valid) {
            out.h[gi] = vh;
            out.hu[gi] = vhu;
            out.hv[gi] = vhv;
            const double w = sa.w, keep = sa.keep;
            if (fp::nz(keep)) {
                acc.h[gi] = w * vh + keep * acc.h[gi];
                acc.hu[gi] = w * vhu + keep * acc.hu[gi];
                acc.hv[gi] = w * vhv + keep * acc.hv[gi];
            } else {
                acc.h[gi] = w * vh;
                acc.hu[gi] = w * vhu;
                acc.hv[gi] = w * vhv;
            }
        }
        return;
    }

    // ---- wet/dry correction (wetting_drying.rs:194-215) ----
    if (P.has_wet_dry) {
        __syncthreads();  // s_q is free again
        if (valid && fp::lt(vh, P.h_dry)) atomicOr(&s_flag[e][1], 1);
        s_q[e][0][i] = vh;
        s_q[e][1][i] = vhu;
        s_q[e][2][i] = vhv;
        __syncthreads();
        const bool needs = s_flag[e][1] != 0;
        if (valid && needs && i == 0) {
            // element_mean and positivity_limit_element
            // (src/solver/limiters/swe_2d.rs:135-203), in node order
            const double* mass = &T.mass[k * NN];
            double sh = 0.0, shu = 0.0, shv = 0.0, hmin = INFINITY;
            for (int p = 0; p < NN; ++p) {
                sh += mass[p] * s_q[e][0][p];
                shu += mass[p] * s_q[e][1][p];
                shv += mass[p] * s_q[e][2][p];
                hmin = lmin(s_q[e][0][p], hmin);
            }
            const double inv_area = T.inv_area[k];
            const double h_avg = sh * inv_area;
            s_red[e][0] = h_avg;
            s_red[e][1] = shu * inv_area;
            s_red[e][2] = shv * inv_area;
            double theta = 1.0;
            if (fp::gt0(h_avg) && fp::lt0(hmin)) {
                theta = h_avg / (h_avg - hmin);
                theta = fp::lt0(theta) ? 0.0 : (fp::gt(theta, 1.0) ? 1.0 : theta);
            }
            s_red[e][3] = theta;
            s_red[e][4] = hmin;
            if (fp::lt0(h_avg)) atomicAdd((unsigned long long*)&cm->clips, 1ull);
        }
        __syncthreads();
        if (valid && needs) {
            const double h_avg = s_red[e][0];
            if (fp::le0(h_avg)) {
                vh = vhu = vhv = 0.0;
            } else {
                if (fp::lt0(s_red[e][4])) {
                    const double th = s_red[e][3];
                    vh = th * (vh - h_avg) + h_avg;
                    vhu = th * (vhu - s_red[e][1]) + s_red[e][1];
                    vhv = th * (vhv - s_red[e][2]) + s_red[e][2];
                    vh = fp::max0(vh);
                }
                if (fp::lt(h_avg, P.h_dry)) vhu = vhv = 0.0;
            }
        }
        if (valid) correct_node(P, vh, vhu, vhv);
    }
    if (valid) {
        out.h[gi] = vh;
        out.hu[gi] = vhu;
        out.hv[gi] = vhv;
        double uo, vo;
        node_velocity(vh, vhu, vhv, h_min, uo, vo);
        out.u[gi] = uo;
        out.v[gi] = vo;
        if (check_finite && !(fp::finite(vh) && fp::finite(vhu) && fp::finite(vhv)))
            cm->nonfinite = 1;
    }
}

// finish_where over every element: state ← acc, then the wet/dry correction
// LISTED: the end of the substeps of lp's elements, and a non-finite
// result flagged in ctl
template <int N1, bool LISTED>
__global__ void __launch_bounds__(Cfg<N1>::THREADS)
    finish_kernel(DevTables T, Physics P, DevBuf acc, DevBuf state, StepCtl* ctl, LtsPass lp) {
    using C = Cfg<N1>;
    constexpr int NN = C::NN, EPB = C::EPB;
    __shared__ double s_v[EPB][3][NN];
    __shared__ int s_flag[EPB];
    __shared__ double s_red[EPB][5];
    const int tid = threadIdx.x;
    const int e = tid / NN, i = tid % NN;
    int64_t k = (int64_t)blockIdx.x * EPB + e;
    if (LISTED) k = k < lp.n ? (int64_t)lp.list[k] : T.K;
    const bool valid = k < T.K;
    const int64_t gi = k * NN + i;
    StepCtl* const cm = ctl + ((T.elem_member && valid) ? T.elem_member[k] : 0);  // the member's
    if (i == 0) s_flag[e] = 0;
    double vh = 0, vhu = 0, vhv = 0;
    if (valid) {
        vh = acc.h[gi];
        vhu = acc.hu[gi];
        vhv = acc.hv[gi];
    }
    s_v[e][0][i] = vh;
    s_v[e][1][i] = vhu;
    s_v[e][2][i] = vhv;
    __syncthreads();
    if (P.has_wet_dry) {
        if (valid && fp::lt(vh, P.h_dry)) atomicOr(&s_flag[e], 1);
        __syncthreads();
        const bool needs = s_flag[e] != 0;
        if (valid && needs && i == 0) {
            const double* mass = &T.mass[k * NN];
            double sh = 0.0, shu = 0.0, shv = 0.0, hmin = INFINITY;
            for (int p = 0; p < NN; ++p) {
                sh += mass[p] * s_v[e][0][p];
                shu += mass[p] * s_v[e][1][p];
                shv += mass[p] * s_v[e][2][p];
                hmin = lmin(s_v[e][0][p], hmin);
            }
            const double inv_area = T.inv_area[k];
            const double h_avg = sh * inv_area;
            s_red[e][0] = h_avg;
            s_red[e][1] = shu * inv_area;
            s_red[e][2] = shv * inv_area;
            double theta = 1.0;
            if (fp::gt0(h_avg) && fp::lt0(hmin)) {
                theta = h_avg / (h_avg - hmin);
                theta = fp::lt0(theta) ? 0.0 : (fp::gt(theta, 1.0) ? 1.0 : theta);
            }
            s_red[e][3] = theta;
            s_red[e][4] = hmin;
            if (fp::lt0(h_avg)) atomicAdd((unsigned long long*)&cm->clips, 1ull);
        }
        __syncthreads();
        if (valid && needs) {
            const double h_avg = s_red[e][0];
            if (fp::le0(h_avg)) {
                vh = vhu = vhv = 0.0;
            } else {
                if (fp::lt0(s_red[e][4])) {
                    const double th = s_red[e][3];
                    vh = th * (vh - h_avg) + h_avg;
                    vhu = th * (vhu - s_red[e][1]) + s_red[e][1];
                    vhv = th * (vhv - s_red[e][2]) + s_red[e][2];
                    vh = fp::max0(vh);
                }
                if (fp::lt(h_avg, P.h_dry)) vhu = vhv = 0.0;
            }
        }
        if (valid) correct_node(P, vh, vhu, vhv);
    }
    if (valid) {
        state.h[gi] = vh;
        state.hu[gi] = vhu;
        state.hv[gi] = vhv;
        double uo, vo;
        node_velocity(vh, vhu, vhv, P.h_min, uo, vo);
        state.u[gi] = uo;
        state.v[gi] = vo;
        if (LISTED && !(fp::finite(vh) && fp::finite(vhu) && fp::finite(vhv))) cm->nonfinite = 1;
    }
}

// Per element, whether every node is deeper than each of three depths
// (bits 0, 1, 2): the line-local test and the two depths of the coarse
// step's bound (SWEPhysics2D::line_local and coarse_step_bound,
// src/physics/builder.rs:560-632)
__global__ void depth_flags_kernel(const double* h, int64_t K, int nn, double d0, double d1,
                                   double d2, uint8_t* flags) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    bool a = true, b = true, c = true;
    for (int i = 0; i < nn; ++i) {
        const double x = h[k * nn + i];
        a = a && fp::gt(x, d0);
        b = b && fp::gt(x, d1);
        c = c && fp::gt(x, d2);
    }
    flags[k] = (uint8_t)((a ? 1 : 0) | (b ? 2 : 0) | (c ? 4 : 0));
}

// The point-implicit damping of a stage value over dt with the rates frozen
// at `from` (apply_implicit_damping_2d, src/solver/algorithms/
// wetting_drying.rs:376-389: damp_node at every node), then the stage's
// node velocities
__global__ void damping_kernel(DevTables T, Physics P, DevBuf stage, DevBuf from, double dt,
                               int64_t n) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n) return;
    const double h = stage.h[g];
    double hu = stage.hu[g], hv = stage.hv[g];
    const double g_n2 = P.friction == 2 ? T.g_n2[g] : P.g_n2;
    damp(P, g_n2, h, hu, hv, DampIn{from.h[g], from.hu[g], from.hv[g], from.u[g], from.v[g]},
         dt);
    stage.hu[g] = hu;
    stage.hv[g] = hv;
    double u, v;
    node_velocity(h, hu, hv, P.h_min, u, v);
    stage.u[g] = u;
    stage.v[g] = v;
}

// node velocities of a buffer (after an upload)
__global__ void velocity_kernel(DevBuf b, int64_t n, double h_min) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n) return;
    double u, v;
    node_velocity(b.h[g], b.hu[g], b.hv[g], h_min, u, v);
    b.u[g] = u;
    b.v[g] = v;
}

// ---------------------------------------------------------------------------
// the time step (src/solver/rhs/swe_2d.rs:2072-2115, 1346-1367, 2165-2258)

// The dt pass. An element's step needs only the largest of its nodes' rates
// (its own nodes and the neighbours' face nodes, each with its own metric),
// so the rates are first taken in single precision — on the FP32 and
// integer pipes, which run 64 times faster than the FP64 pipe — with a bound
// on their error; only the rates that can still be the largest are then
// computed in FP64, by dense lanes from a list in shared memory, and their
// maximum is the exact one. One lane per element then takes the positivity
// sums in node order, the reference's order.
//
// node_rate_f32 (point.cuh) is within 2⁻²⁰·B of the FP64 rate, B its error
// scale; a node whose r₃₂ + δ·B is below the largest r₃₂ − δ·B of its
// element (δ = 2⁻¹⁶, sixteen times the bound) cannot hold the maximum.
template <int N1>
struct DtCfg {
    static constexpr int NN = N1 * N1;
    // elements per block, one lane of warp 0 each: 16, so that a dt block
    // (256 threads at N = 3, 40 registers) fits on an SM beside two blocks
    // of the face pass it runs with
    static constexpr int EPB = 16;
    static constexpr int THREADS = EPB * NN;
    static constexpr int PITCH = NN + 1;  // odd row pitch: lanes spread over the banks
    static constexpr int SLOTS = NN + 4 * N1;  // own nodes, then neighbours' face nodes
};

// The element's dt from its largest rate and its nodes' depths and mass
// weights (element_dt, swe_2d.rs:2072-2115, with PositivityBound::element_cfl
// and positivity_relaxation, swe_2d.rs:2220-2258)
template <int N1>
__device__ __forceinline__ double element_dt(const DtParams& D, int order, double weight_ratio,
                                             double rmax, const double* h, const double* mass) {
    constexpr int NN = N1 * N1;
    double cfl = D.cfl;
    if (D.positivity) {
        double water = 0.0, water_b = 0.0;
        bool shallow = false;
#pragma unroll
        for (int p = 0; p < NN; ++p) {
            const double hp = h[p];
            shallow = shallow || fp::le(hp, D.shallow);
            const double wi = mass[p] * fp::max0(hp);
            water += wi;
            constexpr int last = N1 - 1;
            if (p % N1 == 0 || p % N1 == last || p / N1 == 0 || p / N1 == last) water_b += wi;
        }
        // f64::min drops the NaN of 0/0
        const double ratio =
            fp::le0(water_b) ? weight_ratio : lmin(water / water_b, weight_ratio);
        const double rho = lmax(0.9 * ratio, 1.0);
        const double cap = shallow ? D.max_cfl_subcells : D.max_cfl;
        cfl = lmin(cfl, lmin(D.bound_cfl * rho, cap));
    }
    return fp::lt(rmax, 1e-14) ? INFINITY : cfl / ((2.0 * (double)order + 1.0) * rmax);
}

// LISTED: the elements list[0..n_list) (any order, any subset), else all
template <int N1, bool LISTED>
__global__ void __launch_bounds__(DtCfg<N1>::THREADS)
    dt_kernel(DevTables T, Physics P, DevBuf q, DtParams D, double* dt_el, StepCtl* ctl,
              const int* active, const int32_t* list, int64_t n_list) {
    using C = DtCfg<N1>;
    constexpr int NN = C::NN, EPB = C::EPB, PITCH = C::PITCH, SLOTS = C::SLOTS;
    __shared__ int64_t s_k[EPB];                      // the block's elements
    __shared__ float s_r[EPB][SLOTS];                 // r₃₂, −1 for a dry node
    __shared__ float s_b[EPB][SLOTS];                 // δ·B
    __shared__ unsigned int s_lo[EPB];                // the element's largest r₃₂ − δ·B (bits)
    __shared__ unsigned long long s_rmax[EPB];        // its largest exact rate (bits)
    __shared__ short s_list[EPB * SLOTS];             // candidates: e·SLOTS + slot
    __shared__ int s_count;
    __shared__ double s_h[EPB * PITCH];
    __shared__ double s_mass[EPB * PITCH];
    if (!*active) return;
    const int tid = threadIdx.x;
    const int e = tid / NN, i = tid % NN;
    const int64_t at = (int64_t)blockIdx.x * EPB + e;
    const int64_t k = LISTED ? (at < n_list ? (int64_t)list[at] : T.K) : at;
    if (i == 0) s_k[e] = k;
    const int64_t gi = k * NN + i;
    const double g = P.g, h_min = P.h_min;
    const float g32 = f32_trunc(g);
    constexpr float kDelta = 1.0f / 65536.0f;      // δ = 2⁻¹⁶
    constexpr float kFloor = 1e-30f;               // the sub-float-range terms
    if (tid < EPB) {
        s_lo[tid] = 0u;
        s_rmax[tid] = 0ull;  // +0: a dry node's rate
    }
    if (tid == 0) s_count = 0;
    double h = 0.0, mass = 0.0;
    // single-precision rates of the node and of the neighbour face nodes it takes
    auto slot_rate = [&](int slot, double hs, double us, double vs, const float* m) {
        float r = -1.0f, b = 0.0f;
        if (fp::gt(hs, h_min)) {
            node_rate_f32(hs, us, vs, m, g32, r, b);
            b = kDelta * b + kFloor;
        }
        s_r[e][slot] = r;
        s_b[e][slot] = b;
    };
    if (k < T.K) {
        h = q.h[gi];
        mass = T.mass[gi];
        slot_rate(i, h, q.u[gi], q.v[gi], &T.dtm32_own[gi * 6]);
        for (int it = i; it < 4 * N1; it += NN) {
            const int64_t o = k * 4 * N1 + it;
            const int64_t nb = T.nb_face_node[o];
            if (nb < 0) {
                s_r[e][NN + it] = -1.0f;
                s_b[e][NN + it] = 0.0f;
                continue;
            }
            slot_rate(NN + it, q.h[nb], q.u[nb], q.v[nb], &T.dtm32_face[o * 6]);
        }
    }
    s_h[e * PITCH + i] = h;
    s_mass[e * PITCH + i] = mass;
    __syncthreads();
    // the element's threshold: its largest r₃₂ − δ·B (non-negative floats
    // order as their bits)
    if (k < T.K) {
        for (int sl = i; sl < SLOTS; sl += NN) {
            const float r = s_r[e][sl];
            if (r >= 0.0f) atomicMax(&s_lo[e], __float_as_uint(fmaxf(r - s_b[e][sl], 0.0f)));
        }
    }
    __syncthreads();
    if (k < T.K) {
        const float lo = __uint_as_float(s_lo[e]);
        for (int sl = i; sl < SLOTS; sl += NN) {
            const float r = s_r[e][sl];
            if (r >= 0.0f && r + s_b[e][sl] >= lo)
                s_list[atomicAdd(&s_count, 1)] = (short)(e * SLOTS + sl);
        }
    }
    __syncthreads();
    // exact rates of the candidates, one per lane
    const int n_cand = s_count;
    for (int c = tid; c < n_cand; c += C::THREADS) {
        const int es = s_list[c];
        const int ce = es / SLOTS, sl = es % SLOTS;
        const int64_t kc = s_k[ce];
        int64_t node;
        const double* m;
        if (sl < NN) {
            node = kc * NN + sl;
            m = &T.dtm_own[node * 6];
        } else {
            const int64_t o = kc * 4 * N1 + (sl - NN);
            node = T.nb_face_node[o];
            m = &T.dtm_face[o * 6];
        }
        const double r = node_rate(q.h[node], q.u[node], q.v[node], m, g);
        atomicMax(&s_rmax[ce], (unsigned long long)fp::bits(r));  // r ≥ +0
    }
    __syncthreads();
    if (tid >= 32) return;  // warp 0: lane l < EPB finishes the block's element l
    const int64_t kl = tid < EPB ? s_k[tid] : T.K;
    unsigned long long dt_bits = 0x7FF0000000000000ull;  // +∞
    int member = -1;
    if (kl < T.K) {
        const double rmax = fp::from_bits((int64_t)s_rmax[tid]);
        const double dt = element_dt<N1>(D, P.order, T.weight_ratio[kl], rmax, &s_h[tid * PITCH],
                                         &s_mass[tid * PITCH]);
        if (dt_el) dt_el[kl] = dt;
        dt_bits = (unsigned long long)fp::bits(dt);
        member = T.elem_member ? T.elem_member[kl] : 0;
    }
    // Each member's smallest step over the warp, then one atomic per member
    // present: members are contiguous element ranges, so lane l gathers the
    // lanes above it while they share its member, and the first lane of each
    // run holds that run's minimum. dt ≥ 0, so its bits order as the values.
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const unsigned long long o = __shfl_down_sync(0xffffffffu, dt_bits, off);
        const int om = __shfl_down_sync(0xffffffffu, member, off);
        if (tid + off < 32 && om == member && o < dt_bits) dt_bits = o;
    }
    const int below = __shfl_up_sync(0xffffffffu, member, 1);
    if (member >= 0 && (tid == 0 || below != member)) atomicMin(&ctl[member].dt_bits, dt_bits);
}

// ---------------------------------------------------------------------------
// the run's clock on the device (Simulation::run_with_callback's loop body,
// src/simulation/runner.rs:355-450)

constexpr int kFailDtMin = 4, kFailMaxSteps = 5, kFailNonFinite = 3;

// Whether the step runs: no failure, time left before the target, steps left
__global__ void step_begin(StepCtl* ctl, int n) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    StepCtl* c = ctl + m;
    c->dt_bits = 0x7FF0000000000000ull;  // +∞
    bool run = c->failure == 0 && c->t < c->target;
    if (run && c->max_steps > 0 && c->steps >= c->max_steps) {
        c->failure = kFailMaxSteps;
        run = false;
    }
    c->active = run ? 1 : 0;
    // the first stage's time needs no dt (its offset is 0 in every scheme):
    // set here, a pass of the first stage can start beside the dt pass
    if (run && c->st_c[0] == 0.0) c->stage[0].time = c->t;
}

// dt from the element steps, capped, checked, fitted to land on the target;
// the stages' times and weights (element_stage, src/time/multirate.rs:169-200)
__global__ void step_dt(StepCtl* ctl, int n) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    StepCtl* c = ctl + m;
    if (!c->active) return;
    double dt = __longlong_as_double((long long)c->dt_bits);
    if (c->dt_max > 0.0) dt = fmin(dt, c->dt_max);
    if (c->dt_min > 0.0 && dt < c->dt_min) {
        c->failure = kFailDtMin;
        c->active = 0;
        c->dt = dt;
        return;
    }
    c->dt_min_used = fmin(c->dt_min_used, dt);
    c->dt_max_used = fmax(c->dt_max_used, dt);
    const bool landed = c->t + dt * (1.0 + 1e-9) >= c->target;
    if (landed) dt = c->target - c->t;
    c->landed = landed ? 1 : 0;
    c->dt = dt;
    for (int s = 0; s < c->scheme_stages; ++s) {
        StageArgs& a = c->stage[s];
        if (s > 0 || c->st_c[0] != 0.0)  // the first stage's time from step_begin
            a.time = __dadd_rn(c->t, __dmul_rn(c->st_c[s], dt));  // rounded apart, as the reference
        a.a = c->st_start[s];
        a.b = c->st_input[s];
        a.c = c->st_beta[s] * dt;
        a.w = 1.0;
        a.keep = 0.0;
    }
}

__global__ void step_end(StepCtl* ctl, int n) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    StepCtl* c = ctl + m;
    if (!c->active) return;
    c->t = c->landed ? c->target : c->t + c->dt;
    c->steps += 1;
    if (c->nonfinite) {
        c->failure = kFailNonFinite;
        c->active = 0;
    }
}

}  // namespace DGSWE_NS
}  // namespace dgswe
