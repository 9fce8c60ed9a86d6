// The discrete adjoint of one stage (kernels.cuh's face_kernel +
// stage_kernel in kPost mode), for the SSP-RK steps of a WetDry run.
//
// Per stage, given λ of the stage output:
//  - stage_adjoint_kernel<N1>: per element, the reverse of the wet/dry
//    correction (correct_node and the element limiter, its branches as the
//    forward took them), the point-implicit damping, the Shu–Osher
//    combination, Coriolis and 1/J, the lift of the face fluxes (λ of each
//    face slot), and the volume term: the split-form pair fluxes and the
//    bed slope, or on subcell elements the subcell reconstruction, interface
//    HLL and bed/metric terms. It writes λ of the stage input for its own
//    element; what lands on a neighbour's node (subcell outer nodes) goes
//    through atomics;
//  - face_adjoint_kernel<N1>: per face node, the reverse of the hydrostatic
//    HLL flux (both sides) or of the boundary flux (wall ghost,
//    characteristic state with the tide's amplitude and phase);
//  - adjoint_combine_kernel: λ of the input node velocity folded into its
//    h, hu, hv (node_velocity), all contributions summed.
// The forward values the reverse needs come from a recomputation of the
// stage (stage_kernel's `keep` output: the combination and the damped
// momentum) and from the stage input itself. The time step is fixed: dt
// and the stage weights are the forward's.
#pragma once

#include "adjoint_point.cuh"

namespace dgswe {
namespace DGSWE_NS {

// The stage adjoint runs as two passes: kAdjWet over the mesh, reversing
// the elements without subcells (the split-form pairs), and kAdjSub over
// the list of those with subcells (subcell_list_kernel, the same test).
// Every element belongs to exactly one pass, and the two write disjoint
// nodes and face slots (their sums into neighbours are atomic), so they
// run side by side. Apart, the wet pass needs neither the subcells'
// scratch nor the array where λ lands from an element's other nodes, and
// its registers are the pair path's alone, so more of its blocks fit on an
// SM; the subcell pass's work is the list's, its other blocks leave at
// once. The few subcell elements' reverse is long (each warp's FP64
// instructions in sequence), so beside the wet pass it costs no time of
// its own.
enum { kAdjWet = 0, kAdjSub = 1 };

template <int N1, int PATH>
struct AdjCfg {
    static constexpr int NN = N1 * N1;
    static constexpr int NP = N1 - 1;
    static constexpr int NA = 2 * (N1 - 1);
    static constexpr int EPB = (64 / NN) > 0 ? (64 / NN) : 1;
    static constexpr int THREADS = EPB * NN;
    // per pair slot a row of 7, the pair's factors for its two nodes; the
    // bed-slope weights (2 per node); each node's λ of the RHS (3 per node)
    static constexpr int ROW = 7;
    static constexpr int PAIR = NN * NP * ROW + 5 * NN;
    static constexpr int FACES = 2 * NN * 8;                    // subcell faces
    static constexpr int IFL = 2 * N1 * (N1 - 1) * 6;           // subcell interface fluxes
    static constexpr int SUB = 2 * FACES + IFL;                 // faces, their λ, interfaces' λ
    static constexpr int VOL = PATH == kAdjWet ? PAIR : (PAIR > SUB ? PAIR : SUB);
    static constexpr int X = VOL > 6 * NN ? VOL : 6 * NN;       // the limiter's scratch too
    static constexpr int LAND = PATH == kAdjSub ? NN : 1;
    // the wet pass: 10 blocks per SM (≤ 102 registers); the subcell pass:
    // 8 (≤ 128 registers; shared memory ≈ 27 KB a block)
    static constexpr int MIN_BLOCKS = PATH == kAdjWet ? 10 : 8;
};

// The node's face slots in the reference's face order (as the forward's lift)
template <int N1>
__device__ __forceinline__ void node_face_slots(int a, int j, int64_t k, int64_t& s_a,
                                                int64_t& s_b) {
    int f_a = j == 0 ? 0 : (j == N1 - 1 ? 2 : -1);
    int f_b = a == N1 - 1 ? 1 : (a == 0 ? 3 : -1);
    if (f_a == 2 && f_b == 1) {
        f_a = 1;
        f_b = 2;
    }
    auto slot = [&](int f) -> int64_t {
        if (f < 0) return -1;
        const int fi = f == 0 ? a : (f == 1 ? j : (f == 2 ? N1 - 1 - a : N1 - 1 - j));
        return (k * 4 + f) * N1 + fi;
    };
    s_a = slot(f_a);
    s_b = slot(f_b);
}

template <int N1, int PATH>
__global__ void __launch_bounds__(AdjCfg<N1, PATH>::THREADS, AdjCfg<N1, PATH>::MIN_BLOCKS)
    stage_adjoint_kernel(DevTables T, Physics P, StageExtra X, DevBuf in, DevBuf keep, AdjStage A,
                         const StepCtl* ctl, int slot) {
    using C = AdjCfg<N1, PATH>;
    constexpr int NN = C::NN, NP = C::NP, NA = C::NA, EPB = C::EPB;
    __shared__ double s_q[EPB][6][NN];        // stage input: h, hu, hv, u, v, b
    __shared__ double s_l[EPB][6][C::LAND];   // λ landing from the element's other nodes
    __shared__ double s_x[EPB][C::X];         // limiter, then the pair or subcell scratch
    __shared__ int s_flag[EPB][2];
    __shared__ double s_red[EPB][12];
    __shared__ int s_arg[EPB];
    __shared__ int s_live[EPB];

    const int tid = threadIdx.x;
    const int e = tid / NN, i = tid % NN;
    // the subcell pass takes its elements from the stage's subcell list;
    // its blocks past the list's end leave at once
    int64_t k;
    if (PATH == kAdjSub) {
        const unsigned long long n_sub = A.sub_count[slot];
        const unsigned long long at = (unsigned long long)blockIdx.x * EPB;
        if (at >= n_sub) return;
        k = at + e < n_sub ? A.sub_list[slot * T.K + (int64_t)(at + e)] : T.K;
    } else {
        k = (int64_t)blockIdx.x * EPB + e;
    }
    bool valid = k < T.K;
    const int64_t gi = k * NN + i;
    const int a = i % N1, j = i / N1;
    const double g = P.g, h_min = P.h_min, sqrt_g = P.sqrt_g, half_g = P.half_g;

    if (i == 0) {
        s_flag[e][0] = 0;
        s_flag[e][1] = 0;
        s_live[e] = 0;
    }
    // the node's input, λ of its output and the kept values, loaded together
    // (one memory latency), though an element of the other pass uses none
    double h = 0, hu = 0, hv = 0, u = 0, v = 0, b = 0;
    double lo_h = 0, lo_hu = 0, lo_hv = 0;
    double vh = 0, vhu = 0, vhv = 0, dhu = 0, dhv = 0;
    if (valid) {
        h = in.h[gi];
        hu = in.hu[gi];
        hv = in.hv[gi];
        u = in.u[gi];
        v = in.v[gi];
        b = P.has_bed ? T.bed[gi] : 0.0;
        lo_h = A.lo_h[gi];
        lo_hu = A.lo_hu[gi];
        lo_hv = A.lo_hv[gi];
        vh = keep.h[gi];
        vhu = keep.hu[gi];
        vhv = keep.hv[gi];
        dhu = keep.u[gi];
        dhv = keep.v[gi];
    }
    s_q[e][0][i] = h;
    s_q[e][1][i] = hu;
    s_q[e][2][i] = hv;
    s_q[e][3][i] = u;
    s_q[e][4][i] = v;
    s_q[e][5][i] = b;
    if (PATH == kAdjSub) {
#pragma unroll
        for (int c = 0; c < 6; ++c) s_l[e][c][i] = 0.0;
    }
    __syncthreads();
    if (valid && P.formulation == kWetDry && fp::lt(h, P.subcell_depth)) atomicOr(&s_flag[e][0], 1);
    __syncthreads();
    // this pass's elements; a block with none of them leaves together
    if ((PATH == kAdjSub) != (s_flag[e][0] != 0)) valid = false;
    // λ of the stage output. An element whose output λ is zero at every node
    // sends zero back through its whole reverse (linear in λ, with finite
    // partials): its nodes' and face slots' λ are written as zeros, its
    // sums (base, g·n², bed, neighbours) are left, and it takes no further
    // part; a block without a live element leaves
    if (valid && (fp::nz(lo_h) || fp::nz(lo_hu) || fp::nz(lo_hv))) s_live[e] = 1;
    __syncthreads();
    if (valid && s_live[e] == 0) {
        A.li_h[gi] = 0.0;
        A.li_hu[gi] = 0.0;
        A.li_hv[gi] = 0.0;
        A.li_u[gi] = 0.0;
        A.li_v[gi] = 0.0;
        int64_t s_a, s_b;
        node_face_slots<N1>(a, j, k, s_a, s_b);
        if (s_a >= 0) A.lf_h[s_a] = A.lf_hu[s_a] = A.lf_hv[s_a] = 0.0;
        if (s_b >= 0) A.lf_h[s_b] = A.lf_hu[s_b] = A.lf_hv[s_b] = 0.0;
        valid = false;
    }
    if (!__syncthreads_or(valid ? 1 : 0)) return;
    constexpr bool sub = PATH == kAdjSub;
    const bool affine = valid ? T.affine[k] != 0 : true;
    // the element's member's stage weights (an ensemble: one StepCtl each)
    const StageArgs sa = ctl[(T.elem_member && valid) ? T.elem_member[k] : 0].stage[slot];

    // λ of this node's input values (registers)
    double Lh = 0, Lhu = 0, Lhv = 0, Lu = 0, Lv = 0, Lb = 0;

    // ---- the wet/dry correction, reversed ----

    double ldh = lo_h, ldhu = lo_hu, ldhv = lo_hv;  // λ of (vh, dhu, dhv)
    if (P.has_wet_dry) {
        if (valid && fp::lt(vh, P.h_dry)) atomicOr(&s_flag[e][1], 1);
        s_x[e][0 * NN + i] = vh;
        s_x[e][1 * NN + i] = dhu;
        s_x[e][2 * NN + i] = dhv;
        __syncthreads();
        const bool needs = s_flag[e][1] != 0;
        if (valid && needs && i == 0) {
            // the forward's element_mean and positivity_limit_element
            const double* mass = &T.mass[k * NN];
            double sh = 0.0, shu = 0.0, shv = 0.0, hmin = INFINITY;
            int arg = 0;
            for (int p = 0; p < NN; ++p) {
                sh += mass[p] * s_x[e][0 * NN + p];
                shu += mass[p] * s_x[e][1 * NN + p];
                shv += mass[p] * s_x[e][2 * NN + p];
                if (fp::lt(s_x[e][0 * NN + p], hmin)) {
                    hmin = s_x[e][0 * NN + p];
                    arg = p;
                }
            }
            const double inv_area = T.inv_area[k];
            const double h_avg = sh * inv_area;
            double theta = 1.0, theta_raw = 1.0;
            if (fp::gt0(h_avg) && fp::lt0(hmin)) {
                theta_raw = h_avg / (h_avg - hmin);
                theta = fp::lt0(theta_raw) ? 0.0 : (fp::gt(theta_raw, 1.0) ? 1.0 : theta_raw);
            }
            s_red[e][0] = h_avg;
            s_red[e][1] = shu * inv_area;
            s_red[e][2] = shv * inv_area;
            s_red[e][3] = theta;
            s_red[e][4] = hmin;
            s_red[e][5] = theta == theta_raw ? 1.0 : 0.0;  // θ not clamped
            s_arg[e] = arg;
        }
        __syncthreads();
        const double h_avg = s_red[e][0], theta = s_red[e][3], hmin = s_red[e][4];
        const bool zeroed = needs && fp::le0(h_avg);
        const bool scaled = needs && !zeroed && fp::lt0(hmin);
        const bool mom0 = needs && !zeroed && fp::lt(h_avg, P.h_dry);
        double wh = vh, whu = dhu, whv = dhv, pre = vh;
        if (valid && needs) {
            if (zeroed) {
                wh = whu = whv = 0.0;
            } else {
                if (scaled) {
                    pre = theta * (vh - h_avg) + h_avg;
                    wh = fp::max0(pre);
                    whu = theta * (dhu - s_red[e][1]) + s_red[e][1];
                    whv = theta * (dhv - s_red[e][2]) + s_red[e][2];
                }
                if (mom0) whu = whv = 0.0;
            }
        }
        double lwh = 0.0, lwhu = 0.0, lwhv = 0.0;
        if (valid) correct_node_rev(P, wh, whu, whv, lo_h, lo_hu, lo_hv, lwh, lwhu, lwhv);
        if (mom0) lwhu = lwhv = 0.0;
        const double lpre = (scaled && fp::gt0(pre)) ? lwh : 0.0;
        if (!needs) {
            ldh = lwh;
            ldhu = lwhu;
            ldhv = lwhv;
        } else if (zeroed) {
            ldh = ldhu = ldhv = 0.0;
        } else if (scaled) {
            ldh = theta * lpre;
            ldhu = theta * lwhu;
            ldhv = theta * lwhv;
        } else {
            ldh = lwh;
            ldhu = lwhu;
            ldhv = lwhv;
        }
        s_x[e][3 * NN + i] = lpre;
        s_x[e][4 * NN + i] = lwhu;
        s_x[e][5 * NN + i] = lwhv;
        __syncthreads();
        if (valid && scaled && i == 0) {
            double tb = 0.0, sp = 0.0, spu = 0.0, spv = 0.0;
            for (int p = 0; p < NN; ++p) {
                tb += s_x[e][3 * NN + p] * (s_x[e][0 * NN + p] - h_avg) + s_x[e][4 * NN + p] * (s_x[e][1 * NN + p] - s_red[e][1]) +
                      s_x[e][5 * NN + p] * (s_x[e][2 * NN + p] - s_red[e][2]);
                sp += s_x[e][3 * NN + p];
                spu += s_x[e][4 * NN + p];
                spv += s_x[e][5 * NN + p];
            }
            double h_avg_b = (1.0 - theta) * sp, hmin_b = 0.0;
            if (s_red[e][5] != 0.0) {  // dθ: θ = h_avg/(h_avg − hmin)
                const double d = h_avg - hmin;
                h_avg_b += tb * (-hmin) / (d * d);
                hmin_b = tb * h_avg / (d * d);
            }
            const double inv_area = T.inv_area[k];
            s_red[e][6] = h_avg_b * inv_area;
            s_red[e][7] = (1.0 - theta) * spu * inv_area;
            s_red[e][8] = (1.0 - theta) * spv * inv_area;
            s_red[e][9] = hmin_b;
        }
        __syncthreads();
        if (valid && scaled) {
            const double m = T.mass[gi];
            ldh += m * s_red[e][6];
            ldhu += m * s_red[e][7];
            ldhv += m * s_red[e][8];
            if (i == s_arg[e]) ldh += s_red[e][9];
        }
    }

    // ---- damping, the combination, Coriolis, 1/J: reversed ----
    double lvh = ldh, lvhu = ldhu, lvhv = ldhv;  // λ of the combination
    if (valid && (P.friction || P.has_wet_dry)) {
        const double g_n2 = P.friction == 2 ? T.g_n2[gi] : P.g_n2;
        DampIn fromb{};
        double gb = 0.0;
        lvhu = 0.0;
        lvhv = 0.0;
        damp_rev(P, g_n2, vh, vhu, vhv, DampIn{h, hu, hv, u, v}, sa.c, ldhu, ldhv, lvh, lvhu, lvhv,
                 fromb, gb);
        Lh += fromb.h;
        Lhu += fromb.hu;
        Lhv += fromb.hv;
        Lu += fromb.u;
        Lv += fromb.v;
        if (P.friction) A.lgn2[gi] += gb;
    }
    double lrh = 0.0, lrhu = 0.0, lrhv = 0.0;  // λ of the volume + surface RHS
    if (valid) {
        if (fp::nz(sa.a)) {
            A.lb_h[gi] += sa.a * lvh;
            A.lb_hu[gi] += sa.a * lvhu;
            A.lb_hv[gi] += sa.a * lvhv;
        }
        if (fp::nz(sa.b)) {
            Lh += sa.b * lvh;
            Lhu += sa.b * lvhu;
            Lhv += sa.b * lvhv;
        }
        double lFh = 0.0, lFhu = 0.0, lFhv = 0.0;
        if (fp::nz(sa.c)) {
            lFh = sa.c * lvh;
            lFhu = sa.c * lvhu;
            lFhv = sa.c * lvhv;
        }
        if (P.has_coriolis) {
            const double f = P.coriolis_field ? T.fcor[gi] : P.f0;
            Lhv += f * lFhu;
            Lhu -= f * lFhv;
        }
        const double jinv = T.jinv[gi];
        lrh = jinv * lFh;
        lrhu = jinv * lFhu;
        lrhv = jinv * lFhv;
        // the lift: rh −= sJ·LIFT·F* per face slot of the node
        int64_t s_a, s_b;
        node_face_slots<N1>(a, j, k, s_a, s_b);
        if (s_a >= 0) {
            const double c = T.lift_scale[s_a];
            A.lf_h[s_a] = -c * lrh;
            A.lf_hu[s_a] = -c * lrhu;
            A.lf_hv[s_a] = -c * lrhv;
        }
        if (s_b >= 0) {
            const double c = T.lift_scale[s_b];
            A.lf_h[s_b] = -c * lrh;
            A.lf_hu[s_b] = -c * lrhu;
            A.lf_hv[s_b] = -c * lrhv;
        }
    }

    // ---- the volume term, reversed ----
    double* faces = &s_x[e][0];                    // subcell [dir][line][pos][8]
    double* faces_b = &s_x[e][C::FACES];           // their λ
    double* ifl_b = &s_x[e][2 * C::FACES];         // λ of the interface fluxes [..][6]
    constexpr int ROW = C::ROW;
    // pair path: [slot][λp, λm, m0, m1, λu, λv, m] — λ of the pair's
    // pressure and mass flux, its metric, λ of its velocity sums and its mass
    // flux; each node takes λp·h(other node), λm·(m0, m1) and (λu, λv)·m
    double* lp = &s_x[e][0];
    double* s_ab = &s_x[e][NN * NP * ROW];         // pair path: bed-slope weights −h·λr [2][NN]
    double* s_lr = &s_x[e][NN * NP * ROW + 2 * NN];  // pair path: λ of the RHS [3][NN]
    auto node_side = [&](int n) {
        return Sd{s_q[e][0][n], s_q[e][3][n], s_q[e][4][n], s_q[e][5][n]};
    };
    __syncthreads();
    const bool work = valid;  // live elements only (above)
    // step 1: pair slots' λ, or the subcell faces (forward)
    if (work && !sub) {
        if (P.has_bed) {
            Lh -= T.gdb[gi * 2] * lrhu + T.gdb[gi * 2 + 1] * lrhv;
        }
        s_ab[i] = -h * lrhu;
        s_ab[NN + i] = -h * lrhv;
        s_lr[i] = lrh;
        s_lr[NN + i] = lrhu;
        s_lr[2 * NN + i] = lrhv;
    } else if (work && sub) {
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
                reconstruct(l, q, r, x_l, P.x[pos], x_r, X.xl[pos], X.xr[pos], P.subcell_h_dry, fl,
                            fr);
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
    // step 2: each owned pair's reverse; or the subcells' sums and bed terms
    if (work && !sub) {
        const double two_g = P.two_g;
#pragma unroll
        for (int q = 0; q < NP; ++q) {
            const int sl = i * NP + q;
            const int8_t* own = &T.sched_owned[sl * 5];
            const int na = own[0], nc = own[1];
            const double hm0 = T.pair_hm[(gi * NP + q) * 2];
            const double hm1 = T.pair_hm[(gi * NP + q) * 2 + 1];
            // λ of the pair's flux: its two nodes' λ of the RHS, each times
            // its accumulation coefficient (−coef into h, −coef/2 into hu, hv)
            const double* pc = &T.pair_coef[sl * 4];
            const double f0 = -(pc[0] * s_lr[na] + pc[1] * s_lr[nc]);
            const double f1 = -(pc[2] * s_lr[NN + na] + pc[3] * s_lr[NN + nc]);
            const double f2 = -(pc[2] * s_lr[2 * NN + na] + pc[3] * s_lr[2 * NN + nc]);
            const double mass = (s_q[e][1][na] + s_q[e][1][nc]) * hm0 +
                                (s_q[e][2][na] + s_q[e][2][nc]) * hm1;
            const double lmass =
                f0 + f1 * (s_q[e][3][na] + s_q[e][3][nc]) + f2 * (s_q[e][4][na] + s_q[e][4][nc]);
            const double lgp2 = (f1 * hm0 + f2 * hm1) * two_g;
            double* o = &lp[sl * ROW];
            o[0] = lgp2;
            o[1] = lmass;
            o[2] = hm0;
            o[3] = hm1;
            o[4] = f1;
            o[5] = f2;
            o[6] = mass;
        }
    } else if (work && sub) {
#pragma unroll
        for (int dir = 0; dir < 2; ++dir) {
            const int line = dir == 0 ? j : a;
            const int pos = dir == 0 ? a : j;
            const double iw = X.inv_w[pos];
            if (pos + 1 < N1) {
                double* o = &ifl_b[((dir * N1 + line) * (N1 - 1) + pos) * 6];
                o[0] = -iw * lrh;
                o[1] = -iw * lrhu;
                o[2] = -iw * lrhv;
            }
            if (pos > 0) {
                double* o = &ifl_b[((dir * N1 + line) * (N1 - 1) + pos - 1) * 6];
                o[3] = iw * lrh;
                o[4] = iw * lrhu;
                o[5] = iw * lrhv;
            }
            const double* f = &faces[((dir * N1 + line) * N1 + pos) * 8];
            double* fb = &faces_b[((dir * N1 + line) * N1 + pos) * 8];
            const double lh = f[0], lb = f[3], rhh = f[4], rb = f[7];
            const double w_a = P.w[pos];
#if DGSWE_FAST_PATH
            const double kb = -0.5 * g * iw;
            const double km = 0.25 * g * iw;
            (void)w_a;
#else
            const double kb = -0.5 * g / w_a;
            const double km = 0.25 * g / w_a;
#endif
            double m0[N1], m1[N1];
            line_metric<N1>(T, k, dir, line, m0, m1);
            double lbed;
            double llh = 0.0, llb = 0.0, lrh_ = 0.0, lrb = 0.0;
            if (affine) {
                lbed = lrhu * m0[0] + lrhv * m1[0];
            } else {
                double i0[N1 + 1], i1[N1 + 1];
                telescoped<N1>(P, m0, m1, false, i0, i1);
                const double ml0 = i0[pos], ml1 = i1[pos], mr0 = i0[pos + 1], mr1 = i1[pos + 1];
                lbed = lrhu * 0.5 * (ml0 + mr0) + lrhv * 0.5 * (ml1 + mr1);
                const double lmet = lrhu * (mr0 - ml0) + lrhv * (mr1 - ml1);
                // metric = km·((rhh + h)(b − rb) + (lh + h)(b − lb))
                const double k2 = lmet * km;
                lrh_ += k2 * (b - rb);
                Lh += k2 * ((b - rb) + (b - lb));
                Lb += k2 * ((rhh + h) + (lh + h));
                lrb -= k2 * (rhh + h);
                llh += k2 * (b - lb);
                llb -= k2 * (lh + h);
            }
            // bed = kb·(lh + rhh)(rb − lb)
            const double k1 = lbed * kb;
            llh += k1 * (rb - lb);
            lrh_ += k1 * (rb - lb);
            lrb += k1 * (lh + rhh);
            llb -= k1 * (lh + rhh);
            fb[0] = llh;
            fb[1] = 0.0;
            fb[2] = 0.0;
            fb[3] = llb;
            fb[4] = lrh_;
            fb[5] = 0.0;
            fb[6] = 0.0;
            fb[7] = lrb;
        }
    }
    __syncthreads();
    // step 3: gather the pairs' λ and the bed slope's; or the interface HLLs
    if (work && !sub) {
#pragma unroll
        for (int q = 0; q < NA; ++q) {
            const int sl = T.sched_slot[i * NA + q];
            const int8_t* own = &T.sched_owned[sl * 5];
            const int other = own[0] == i ? own[1] : own[0];
            const double* o = &lp[sl * ROW];
            Lh += o[0] * s_q[e][0][other];
            Lhu += o[1] * o[2];
            Lhv += o[1] * o[3];
            Lu += o[4] * o[6];
            Lv += o[5] * o[6];
        }
        if (P.has_bed && A.lbed) {
            // gdb_i = g Σ_dir Σ_c D[pos_i][pos_c] B_c w(i, c), transposed: this
            // node as c, the coefficients from the gdb_t table
            const double* t = &T.gdb_t[gi * 4 * N1];
#pragma unroll
            for (int dir = 0; dir < 2; ++dir) {
                const int line = dir == 0 ? j : a;
#pragma unroll
                for (int pa = 0; pa < N1; ++pa) {
                    const int n = line_node(N1, dir, line, pa);
                    const double* c = &t[(dir * N1 + pa) * 2];
                    Lb += c[0] * s_ab[n] + c[1] * s_ab[NN + n];
                }
            }
        }
    } else if (work && sub) {
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
            const double* fa_ = &faces[((dir * N1 + line) * N1 + pos) * 8 + 4];
            const double* fb_ = &faces[((dir * N1 + line) * N1 + pos + 1) * 8];
            const double* o = &ifl_b[((dir * N1 + line) * (N1 - 1) + pos) * 6];
            Sd sa_{}, sb_{};
            hydro_hll_rev(Sd{fa_[0], fa_[1], fa_[2], fa_[3]}, Sd{fb_[0], fb_[1], fb_[2], fb_[3]}, mx,
                          my, norm, mx * inv, my * inv, g, sqrt_g, half_g, h_min,
                          F3{o[0], o[1], o[2]}, F3{o[3], o[4], o[5]}, sa_, sb_);
            double* ba = &faces_b[((dir * N1 + line) * N1 + pos) * 8 + 4];
            double* bb = &faces_b[((dir * N1 + line) * N1 + pos + 1) * 8];
            ba[0] += sa_.h;
            ba[1] += sa_.u;
            ba[2] += sa_.v;
            ba[3] += sa_.b;
            bb[0] += sb_.h;
            bb[1] += sb_.u;
            bb[2] += sb_.v;
            bb[3] += sb_.b;
        }
    }
    __syncthreads();
    // step 4: the subcell reconstructions, reversed
    if (work && sub) {
#pragma unroll
        for (int dir = 0; dir < 2; ++dir) {
            const int line = dir == 0 ? j : a;
            const int pos = dir == 0 ? a : j;
            const Sd q = node_side(i);
            Sd l{}, r{};
            double x_l = 0.0, x_r = 0.0;
            bool have_l = true, have_r = true;
            int n_l = -1, n_r = -1;
            int64_t og_l = -1, og_r = -1;
            if (pos > 0) {
                n_l = line_node(N1, dir, line, pos - 1);
                l = node_side(n_l);
                x_l = P.x[pos - 1];
            } else {
                const int face = dir == 0 ? 3 : 0;
                const int fi = dir == 0 ? N1 - 1 - line : line;
                const int64_t o = (k * 4 + face) * N1 + fi;
                og_l = T.outer_idx[o];
                have_l = og_l >= 0;
                if (have_l) {
                    l = Sd{in.h[og_l], in.u[og_l], in.v[og_l], P.has_bed ? T.bed[og_l] : 0.0};
                    x_l = -1.0 - T.outer_dist[o];
                }
            }
            if (pos + 1 < N1) {
                n_r = line_node(N1, dir, line, pos + 1);
                r = node_side(n_r);
                x_r = P.x[pos + 1];
            } else {
                const int face = dir == 0 ? 1 : 2;
                const int fi = dir == 0 ? line : N1 - 1 - line;
                const int64_t o = (k * 4 + face) * N1 + fi;
                og_r = T.outer_idx[o];
                have_r = og_r >= 0;
                if (have_r) {
                    r = Sd{in.h[og_r], in.u[og_r], in.v[og_r], P.has_bed ? T.bed[og_r] : 0.0};
                    x_r = 1.0 + T.outer_dist[o];
                }
            }
            const double* fb = &faces_b[((dir * N1 + line) * N1 + pos) * 8];
            const Sd lb{fb[0], fb[1], fb[2], fb[3]}, rb{fb[4], fb[5], fb[6], fb[7]};
            if (have_l && have_r) {
                Sd mb{}, cb{}, pb{};
                reconstruct_rev(l, q, r, x_l, P.x[pos], x_r, X.xl[pos], X.xr[pos], P.subcell_h_dry,
                                lb, rb, mb, cb, pb);
                Lh += cb.h;
                Lu += cb.u;
                Lv += cb.v;
                Lb += cb.b;
                if (n_l >= 0) {
                    atomicAdd(&s_l[e][0][n_l], mb.h);
                    atomicAdd(&s_l[e][3][n_l], mb.u);
                    atomicAdd(&s_l[e][4][n_l], mb.v);
                    atomicAdd(&s_l[e][5][n_l], mb.b);
                } else {
                    atomicAdd(&A.lx_h[og_l], mb.h);
                    atomicAdd(&A.lx_u[og_l], mb.u);
                    atomicAdd(&A.lx_v[og_l], mb.v);
                    if (P.has_bed && A.lbed) atomicAdd(&A.lbed[og_l], mb.b);
                }
                if (n_r >= 0) {
                    atomicAdd(&s_l[e][0][n_r], pb.h);
                    atomicAdd(&s_l[e][3][n_r], pb.u);
                    atomicAdd(&s_l[e][4][n_r], pb.v);
                    atomicAdd(&s_l[e][5][n_r], pb.b);
                } else {
                    atomicAdd(&A.lx_h[og_r], pb.h);
                    atomicAdd(&A.lx_u[og_r], pb.u);
                    atomicAdd(&A.lx_v[og_r], pb.v);
                    if (P.has_bed && A.lbed) atomicAdd(&A.lbed[og_r], pb.b);
                }
            } else {  // no reconstruction: both faces are the node's state
                Lh += lb.h + rb.h;
                Lu += lb.u + rb.u;
                Lv += lb.v + rb.v;
                Lb += lb.b + rb.b;
            }
        }
    }
    __syncthreads();
    if (valid) {
        // λ landed from the element's other nodes (the subcell pass only)
        auto land = [&](int c) { return PATH == kAdjSub ? s_l[e][c][i] : 0.0; };
        A.li_h[gi] = Lh + land(0);
        A.li_hu[gi] = Lhu + land(1);
        A.li_hv[gi] = Lhv + land(2);
        A.li_u[gi] = Lu + land(3);
        A.li_v[gi] = Lv + land(4);
        const double lb_all = Lb + land(5);
        if (P.has_bed && A.lbed && lb_all != 0.0) atomicAdd(&A.lbed[gi], lb_all);
    }
}

// The face fluxes' reverse: every interior edge node once (both sides) and
// every boundary face node
template <int N1>
__global__ void __launch_bounds__(256)
    face_adjoint_kernel(DevTables T, Physics P, DevBuf in, AdjStage A, const StepCtl* ctl,
                        int slot) {
    const int64_t item = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n_int = T.n_edges * N1;
    if (item >= n_int + T.n_bfaces * N1) return;
    constexpr int NN = N1 * N1;
    const double g = P.g, h_min = P.h_min, sqrt_g = P.sqrt_g, half_g = P.half_g;
    auto add = [&](int64_t gn, double lh, double lhu, double lhv, double lu, double lv,
                   double lb) {
        if (lh != 0.0) atomicAdd(&A.lx_h[gn], lh);
        if (lhu != 0.0) atomicAdd(&A.lx_hu[gn], lhu);
        if (lhv != 0.0) atomicAdd(&A.lx_hv[gn], lhv);
        if (lu != 0.0) atomicAdd(&A.lx_u[gn], lu);
        if (lv != 0.0) atomicAdd(&A.lx_v[gn], lv);
        if (P.has_bed && A.lbed && lb != 0.0) atomicAdd(&A.lbed[gn], lb);
    };
    if (item < n_int) {
        const int64_t e = item / N1;
        const int fi = (int)(item % N1);
        const int64_t L = T.edge_left[e], R = T.edge_right[e];
        const int64_t kl = L >> 2, kr = R >> 2;
        const int fl = (int)(L & 3), fr = (int)(R & 3);
        const int rfi = N1 - 1 - fi;
        const int64_t sl = (L * N1) + fi, sr = (R * N1) + rfi;
        // the right slot stored −fb
        const F3 la{A.lf_h[sl], A.lf_hu[sl], A.lf_hv[sl]};
        const F3 lb{-A.lf_h[sr], -A.lf_hu[sr], -A.lf_hv[sr]};
        // (the states are loaded before the test below, so that one memory
        // latency covers both)
        const int64_t gl = kl * NN + P.face_node[fl][fi], gr = kr * NN + P.face_node[fr][rfi];
        const Q ql = load_q(in, T, P, gl), qr = load_q(in, T, P, gr);
        // zero λ on both sides sends zero back (linear in λ)
        if (!(fp::nz(la.h) || fp::nz(la.hu) || fp::nz(la.hv) || fp::nz(lb.h) || fp::nz(lb.hu) ||
              fp::nz(lb.hv)))
            return;
        const double* geo = &T.edge_geo[e * 5];
        Sd ab{}, bb{};
        hydro_hll_rev(side(ql), side(qr), geo[0], geo[1], geo[2], geo[3], geo[4], g, sqrt_g, half_g,
                      h_min, la, lb, ab, bb);
        add(gl, ab.h, 0.0, 0.0, ab.u, ab.v, ab.b);
        add(gr, bb.h, 0.0, 0.0, bb.u, bb.v, bb.b);
        return;
    }
    const int64_t bfi = (item - n_int) / N1;
    const int fi = (int)((item - n_int) % N1);
    const int64_t B = T.bface[bfi];
    const int64_t k = B >> 2;
    const int face = (int)(B & 3);
    const int64_t sl = B * N1 + fi;
    const F3 lfs{A.lf_h[sl], A.lf_hu[sl], A.lf_hv[sl]};
    if (!(fp::nz(lfs.h) || fp::nz(lfs.hu) || fp::nz(lfs.hv))) return;  // zero λ: zero back
    const int64_t gn = k * NN + P.face_node[face][fi];
    const Q qi = load_q(in, T, P, gn);
    const double* geo = &T.bface_geo[bfi * 5];
    const double nx = geo[0], ny = geo[1];
    const int ci = T.bface_cond[bfi];
    const Condition& c = T.cond ? T.cond[ci] : P.cond[ci];
    double u, v;
    interior_velocity(qi, h_min, u, v);
    if (c.kind == kBcWall) {
        const Q qe = wall_ghost(qi, u, v, nx, ny, c.wall_h_min, h_min);
        Sd sib{}, seb{};
        hydro_hll_rev(side(qi), side(qe), nx, ny, geo[2], geo[3], geo[4], g, sqrt_g, half_g, h_min,
                      lfs, F3{0.0, 0.0, 0.0}, sib, seb);
        Q qib{sib.h, 0.0, 0.0, 0.0, 0.0, sib.b};
        const Q qeb{seb.h, 0.0, 0.0, seb.u, seb.v, seb.b};
        double ub = sib.u, vb = sib.v;  // the node velocity is the interior velocity
        wall_ghost_rev(qi, u, v, nx, ny, c.wall_h_min, h_min, qe, qeb, qib, ub, vb);
        add(gn, qib.h, qib.hu, qib.hv, ub, vb, qib.b);
    } else {
        const double t = ctl[T.elem_member ? T.elem_member[k] : 0].stage[slot].time;
        const double eta = tide_elevation(c, t);
        const Q qb = characteristic_state(qi, u, v, eta, nx, ny, c.elevation_only, g, h_min);
        Q qbb{};
        wflux_same_rev(qb, nx, ny, g, lfs, qbb);
        Q qib{};
        double ub = 0.0, vb = 0.0, etab = 0.0;
        characteristic_state_rev(qi, u, v, eta, nx, ny, c.elevation_only, g, h_min, qbb, qib, ub,
                                 vb, etab);
        add(gn, qib.h, qib.hu, qib.hv, ub, vb, qib.b);
        if (A.ltide && etab != 0.0) {
            double gr[2 * kMaxConstituents] = {};
            tide_elevation_rev(c, t, etab, gr);
            for (int m = 0; m < 2 * c.n_constituents; ++m)
                atomicAdd(&A.ltide[ci * 2 * kMaxConstituents + m], gr[m]);
        }
    }
}

// The subcell elements of a step's three stage inputs h0, h1, h2 (a node
// shallower than the subcell depth, in the WetDry formulation): stage s's
// list at A.sub_list + s·K, its length in A.sub_count[s] (zeroed before).
// One thread per element; the lists' order does not matter.
__global__ void subcell_list_kernel(DevTables T, Physics P, const double* h0, const double* h1,
                                    const double* h2, AdjStage A, int nn) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= T.K || P.formulation != kWetDry) return;
    const double* hs[3] = {h0, h1, h2};
#pragma unroll
    for (int s = 0; s < 3; ++s) {
        bool sub = false;
        for (int i = 0; i < nn; ++i) sub |= fp::lt(hs[s][k * nn + i], P.subcell_depth);
        if (sub) A.sub_list[s * T.K + (int64_t)atomicAdd(&A.sub_count[s], 1ull)] = k;
    }
}

// λ of the stage input: own element + faces and neighbours, the node
// velocity folded into h, hu, hv; clears the atomic accumulators. For the
// step's first stage (`base_h` set) λ of the step's start state: that plus
// the three stages' base terms, whose sums are cleared
__global__ void adjoint_combine_kernel(DevBuf in, AdjStage A, double* out_h, double* out_hu,
                                       double* out_hv, double* base_h, double* base_hu,
                                       double* base_hv, int64_t n, double h_min) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n) return;
    // every load first, so that one memory latency covers them all
    double bh = 0.0, bhu = 0.0, bhv = 0.0;
    if (base_h) {
        bh = base_h[g];
        bhu = base_hu[g];
        bhv = base_hv[g];
    }
    double lh = A.li_h[g] + A.lx_h[g], lhu = A.li_hu[g] + A.lx_hu[g], lhv = A.li_hv[g] + A.lx_hv[g];
    const double lu = A.li_u[g] + A.lx_u[g], lv = A.li_v[g] + A.lx_v[g];
    node_velocity_rev(in.h[g], in.hu[g], in.hv[g], h_min, lu, lv, lh, lhu, lhv);
    if (base_h) {
        lh = lh + bh;
        lhu = lhu + bhu;
        lhv = lhv + bhv;
        base_h[g] = 0.0;
        base_hu[g] = 0.0;
        base_hv[g] = 0.0;
    }
    out_h[g] = lh;
    out_hu[g] = lhu;
    out_hv[g] = lhv;
    A.lx_h[g] = 0.0;
    A.lx_hu[g] = 0.0;
    A.lx_hv[g] = 0.0;
    A.lx_u[g] = 0.0;
    A.lx_v[g] = 0.0;
}

// η = Σ w_i (h_i + B_i) at each station (its element's nodes, Lagrange
// weights), into eta[s]
__global__ void station_eval_kernel(const double* h, const double* bed, const int64_t* node0,
                                    const double* w, int n_stations, int nn, double* eta) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n_stations) return;
    double acc = 0.0;
    for (int i = 0; i < nn; ++i) {
        const int64_t gn = node0[s] + i;
        acc += w[(int64_t)s * nn + i] * (h[gn] + (bed ? bed[gn] : 0.0));
    }
    eta[s] = acc;
}

// λ of the misfit Σ (η − η_obs)² at one step: 2(η − η_obs)·w into h and B
__global__ void station_seed_kernel(const double* eta, const double* obs, const int64_t* node0,
                                    const double* w, int n_stations, int nn, double* lh,
                                    double* lbed) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_stations * nn) return;
    const int s = t / nn, i = t % nn;
    const double r = 2.0 * (eta[s] - (obs ? obs[s] : 0.0)) * w[t];
    atomicAdd(&lh[node0[s] + i], r);
    if (lbed) atomicAdd(&lbed[node0[s] + i], r);
}

}  // namespace DGSWE_NS
}  // namespace dgswe
