// Device-side data of a dgswe handle shared by the host runtime and the
// kernel translation units: table pointers, physics constants, stage
// arguments and the step control block. Plain structs, passed to kernels by
// value.
#pragma once

#include <cstdint>

namespace dgswe {

constexpr int kMaxConstituents = 8;
constexpr int kMaxConditions = 8;
constexpr int kMaxStages = 4;
// stage argument slots: 0..3 the device-driven step's stages, 4 host calls
constexpr int kHostSlot = 4;
constexpr int kArgSlots = 5;

struct DevBuf {
    double *h, *hu, *hv;  // conserved
    double *u, *v;        // node velocity (hu, hv)/h, 0 at h ≤ h_min
};

struct DevTables {
    int64_t K = 0;
    int64_t n_edges = 0, n_bfaces = 0;
    const double *bed, *jinv, *pair_hm, *gdb, *contra, *lift_scale, *outer_dist;
    const double *fcor, *g_n2, *mass, *inv_area, *weight_ratio, *dtm_own, *dtm_face;
    const float *dtm32_own, *dtm32_face;  // dtm_own, dtm_face truncated to floats
    const double *edge_geo, *bface_geo;
    const int64_t *outer_idx, *nb_face_node, *edge_left, *edge_right, *bface;
    const int32_t* bface_cond;
    const uint8_t* affine;
    // order-N schedule: owned pairs (a, c, dir, pa, pc as int8 x5) and the
    // accumulation (slot, coefficient) of every node
    const int8_t* sched_owned;  // [nn][n1-1][5]
    const int32_t* sched_slot;  // [nn][2(n1-1)]
    const double* sched_coef;   // [nn][2(n1-1)]
    const double* sched_hcoef;  // [nn][2(n1-1)] sched_coef / 2
    const double* pair_coef;    // [nn·(n1-1)][4] per owned slot: both nodes' coefficients, halves
    // An ensemble's concatenated members: each element's member (its
    // StepCtl is ctl[member]) and the members' boundary conditions, which
    // bface_cond indexes. Both null for one mesh (ctl[0], Physics::cond).
    const int32_t* elem_member = nullptr;
    const struct Condition* cond = nullptr;
    // The adjoint's transpose of the bed slope: per node c, for each
    // direction and line position p, g·D[p][pos_c]·w (x and y) of the node i
    // at p, so that ∂(g∇B)_i/∂B_c is a table entry (adjoint handles only)
    const double* gdb_t = nullptr;  // [K·nn][2][n1][2]
    // Per-node tides (BoundaryTides): each boundary face node's slot (−1:
    // not a per-node tide), the conditions' constituents and their slots'
    // constants, mean levels and source depths
    const int32_t* bface_slot = nullptr;  // [B·n1]
    const double *nt_omega = nullptr, *nt_frate = nullptr, *nt_coef = nullptr;
    const double *nt_mean = nullptr, *nt_depth = nullptr;
    // parent series: snapshot times, values (f32) and each slot's parent
    // depth (per-node tides and parents share bface_slot and nt_depth)
    const double* pt_times = nullptr;
    const float* pt_values = nullptr;
    // the nesting relaxation band: its nodes (flat index) and their slots,
    // the parent's series and each slot's weight and depth, the options,
    // and the source of the current stage per node ([3][K·nn], 0 off the
    // band) that the stage kernel adds after Coriolis
    int64_t rx_n = 0;
    const int64_t* rx_node = nullptr;
    const int32_t* rx_slot = nullptr;
    const double *rx_weight = nullptr, *rx_depth = nullptr, *rx_times = nullptr;
    const float* rx_values = nullptr;
    int rx_n_times = 0, rx_cubic = 0, rx_velocity = 0, rx_momentum_only = 0;
    double rx_ref_level = 0.0, rx_max_ratio = 0.0, rx_ramp = 0.0, rx_rate = 0.0, rx_wet = 0.0;
    double* rx_src = nullptr;
    // the weather (GriddedAtmosphere2D): its snapshot times (Unix s) and
    // values ([time][5][K·nn] f32: u, v, ∂p/∂x, ∂p/∂y, p − p_ref), the Unix
    // time of simulation time 0 and the options. With at_source its momentum
    // source goes into rx_src, which the band's kernel then adds to.
    int at_n_times = 0, at_source = 0, at_wind = 0, at_pressure = 0, at_level = 0, at_drag = 0;
    const double* at_times = nullptr;
    const float* at_values = nullptr;
    double at_epoch = 0.0, at_cd = 0.0, at_rho_air = 0.0, at_rho_water = 0.0, at_h_min = 0.0;
    double at_ramp = 0.0;
};

struct Constituent {
    double amplitude, omega, phase, f, f_rate, u_deg, u_rate_deg, v0_deg;
};

struct Condition {
    int kind;
    int elevation_only;
    int n_constituents;
    double wall_h_min;
    double mean, ramp;
    Constituent c[kMaxConstituents];
    // per-node tides (kind 2): the condition's constituents from nt_omega0
    // in DevTables::nt_omega / nt_frate, its slots from nt_slot0, their
    // constants from nt_coef0 in DevTables::nt_coef ([slot][n][6])
    int nt_n, nt_velocity, nt_use_mean, nt_omega0;
    int64_t nt_slot0, nt_coef0;
    double nt_max_ratio;
    // a parent model (kind 3): its snapshot times from pt_time0 in
    // DevTables::pt_times, its slots from pt_slot0, their series from
    // pt_val0 in DevTables::pt_values ([slot][time][3]); the nt_ fields'
    // velocity, transport ratio and slot base serve it too
    int pt_n_times, pt_cubic;
    int64_t pt_time0, pt_val0;
    double pt_reference_level;
    // InverseBarometer: the external η raised by raise_factor times the
    // weather's level at the face node (characteristic kinds)
    int raise;
    double raise_factor;
};

struct Physics {
    int order, n1, nn;
    int formulation;
    double g, h_min;
    double sqrt_g, half_g, two_g;  // √g, g/2 and 2g, computed once on the host
    double subcell_depth, subcell_h_dry;
    int has_bed;
    int has_wet_dry;
    double h_dry, relaxation_time, max_velocity;
    int friction;  // 0 none, 1 uniform, 2 per node
    double g_n2, manning_h_min;
    int has_coriolis, coriolis_field;
    double f0;
    int n_conditions;
    Condition cond[kMaxConditions];
    double x[5], w[5], d[25];  // GLL nodes, weights, D
    int face_node[4][5];
    // launch shapes (dgswe_autotune): the face kernel's threads per block
    // and the stage kernel's shape (0: ⌊128/nn⌋ elements a block, 5 blocks
    // per SM; 1: ⌊64/nn⌋ elements a block, 10 blocks per SM)
    int face_threads = 256;
    int stage_shape = 0;
};

// Subcell bounds x_l, x_r of each GLL subcell (sums of the weights from
// −1, in order) and the reciprocal weights
struct StageExtra {
    double xl[5], xr[5], inv_w[5];
    // a RHS that keeps its subcell mass fluxes: [K][2·n1·(n1 − 1)], NaN in
    // the elements without subcells (null: not kept)
    double* subcell_mass = nullptr;
    // the elements [k_first, k_last) a whole-mesh stage pass covers (a pass
    // in chunks, each chunk's result copied out while the next runs)
    int64_t k_first = 0, k_last = INT64_MAX;
};

// The element step's parameters: the CFL and the positivity bound of a
// wet/dry run (PositivityBound, src/solver/rhs/swe_2d.rs:2165-2212)
struct DtParams {
    double cfl;
    double bound_cfl, max_cfl, max_cfl_subcells, shallow;
    int positivity;
};

struct StageArgs {
    double time, a, b, c, w, keep;
};

// One pass of a multirate coarse step on the device: a finest substep's
// stage over the elements whose stage rate is at least the substep's depth
// (a prefix of the rate-sorted order), with the faces they read, or the end
// of the substeps of the elements whose level is at least it. Each element
// takes its stage from its level (element_stage, src/time/multirate.rs:169-200).
struct LtsPass {
    const int32_t* list = nullptr;    // the pass's elements
    int64_t n = 0;
    const int32_t* edges = nullptr;   // the interior edges they read
    int64_t n_edges = 0;
    const int32_t* bfaces = nullptr;  // and boundary faces
    int64_t n_bfaces = 0;
    const uint8_t* level = nullptr;   // [K]
    const uint8_t* rate = nullptr;    // [K] the stage's rates
    double t = 0.0, dt = 0.0;         // the coarse step
    int finest = 0, substep = 0, depth = 0, last = 0;
    double start = 0.0, input = 0.0, beta = 0.0, c = 0.0;  // the stage's Shu–Osher weights
};

// Step control (device memory): the run's clock, the step's dt and stage
// arguments, and the failure flags. Written by the step kernels of a
// device-driven run or by the host between host-driven calls.
struct StepCtl {
    StageArgs stage[kArgSlots];
    double t, dt, target, t_end;
    double dt_max, dt_min, cfl;
    double dt_min_used, dt_max_used;
    unsigned long long dt_bits;  // atomicMin of the element steps
    long long steps, max_steps, clips;
    int active;     // the current step runs
    int landed;
    int nonfinite;  // the state stopped being finite
    int failure;    // 0, or the dgswe_status that stopped the run
    int always;     // 1: a flag host-driven calls point kernels at
    int scheme_stages;
    double st_start[kMaxStages], st_input[kMaxStages], st_beta[kMaxStages], st_c[kMaxStages];
};

// The adjoint of one stage (adjoint_kernels.cuh): λ arrays per node, or per
// face slot for the face fluxes
struct AdjStage {
    const double *lo_h, *lo_hu, *lo_hv;          // of the stage output (read)
    double *li_h, *li_hu, *li_hv, *li_u, *li_v;  // of the stage input, own element (written)
    double *lb_h, *lb_hu, *lb_hv;                // of the stage's base state (added)
    double *lf_h, *lf_hu, *lf_hv;                // of the face fluxes, per face slot (written)
    double *lx_h, *lx_hu, *lx_hv, *lx_u, *lx_v;  // of the stage input from faces and
                                                 // neighbouring elements (atomic)
    double* lbed;                                // of the bed elevation (atomic)
    double* lgn2;                                // of g·n² per node (added)
    double* ltide;                               // [condition][constituent][amplitude, phase]
    int64_t* sub_list;                           // [3][K] each stage's subcell elements
    unsigned long long* sub_count;               // [3] their numbers
};

}  // namespace dgswe
