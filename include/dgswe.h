/*
 * dgswe.h — C ABI of the GB300 (sm_103a) FP64 2D shallow-water nodal-DG
 * stage: the split-form `WetDry` right-hand side on unstructured quads with
 * its SSP Runge–Kutta stage update, numerical flux, sources and wet/dry
 * limiter.
 *
 * This is the boundary a host in another language binds (a Rust
 * `CaseDevice` implementation through `extern "C"`, Python through ctypes):
 * plain C structs, plain pointers and sizes, `int` status codes, no C++
 * types and no exceptions across it. Every entry point below names the
 * reference interface it replaces (EmilLindfors/dgcom, paths relative to
 * that repository).
 *
 * Conventions
 *  - A solution crosses the ABI as the reference's SoA layout
 *    (`SWESolution2D::data[var][k·n_nodes + i]`,
 *    src/solver/core/system_solution.rs:135-142): three arrays h, hu, hv of
 *    n_elements·(order+1)² doubles, node i = j·(order+1) + a with r fastest
 *    (src/operators/operators_2d.rs:388-412).
 *  - Arrays passed in a `dgswe_form` are copied by `dgswe_create`; the caller
 *    keeps ownership. The handle owns all device memory it uses, except the
 *    one fixed working array of dgswe_compute_rhs_noalloc, which belongs to
 *    the library (64 MiB on every device where its device code is loaded).
 *  - A handle is used by one host thread at a time; each handle has its own
 *    CUDA stream.
 *  - Every function returns DGSWE_OK (0) or a status; the handle keeps a
 *    message (`dgswe_last_error`).
 */
#ifndef DGSWE_H
#define DGSWE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DGSWE_ABI_VERSION 4u

/* ---- status codes ------------------------------------------------------ */
enum dgswe_status {
    DGSWE_OK = 0,
    DGSWE_ERR_INVALID = 1,     /* invalid input: form, sizes, pointers, buffer ids */
    DGSWE_ERR_CUDA = 2,        /* a CUDA call failed (message names it) */
    DGSWE_ERR_NONFINITE = 3,   /* the state is not finite: the run blew up */
    DGSWE_ERR_DT_MIN = 4,      /* time step below the run's dt_min */
    DGSWE_ERR_MAX_STEPS = 5,   /* the run's step limit was reached */
    DGSWE_ERR_STOPPED = 6,     /* the stop flag was set */
    DGSWE_ERR_UNSUPPORTED = 7, /* physics this device does not run */
    DGSWE_ERR_NO_DEVICE = 8    /* no CUDA device (or not the requested one) */
};

/* ---- physics as data (src/physics/device.rs:27-62) ---------------------- */

/* SWEFormulation2D (src/solver/rhs/swe_2d.rs:42-90): the split forms. */
enum dgswe_formulation {
    DGSWE_WET_DRY = 0,
    DGSWE_ENTROPY_STABLE = 1,
    DGSWE_ENTROPY_CONSERVATIVE = 2
};

/* DeviceBoundary2D (src/boundary/boundary_2d.rs:213-231). */
enum dgswe_boundary_kind {
    DGSWE_BC_WALL = 0,           /* Reflective2D: free-slip mirror ghost state */
    DGSWE_BC_CHARACTERISTIC = 1, /* CharacteristicOBC with a uniform harmonic tide */
    DGSWE_BC_NODE_TIDES = 2,     /* CharacteristicOBC with harmonic constants per boundary
                                    node (DeviceExternal2D::Tides, BoundaryTides) */
    DGSWE_BC_PARENT = 3          /* CharacteristicOBC with a parent model's series per
                                    boundary node (DeviceExternal2D::Parent, OceanModelState) */
};

/* ElevationOnly (src/boundary/characteristic.rs:347-355). */
enum dgswe_elevation_only {
    DGSWE_AT_REST = 0,
    DGSWE_INCOMING_WAVE = 1
};

/* DeviceFriction2D: Manning (src/source/swe_2d/friction.rs:195-348) or
 * SpatiallyVaryingManning2D (friction.rs:463-620). */
enum dgswe_friction {
    DGSWE_FRICTION_NONE = 0,
    DGSWE_FRICTION_MANNING = 1,      /* uniform n */
    DGSWE_FRICTION_MANNING_NODES = 2 /* n per node (manning_n_nodes) */
};

/* DragCoefficient (src/source/swe_2d/wind.rs:64-158), by its device code
 * (DragCoefficient::device_code, wind.rs:108-128). */
enum dgswe_drag {
    DGSWE_DRAG_CONSTANT = 0,      /* drag_cd */
    DGSWE_DRAG_LARGE_POND = 1,    /* 1.2e-3 to 11 m/s, then (0.49 + 0.065 min(|U|, 25))·1e-3 */
    DGSWE_DRAG_WU = 2,            /* (0.8 + 0.065 |U|)·1e-3 */
    DGSWE_DRAG_SMITH = 3,         /* (0.61 + 0.063 |U|)·1e-3 */
    DGSWE_DRAG_YELLAND_TAYLOR = 4 /* 1.1e-3 to 6 m/s, then (0.50 + 0.071 |U|)·1e-3 */
};

/* SspScheme (src/time/integrator.rs:226-298). */
enum dgswe_scheme {
    DGSWE_SSP_RK3 = 0,
    DGSWE_SSP_RK43 = 1
};

/* Device arithmetic, FP64 throughout. FAST contracts multiply-adds into FMA,
 * takes square roots and reciprocals within an ulp of the correctly rounded
 * value (a single-precision seed refined in FP64) and the Manning rate's
 * h^(-4/3) from one third-order FP64 step, with no division; EXACT keeps
 * every multiply and add separately rounded, uses IEEE division and square
 * root and follows the reference's cube root
 * (src/source/swe_2d/friction.rs:39-70). */
enum dgswe_numerics {
    DGSWE_NUMERICS_FAST = 0,
    DGSWE_NUMERICS_EXACT = 1
};

/* One tidal constituent of a uniform HarmonicTide
 * (src/boundary/harmonic_tide.rs:124-136) with its nodal drift
 * (src/tides/astronomy.rs:240-270): its term at time t is
 *   (f + f_rate·t)·amplitude·cos(2π t/period + phase + (v0_deg + u_deg + u_rate_deg·t)·π/180).
 * Without nodal corrections f = 1 and the other drift terms are 0. */
typedef struct dgswe_tide_constituent {
    double amplitude;  /* m */
    double period;     /* s */
    double phase;      /* rad, internal phase φ = −G (Greenwich lag) */
    double f;          /* nodal factor at t = 0 */
    double f_rate;     /* its drift per second */
    double u_deg;      /* nodal phase at t = 0 (deg) */
    double u_rate_deg; /* its drift per second (deg/s) */
    double v0_deg;     /* equilibrium argument at t = 0 (deg) */
} dgswe_tide_constituent;

/* The condition of the boundary faces tagged `tag`. */
/* BoundaryTides (src/boundary/tidal_atlas.rs:855-1070) as plain data: an
 * atlas's tide at the forced boundary nodes, in the order of its slots. The
 * external state of slot s at time t is, with f_j = 1 + f_rate_j·t and the
 * constants c = coefficients[s][j] = (C_η, S_η, C_u, S_u, C_v, S_v),
 *   (η, u, v) = (mean_s, 0, 0) + ramp(t)·Σ_j f_j (C cos ω′_j t + S sin ω′_j t)
 * (tide_term, tide_level), with (u, v) only if velocity ≠ 0, scaled by
 * D_source/D_child within [1/r, r] where max_transport_ratio r > 0
 * (tide_state). A boundary face node takes the slot slot_of_node gives its
 * flat mesh node, or else the slot nearest to it. */
typedef struct dgswe_node_tides {
    int32_t n_constituents;
    const double* omega;          /* [n] ω′ = ω + u̇ (rad/s) */
    const double* f_rate;         /* [n] ḟ/f₀ (1/s) */
    int64_t n_slots;
    const double* positions;      /* [n_slots][2] x, y of the forced nodes */
    const double* coefficients;   /* [n_slots][n][6] */
    const double* mean;           /* [n_slots] Z0 (use_mean), or NULL */
    const double* source_depth;   /* [n_slots] the source's still-water depth, or NULL */
    const uint32_t* slot_of_node; /* [n_elements·(N+1)²] or NULL; 0xFFFFFFFF: none */
    int32_t velocity;             /* the tides carry (u, v) */
    int32_t use_mean;             /* add mean (not ramped) */
    double max_transport_ratio;   /* ≤ 0: no transport scaling */
    double ramp_duration;         /* s; ≤ 0: no ramp */
} dgswe_node_tides;

/* OceanModelState's boundary data (src/boundary/ocean_nesting.rs:540-900)
 * as plain data: a parent model's ζ, u, v (f32, as the reference stores
 * them) per slot and snapshot, the snapshots' simulation times. At time t
 * the snapshots' Lagrange weights w (linear between the bracketing two, or
 * cubic through up to four: TimeStencil, src/io/field_series.rs:26-90) give
 *   ζ, u, v = ramp(t)·Σ w_k values_k,  η = ζ + ramp(t)·reference_level
 * (parent_term, parent_state), with (u, v) only if velocity ≠ 0, scaled by
 * D_parent/D_child within [1/r, r] where max_transport_ratio r > 0 and the
 * parent depth is finite. A boundary face node takes the slot slot_of_node
 * gives its flat node, or else the nearest slot marked on_boundary. The
 * run's times must lie within [times[0], times[n_times − 1]]. */
typedef struct dgswe_parent_series {
    int64_t n_slots;
    const double* positions;      /* [n_slots][2] */
    const uint8_t* on_boundary;   /* [n_slots] slots a face node may take by position; NULL: all */
    const uint32_t* slot_of_node; /* [n_elements·(N+1)²] or NULL; 0xFFFFFFFF: none */
    int64_t n_times;
    const double* times;          /* [n_times] strictly increasing (simulation seconds) */
    const float* values;          /* [n_slots][n_times][3] ζ, u, v */
    const double* parent_depth;   /* [n_slots] (NaN: unknown), or NULL */
    int32_t cubic;                /* TimeInterpolation::Cubic, else Linear */
    int32_t velocity;             /* the parent carries (u, v) */
    double reference_level;       /* the datum shift, ramped with ζ */
    double max_transport_ratio;   /* ≤ 0: no transport scaling */
    double ramp_duration;         /* s; ≤ 0: no ramp */
} dgswe_parent_series;

/* NestingRelaxation2D (src/boundary/ocean_nesting.rs:900-1065; the device
 * source DeviceSource2D::NestingRelaxation) as plain data: at every node
 * whose slot (parent->slot_of_node, required) has weight w > 0, the source
 *   γ (q_parent − q),  γ = w·rate
 * with the parent's η, u, v there (as the parent boundary evaluates them;
 * without currents the node's own velocity), zero where the node or the
 * parent is shallower than wet_depth; with momentum_only the depth is kept
 * and the momentum relaxed at the node's depth (relaxation_source). It is
 * added to the RHS after Coriolis. */
typedef struct dgswe_relaxation {
    const dgswe_parent_series* parent;
    const double* weight;   /* [parent->n_slots] band weight; 1 on the boundary */
    double rate;            /* 1/τ (1/s) */
    double wet_depth;       /* m */
    int32_t momentum_only;
} dgswe_relaxation;

/* GriddedAtmosphere2D (src/source/swe_2d/gridded_atmosphere.rs:60-900) as a
 * device holds it: a weather model's snapshots regridded onto the mesh
 * nodes (GriddedAtmosphere2D::regridded), each node's
 *   (u, v, ∂p/∂x, ∂p/∂y, p − p_ref)
 * in f32, the wind in the mesh axes, unramped. At simulation time t the
 * snapshots' linear time weights at epoch_unix + t (TimeStencil,
 * TimeInterpolation::Linear) sum them in turn from zero (add_snapshot), and
 * the ramp is tidal_ramp(t, ramp_duration). As a source term
 * (DeviceSource2D::Atmosphere, when `source` ≠ 0) every node at least h_min
 * deep gets
 *   (S_hu, S_hv) = (τ − h ∇p)/ρ_water,  τ = ρ_air C_d(|U|) |U| U,
 * with U = ramp·(u, v) if `wind` and ∇p = ramp·(∂p/∂x, ∂p/∂y) if `pressure`
 * (atmosphere_source), added to the RHS after Coriolis and the relaxation
 * band. A characteristic boundary with `raise` reads its inverse-barometer
 * level −ramp·(p − p_ref)/(ρ_water g), g = 9.81, at each face node
 * (DeviceLevel::Atmosphere, inverse_barometer_level), 0 unless `level`.
 * The run's times must lie within the snapshots'. */
typedef struct dgswe_atmosphere {
    int64_t n_times;
    const double* times;      /* [n_times] strictly increasing Unix seconds */
    double epoch_unix;        /* Unix time of simulation time 0 (ModelClock) */
    const float* values;      /* [n_times][n_elements·(N+1)²][5] */
    int32_t source;           /* add the momentum source (else only boundaries read it) */
    int32_t wind;             /* the source applies the wind stress */
    int32_t pressure;         /* the source applies the pressure gradient */
    int32_t level;            /* the level is the pressure's (has_level); else 0 */
    int32_t drag;             /* dgswe_drag */
    double drag_cd;           /* DGSWE_DRAG_CONSTANT's C_d */
    double rho_air;           /* kg/m³ */
    double rho_water;         /* kg/m³ */
    double h_min;             /* nodes shallower than this are not forced */
    double ramp_duration;     /* s; ≤ 0: no ramp */
} dgswe_atmosphere;

typedef struct dgswe_boundary {
    int32_t tag;            /* the face tag this condition applies to */
    int32_t kind;           /* dgswe_boundary_kind */
    double wall_h_min;      /* Reflective2D::h_min (wall) */
    int32_t elevation_only; /* dgswe_elevation_only (characteristic) */
    int32_t n_constituents; /* characteristic: harmonic tide terms */
    const dgswe_tide_constituent* constituents;
    double mean_elevation;  /* η₀ (m), not ramped */
    double ramp_duration;   /* s; ≤ 0: no ramp (src/boundary/harmonic_tide.rs:24-32) */
    const dgswe_node_tides* node_tides; /* DGSWE_BC_NODE_TIDES: the tide per node */
    const dgswe_parent_series* parent;  /* DGSWE_BC_PARENT: the parent per node */
    /* InverseBarometer (src/boundary/characteristic.rs:273-340): a
     * characteristic boundary's external η raised by raise_factor times the
     * form's atmosphere's level at each face node (DeviceBoundary2D's
     * `raise`); 0: not raised */
    int32_t raise;
    double raise_factor;
} dgswe_boundary;

/* SWEDeviceForm2D (src/physics/device.rs:27-62) as plain data, with the
 * mesh as Mesh2D::from_quads takes it (src/mesh/core/mesh2d.rs:456-470). */
typedef struct dgswe_form {
    uint32_t abi_version;     /* DGSWE_ABI_VERSION */
    int32_t order;            /* polynomial order N, 1..4 */

    int64_t n_vertices;
    const double* vertices;   /* [n_vertices][2] x, y */
    int64_t n_elements;
    const int64_t* elements;  /* [n_elements][4] vertex indices, counter-clockwise */
    int64_t n_periodic;
    const int64_t* periodic;  /* [n_periodic][4] (element_a, face_a, element_b, face_b) */
    const int32_t* face_tags; /* [n_elements][4] tag of each boundary face; NULL: tag 0 */

    const double* bathymetry; /* [n_elements·(N+1)²] bed elevation B; NULL: flat 0 */

    double g;                 /* gravity (ShallowWater2D::g) */
    double h_min;             /* velocity threshold (ShallowWater2D::h_min) */
    int32_t formulation;      /* dgswe_formulation */
    double subcell_depth;     /* WetDry: subcells where a node is shallower */
    double subcell_h_dry;     /* WetDry: the subcells' dry-node depth */

    int32_t has_wet_dry;      /* WetDryConfig after every stage (wetting_drying.rs:51-175) */
    double wet_dry_h_dry;
    double wet_dry_relaxation_time;
    double wet_dry_max_velocity;
    double positivity_h_dry;  /* h_dry of the positivity-bounded step; ≤ 0: no bound */

    int32_t friction;         /* dgswe_friction */
    double friction_g;        /* the law's g (g·n² per node) */
    double manning_n;         /* uniform n */
    double manning_h_min;     /* depth floor of the law */
    const double* manning_n_nodes; /* [n_elements·(N+1)²] n per node (MANNING_NODES) */

    int32_t has_coriolis;     /* CoriolisSource2D (src/source/swe_2d/coriolis.rs:151-175) */
    double coriolis_f0;
    double coriolis_beta;
    double coriolis_y0;

    int32_t n_boundaries;
    const dgswe_boundary* boundaries;

    int32_t numerics;         /* dgswe_numerics */

    /* Local time stepping (SWEDeviceForm2D::line_local_depth,
     * src/physics/device.rs:62-66): elements whose every node is deeper than
     * line_local_depth + 1 m read only their GLL lines in a stage, so the
     * stage rates spread node by node; has_line_local = 0: no element does
     * (the rates spread one face per stage). */
    int32_t has_line_local;
    double line_local_depth;

    /* A nesting relaxation band towards a parent model, or NULL */
    const dgswe_relaxation* relaxation;

    /* A weather model's wind and air pressure (the source term and the
     * boundaries' inverse-barometer level), or NULL */
    const dgswe_atmosphere* atmosphere;
} dgswe_form;

/* ---- stages and runs ---------------------------------------------------- */

/* Device solution buffers: 0 is the state, 1.. stage values. */
#define DGSWE_STATE 0
#define DGSWE_N_BUFFERS 6

/* One stage pass over every element (ElementStage,
 * src/time/multirate.rs:169-200):
 *   out = a·base + b·input + c·F(input)   (a term only where its weight ≠ 0),
 * then the point-implicit damping with weight c, then either
 *   acc ← w·out + keep·acc   (accumulate ≠ 0; the acc term only if keep ≠ 0)
 * or the post-processing (wet/dry correction) of out. */
typedef struct dgswe_stage_plan {
    int32_t base;       /* buffer id of the step start */
    int32_t input;      /* buffer id of the RHS argument */
    int32_t out;        /* buffer id written */
    int32_t acc;        /* buffer id summed into (accumulate ≠ 0) */
    double time;        /* stage time (boundary data) */
    double a, b, c;
    int32_t accumulate;
    double w, keep;
} dgswe_stage_plan;

/* DeviceRun (src/case/run.rs:273-289) as plain data. */
typedef struct dgswe_run_config {
    int32_t scheme;            /* dgswe_scheme */
    double cfl;
    double t_start, t_end;     /* span (s) */
    double interval;           /* callback interval (s); ≤ 0: every step */
    double dt_max;             /* ≤ 0: none */
    double dt_min;             /* ≤ 0: none */
    int64_t max_steps;         /* ≤ 0: none */
    const volatile int32_t* stop; /* nonzero stops the run at its next step; NULL: none */
    int32_t levels;            /* local time stepping: levels below the coarsest
                                  (DeviceRun::levels, ≤ DGSWE_MAX_LEVELS); 0: global steps */
} dgswe_run_config;

#define DGSWE_MAX_LEVELS 8

/* DeviceRunReport (src/case/run.rs:292-300) with its SimulationResult. */
typedef struct dgswe_report {
    int32_t success;
    double final_time;
    int64_t n_steps;
    double dt_min_used;
    double dt_max_used;
    double wall_time;
    int64_t negative_depth_clips;
    char message[256];
    char device[128];
} dgswe_report;

/* The run's callback: the state on the host at time t (n values per field).
 * The arrays are valid during the call only. */
typedef void (*dgswe_callback)(void* user, double t, const double* h,
                               const double* hu, const double* hv, int64_t n);

/* Per-kernel timing of device-driven steps (dgswe_profile_steps). */
typedef struct dgswe_profile {
    int64_t steps;          /* steps timed */
    double total_ms;        /* device time from the first launch to the last */
    double face_ms;         /* summed durations of the face kernels */
    double stage_ms;        /* of the element stage kernels */
    double dt_ms;           /* of the element time-step kernels */
    double control_ms;      /* of the one-thread clock kernels */
    int64_t face_launches, stage_launches, dt_launches, control_launches;
    double t_final;         /* model time after the steps */
} dgswe_profile;

/* What dgswe_check_form found in a form (no device involved). */
typedef struct dgswe_form_info {
    int64_t n_elements;
    int64_t n_interior_edges;  /* each counted once */
    int64_t n_periodic_edges;  /* interior edges whose faces do not share vertices */
    int64_t n_boundary_faces;
    int64_t n_affine;          /* parallelogram elements */
    double min_jacobian;       /* smallest J at any node */
    double area;               /* Σ of the element areas (Σ w_i J_i) */
    double table_checksum;     /* Σ of every static device table value */
} dgswe_form_info;

typedef struct dgswe_handle dgswe_handle;

/* ---- entry points ------------------------------------------------------- */

/* Validates `form` and builds its connectivity, geometry and static tables
 * on the host only, without touching a device, into `info` (may be NULL);
 * `message` (may be NULL) receives the reason of a failure. The device
 * path's counterpart of `dgcom check` (src/case/cli.rs:126-134). */
int dgswe_check_form(const dgswe_form* form, dgswe_form_info* info, char* message,
                     size_t message_size);

/* ABI version of the library (DGSWE_ABI_VERSION it was built with). */
uint32_t dgswe_abi_version(void);

/* Text of a status code. */
const char* dgswe_status_string(int status);

/* The device's physics from `form` on CUDA device `device`: the handle of
 * a run. Replaces GpuSWE2D::from_form (gpu/src/swe2d.rs:3360) behind
 * CaseDevice::run_2d (src/case/run.rs:179-192); refuses physics without a
 * device form as SWEPhysics2D::device_form does (src/physics/device.rs:79-142). */
int dgswe_create(const dgswe_form* form, int device, dgswe_handle** out);

/* Frees the handle and its device memory. NULL is ignored. */
void dgswe_destroy(dgswe_handle* handle);

/* The message of the handle's last failure ("" if none). */
const char* dgswe_last_error(const dgswe_handle* handle);

/* Values per field of a solution: n_elements·(N+1)². */
int64_t dgswe_n_values(const dgswe_handle* handle);

/* Copies a solution into / out of a device buffer (DGSWE_STATE: the state).
 * Replaces DeviceState::upload / download (gpu/src/case.rs:36-70). */
int dgswe_upload(dgswe_handle* handle, int32_t buffer, const double* h,
                 const double* hu, const double* hv, int64_t n);
int dgswe_download(dgswe_handle* handle, int32_t buffer, double* h, double* hu,
                   double* hv, int64_t n);

/* The RHS of buffer `input` at `time` into out_* (host): PhysicsModule::
 * compute_rhs_into (src/physics/builder.rs:425-434) →
 * compute_rhs_swe_2d_parallel_into (src/solver/rhs/swe_2d.rs:1478-1488). */
int dgswe_compute_rhs(dgswe_handle* handle, int32_t input, double time,
                      double* out_h, double* out_hu, double* out_hv, int64_t n);

/* compute_rhs_swe_2d_mass_fluxes_into (src/solver/rhs/swe_2d.rs:1042-1075;
 * BarotropicPhysics::compute_rhs_mass_fluxes_into, src/physics/builder.rs:
 * 785-817): dgswe_compute_rhs that also writes the numerical mass flux of
 * every element face node, face_mass[(k·4 + face)·(N+1) + fi] = F*_h along
 * the element's outward unit normal (n_face = n_elements·4·(N+1)), and of
 * every subcell interface of the elements that take the subcells,
 * subcell_mass[k·2(N+1)N + (dir·(N+1) + line)·N + a] (the interface between
 * nodes a and a + 1 of the line, metric-scaled; n_sub = n_elements·2(N+1)N),
 * NaN in every other element. Either output may be NULL. */
int dgswe_compute_rhs_mass_fluxes(dgswe_handle* handle, int32_t input, double time,
                                  double* out_h, double* out_hu, double* out_hv, int64_t n,
                                  double* face_mass, int64_t n_face, double* subcell_mass,
                                  int64_t n_sub);

/* One stage pass over every element: LocalTimeStepping::stage_where
 * (src/physics/builder.rs:652-737). */
int dgswe_stage(dgswe_handle* handle, const dgswe_stage_plan* plan);

/* End of a substep over every element: state ← acc, then the post-processing
 * (LocalTimeStepping::finish_where, src/physics/builder.rs:739-782). */
int dgswe_finish(dgswe_handle* handle, int32_t acc);

/* Point-implicit damping of a stage value (PhysicsModule::implicit_damping,
 * src/physics/builder.rs:501-504; apply_implicit_damping_2d,
 * src/solver/algorithms/wetting_drying.rs:376-389): buffer `stage`, formed
 * from an RHS at buffer `from` with weight dt on it, damped over dt by the
 * bottom friction and the wet/dry thin-layer relaxation with the rates
 * frozen at `from` (damp_node at every node); the stage's node velocities
 * follow. Without friction or a wet/dry correction nothing changes. */
int dgswe_implicit_damping(dgswe_handle* handle, int32_t stage, int32_t from, double dt);

/* The wet/dry correction of a buffer in place (PhysicsModule::post_process,
 * src/physics/builder.rs:488-499): per element, the positivity limiter where
 * a node is below h_dry, then correct_node at every node; clipped elements
 * add to dgswe_negative_depth_clips. */
int dgswe_post_process(dgswe_handle* handle, int32_t buffer);

/* Every element's stable step at `cfl` for `scheme` (element_dt_swe_2d,
 * src/solver/rhs/swe_2d.rs:2018-2043, with the positivity bound of a
 * wet/dry run) into dt_elements (n_elements values; may be NULL), and their
 * minimum (min_element_dt_swe_2d, swe_2d.rs:2045-2068) into dt_min (may be
 * NULL). Reads the state buffer. */
int dgswe_element_dt(dgswe_handle* handle, double cfl, int32_t scheme,
                     double* dt_elements, double* dt_min);

/* One global SSP step of dt from t on the state, the stages fused per
 * element (MultirateStepper::step with one level,
 * src/time/multirate.rs:1285-1315). */
int dgswe_step(dgswe_handle* handle, int32_t scheme, double t, double dt);

/* One global SSP step of a state the caller holds on the host, as the
 * reference's CPU solver steps its SWESolution2D in place
 * (SSPRK3::step_with_relaxation, src/time/integrator.rs:472-500, with the
 * step of compute_dt_ssp): uploads h, hu, hv (n = dgswe_n_values each),
 * takes the positivity-bounded CFL step at `cfl` on the device (capped at
 * dt_max when it is > 0; it lands on the end of any forcing series'
 * snapshots rather than leave them), advances the state from t and writes
 * it back into the same arrays, and the step taken into dt_out (may be
 * NULL). The upload runs in element chunks, and as each chunk arrives the
 * dt pass and the first stage's face fluxes run for what reads nothing
 * later; the last stage runs in element chunks, each copied back while the
 * next one computes. Page-locked host arrays give the full overlap. The
 * handle's first call builds the chunks' ready lists (host work and device
 * memory in proportion to the mesh) and its copy stream. The
 * result is that of dgswe_upload, dgswe_element_dt,
 * dgswe_step and dgswe_download, bit for bit; the state buffer holds it
 * too. DGSWE_ERR_NONFINITE if the new state is not finite. */
int dgswe_step_host(dgswe_handle* handle, int32_t scheme, double t, double cfl, double dt_max,
                    double* h, double* hu, double* hv, int64_t n, double* dt_out);

/* Simulation::run_with_callback (src/simulation/runner.rs:264-500) on the
 * state: dt from the positivity-bounded element steps, capped by dt_max,
 * landing on every callback time and the end; the callback gets the state
 * on the host at the start, every interval and the end. */
int dgswe_run(dgswe_handle* handle, const dgswe_run_config* run,
              dgswe_callback callback, void* user, dgswe_report* report);

/* Elements emptied because their mean depth went negative, summed over
 * every stage so far (SWEPhysics2D::negative_depth_clips,
 * src/physics/builder.rs:204). */
int64_t dgswe_negative_depth_clips(const dgswe_handle* handle);

/* ---- local time stepping -------------------------------------------------
 * dgswe_run with run->levels > 0 takes multirate coarse steps (Multirate on
 * the scheme, src/time/multirate.rs): every element steps at dt/2^level of
 * the coarse step dt, levels from the element steps every coarse step (the
 * host plans, as the reference's MultirateStepper does; the device runs each
 * finest substep's stage passes over prefixes of level-sorted element and
 * face lists). One level is the global scheme, bit for bit. */

/* The LocalTimeStepping passes, for a host that runs its own multirate
 * stepper (the reference's Simulation with Multirate drives its device
 * backend this way, gpu/src/swe2d.rs:4403-4660):
 *   begin_coarse_step  LocalTimeStepping::begin_coarse_step: the coarse
 *                      step's levels [n_elements] and every stage's rates
 *                      [n_stages][n_elements], each between its element's
 *                      level and the finest level; the library orders the
 *                      passes' elements and faces by them;
 *   stage_where        LocalTimeStepping::stage_where with its StagePlan
 *                      (src/time/multirate.rs:207-260): the elements whose
 *                      rate of `stage` is at least `depth`, each with its
 *                      element_stage;
 *   finish_where       LocalTimeStepping::finish_where: state ← acc and the
 *                      post-processing on the elements whose level is at
 *                      least `depth`;
 *   depth_flags        per element, whether every node of `buffer` is
 *                      deeper than d0, d1, d2 (bits 0, 1, 2): line_local's
 *                      and coarse_step_bound's tests. */
typedef struct dgswe_multirate_stage {
    double t, dt;                    /* the coarse step (StagePlan::step) */
    int32_t finest, substep, depth;  /* 2^finest finest substeps; this one and its depth */
    int32_t stage, last;             /* the stage (0-based); whether it is the scheme's last */
    double start, input, beta, c;    /* its Shu–Osher weights (ShuOsherStage) */
    int32_t base, input_buffer, out, acc; /* buffer ids: the substep start, the RHS argument,
                                             the stage value, the substep sum (last stage) */
} dgswe_multirate_stage;

int dgswe_begin_coarse_step(dgswe_handle* handle, int32_t n_stages, const uint8_t* levels,
                            const uint8_t* rates);
int dgswe_stage_where(dgswe_handle* handle, const dgswe_multirate_stage* plan);
int dgswe_finish_where(dgswe_handle* handle, int32_t acc, int32_t depth);
int dgswe_depth_flags(dgswe_handle* handle, int32_t buffer, double d0, double d1, double d2,
                      uint8_t* flags);

/* MultirateStats (src/time/multirate.rs:785-860) of the handle's last run */
typedef struct dgswe_multirate_stats {
    int64_t steps;                /* coarse steps */
    int64_t element_evaluations;  /* element RHS evaluations */
    int64_t global_evaluations;   /* those of global steps at the finest level */
    int32_t finest_level;         /* largest level used */
    double model_seconds;
    double ideal_evaluations;     /* every element at its own stable step */
    double level_evaluations;     /* every stage at the element's level */
    int64_t line_local_elements;  /* summed over the coarse steps */
    int64_t plans;                /* coarse steps whose levels or rates changed */
    double plan_seconds;          /* host time planning them (and copying the plans) */
    double device_seconds;        /* device time of the coarse steps' passes */
} dgswe_multirate_stats;

int dgswe_multirate_stats_get(const dgswe_handle* handle, dgswe_multirate_stats* out);

/* The level planner alone, on the host (no device): MultirateStepper's
 * level assignment (assign_levels, the landing fit, the jump limit, the
 * stage rates and the kept plan) on a form's mesh, for the scheme's stages
 * and up to max_levels levels. */
typedef struct dgswe_planner dgswe_planner;

typedef struct dgswe_plan_result {
    double dt;                 /* the coarse step, fitted to the landing */
    double stable_step;        /* the step the elements (and the cap) allow */
    int32_t finest;            /* finest level */
    int64_t evaluations;       /* element RHS evaluations per coarse step */
    int64_t level_evaluations; /* the same with every stage at the element's level */
    double inverse_dt_sum;     /* Σ 1/element dt over the finite ones */
} dgswe_plan_result;

int dgswe_planner_create(const dgswe_form* form, int32_t max_levels, int32_t scheme,
                         dgswe_planner** out);
void dgswe_planner_destroy(dgswe_planner* planner);
/* element_dt [n_elements] (∞: unlimited); line_local [n_elements] flags or
 * NULL (no line-local elements: the rates spread one face per stage);
 * dt_cap, landing ≤ 0: none. levels [n_elements], rates
 * [n_stages][n_elements] and order [(n_stages + 1)][n_elements] (each key's
 * elements, largest key first: the device's pass order; key j < n_stages is
 * stage j's rate, the last the level) may be NULL. */
int dgswe_planner_assign(dgswe_planner* planner, const double* element_dt,
                         const uint8_t* line_local, double dt_cap, double landing,
                         dgswe_plan_result* result, uint8_t* levels, uint8_t* rates,
                         int32_t* order);
/* The planner's pieces on given levels [n_elements]: with limit ≠ 0 the
 * jump limit first (face neighbours' levels differ by at most one, the
 * coarser side refined; `levels` is updated), then every stage's rates into
 * rates [n_stages][n_elements] (may be NULL), node by node over the GLL
 * lines where line_local marks an element (NULL: one face per stage). */
int dgswe_planner_spread(dgswe_planner* planner, uint8_t* levels, int32_t limit,
                         const uint8_t* line_local, uint8_t* rates);

/* Launch shapes of a handle's kernels, chosen by timing them on its own
 * mesh and state (an autotuner): the face kernel's threads per
 * block (64, 128 or 256) and the stage kernel's elements per block
 * (shape 0: ⌊128/(N+1)²⌋ at 5 blocks per SM; 1: ⌊64/(N+1)²⌋ at 10; 2:
 * ⌊128/(N+1)²⌋ at 6). The shapes change no result (tests compare them bit
 * for bit). No reference counterpart. */
typedef struct dgswe_tuning {
    int32_t face_threads;      /* chosen */
    int32_t stage_threads;     /* chosen: elements per block × (N+1)² */
    double face_ms[3];         /* one face pass at 64, 128, 256 threads */
    double stage_ms[3];        /* one RHS stage at the three shapes */
} dgswe_tuning;

/* Times `repeats` face passes and RHS stages of buffer 0 at each shape
 * (CUDA events on the handle's stream; the state is not changed), keeps the
 * fastest shapes for every later launch and returns them. force_face /
 * force_stage ≥ 0 set a shape without timing (threads; shape 0, 1 or 2). */
int dgswe_autotune(dgswe_handle* handle, int32_t repeats, int32_t force_face,
                   int32_t force_stage, dgswe_tuning* out);

/* Times n_steps device-driven steps of the state from run->t_start (the
 * run's scheme, cfl and dt_max; no end time), every kernel bracketed by CUDA
 * events on the handle's stream, into `out`. The GPU counterpart of the
 * reference's DG_PROFILE scope timers (src/profiling.rs:1-90); advances the
 * state like dgswe_run. */
int dgswe_profile_steps(dgswe_handle* handle, const dgswe_run_config* run,
                        int64_t n_steps, dgswe_profile* out);

/* The RHS of a state already on the device, without allocating anything.
 * No counterpart in the reference: it exists for callers that cannot call
 * cudaMalloc while they step — a host that hands the whole device budget to
 * its own pool up front, or a hot loop where an allocation would synchronise
 * the device or fail halfway through a run. h/hu/hv and out_* are device
 * pointers of n = dgswe_n_values() doubles each, owned by the caller; the
 * result is dgswe_compute_rhs's, bit for bit, and `time` must lie within the
 * snapshots of any forcing series the form holds, as there. Its working
 * memory (the face fluxes and the node velocities, n_elements·(12(N+1) +
 * 2(N+1)²) doubles) lives in one 64 MiB array inside the library, so meshes
 * up to ≈ 104,000 elements at N = 3 (≈ 155,000 at N = 2) fit; larger ones
 * are refused with DGSWE_ERR_INVALID. Every GPU on which the library's
 * device code is loaded holds that array until the process exits. Every
 * call shares it: calls that overlap on the GPU (other streams, other
 * handles, other host threads) race. Each call writes every value it reads,
 * so nothing needs clearing between calls.
 * The call runs on the handle's own stream and does not wait for other
 * streams: finish (or order by an event) the work that writes h/hu/hv
 * before calling. It returns when the RHS is complete. A handle's first
 * call looks up the array's device address (cudaGetSymbolAddress, with the
 * handle's device current) and keeps it on the handle: make that first call
 * before any stream capture. */
int dgswe_compute_rhs_noalloc(dgswe_handle* handle, const double* h, const double* hu,
                              const double* hv, double time, double* out_h, double* out_hu,
                              double* out_hv, int64_t n);

/* ---------------------------------------------------------------------------
 * The Standard-kernel helpers of the reference's RHS bench
 * (benches/rhs_swe_2d_bench.rs), on the device.
 *
 * Each applies one helper of src/solver/simd/kernels.rs to n_elements
 * elements at once: element e's vectors start at e·n_nodes (e·n_face_nodes
 * for face data) in device arrays of the caller's; a matrix (D, LIFT) is one
 * row-major device array shared by all elements. Every product and sum is
 * rounded on its own, in the helper's order, so each element's result is
 * the reference's helper's bit for bit (its scalar and SIMD forms agree).
 * `device` is the GPU the pointers live on. Each call runs on the default
 * stream and returns when it is complete. Errors: DGSWE_ERR_INVALID (NULL
 * pointers, sizes), DGSWE_ERR_NO_DEVICE, DGSWE_ERR_CUDA; the text of the
 * calling thread's last failure is dgswe_helpers_last_error(). */

/* out = D·flux per element for h, hu, hv (n_nodes ≤ 64). Replaces
 * apply_diff_matrix / apply_diff_matrix_scalar
 * (src/solver/simd/kernels.rs:31-61, 315-359). */
int dgswe_apply_diff_matrix(int device, const double* d, const double* flux_h,
                            const double* flux_hu, const double* flux_hv, double* out_h,
                            double* out_hu, double* out_hv, int64_t n_nodes, int64_t n_elements);

/* out += scale[e]·LIFT·flux_diff per element (LIFT n_nodes × n_face_nodes).
 * Replaces apply_lift / apply_lift_scalar (src/solver/simd/kernels.rs:74-104,
 * 361-389), whose one `scale` becomes one per element. */
int dgswe_apply_lift(int device, const double* lift, const double* flux_diff_h,
                     const double* flux_diff_hu, const double* flux_diff_hv, double* out_h,
                     double* out_hu, double* out_hv, int64_t n_nodes, int64_t n_face_nodes,
                     const double* scale, int64_t n_elements);

/* out_hu += f·hv, out_hv += −f·hu over n_values nodes. Replaces
 * coriolis_source / coriolis_source_scalar (src/solver/simd/kernels.rs:
 * 117-131, 391-403). */
int dgswe_coriolis_source(int device, const double* hu, const double* hv, double* out_hu,
                          double* out_hv, double f, int64_t n_values);

/* out = −(dfx_dr·rx + dfx_ds·sx + dfy_dr·ry + dfy_ds·sy) per element, with
 * `derivatives` the reference's twelve inputs in its argument order
 * (dfx_dr_h, dfx_dr_hu, dfx_dr_hv, dfx_ds_h, …, dfy_ds_hv) and `metric`
 * the element's (rx, sx, ry, sy), four per element. Replaces
 * combine_derivatives / combine_derivatives_scalar
 * (src/solver/simd/kernels.rs:184-224, 405-440). */
int dgswe_combine_derivatives(int device, const double* const derivatives[12], double* out_h,
                              double* out_hu, double* out_hv, const double* metric,
                              int64_t n_nodes, int64_t n_elements);

/* The text of the calling thread's last helper failure ("" if none). */
const char* dgswe_helpers_last_error(void);

/* ---------------------------------------------------------------------------
 * Ensembles: independent runs advanced together.
 *
 * No counterpart in the reference, which runs one case per
 * CaseDevice::run_2d call (src/case/run.rs:179-212); a member is what one
 * such call would run. Members may differ in mesh (size and shape), order,
 * bathymetry, Manning coefficient (uniform or per node) and boundary data
 * (tide constituents, walls); every other physics option must equal member
 * 0's, or create fails with DGSWE_ERR_INVALID. Each member takes its own
 * time step from its own CFL limit. All members' device data lives in one
 * set of tables per order, and one CUDA graph advances every member by one
 * step. A member's result equals a dgswe_run of that member alone over the
 * same steps, bit for bit. */
typedef struct dgswe_ensemble dgswe_ensemble;

/* Copies n_members forms (the same rules as dgswe_create for each) to the
 * device. *out is set even on failure, for dgswe_ensemble_last_error;
 * destroy it either way. */
int dgswe_ensemble_create(const dgswe_form* forms, int n_members, int device,
                          dgswe_ensemble** out);
void dgswe_ensemble_destroy(dgswe_ensemble* ensemble);
const char* dgswe_ensemble_last_error(const dgswe_ensemble* ensemble);
int dgswe_ensemble_n_members(const dgswe_ensemble* ensemble);
/* Values per variable of one member: its n_elements·(order+1)² */
int64_t dgswe_ensemble_n_values(const dgswe_ensemble* ensemble, int member);
/* One member's state, host or device pointers, n = dgswe_ensemble_n_values */
int dgswe_ensemble_upload(dgswe_ensemble* ensemble, int member, const double* h,
                          const double* hu, const double* hv, int64_t n);
int dgswe_ensemble_download(dgswe_ensemble* ensemble, int member, double* h, double* hu,
                            double* hv, int64_t n);
/* Advances every member by n_steps SSP steps (run->scheme, run->cfl,
 * run->dt_max, run->dt_min; t_end, interval and stop are not used), all
 * from run->t_start, or each from its own time (0 before its first run)
 * when run->t_start is NaN: two runs of n steps with the second from NaN
 * equal one run of 2n. Negative-depth clips add up over runs. reports (n_members entries) and profile may be NULL;
 * profile->total_ms is the device time of all the steps. A member whose
 * step fails (non-finite state, dt below dt_min) stops there and the others
 * go on; the call then returns that member's status. */
int dgswe_ensemble_run(dgswe_ensemble* ensemble, const dgswe_run_config* run, int64_t n_steps,
                       dgswe_report* reports, dgswe_profile* profile);

/* ---------------------------------------------------------------------------
 * The discrete adjoint of a WetDry SSP-RK3 run.
 *
 * No counterpart in the reference, which has no adjoint. The functional is
 * a station misfit, J = Σ_{n=1..N} Σ_s (η_s(q_n) − η_obs[n][s])², with
 * η = h + B interpolated at station s inside its element and q_n the state
 * after step n. The reverse sweep gives ∂J/∂ of the initial state, of the
 * bed elevation B per node, of Manning's n per node (per element: sum an
 * element's nodes) and of each boundary condition's tide constituents
 * (amplitude and phase). These are exact derivatives of the steps the
 * forward sweep took: its time steps and every branch (wet/dry tests, the
 * limiter, the HLL wave speeds) stay fixed. Where the bed of coincident
 * nodes of two elements is equal, the face bed max(B⁻, B⁺) has a kink; the
 * derivative given is exact for perturbations that keep coincident nodes
 * equal (a continuous bed). Step-start states are stored in HBM within
 * memory_budget; when all N do not fit, a two-level checkpointing stores
 * every s-th one and replays each segment from it: keeping each step's
 * stage inputs with their node velocities and the kept values when the
 * budget holds 10 states a step of the segment (full segments), else its
 * step-start states only. */
#define DGSWE_MAX_CONSTITUENTS 8

typedef struct dgswe_adjoint dgswe_adjoint;

typedef struct dgswe_adjoint_config {
    int32_t scheme;           /* DGSWE_SSP_RK3 */
    double cfl;               /* the forward's CFL when no time steps are given */
    double t_start;
    int64_t n_steps;          /* N */
    int32_t n_stations;
    const double* stations;   /* [n_stations][2] x, y; copied */
    double memory_budget;     /* bytes of HBM for stored states; ≤ 0: free memory − 2 GiB */
    const int32_t* station_member; /* [n_stations] each station's member (an ensemble's
                                      adjoint); NULL: member 0 */
    int64_t checkpoint_every;  /* checkpoint interval s (steps); ≤ 0: every step if the
                                  budget holds them all, else the interval that needs
                                  the least memory */
} dgswe_adjoint_config;

typedef struct dgswe_adjoint_stats {
    double J;                 /* of the last forward sweep */
    double forward_ms;        /* device time of the forward sweep */
    double reverse_ms;        /* of the reverse sweep */
    double forward_wall_s, reverse_wall_s;
    int64_t stride;           /* checkpoint interval; 1: every step-start state stored */
    int32_t full_segments;    /* the replay keeps every step's reverse data: each step is
                                 computed once in the reverse sweep, not twice */
    int64_t recomputed_steps; /* forward steps the reverse sweep recomputed */
    int64_t stored_states;
    double stored_bytes;
} dgswe_adjoint_stats;

/* A form (the WetDry formulation) and the run's shape; the stations are
 * located in the mesh here (DGSWE_ERR_INVALID if one is outside). *out is
 * set even on failure; destroy it either way. */
int dgswe_adjoint_create(const dgswe_form* form, int device, const dgswe_adjoint_config* config,
                         dgswe_adjoint** out);
/* The adjoint of an ensemble run (dgswe_ensemble_create's members, all of
 * one order) in one batched sweep: each member takes its own CFL steps (or
 * given ones) and its stations (config->station_member); J is the sum of
 * the members' misfits. The state, the initial state and the per-node
 * gradients are the members' arrays concatenated (member m's first value
 * at dgswe_adjoint_member_offset(m)); time steps are [N][n_members];
 * tide gradients are per boundary condition, the members' conditions
 * concatenated in member order. Each member's gradients equal those of its
 * own single-mesh adjoint. */
int dgswe_adjoint_create_ensemble(const dgswe_form* forms, int n_members, int device,
                                  const dgswe_adjoint_config* config, dgswe_adjoint** out);
/* Member m's first value in the concatenated arrays (−1: no such member) */
int64_t dgswe_adjoint_member_offset(const dgswe_adjoint* adjoint, int member);
/* Each member's part of J from the last forward sweep [n_members] */
int dgswe_adjoint_member_misfit(const dgswe_adjoint* adjoint, double* J);
void dgswe_adjoint_destroy(dgswe_adjoint* adjoint);
const char* dgswe_adjoint_last_error(const dgswe_adjoint* adjoint);
int64_t dgswe_adjoint_n_values(const dgswe_adjoint* adjoint);
/* Each station's element and its (order+1)² interpolation weights */
int dgswe_adjoint_stations(const dgswe_adjoint* adjoint, int64_t* element, double* weights);
/* The forward sweep from (h0, hu0, hv0): N steps of SSP-RK3 with the given
 * time steps dts[N] ([N][n_members] for an ensemble), or (dts NULL) with
 * the CFL steps, written to dts_out.
 * eta_obs [N][n_stations] (NULL: zero) enters J; eta_out gets the
 * stations' η after each step. Any output may be NULL. */
int dgswe_adjoint_forward(dgswe_adjoint* adjoint, const double* h0, const double* hu0,
                          const double* hv0, const double* dts, const double* eta_obs,
                          double* eta_out, double* dts_out, double* J);
/* The reverse sweep of the last forward sweep: ∂J/∂h0, ∂J/∂hu0, ∂J/∂hv0,
 * ∂J/∂B and ∂J/∂n per node (n_values each), and ∂J/∂(amplitude, phase)
 * as [n_boundaries][DGSWE_MAX_CONSTITUENTS][2]. Any output may be NULL;
 * with grad_bed NULL the sweep does not form the bed's λ at all, which
 * saves its arithmetic and atomics. */
int dgswe_adjoint_reverse(dgswe_adjoint* adjoint, double* grad_h0, double* grad_hu0,
                          double* grad_hv0, double* grad_bed, double* grad_manning,
                          double* grad_tide);
/* New parameter values for the next forward sweep, in the gradients'
 * layout: Manning's n per node [n_values] (the form's friction must be
 * DGSWE_FRICTION_MANNING_NODES, or any Manning law in an ensemble) and the
 * tide constituents' (amplitude, phase) [n_conditions][DGSWE_MAX_CONSTITUENTS][2]
 * (the phase as dgswe_tide_constituent.phase; entries beyond a
 * condition's n_constituents are ignored). Either may be NULL: unchanged.
 * A calibration loop calls forward, reverse and this in turn. */
int dgswe_adjoint_set_parameters(dgswe_adjoint* adjoint, const double* manning_n,
                                 const double* tide);
int dgswe_adjoint_get_stats(const dgswe_adjoint* adjoint, dgswe_adjoint_stats* out);

#ifdef __cplusplus
}
#endif

#endif /* DGSWE_H */
