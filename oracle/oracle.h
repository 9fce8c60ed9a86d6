/*
 * Oracle — test infrastructure only. The C entry points of the CPU
 * restatement of the reference's 2D split-form shallow-water path
 * (EmilLindfors/dgcom), mirroring the CUDA library's ABI (include/dgswe.h)
 * one for one so that the tests call both the same way. Only the tests, the
 * smoke check and the bench's CPU-baseline leg load it.
 */
#ifndef DGSWE_ORACLE_H
#define DGSWE_ORACLE_H

#include "../include/dgswe.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_handle oracle_handle;

int oracle_set_threads(int n);
int oracle_create(const dgswe_form* form, int device, oracle_handle** out);
void oracle_destroy(oracle_handle* h);
int64_t oracle_n_values(const oracle_handle* h);
int oracle_upload(oracle_handle* h, int32_t buffer, const double* hh, const double* hu,
                  const double* hv, int64_t n);
int oracle_download(oracle_handle* h, int32_t buffer, double* hh, double* hu, double* hv, int64_t n);
int oracle_compute_rhs(oracle_handle* h, int32_t input, double time, double* out_h, double* out_hu,
                       double* out_hv, int64_t n);
int oracle_compute_rhs_mass_fluxes(oracle_handle* h, int32_t input, double time, double* oh,
                                   double* ohu, double* ohv, int64_t n, double* face_mass,
                                   int64_t n_face, double* subcell_mass, int64_t n_sub);
int oracle_subcell_divergence(oracle_handle* h, int64_t k, const double* hu, const double* hv,
                              const double* interfaces, const double* face, double* div);
int oracle_stage(oracle_handle* h, const dgswe_stage_plan* plan);
int oracle_finish(oracle_handle* h, int32_t acc);
int oracle_implicit_damping(oracle_handle* h, int32_t stage, int32_t from, double dt);
int oracle_post_process(oracle_handle* h, int32_t buffer);
int oracle_element_dt(oracle_handle* h, double cfl, int32_t scheme, double* dt_elements,
                      double* dt_min);
int oracle_step(oracle_handle* h, int32_t scheme, double t, double dt);
int oracle_run(oracle_handle* h, const dgswe_run_config* run, dgswe_callback cb, void* user,
               dgswe_report* report);
int64_t oracle_negative_depth_clips(const oracle_handle* h);
/* MultirateStats of the last run with local time stepping (run->levels > 0) */
/* TimeStencil::new: the snapshots and weights at t (returns how many; 0: outside) */
int oracle_time_stencil(const double* times, int64_t n, double t, int cubic, int64_t* idx,
                        double* w);
int oracle_multirate_stats_get(const oracle_handle* h, dgswe_multirate_stats* out);

/* pointwise functions for the known-answer tests */
double oracle_manning_cbrt(double x);
double oracle_tidal_ramp(double t, double duration);
double oracle_hypot(double x, double y);
double oracle_drag_coefficient(int kind, double cd, double speed);
void oracle_atmosphere_source(double h, double u, double v, double px, double py, int drag,
                              double cd, double rho_air, double rho_water, double h_min,
                              double out[2]);
double oracle_inverse_barometer_level(double p, double ramp, double rho_water);
void oracle_characteristic_state(const double interior[3], double h_e, double un_e, double ut_e,
                                 double nx, double ny, double g, double h_min, double out[3]);
void oracle_desingularized_velocity(double h_dry, double h, double hu, double hv, double out[2]);
double oracle_thin_layer_rate(double h_dry, double relaxation_time, double h);
void oracle_correct_node(double h_dry, double max_velocity, double h, double io[2]);
void oracle_wintermeyer_flux(const double l[6], const double r[6], double m0, double m1, double g,
                             double out[3]);
void oracle_hydrostatic_hll(const double a[4], const double b[4], double m0, double m1, double g,
                            double h_min, double fa[3], double fb[3]);
void oracle_gll(int order, double* nodes, double* weights, double* d);
double oracle_positivity_cfl(int order);
void oracle_positivity_bound(int order, int scheme, double out[3]);
int oracle_wet_dry_element(int nn, double* h, double* hu, double* hv, const double* mass,
                           double h_dry, double max_velocity);
void oracle_damp_nodes(int64_t n, const double* h, double* hu, double* hv, const double* fh,
                       const double* fhu, const double* fhv, double dt, double g, double manning_n,
                       double h_dry, double relaxation_time);
double oracle_tide_elevation(const dgswe_boundary* b, double t);

/* the Standard-kernel helpers of the reference's RHS bench, one element */
void oracle_apply_diff_matrix(const double* d, const double* fh, const double* fhu,
                              const double* fhv, double* oh, double* ohu, double* ohv, int64_t n);
void oracle_apply_lift(const double* lift, const double* dh, const double* dhu, const double* dhv,
                       double* oh, double* ohu, double* ohv, int64_t n, int64_t nf, double scale);
void oracle_coriolis_source(const double* hu, const double* hv, double* ohu, double* ohv, double f,
                            int64_t n);
void oracle_combine_derivatives(const double* const in[12], double* oh, double* ohu, double* ohv,
                                double rx, double sx, double ry, double sy, int64_t n);

#ifdef __cplusplus
}
#endif

#endif
