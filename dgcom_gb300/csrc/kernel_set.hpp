// The launchers of one numerics variant of the kernels, as a table the
// host runtime picks from at dgswe_create.
#pragma once

#include <cuda_runtime.h>

#include "device.hpp"

namespace dgswe {

struct KernelSet {
    void (*face)(int n1, const DevTables&, const Physics&, const DevBuf& in, double* fh,
                 double* fhu, double* fhv, const StepCtl* ctl, int slot, const int* active,
                 cudaStream_t);
    void (*stage)(int n1, const DevTables&, const Physics&, const StageExtra&, const DevBuf& in,
                  const DevBuf& base, const DevBuf& out, const DevBuf& acc, const double* fh,
                  const double* fhu, const double* fhv, StepCtl* ctl, int slot, int mode,
                  int check_finite, const int* active, cudaStream_t);
    void (*finish)(int n1, const DevTables&, const Physics&, const DevBuf& acc,
                   const DevBuf& state, StepCtl* ctl, cudaStream_t);
    void (*dt)(int n1, const DevTables&, const Physics&, const DevBuf& q, const DtParams&,
               double* dt_el, StepCtl* ctl, const int* active, cudaStream_t);
    void (*velocity)(const DevBuf&, int64_t n, double h_min, cudaStream_t);
    // a kPost stage that also keeps the combination and the damped momentum
    // (the adjoint's recomputation)
    void (*stage_keep)(int n1, const DevTables&, const Physics&, const StageExtra&,
                       const DevBuf& in, const DevBuf& base, const DevBuf& out, const double* fh,
                       const double* fhu, const double* fhv, StepCtl* ctl, int slot,
                       int check_finite, const DevBuf& keep, cudaStream_t);
    // the adjoint of one stage (adjoint_kernels.cuh): the wet elements'
    // pass (`subcells` 0) or the listed subcell elements' (1)
    void (*stage_adjoint)(int n1, const DevTables&, const Physics&, const StageExtra&,
                          const DevBuf& in, const DevBuf& keep, const AdjStage&,
                          const StepCtl* ctl, int slot, int subcells, cudaStream_t);
    void (*face_adjoint)(int n1, const DevTables&, const Physics&, const DevBuf& in,
                         const AdjStage&, const StepCtl* ctl, int slot, cudaStream_t);
    // out = λ of the stage input; with `base` (the first stage), + base,
    // which is cleared
    void (*adjoint_combine)(const DevBuf& in, const AdjStage&, double* out_h, double* out_hu,
                            double* out_hv, double* const* base, int64_t n, double h_min,
                            cudaStream_t);
    void (*station_eval)(const double* h, const double* bed, const int64_t* node0,
                         const double* w, int n_stations, int nn, double* eta, cudaStream_t);
    void (*station_seed)(const double* eta, const double* obs, const int64_t* node0,
                         const double* w, int n_stations, int nn, double* lh, double* lbed,
                         cudaStream_t);
    // the run's clock, one thread per StepCtl of ctl[0..n)
    void (*step_begin)(StepCtl*, int n, cudaStream_t);
    void (*step_dt)(StepCtl*, int n, cudaStream_t);
    void (*step_end)(StepCtl*, int n, cudaStream_t);
    // a multirate pass (LtsPass): the listed faces, the listed elements'
    // stage (mode kModePost, or kModeAccumulate for the last stage), the
    // end of the listed elements' substeps
    void (*face_listed)(int n1, const DevTables&, const Physics&, const DevBuf& in, double* fh,
                        double* fhu, double* fhv, StepCtl* ctl, const LtsPass&, cudaStream_t);
    void (*stage_listed)(int n1, const DevTables&, const Physics&, const StageExtra&,
                         const DevBuf& in, const DevBuf& base, const DevBuf& out,
                         const DevBuf& acc, const double* fh, const double* fhu,
                         const double* fhv, StepCtl* ctl, int mode, const LtsPass&, cudaStream_t);
    void (*finish_listed)(int n1, const DevTables&, const Physics&, const DevBuf& acc,
                          const DevBuf& state, StepCtl* ctl, const LtsPass&, cudaStream_t);
    // per element: every node deeper than d0, d1, d2 (bits 0, 1, 2)
    void (*depth_flags)(const double* h, int64_t K, int nn, double d0, double d1, double d2,
                        uint8_t* flags, cudaStream_t);
    // the subcell elements of a step's three stage inputs, one list each,
    // for the stage adjoint's subcell pass
    void (*subcell_list)(const DevTables&, const Physics&, const double* h0, const double* h1,
                         const double* h2, const AdjStage&, int nn, cudaStream_t);
    // the point-implicit damping of `stage` over dt, rates frozen at `from`
    // (n values), and the stage's node velocities
    void (*implicit_damping)(const DevTables&, const Physics&, const DevBuf& stage,
                             const DevBuf& from, double dt, int64_t n, cudaStream_t);
    // a global stage's face fluxes of the listed interior edges and boundary
    // faces, without the node sources (a stage taken in parts as its input
    // arrives); the node sources alone (weather, relaxation band)
    void (*face_ready)(int n1, const DevTables&, const Physics&, const DevBuf& in, double* fh,
                       double* fhu, double* fhv, const StepCtl* ctl, int slot, const int* active,
                       const int32_t* edges, int64_t n_edges, const int32_t* bfaces,
                       int64_t n_bfaces, cudaStream_t);
    void (*node_sources)(const DevTables&, const Physics&, const DevBuf& in, const StepCtl* ctl,
                         int slot, cudaStream_t);
    // the dt pass over the listed elements
    void (*dt_listed)(int n1, const DevTables&, const Physics&, const DevBuf& q, const DtParams&,
                      double* dt_el, StepCtl* ctl, const int* active, const int32_t* list,
                      int64_t n, cudaStream_t);
};

// kernels_fast.cu: FMA contraction, division-free Manning rate
const KernelSet* kernels_fast();
// kernels_exact.cu: every operation separately rounded, the reference's cube root
const KernelSet* kernels_exact();

// stage modes of the stage kernel
enum { kModeRhsOnly = 0, kModePost = 1, kModeAccumulate = 2 };

}  // namespace dgswe
