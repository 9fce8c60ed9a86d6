// The internals of a dgswe handle, shared by the C ABI of one mesh (api.cu)
// and the adjoint driver (adjoint.cu), which works on a handle's tables,
// buffers and step control.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <utility>
#include <vector>

#include "../../include/dgswe.h"
#include "device.hpp"
#include "kernel_set.hpp"
#include "multirate.hpp"
#include "setup.hpp"

namespace dgswe {
namespace host {

constexpr int kRhsBuffer = DGSWE_N_BUFFERS;  // scratch buffer of dgswe_compute_rhs

}  // namespace host

// dgswe_step_host's upload and last stage run in this many element chunks
constexpr int kHostChunks = 8;

namespace host {

struct DeviceBuffer {
    double* base = nullptr;  // one allocation of 5 fields
    DevBuf view{};
};

}  // namespace host
}  // namespace dgswe

struct dgswe_handle {
    using Operators = dgswe::Operators;
    using KernelSet = dgswe::KernelSet;
    using DevTables = dgswe::DevTables;
    using Physics = dgswe::Physics;
    using StageExtra = dgswe::StageExtra;
    using StepCtl = dgswe::StepCtl;
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string error;
    dgswe_form form{};
    std::vector<dgswe_tide_constituent> constituents;
    Operators* ops = nullptr;
    int n1 = 0, nn = 0;
    int64_t K = 0, n_values = 0;
    const KernelSet* ks = nullptr;
    DevTables T{};
    Physics P{};
    StageExtra X{};
    std::vector<void*> allocations;
    dgswe::host::DeviceBuffer buf[DGSWE_N_BUFFERS + 1];
    double *fb_h = nullptr, *fb_hu = nullptr, *fb_hv = nullptr;
    double* dt_el = nullptr;
    double* sub_mass = nullptr;  // subcell mass fluxes (dgswe_compute_rhs_mass_fluxes), lazily
    StepCtl* ctl = nullptr;    // device
    StepCtl* h_ctl = nullptr;  // pinned host mirror
    std::string device_name;
    // graph of one device-driven step
    cudaGraphExec_t step_graph = nullptr;
    int graph_scheme = -1;
    double graph_cfl = -1.0;
    // local time stepping: the mesh's face neighbours and the device tables'
    // edges on the host, the level planner and its plan on the device
    std::vector<std::array<int64_t, 4>> nb;
    std::vector<std::array<int8_t, 4>> nb_face;
    std::vector<int64_t> h_edge_left, h_edge_right, h_bface;
    dgswe::MultiratePlanner* planner = nullptr;
    int planner_levels = -1, planner_stages = -1;
    uint64_t plan_uploaded = 0;
    uint8_t *d_level = nullptr, *d_rate = nullptr, *d_flags = nullptr;
    int32_t *d_order = nullptr, *d_edges = nullptr, *d_bfaces = nullptr;
    dgswe_multirate_stats mr_stats{};
    cudaEvent_t ev_lts[2] = {nullptr, nullptr};
    // the level planner on the device (multirate_plan.cu): the face
    // neighbours, scratch, the kept plan's inputs and limited levels, the
    // pinned host copy of its scalars and counts
    struct {
        int64_t* nb = nullptr;
        int8_t* nb_face = nullptr;
        uint8_t *level_tmp = nullptr, *memo_level = nullptr, *memo_line = nullptr;
        uint8_t *memo_limited = nullptr, *node_a = nullptr, *node_b = nullptr;
        int64_t *sort_counts = nullptr, *at_least = nullptr;
        void* scalars = nullptr;
        void* host = nullptr;
        bool memo_valid = false, memo_lines = false;
        int memo_finest = -1;
    } dplan;
    // the times every parent series covers (a run must stay within them)
    std::pair<double, double> parent_range{-INFINITY, INFINITY};
    // device address of dgswe_compute_rhs_noalloc's working array, looked up
    // by the handle's first call to it (not memory the handle owns)
    double* noalloc_scratch = nullptr;
    // dgswe_step_host: the stream that copies the state in and out beside
    // the compute, and one event per chunk (created on first use)
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t chunk_done[dgswe::kHostChunks] = {};
    // per upload chunk, what the first stage can take once that chunk has
    // arrived (everything it reads in it or before it): the elements' dt
    // pass, the interior edges' and boundary faces' fluxes (ready_*[off[c]
    // .. off[c+1]), built on first use)
    const int32_t *ready_elems = nullptr, *ready_edges = nullptr, *ready_bfaces = nullptr;
    int64_t ready_elem_off[dgswe::kHostChunks + 1] = {};
    int64_t ready_edge_off[dgswe::kHostChunks + 1] = {};
    int64_t ready_bface_off[dgswe::kHostChunks + 1] = {};
    bool ready_built = false;
    // the dt pass's own stream, beside the first stage's face pass, and the
    // fork and join between them (created on first use)
    cudaStream_t dt_stream = nullptr;
    cudaEvent_t dt_fork = nullptr, dt_join = nullptr;

    ~dgswe_handle() {
        for (cudaEvent_t e : chunk_done)
            if (e) cudaEventDestroy(e);
        if (copy_stream) cudaStreamDestroy(copy_stream);
        for (cudaEvent_t e : {dt_fork, dt_join})
            if (e) cudaEventDestroy(e);
        if (dt_stream) cudaStreamDestroy(dt_stream);
        delete planner;
        if (dplan.host) cudaFreeHost(dplan.host);
        for (cudaEvent_t e : ev_lts)
            if (e) cudaEventDestroy(e);
        if (step_graph) cudaGraphExecDestroy(step_graph);
        for (void* p : allocations) cudaFree(p);
        if (h_ctl) cudaFreeHost(h_ctl);
        if (stream) cudaStreamDestroy(stream);
        delete ops;
    }
};


namespace dgswe {
namespace host {

// Records `status` and the message on the handle; returns the status
int fail(dgswe_handle* h, int status, const char* fmt, ...);
// Allocates buffer `id` (5 fields of n_values doubles) on first use
int ensure_buffer(dgswe_handle* h, int id);
int sync(dgswe_handle* h);
// One stage: the face pass, then the element stage
void launch_stage(dgswe_handle* h, int in, int base, int out, int acc, int slot, int mode,
                  int check_finite, const int* active);
const int* always(dgswe_handle* h);
// The device clock of a run from run->t_start towards `target`
int begin_run(dgswe_handle* h, const dgswe_run_config* run, double target);
// dgswe_run with local time stepping (run->levels > 0; multirate_run.cu)
int run_multirate(dgswe_handle* h, const dgswe_run_config* run, dgswe_callback callback,
                  void* user, dgswe_report* report);
// A coarse step's plan made on the device (multirate_plan.cu) from the
// element steps in h->dt_el and the depth flags in h->d_flags, into the
// handle's plan arrays and the planner's counts: the fitted coarse step and
// the stable step before the fit
int device_plan(dgswe_handle* h, int n_stages, bool lines, bool bounded, double dt_max,
                double landing, double& fitted_dt, double& stable_dt);

}  // namespace host
}  // namespace dgswe

#define CK(call)                                                                             \
    do {                                                                                     \
        cudaError_t err_ = (call);                                                           \
        if (err_ != cudaSuccess)                                                             \
            return fail(h, DGSWE_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(err_)); \
    } while (0)
