// The internals of an ensemble (ensemble.cu), shared with the adjoint
// driver (adjoint.cu), which runs the adjoint over an ensemble's order group.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/dgswe.h"
#include "device.hpp"
#include "kernel_set.hpp"
#include "setup.hpp"

namespace dgswe {
namespace host {

constexpr int kEnsBuffers = 4;  // state and the stage outputs of SSP-RK(4,3)

struct Group {
    int n1 = 0, nn = 0;
    int64_t K = 0, n_values = 0;
    Operators* ops = nullptr;
    DevTables T{};
    Physics P{};
    StageExtra X{};
    double* buf_base[kEnsBuffers] = {};
    DevBuf buf[kEnsBuffers]{};
    double *fb_h = nullptr, *fb_hu = nullptr, *fb_hv = nullptr;
    std::vector<int> members;
};

struct Member {
    int group = -1;
    int64_t k0 = 0, K = 0, node0 = 0, n_values = 0;
};

}  // namespace host
}  // namespace dgswe

struct dgswe_ensemble {
    using Group = dgswe::host::Group;
    using Member = dgswe::host::Member;
    using KernelSet = dgswe::KernelSet;
    using StepCtl = dgswe::StepCtl;
    int device = 0;
    cudaStream_t stream = nullptr, side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr, t0 = nullptr, t1 = nullptr;
    std::string error, device_name;
    dgswe_form form0{};  // the shared physics (array pointers cleared)
    const KernelSet* ks = nullptr;
    int n_members = 0;
    std::vector<Member> members;
    std::vector<int> cond_base;  // each member's first condition in T.cond
    std::vector<Group> groups;
    StepCtl* ctl = nullptr;    // device, one per member
    StepCtl* h_ctl = nullptr;  // pinned host mirror
    int* always = nullptr;     // device 1: the launches' activity flag
    std::vector<void*> allocations;
    cudaGraphExec_t graph = nullptr;
    int graph_scheme = -1;
    double graph_cfl = -1.0;

    ~dgswe_ensemble() {
        if (graph) cudaGraphExecDestroy(graph);
        for (void* p : allocations) cudaFree(p);
        if (h_ctl) cudaFreeHost(h_ctl);
        for (cudaEvent_t e : {fork, join, t0, t1})
            if (e) cudaEventDestroy(e);
        if (side) cudaStreamDestroy(side);
        if (stream) cudaStreamDestroy(stream);
        for (Group& g : groups) delete g.ops;
    }
};

