// The multirate level planner on the device: the host planner's rules
// (multirate.cpp, each after the reference's MultirateStepper,
// src/time/multirate.rs:527-778, 1088-1113) as kernels over the element
// steps and depth flags the dt pass leaves on the device, so that a coarse
// step's plan never crosses the host link: only a few scalars (the step
// bounds, the limit's progress, the pass counts) come back.
//
//  - plan_scan_kernel: the smallest and largest finite element step, the
//    longest step of an element in water (coarse_step_bound), Σ 1/dt and
//    the line-local count;
//  - plan_level_kernel: each element's level for a coarse step (the
//    smallest ℓ with dt/2^ℓ ≤ its step: assign_levels, levels_for_step);
//  - plan_memo_kernel: whether the levels and line flags are the last
//    plan's (the kept plan);
//  - plan_limit_kernel: one Jacobi sweep of the jump limit, repeated until
//    nothing changes (limit_level_jumps);
//  - plan_spread_faces_kernel / plan_spread_lines_kernel: one stage's rates
//    (spread_over_stencil, spread_over_lines);
//  - sort_count / sort_offsets / sort_scatter: the passes' orders, a stable
//    counting sort by key, largest first, index order within a key (tiles
//    of 1024 items; ranks within a tile from warp ballots), with each
//    key's count of items at or above it.
//
// Integer and compare work only, besides the steps' Σ 1/dt (a statistic):
// the plan is the host planner's bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/dgswe.h"
#include "device.hpp"
#include "handle.hpp"
#include "multirate.hpp"

namespace dgswe {
namespace {

constexpr int kThreads = 256;
constexpr int kSortTile = 1024;
constexpr int kKeys = kMaxLevels + 1;
constexpr unsigned long long kInfBits = 0x7FF0000000000000ull;

struct PlanScalars {
    unsigned long long lo, hi, b2, b4;  // bit patterns of non-negative steps
    double inv_sum;
    unsigned long long n_line_local;
    int finest;
    int changed;
    unsigned long long pow2_sum;
};

__device__ __forceinline__ bool finite_bits(unsigned long long b) {
    return (b & 0x7FF0000000000000ull) != 0x7FF0000000000000ull;
}

__global__ void plan_scan_kernel(const double* __restrict__ dt, const uint8_t* __restrict__ flags,
                                 int64_t K, PlanScalars* s) {
    unsigned long long lo = kInfBits, hi = 0, b2 = 0, b4 = 0, nll = 0;
    double inv = 0.0;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < K;
         k += (int64_t)gridDim.x * blockDim.x) {
        const uint8_t f = flags[k];
        nll += f & 1;
        const double d = dt[k];
        const unsigned long long b = (unsigned long long)__double_as_longlong(d);
        if (!finite_bits(b)) continue;
        lo = b < lo ? b : lo;
        hi = b > hi ? b : hi;
        if (f & 2) b2 = b > b2 ? b : b2;
        if (f & 4) b4 = b > b4 ? b : b4;
        inv += 1.0 / d;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const unsigned long long olo = __shfl_down_sync(0xffffffffu, lo, off);
        const unsigned long long ohi = __shfl_down_sync(0xffffffffu, hi, off);
        const unsigned long long ob2 = __shfl_down_sync(0xffffffffu, b2, off);
        const unsigned long long ob4 = __shfl_down_sync(0xffffffffu, b4, off);
        nll += __shfl_down_sync(0xffffffffu, nll, off);
        inv += __shfl_down_sync(0xffffffffu, inv, off);
        lo = olo < lo ? olo : lo;
        hi = ohi > hi ? ohi : hi;
        b2 = ob2 > b2 ? ob2 : b2;
        b4 = ob4 > b4 ? ob4 : b4;
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&s->lo, lo);
        atomicMax(&s->hi, hi);
        atomicMax(&s->b2, b2);
        atomicMax(&s->b4, b4);
        atomicAdd(&s->n_line_local, nll);
        atomicAdd(&s->inv_sum, inv);
    }
}

// assign_levels / levels_for_step (multirate.rs:527-583) at coarse step dt
// with at most L levels; the finest level reached into *finest if given
__global__ void plan_level_kernel(const double* __restrict__ dt_el, int64_t K, double dt, int L,
                                  uint8_t* __restrict__ level, int* finest) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    int l = 0;
    double dl = dt;
    const double e = dt_el[k];
    while (l < L && dl > e) {
        dl *= 0.5;
        l += 1;
    }
    level[k] = (uint8_t)l;
    if (finest && l > 0) atomicMax(finest, l);
}

__global__ void plan_memo_kernel(const uint8_t* __restrict__ level, const uint8_t* __restrict__ memo,
                                 const uint8_t* __restrict__ flags,
                                 const uint8_t* __restrict__ memo_line, int lines, int64_t K,
                                 int* diff) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    if (level[k] != memo[k] || (lines && (flags[k] & 1) != memo_line[k])) *diff = 1;
}

__global__ void plan_save_memo_kernel(const uint8_t* __restrict__ level,
                                      const uint8_t* __restrict__ flags, int lines, int64_t K,
                                      uint8_t* __restrict__ memo, uint8_t* __restrict__ memo_line) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    memo[k] = level[k];
    if (lines) memo_line[k] = flags[k] & 1;
}

// to[k] = max(from[k], from[j] − 1) over the face neighbours j
// (limit_level_jumps, multirate.rs:745-752)
__global__ void plan_limit_kernel(const int64_t* __restrict__ nb, const uint8_t* __restrict__ from,
                                  uint8_t* __restrict__ to, int64_t K, int* changed) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    uint8_t m = from[k];
#pragma unroll
    for (int f = 0; f < 4; ++f) {
        const int64_t j = nb[k * 4 + f];
        if (j < 0) continue;
        const uint8_t v = from[j];
        const uint8_t dropped = v > 0 ? (uint8_t)(v - 1) : 0;
        m = m > dropped ? m : dropped;
    }
    to[k] = m;
    if (m != from[k]) *changed = 1;
}

// to[k] = the largest `from` over k and its face neighbours
// (spread_over_stencil, multirate.rs:617-676)
__global__ void plan_spread_faces_kernel(const int64_t* __restrict__ nb,
                                         const uint8_t* __restrict__ from,
                                         uint8_t* __restrict__ to, int64_t K) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    uint8_t m = from[k];
#pragma unroll
    for (int f = 0; f < 4; ++f) {
        const int64_t j = nb[k * 4 + f];
        if (j >= 0) m = m > from[j] ? m : from[j];
    }
    to[k] = m;
}

__global__ void plan_fill_nodes_kernel(const uint8_t* __restrict__ level, int nn, int64_t K,
                                       uint8_t* __restrict__ node) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= K * nn) return;
    node[g] = level[g / nn];
}

struct FaceNodes {
    int n[4][5];
};

// One stage of node rates (spread_over_lines, multirate.rs:678-743): a
// line-local element's node follows its two GLL lines and, on a face, the
// neighbour's coincident node; any other element follows all of its own
// nodes and its neighbours' shared-face nodes and the nodes one in from them
__global__ void plan_spread_lines_kernel(const int64_t* __restrict__ nb,
                                         const int8_t* __restrict__ nb_face,
                                         const uint8_t* __restrict__ flags, FaceNodes fn, int n1,
                                         const uint8_t* __restrict__ from, uint8_t* __restrict__ to,
                                         uint8_t* __restrict__ rate, int64_t K) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    const int nn = n1 * n1;
    const uint8_t* own = from + k * nn;
    uint8_t* out = to + k * nn;
    auto inner = [n1](int face, int node) {
        switch (face) {
            case 0: return node + n1;
            case 1: return node - 1;
            case 2: return node - n1;
            default: return node + 1;
        }
    };
    if (!(flags[k] & 1)) {
        uint8_t m = 0;
        for (int i = 0; i < nn; ++i) m = m > own[i] ? m : own[i];
        for (int f = 0; f < 4; ++f) {
            const int64_t j = nb[k * 4 + f];
            if (j < 0) continue;
            const uint8_t* other = from + j * nn;
            const int of = nb_face[k * 4 + f];
            for (int fi = 0; fi < n1; ++fi) {
                const int node = fn.n[of][fi];
                const uint8_t a = other[node], b = other[inner(of, node)];
                const uint8_t ab = a > b ? a : b;
                m = m > ab ? m : ab;
            }
        }
        for (int i = 0; i < nn; ++i) out[i] = m;
        rate[k] = m;
        return;
    }
    for (int r = 0; r < n1; ++r) {  // r-lines (rows)
        uint8_t m = 0;
        for (int i = 0; i < n1; ++i) m = m > own[r * n1 + i] ? m : own[r * n1 + i];
        for (int i = 0; i < n1; ++i) out[r * n1 + i] = m;
    }
    for (int c = 0; c < n1; ++c) {  // s-lines (columns)
        uint8_t m = 0;
        for (int r = 0; r < n1; ++r) m = m > own[r * n1 + c] ? m : own[r * n1 + c];
        for (int r = 0; r < n1; ++r) out[r * n1 + c] = out[r * n1 + c] > m ? out[r * n1 + c] : m;
    }
    for (int f = 0; f < 4; ++f) {
        const int64_t j = nb[k * 4 + f];
        if (j < 0) continue;
        const uint8_t* other = from + j * nn;
        const int of = nb_face[k * 4 + f];
        for (int fi = 0; fi < n1; ++fi) {
            const int node = fn.n[f][fi];
            const uint8_t o = other[fn.n[of][n1 - 1 - fi]];
            out[node] = out[node] > o ? out[node] : o;
        }
    }
    uint8_t m = 0;
    for (int i = 0; i < nn; ++i) m = m > out[i] ? m : out[i];
    rate[k] = m;
}

// Σ 2^a[i] (the evaluations of a pass set)
__global__ void plan_pow2_sum_kernel(const uint8_t* __restrict__ a, int64_t n,
                                     unsigned long long* sum) {
    unsigned long long s = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        s += 1ull << a[i];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(sum, s);
}

// The sort key of item i: an element's own value (mode 0), an interior
// edge's larger side (mode 1, edge_left/edge_right), a boundary face's
// element (mode 2, bface)
__device__ __forceinline__ int sort_key(int mode, const uint8_t* a, const int64_t* l,
                                        const int64_t* r, int64_t i) {
    if (mode == 0) return a[i];
    const int x = a[l[i] >> 2];
    if (mode == 2) return x;
    const int y = a[r[i] >> 2];
    return x > y ? x : y;
}

__global__ void __launch_bounds__(kSortTile)
    sort_count_kernel(int mode, const uint8_t* __restrict__ a, const int64_t* __restrict__ l,
                      const int64_t* __restrict__ r, int64_t n, int V, int64_t* counts) {
    __shared__ int hist[kKeys];
    if (threadIdx.x < V) hist[threadIdx.x] = 0;
    __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * kSortTile + threadIdx.x;
    if (i < n) atomicAdd(&hist[sort_key(mode, a, l, r, i)], 1);
    __syncthreads();
    if (threadIdx.x < V) counts[(int64_t)blockIdx.x * V + threadIdx.x] = hist[threadIdx.x];
}

// counts [nblk][V] → each tile's first slot per key (in place): keys in
// descending order, tiles in order; at_least[v] = items with key ≥ v
__global__ void sort_offsets_kernel(int64_t* counts, int64_t nblk, int V, int64_t* at_least) {
    __shared__ int64_t total[kKeys];
    const int v = threadIdx.x;
    if (v < V) {
        int64_t t = 0;
        for (int64_t b = 0; b < nblk; ++b) t += counts[b * V + v];
        total[v] = t;
    }
    __syncthreads();
    if (v < V) {
        int64_t base = 0;
        for (int u = v + 1; u < V; ++u) base += total[u];
        at_least[v] = base + total[v];
        int64_t o = base;
        for (int64_t b = 0; b < nblk; ++b) {
            const int64_t c = counts[b * V + v];
            counts[b * V + v] = o;
            o += c;
        }
    }
}

__global__ void __launch_bounds__(kSortTile)
    sort_scatter_kernel(int mode, const uint8_t* __restrict__ a, const int64_t* __restrict__ l,
                        const int64_t* __restrict__ r, int64_t n, int V,
                        const int64_t* __restrict__ offsets, int32_t* __restrict__ order) {
    __shared__ int warp_count[kSortTile / 32][kKeys];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t i = (int64_t)blockIdx.x * kSortTile + threadIdx.x;
    const int key = i < n ? sort_key(mode, a, l, r, i) : -1;
    int rank = 0;
    for (int v = 0; v < V; ++v) {
        const unsigned m = __ballot_sync(0xffffffffu, key == v);
        if (key == v) rank = __popc(m & ((1u << lane) - 1u));
        if (lane == 0) warp_count[warp][v] = __popc(m);
    }
    __syncthreads();
    if (threadIdx.x < V) {
        int s = 0;
        for (int w = 0; w < kSortTile / 32; ++w) {
            const int c = warp_count[w][threadIdx.x];
            warp_count[w][threadIdx.x] = s;
            s += c;
        }
    }
    __syncthreads();
    if (key >= 0)
        order[offsets[(int64_t)blockIdx.x * V + key] + warp_count[warp][key] + rank] = (int32_t)i;
}

unsigned grid_of(int64_t n, int threads = kThreads) {
    return (unsigned)std::max<int64_t>(1, (n + threads - 1) / threads);
}

double from_bits(unsigned long long b) {
    double d;
    std::memcpy(&d, &b, sizeof d);
    return d;
}

}  // namespace

namespace host {

namespace {

template <class T>
int dev_alloc(dgswe_handle* h, size_t n, T** out) {
    void* p = nullptr;
    CK(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)));
    h->allocations.push_back(p);
    *out = (T*)p;
    return DGSWE_OK;
}

// The device planner's buffers, once per handle
int plan_buffers(dgswe_handle* h) {
    auto& dp = h->dplan;
    if (dp.nb) return DGSWE_OK;
    const size_t K = (size_t)h->K, nn = (size_t)h->nn;
    const size_t E = h->h_edge_left.size(), B = h->h_bface.size();
    const size_t tiles = (std::max(std::max(K, E), B) + kSortTile - 1) / kSortTile;
    int s = DGSWE_OK;
    if ((s = dev_alloc(h, 4 * K, &dp.nb))) return s;
    if ((s = dev_alloc(h, 4 * K, &dp.nb_face))) return s;
    if ((s = dev_alloc(h, K, &dp.level_tmp))) return s;
    if ((s = dev_alloc(h, K, &dp.memo_level))) return s;
    if ((s = dev_alloc(h, K, &dp.memo_line))) return s;
    if ((s = dev_alloc(h, K, &dp.memo_limited))) return s;
    if ((s = dev_alloc(h, K * nn, &dp.node_a))) return s;
    if ((s = dev_alloc(h, K * nn, &dp.node_b))) return s;
    if ((s = dev_alloc(h, tiles * kKeys, &dp.sort_counts))) return s;
    if ((s = dev_alloc(h, (size_t)(3 * kPlanStages + 1) * kKeys, &dp.at_least))) return s;
    uint8_t* sc = nullptr;
    if ((s = dev_alloc(h, sizeof(PlanScalars), &sc))) return s;
    dp.scalars = sc;
    void* p = nullptr;
    CK(cudaMallocHost(&p, sizeof(PlanScalars) + (3 * kPlanStages + 1) * kKeys * sizeof(int64_t)));
    dp.host = p;
    CK(cudaMemcpy(dp.nb, h->nb.data(), 4 * K * sizeof(int64_t), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dp.nb_face, h->nb_face.data(), 4 * K, cudaMemcpyHostToDevice));
    return DGSWE_OK;
}

// A stable counting sort of n items by key, largest first, into order;
// each key's count at or above it into at_least[0..V)
int plan_sort(dgswe_handle* h, int mode, const uint8_t* a, const int64_t* l, const int64_t* r,
              int64_t n, int V, int32_t* order, int64_t* at_least) {
    cudaStream_t st = h->stream;
    if (n == 0) {
        CK(cudaMemsetAsync(at_least, 0, V * sizeof(int64_t), st));
        return DGSWE_OK;
    }
    const int64_t tiles = (n + kSortTile - 1) / kSortTile;
    int64_t* counts = h->dplan.sort_counts;
    sort_count_kernel<<<(unsigned)tiles, kSortTile, 0, st>>>(mode, a, l, r, n, V, counts);
    sort_offsets_kernel<<<1, 32, 0, st>>>(counts, tiles, V, at_least);
    sort_scatter_kernel<<<(unsigned)tiles, kSortTile, 0, st>>>(mode, a, l, r, n, V, counts, order);
    return DGSWE_OK;
}

int read_scalars(dgswe_handle* h, PlanScalars& out) {
    CK(cudaMemcpyAsync(h->dplan.host, h->dplan.scalars, sizeof(PlanScalars),
                       cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    std::memcpy(&out, h->dplan.host, sizeof out);
    return DGSWE_OK;
}

}  // namespace

int device_plan(dgswe_handle* h, int n_stages, bool lines, bool bounded, double dt_max,
                double landing, double& fitted_dt, double& stable_dt) {
    if (int s = plan_buffers(h)) return s;
    auto& dp = h->dplan;
    MultiratePlanner& pl = *h->planner;
    cudaStream_t st = h->stream;
    const int64_t K = h->K;
    const int64_t E = (int64_t)h->h_edge_left.size(), B = (int64_t)h->h_bface.size();
    PlanScalars init{};
    init.lo = kInfBits;
    PlanScalars* ds = (PlanScalars*)dp.scalars;
    CK(cudaMemcpyAsync(ds, &init, sizeof init, cudaMemcpyHostToDevice, st));
    plan_scan_kernel<<<std::min<unsigned>(grid_of(K), 4 * 152), kThreads, 0, st>>>(h->dt_el,
                                                                                   h->d_flags, K, ds);
    PlanScalars sc;
    if (int s = read_scalars(h, sc)) return s;

    // coarse_step_bound (src/physics/builder.rs:611-632) and the cap
    double bound = INFINITY;
    if (bounded) {
        const double longest2 = from_bits(sc.b2), longest4 = from_bits(sc.b4);
        if (longest2 > 0.0) bound = longest2;
        else if (longest4 > 0.0) bound = longest4;
    }
    double cap = dt_max > 0.0 ? std::min(dt_max, bound) : bound;
    if (!std::isfinite(cap)) cap = 0.0;

    // assign_levels (multirate.rs:527-568)
    const int max_levels = std::min(h->planner_levels, kMaxLevels);
    const double lo = from_bits(sc.lo), hi = from_bits(sc.hi);
    int finest = 0;
    double dt = INFINITY;
    if (std::isfinite(lo)) {
        const bool capped = cap > 0.0 && std::isfinite(cap);
        while (finest < max_levels) {
            const double coarser = lo * (double)(2ull << finest);
            if (coarser > hi || (capped && coarser > cap)) break;
            finest += 1;
        }
        dt = lo * (double)(1ull << finest);
    }
    plan_level_kernel<<<grid_of(K), kThreads, 0, st>>>(h->dt_el, K, dt, finest, h->d_level, nullptr);
    stable_dt = dt;
    // the landing: equal steps to the time left, each with its own levels
    if (finest > 0 && landing > 0.0 && std::isfinite(landing) && std::isfinite(dt)) {
        const double steps = std::max(std::ceil(landing / (dt * (1.0 + 1e-9))), 1.0);
        const double fitted = landing / steps;
        if (fitted < dt) {
            dt = fitted;
            CK(cudaMemsetAsync(&ds->finest, 0, sizeof(int), st));
            plan_level_kernel<<<grid_of(K), kThreads, 0, st>>>(h->dt_el, K, dt, max_levels,
                                                               h->d_level, &ds->finest);
            if (int s = read_scalars(h, sc)) return s;
            finest = sc.finest;
        }
    }
    fitted_dt = dt;
    pl.set_step_figures(stable_dt, sc.inv_sum, lines ? (int64_t)sc.n_line_local : 0);

    // the kept plan (multirate.rs:1104-1113): unchanged levels and flags
    if (dp.memo_valid && dp.memo_finest == finest && dp.memo_lines == lines &&
        h->plan_uploaded == pl.version()) {
        CK(cudaMemsetAsync(&ds->changed, 0, sizeof(int), st));
        plan_memo_kernel<<<grid_of(K), kThreads, 0, st>>>(h->d_level, dp.memo_level, h->d_flags,
                                                          dp.memo_line, lines ? 1 : 0, K,
                                                          &ds->changed);
        if (int s = read_scalars(h, sc)) return s;
        if (!sc.changed) {
            CK(cudaMemcpyAsync(h->d_level, dp.memo_limited, (size_t)K, cudaMemcpyDeviceToDevice,
                               st));
            return DGSWE_OK;
        }
    }
    plan_save_memo_kernel<<<grid_of(K), kThreads, 0, st>>>(h->d_level, h->d_flags, lines ? 1 : 0,
                                                           K, dp.memo_level, dp.memo_line);
    // the jump limit, sweep after sweep until nothing changes
    uint8_t* cur = h->d_level;
    uint8_t* nxt = dp.level_tmp;
    for (int sweep = 0; sweep <= 2 * kMaxLevels + 2; ++sweep) {
        CK(cudaMemsetAsync(&ds->changed, 0, sizeof(int), st));
        plan_limit_kernel<<<grid_of(K), kThreads, 0, st>>>(dp.nb, cur, nxt, K, &ds->changed);
        if (int s = read_scalars(h, sc)) return s;
        if (!sc.changed) break;
        std::swap(cur, nxt);
    }
    if (cur != h->d_level)
        CK(cudaMemcpyAsync(h->d_level, cur, (size_t)K, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(dp.memo_limited, h->d_level, (size_t)K, cudaMemcpyDeviceToDevice, st));

    // the stage rates
    unsigned long long* pow2 = &ds->pow2_sum;
    const size_t Ks = (size_t)K;
    if (lines) {
        FaceNodes fn{};
        for (int f = 0; f < 4; ++f)
            for (int i = 0; i < 5; ++i) fn.n[f][i] = h->ops->face_node[f][i];
        plan_fill_nodes_kernel<<<grid_of(K * h->nn), kThreads, 0, st>>>(h->d_level, h->nn, K,
                                                                          dp.node_a);
        uint8_t* from = dp.node_a;
        uint8_t* to = dp.node_b;
        for (int s = 0; s < n_stages; ++s) {
            plan_spread_lines_kernel<<<grid_of(K), kThreads, 0, st>>>(
                dp.nb, dp.nb_face, h->d_flags, fn, h->n1, from, to, h->d_rate + s * Ks, K);
            std::swap(from, to);
        }
    } else {
        for (int s = 0; s < n_stages; ++s)
            plan_spread_faces_kernel<<<grid_of(K), kThreads, 0, st>>>(
                dp.nb, s == 0 ? h->d_level : h->d_rate + (s - 1) * Ks, h->d_rate + s * Ks, K);
    }

    // the evaluations: Σ 2^level over the stages, Σ 2^rate per stage
    unsigned long long zero = 0;
    CK(cudaMemcpyAsync(pow2, &zero, sizeof zero, cudaMemcpyHostToDevice, st));
    plan_pow2_sum_kernel<<<std::min<unsigned>(grid_of(K), 4 * 152), kThreads, 0, st>>>(h->d_level,
                                                                                      K, pow2);
    if (int s = read_scalars(h, sc)) return s;
    const int64_t level_evaluations = (int64_t)n_stages * (int64_t)sc.pow2_sum;
    CK(cudaMemcpyAsync(pow2, &zero, sizeof zero, cudaMemcpyHostToDevice, st));
    plan_pow2_sum_kernel<<<std::min<unsigned>(grid_of(K * n_stages), 4 * 152), kThreads, 0, st>>>(
        h->d_rate, K * n_stages, pow2);

    // the passes' orders and counts
    const int V = finest + 1;
    int64_t* al = dp.at_least;
    for (int j = 0; j <= n_stages; ++j) {
        const uint8_t* key = j < n_stages ? h->d_rate + j * Ks : h->d_level;
        if (int s = plan_sort(h, 0, key, nullptr, nullptr, K, V, h->d_order + j * Ks,
                              al + j * kKeys))
            return s;
    }
    for (int s = 0; s < n_stages; ++s) {
        const uint8_t* r = h->d_rate + s * Ks;
        if (int st2 = plan_sort(h, 1, r, h->T.edge_left, h->T.edge_right, E, V,
                                h->d_edges + s * E, al + (kPlanStages + 1 + s) * kKeys))
            return st2;
        if (int st2 = plan_sort(h, 2, r, h->T.bface, nullptr, B, V, h->d_bfaces + s * B,
                                al + (2 * kPlanStages + 1 + s) * kKeys))
            return st2;
    }
    uint8_t* host = (uint8_t*)dp.host;
    int64_t* counts = (int64_t*)(host + sizeof(PlanScalars));
    CK(cudaMemcpyAsync(host, ds, sizeof(PlanScalars), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(counts, al, (3 * kPlanStages + 1) * kKeys * sizeof(int64_t),
                       cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    std::memcpy(&sc, host, sizeof sc);
    pl.set_device_plan(finest, n_stages, V, counts, counts + (kPlanStages + 1) * kKeys,
                       counts + (2 * kPlanStages + 1) * kKeys, kKeys, (int64_t)sc.pow2_sum,
                       level_evaluations);
    h->plan_uploaded = pl.version();
    dp.memo_valid = true;
    dp.memo_finest = finest;
    dp.memo_lines = lines;
    return DGSWE_OK;
}

}  // namespace host
}  // namespace dgswe
