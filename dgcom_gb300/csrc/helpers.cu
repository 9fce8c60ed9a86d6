// The Standard-kernel helpers that the reference's RHS bench drives
// (benches/rhs_swe_2d_bench.rs; src/solver/simd/kernels.rs:31-224, 314-440),
// as batched device operations behind the C ABI: each applies the helper to
// n_elements elements at once, element e's vectors at offset e·n.
//
// Every product and sum is rounded on its own (__dmul_rn, __dadd_rn), in
// the helper's order, as the reference's scalar code (Rust never contracts
// a multiply and an add) and its SIMD forms (bit for bit with the scalar)
// compute them: each element's result is the reference's, bit for bit.
//
// They are the helpers of the reference's Standard formulation, not of the
// split-form path the library steps with; they are here so that a caller of
// those helpers finds them on the device.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>
#include <string>

#include "../../include/dgswe.h"

namespace {

thread_local std::string g_helper_error;

int helper_fail(int status, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_helper_error = buf;
    return status;
}

int helper_cuda(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return DGSWE_OK;
    return helper_fail(DGSWE_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define HCK(call)                                                  \
    do {                                                           \
        if (int s_ = helper_cuda((call), #call)) return s_;        \
    } while (0)

constexpr int kThreads = 256;
constexpr int kMaxNodes = 64;  // (N+1)² up to order 7

// out[e][i] = Σ_j D[i][j]·f[e][j] for the three fields, j in order from 0.
// One thread per (element, node); the element's flux vectors staged in
// shared memory by the block.
__global__ void diff_matrix_kernel(const double* __restrict__ d, const double* __restrict__ fh,
                                   const double* __restrict__ fhu, const double* __restrict__ fhv,
                                   double* oh, double* ohu, double* ohv, int n, int64_t total) {
    extern __shared__ double s_f[];  // [3][blockDim.x]
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    // a block starts on an element boundary (blockDim.x is a multiple of n)
    if (g < total) {
        s_f[threadIdx.x] = fh[g];
        s_f[blockDim.x + threadIdx.x] = fhu[g];
        s_f[2 * blockDim.x + threadIdx.x] = fhv[g];
    }
    __syncthreads();
    if (g >= total) return;
    const int i = (int)(g % n);
    const int base = threadIdx.x - i;
    double sh = 0.0, shu = 0.0, shv = 0.0;
    for (int j = 0; j < n; ++j) {
        const double dij = __ldg(&d[i * n + j]);
        sh = __dadd_rn(sh, __dmul_rn(dij, s_f[base + j]));
        shu = __dadd_rn(shu, __dmul_rn(dij, s_f[blockDim.x + base + j]));
        shv = __dadd_rn(shv, __dmul_rn(dij, s_f[2 * blockDim.x + base + j]));
    }
    oh[g] = sh;
    ohu[g] = shu;
    ohv[g] = shv;
}

// out[e][i] += scale[e]·(Σ_fi LIFT[i][fi]·diff[e][fi]), fi in order from 0
__global__ void lift_kernel(const double* __restrict__ lift, const double* __restrict__ dh,
                            const double* __restrict__ dhu, const double* __restrict__ dhv,
                            double* oh, double* ohu, double* ohv, const double* __restrict__ scale,
                            int n, int nf, int64_t total) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total) return;
    const int64_t e = g / n;
    const int i = (int)(g % n);
    const double* a = &dh[e * nf];
    const double* b = &dhu[e * nf];
    const double* c = &dhv[e * nf];
    double sh = 0.0, shu = 0.0, shv = 0.0;
    for (int fi = 0; fi < nf; ++fi) {
        const double l = __ldg(&lift[i * nf + fi]);
        sh = __dadd_rn(sh, __dmul_rn(l, a[fi]));
        shu = __dadd_rn(shu, __dmul_rn(l, b[fi]));
        shv = __dadd_rn(shv, __dmul_rn(l, c[fi]));
    }
    const double s = scale[e];
    oh[g] = __dadd_rn(oh[g], __dmul_rn(s, sh));
    ohu[g] = __dadd_rn(ohu[g], __dmul_rn(s, shu));
    ohv[g] = __dadd_rn(ohv[g], __dmul_rn(s, shv));
}

// S_hu += f·hv, S_hv += (−f)·hu
__global__ void coriolis_kernel(const double* __restrict__ hu, const double* __restrict__ hv,
                                double* ohu, double* ohv, double f, int64_t total) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total) return;
    ohu[g] = __dadd_rn(ohu[g], __dmul_rn(f, hv[g]));
    ohv[g] = __dadd_rn(ohv[g], __dmul_rn(-f, hu[g]));
}

struct Twelve {
    const double* p[12];  // dfx_dr (h, hu, hv), dfx_ds, dfy_dr, dfy_ds
};

// out = −(((dfx_dr·rx + dfx_ds·sx) + dfy_dr·ry) + dfy_ds·sy), the element's
// (rx, sx, ry, sy) from `metric`
__global__ void combine_kernel(Twelve in, double* oh, double* ohu, double* ohv,
                               const double* __restrict__ metric, int n, int64_t total) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total) return;
    const int64_t e = g / n;
    const double rx = metric[4 * e], sx = metric[4 * e + 1];
    const double ry = metric[4 * e + 2], sy = metric[4 * e + 3];
    double* out[3] = {oh, ohu, ohv};
#pragma unroll
    for (int v = 0; v < 3; ++v) {
        double div = __dmul_rn(in.p[v][g], rx);
        div = __dadd_rn(div, __dmul_rn(in.p[3 + v][g], sx));
        div = __dadd_rn(div, __dmul_rn(in.p[6 + v][g], ry));
        div = __dadd_rn(div, __dmul_rn(in.p[9 + v][g], sy));
        out[v][g] = -div;
    }
}

unsigned blocks_for(int64_t total, int threads) {
    return (unsigned)((total + threads - 1) / threads);
}

int prepare(int device, const char* what) {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count)
        return helper_fail(DGSWE_ERR_NO_DEVICE, "%s: no CUDA device %d", what, device);
    HCK(cudaSetDevice(device));
    return DGSWE_OK;
}

int finish(const char* what) {
    if (int s = helper_cuda(cudaGetLastError(), what)) return s;
    return helper_cuda(cudaStreamSynchronize(0), what);
}

}  // namespace

extern "C" {

const char* dgswe_helpers_last_error(void) { return g_helper_error.c_str(); }

int dgswe_apply_diff_matrix(int device, const double* d, const double* flux_h,
                            const double* flux_hu, const double* flux_hv, double* out_h,
                            double* out_hu, double* out_hv, int64_t n_nodes, int64_t n_elements) {
    if (!d || !flux_h || !flux_hu || !flux_hv || !out_h || !out_hu || !out_hv || n_nodes < 1 ||
        n_nodes > kMaxNodes || n_elements < 0)
        return helper_fail(DGSWE_ERR_INVALID,
                           "apply_diff_matrix: a NULL pointer, or %lld nodes (1 to %d) and %lld "
                           "elements", (long long)n_nodes, kMaxNodes, (long long)n_elements);
    if (int s = prepare(device, "apply_diff_matrix")) return s;
    const int64_t total = n_nodes * n_elements;
    if (total == 0) return DGSWE_OK;
    const int threads = (int)((kThreads / n_nodes) * n_nodes);  // whole elements a block
    diff_matrix_kernel<<<blocks_for(total, threads), threads, 3 * threads * sizeof(double)>>>(
        d, flux_h, flux_hu, flux_hv, out_h, out_hu, out_hv, (int)n_nodes, total);
    return finish("apply_diff_matrix");
}

int dgswe_apply_lift(int device, const double* lift, const double* flux_diff_h,
                     const double* flux_diff_hu, const double* flux_diff_hv, double* out_h,
                     double* out_hu, double* out_hv, int64_t n_nodes, int64_t n_face_nodes,
                     const double* scale, int64_t n_elements) {
    if (!lift || !flux_diff_h || !flux_diff_hu || !flux_diff_hv || !out_h || !out_hu || !out_hv ||
        !scale || n_nodes < 1 || n_nodes > kMaxNodes || n_face_nodes < 1 ||
        n_face_nodes > n_nodes || n_elements < 0)
        return helper_fail(DGSWE_ERR_INVALID,
                           "apply_lift: a NULL pointer, or %lld nodes, %lld face nodes and %lld "
                           "elements", (long long)n_nodes, (long long)n_face_nodes,
                           (long long)n_elements);
    if (int s = prepare(device, "apply_lift")) return s;
    const int64_t total = n_nodes * n_elements;
    if (total == 0) return DGSWE_OK;
    lift_kernel<<<blocks_for(total, kThreads), kThreads>>>(
        lift, flux_diff_h, flux_diff_hu, flux_diff_hv, out_h, out_hu, out_hv, scale, (int)n_nodes,
        (int)n_face_nodes, total);
    return finish("apply_lift");
}

int dgswe_coriolis_source(int device, const double* hu, const double* hv, double* out_hu,
                          double* out_hv, double f, int64_t n_values) {
    if (!hu || !hv || !out_hu || !out_hv || n_values < 0)
        return helper_fail(DGSWE_ERR_INVALID, "coriolis_source: a NULL pointer or %lld values",
                           (long long)n_values);
    if (int s = prepare(device, "coriolis_source")) return s;
    if (n_values == 0) return DGSWE_OK;
    coriolis_kernel<<<blocks_for(n_values, kThreads), kThreads>>>(hu, hv, out_hu, out_hv, f,
                                                                   n_values);
    return finish("coriolis_source");
}

int dgswe_combine_derivatives(int device, const double* const derivatives[12], double* out_h,
                              double* out_hu, double* out_hv, const double* metric,
                              int64_t n_nodes, int64_t n_elements) {
    if (!derivatives || !out_h || !out_hu || !out_hv || !metric || n_nodes < 1 || n_elements < 0)
        return helper_fail(DGSWE_ERR_INVALID,
                           "combine_derivatives: a NULL pointer, or %lld nodes and %lld elements",
                           (long long)n_nodes, (long long)n_elements);
    Twelve in{};
    for (int c = 0; c < 12; ++c) {
        if (!derivatives[c])
            return helper_fail(DGSWE_ERR_INVALID, "combine_derivatives: derivative %d is NULL", c);
        in.p[c] = derivatives[c];
    }
    if (int s = prepare(device, "combine_derivatives")) return s;
    const int64_t total = n_nodes * n_elements;
    if (total == 0) return DGSWE_OK;
    combine_kernel<<<blocks_for(total, kThreads), kThreads>>>(in, out_h, out_hu, out_hv, metric,
                                                              (int)n_nodes, total);
    return finish("combine_derivatives");
}

}  // extern "C"
