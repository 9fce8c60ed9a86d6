// Oracle — test infrastructure only (see pointwise.hpp). A CPU restatement
// of the reference's 2D shallow-water split-form RHS, its fused SSP stage,
// time-step bound and run loop (EmilLindfors/dgcom), for checking the CUDA
// library and for timing the CPU baseline. Each function cites the
// reference file:line it follows. Built with -ffp-contract=off; OpenMP runs
// the element loops in parallel (each element's result does not depend on
// the thread count, as in the reference's rayon loops).
//
// Parity is pinned only through the reference's own known-answer and
// property tests: the reference is Rust and no Rust toolchain exists where
// this is built, so no output of the reference itself was available.
// The 1D differentiation matrix is the exact Lagrange derivative at the
// reference's GLL nodes evaluated in long double; the reference inverts a
// Vandermonde matrix with faer (src/operators/differentiation.rs:19-36), so
// the last bits of D are not pinned.

#include "oracle.h"

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <string>
#include <unordered_map>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "pointwise.hpp"

namespace oracle {

static const double INF = std::numeric_limits<double>::infinity();

// ---------------------------------------------------------------------------
// Operators (src/operators/operators_2d.rs:114-190, src/polynomial/nodes.rs)

// legendre_and_derivative (src/polynomial/legendre.rs:62-94)
static void legendre_and_derivative(int n, double x, double& p, double& dp) {
    if (n == 0) {
        p = 1.0;
        dp = 0.0;
        return;
    }
    if (n == 1) {
        p = x;
        dp = 1.0;
        return;
    }
    double p_prev = 1.0, p_curr = x;
    for (int k = 1; k < n; ++k) {
        double p_next = ((double)(2 * k + 1) * x * p_curr - (double)k * p_prev) / (double)(k + 1);
        p_prev = p_curr;
        p_curr = p_next;
    }
    p = p_curr;
    if (std::fabs(x - 1.0) < 1e-14)
        dp = (double)(n * (n + 1)) / 2.0;
    else if (std::fabs(x + 1.0) < 1e-14)
        dp = (n % 2 == 0 ? -1.0 : 1.0) * (double)(n * (n + 1)) / 2.0;
    else
        dp = (double)n * (x * p_curr - p_prev) / (x * x - 1.0);
}

static double legendre(int n, double x) {
    double p, dp;
    legendre_and_derivative(n, x, p, dp);
    return p;
}

struct Ops {
    int order = 0, n1 = 0, nn = 0;
    std::vector<double> x1, w1, d1;  // GLL nodes, weights, D row-major
    std::vector<double> nodes_r, nodes_s, w2;
    int face_nodes[4][8];
    std::vector<double> lift;  // [face][node][fi]

    double lift_at(int face, int node, int fi) const { return lift[(face * nn + node) * n1 + fi]; }

    explicit Ops(int order_) : order(order_), n1(order_ + 1), nn((order_ + 1) * (order_ + 1)) {
        const int n = order;
        // gauss_lobatto_nodes (src/polynomial/nodes.rs:17-77)
        x1.resize(n1);
        for (int j = 0; j <= n; ++j) x1[j] = -std::cos(M_PI * (double)j / (double)n);
        x1[0] = -1.0;
        x1[n] = 1.0;
        for (int j = 1; j < n; ++j) {
            double x = x1[j];
            for (int it = 0; it < 100; ++it) {
                double p, dp;
                legendre_and_derivative(n, x, p, dp);
                double update = (1.0 - x * x) * dp / ((double)n * (double)(n + 1) * p);
                if (std::fabs(update) < 1e-15) break;
                x += update;
            }
            x1[j] = x;
        }
        // gauss_lobatto_weights (src/polynomial/nodes.rs:82-103)
        w1.resize(n1);
        double denom = (double)(n * (n + 1));
        for (int j = 0; j < n1; ++j) {
            double p = legendre(n, x1[j]);
            w1[j] = 2.0 / (denom * p * p);
        }
        // D: exact Lagrange derivative at these nodes (barycentric, long double)
        d1.assign(n1 * n1, 0.0);
        std::vector<long double> lam(n1);
        for (int j = 0; j < n1; ++j) {
            long double prod = 1.0L;
            for (int k = 0; k < n1; ++k)
                if (k != j) prod *= ((long double)x1[j] - (long double)x1[k]);
            lam[j] = 1.0L / prod;
        }
        for (int i = 0; i < n1; ++i) {
            long double diag = 0.0L;
            for (int j = 0; j < n1; ++j) {
                if (j == i) continue;
                long double dij = (lam[j] / lam[i]) / ((long double)x1[i] - (long double)x1[j]);
                d1[i * n1 + j] = (double)dij;
                diag -= dij;
            }
            double dd = (double)diag;
            d1[i * n1 + i] = std::fabs(dd) < 1e-14 ? 0.0 : dd;
        }
        // tensor_product_gll_nodes / weights (src/polynomial/legendre_2d.rs:108-144)
        nodes_r.resize(nn);
        nodes_s.resize(nn);
        w2.resize(nn);
        for (int j = 0; j < n1; ++j)
            for (int a = 0; a < n1; ++a) {
                nodes_r[j * n1 + a] = x1[a];
                nodes_s[j * n1 + a] = x1[j];
                w2[j * n1 + a] = w1[a] * w1[j];
            }
        // compute_face_nodes (src/operators/operators_2d.rs:388-412)
        for (int a = 0; a < n1; ++a) face_nodes[0][a] = a;
        for (int j = 0; j < n1; ++j) face_nodes[1][j] = j * n1 + (n1 - 1);
        for (int q = 0; q < n1; ++q) face_nodes[2][q] = (n1 - 1) * n1 + (n1 - 1 - q);
        for (int q = 0; q < n1; ++q) face_nodes[3][q] = (n1 - 1 - q) * n1;
        // compute_lift_matrices (src/operators/operators_2d.rs:445-482):
        // LIFT[face][i][j] = (1/w_i)·(E_f[j][i]·w1[j])
        lift.assign(4 * nn * n1, 0.0);
        for (int face = 0; face < 4; ++face)
            for (int i = 0; i < nn; ++i)
                for (int j = 0; j < n1; ++j) {
                    double e = face_nodes[face][j] == i ? 1.0 : 0.0;
                    double mass_inv = 1.0 / w2[i];
                    lift[(face * nn + i) * n1 + j] = mass_inv * (e * w1[j]);
                }
    }
};

// ---------------------------------------------------------------------------
// Mesh (src/mesh/core/mesh2d.rs:456-620): Mesh2D::from_quads

struct ElementFace {
    int64_t element;
    int face;
};

struct Edge {
    ElementFace left;
    ElementFace right;  // element < 0: boundary
    int32_t tag;
};

struct Mesh {
    std::vector<std::array<double, 2>> vertices;
    std::vector<std::array<int64_t, 4>> elements;
    std::vector<Edge> edges;
    std::vector<std::array<int64_t, 4>> element_edges;
    // FaceLink (src/mesh/core/mesh2d.rs:54-110) unpacked
    struct Link {
        int64_t element = -1;  // -1: boundary
        int face = 0;
        bool left = false, shared = false;
    };
    std::vector<std::array<Link, 4>> links;
    int64_t n_elements = 0;

    std::array<std::array<double, 2>, 4> corners(int64_t k) const {
        std::array<std::array<double, 2>, 4> c;
        for (int i = 0; i < 4; ++i) c[i] = vertices[elements[k][i]];
        return c;
    }

    // Mesh2D::neighbor (src/mesh/core/mesh2d.rs:669-678)
    bool neighbor(int64_t k, int face, ElementFace& nb) const {
        const Edge& e = edges[element_edges[k][face]];
        if (e.left.element == k && e.left.face == face) {
            if (e.right.element < 0) return false;
            nb = e.right;
            return true;
        }
        nb = e.left;
        return true;
    }
};

static std::string build_mesh(const dgswe_form* f, Mesh& m) {
    m.n_elements = f->n_elements;
    m.vertices.resize(f->n_vertices);
    for (int64_t i = 0; i < f->n_vertices; ++i)
        m.vertices[i] = {f->vertices[2 * i], f->vertices[2 * i + 1]};
    m.elements.resize(f->n_elements);
    for (int64_t k = 0; k < f->n_elements; ++k)
        for (int c = 0; c < 4; ++c) {
            int64_t v = f->elements[4 * k + c];
            if (v < 0 || v >= f->n_vertices) return "element uses a vertex that does not exist";
            m.elements[k][c] = v;
        }
    auto face_vertices = [&](ElementFace fc) {
        auto q = m.elements[fc.element];
        return std::make_pair(q[fc.face], q[(fc.face + 1) % 4]);
    };
    auto key = [](std::pair<int64_t, int64_t> p) {
        return std::make_pair(std::min(p.first, p.second), std::max(p.first, p.second));
    };
    std::map<std::pair<int64_t, int>, int64_t> pair_of;
    for (int64_t p = 0; p < f->n_periodic; ++p) {
        for (int s = 0; s < 2; ++s) {
            int64_t e = f->periodic[4 * p + 2 * s];
            int fc = (int)f->periodic[4 * p + 2 * s + 1];
            if (e < 0 || e >= f->n_elements || fc < 0 || fc >= 4) return "invalid periodic face";
            if (!pair_of.emplace(std::make_pair(e, fc), p).second) return "periodic face paired twice";
        }
    }
    struct PairHash {
        size_t operator()(const std::pair<int64_t, int64_t>& p) const {
            return std::hash<int64_t>()(p.first * 1000003 + p.second);
        }
    };
    std::unordered_map<std::pair<int64_t, int64_t>, int64_t, PairHash> edge_of_key;
    edge_of_key.reserve(2 * f->n_elements + 16);
    std::vector<int64_t> edge_of_pair(f->n_periodic, -1);
    m.element_edges.assign(f->n_elements, {-1, -1, -1, -1});
    m.edges.reserve(2 * f->n_elements + 64);
    for (int64_t k = 0; k < f->n_elements; ++k) {
        for (int fc = 0; fc < 4; ++fc) {
            ElementFace face{k, fc};
            auto it = pair_of.find({k, fc});
            if (it != pair_of.end()) {
                int64_t p = it->second;
                if (edge_of_pair[p] < 0) {
                    ElementFace l{f->periodic[4 * p], (int)f->periodic[4 * p + 1]};
                    ElementFace r{f->periodic[4 * p + 2], (int)f->periodic[4 * p + 3]};
                    edge_of_pair[p] = (int64_t)m.edges.size();
                    m.edges.push_back({l, r, 0});
                }
                m.element_edges[k][fc] = edge_of_pair[p];
                continue;
            }
            auto ab = face_vertices(face);
            auto kk = key(ab);
            auto found = edge_of_key.find(kk);
            if (found == edge_of_key.end()) {
                edge_of_key.emplace(kk, (int64_t)m.edges.size());
                m.element_edges[k][fc] = (int64_t)m.edges.size();
                m.edges.push_back({face, {-1, 0}, 0});
            } else {
                Edge& e = m.edges[found->second];
                if (e.right.element >= 0) return "an edge is shared by more than two elements";
                auto lv = face_vertices(e.left);
                if (!(lv.first == ab.second && lv.second == ab.first))
                    return "two faces traverse their shared edge in the same direction";
                e.right = face;
                m.element_edges[k][fc] = found->second;
            }
        }
    }
    for (int64_t p = 0; p < f->n_periodic; ++p)
        for (int s = 0; s < 2; ++s) {
            ElementFace fc{f->periodic[4 * p + 2 * s], (int)f->periodic[4 * p + 2 * s + 1]};
            if (edge_of_key.count(key(face_vertices(fc)))) return "periodic face shared with another";
        }
    for (auto& e : m.edges)
        if (e.right.element < 0)
            e.tag = f->face_tags ? f->face_tags[4 * e.left.element + e.left.face] : 0;
    m.links.assign(f->n_elements, {});
    for (auto& e : m.edges) {
        if (e.right.element < 0) continue;
        auto lv = face_vertices(e.left);
        auto rv = face_vertices(e.right);
        bool shared = rv.first == lv.second && rv.second == lv.first;
        m.links[e.left.element][e.left.face] = {e.right.element, e.right.face, true, shared};
        m.links[e.right.element][e.right.face] = {e.left.element, e.left.face, false, shared};
    }
    return "";
}

// ---------------------------------------------------------------------------
// Geometry (src/operators/geometric.rs:126-221)

struct Metric {
    double x_r, x_s, y_r, y_s, det;
};

// BilinearMetric::at (src/operators/geometric.rs:704-718)
static Metric bilinear_metric(const std::array<std::array<double, 2>, 4>& v, double r, double s) {
    double x0 = v[0][0], y0 = v[0][1], x1 = v[1][0], y1 = v[1][1];
    double x2 = v[2][0], y2 = v[2][1], x3 = v[3][0], y3 = v[3][1];
    Metric m;
    m.x_r = 0.25 * ((1.0 - s) * (x1 - x0) + (1.0 + s) * (x2 - x3));
    m.y_r = 0.25 * ((1.0 - s) * (y1 - y0) + (1.0 + s) * (y2 - y3));
    m.x_s = 0.25 * ((1.0 - r) * (x3 - x0) + (1.0 + r) * (x2 - x1));
    m.y_s = 0.25 * ((1.0 - r) * (y3 - y0) + (1.0 + r) * (y2 - y1));
    m.det = m.x_r * m.y_s - m.x_s * m.y_r;
    return m;
}

// is_parallelogram (src/operators/geometric.rs:722-733)
static bool is_parallelogram(const std::array<std::array<double, 2>, 4>& v) {
    double bx = v[0][0] - v[1][0] + v[2][0] - v[3][0];
    double by = v[0][1] - v[1][1] + v[2][1] - v[3][1];
    double scale = 0.0;
    for (int i = 0; i < 4; ++i) {
        auto a = v[i], b = v[(i + 1) % 4];
        scale = fmax_(scale, std::hypot(b[0] - a[0], b[1] - a[1]));
    }
    return std::hypot(bx, by) <= 1.0e-12 * scale;
}

struct Geometry {
    int nn = 0, n1 = 0;
    std::vector<double> rx, ry, sx, sy, det_j, det_j_inv, mass, area;
    std::vector<double> surface_j, nxv, nyv;  // per face node
    std::vector<uint8_t> affine;

    size_t fidx(int64_t k, int face, int fi) const { return ((size_t)k * 4 + face) * n1 + fi; }
    size_t nidx(int64_t k, int i) const { return (size_t)k * nn + i; }
    // contravariant (src/operators/geometric.rs:309-317)
    void contravariant(int64_t k, int i, double& rx0, double& rx1, double& sx0, double& sx1) const {
        size_t n = nidx(k, i);
        double j = det_j[n];
        rx0 = j * rx[n];
        rx1 = j * ry[n];
        sx0 = j * sx[n];
        sx1 = j * sy[n];
    }
};

static std::string build_geometry(const Mesh& mesh, const Ops& ops, Geometry& g) {
    int64_t K = mesh.n_elements;
    g.nn = ops.nn;
    g.n1 = ops.n1;
    size_t nv = (size_t)K * ops.nn, nf = (size_t)K * 4 * ops.n1;
    g.rx.resize(nv);
    g.ry.resize(nv);
    g.sx.resize(nv);
    g.sy.resize(nv);
    g.det_j.resize(nv);
    g.det_j_inv.resize(nv);
    g.mass.resize(nv);
    g.area.resize(K);
    g.surface_j.resize(nf);
    g.nxv.resize(nf);
    g.nyv.resize(nf);
    g.affine.resize(K);
    bool bad = false;
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < K; ++k) {
        auto v = mesh.corners(k);
        g.affine[k] = is_parallelogram(v) ? 1 : 0;
        double area = 0.0;
        for (int i = 0; i < ops.nn; ++i) {
            Metric m = bilinear_metric(v, ops.nodes_r[i], ops.nodes_s[i]);
            if (!(std::isfinite(m.det) && m.det > 0.0)) bad = true;
            size_t n = g.nidx(k, i);
            g.rx[n] = m.y_s / m.det;
            g.ry[n] = -m.x_s / m.det;
            g.sx[n] = -m.y_r / m.det;
            g.sy[n] = m.x_r / m.det;
            g.det_j[n] = m.det;
            g.det_j_inv[n] = 1.0 / m.det;
            double mass = ops.w2[i] * m.det;
            g.mass[n] = mass;
            area += mass;
        }
        g.area[k] = area;
        for (int face = 0; face < 4; ++face)
            for (int fi = 0; fi < ops.n1; ++fi) {
                int node = ops.face_nodes[face][fi];
                Metric m = bilinear_metric(v, ops.nodes_r[node], ops.nodes_s[node]);
                double vx, vy;
                switch (face) {
                    case 0: vx = m.y_r; vy = -m.x_r; break;
                    case 1: vx = m.y_s; vy = -m.x_s; break;
                    case 2: vx = -m.y_r; vy = m.x_r; break;
                    default: vx = -m.y_s; vy = m.x_s; break;
                }
                double s_j = std::sqrt(vx * vx + vy * vy);
                size_t fn = g.fidx(k, face, fi);
                g.surface_j[fn] = s_j;
                g.nxv[fn] = vx / s_j;
                g.nyv[fn] = vy / s_j;
            }
    }
    if (bad) return "GeometricFactors2D requires a positive finite Jacobian (degenerate, non-convex or clockwise element)";
    return "";
}

// ---------------------------------------------------------------------------
// The model: the form, its boundary conditions and buffers

// TimeStencil::new (src/io/field_series.rs:41-81): the snapshots' Lagrange
// weights at `time`, linear between the bracketing two or cubic through up
// to four; false outside [times[0], times[n − 1]]
static bool time_stencil(const double* times, int64_t n, double time, bool cubic, int64_t idx[4],
                         double w[4], int& len) {
    auto single = [&](int64_t k) {
        idx[0] = k;
        w[0] = 1.0;
        len = 1;
        return true;
    };
    if (n == 0) return false;
    if (n == 1) return single(0);
    if (!(time >= times[0] && time <= times[n - 1])) return false;
    int64_t i1 = std::partition_point(times, times + n, [&](double t) { return t < time; }) - times;
    i1 = i1 < 1 ? 1 : (i1 > n - 1 ? n - 1 : i1);
    int64_t i0 = i1 - 1;
    if (time == times[i0]) return single(i0);
    if (time == times[i1]) return single(i1);
    int64_t lo = cubic ? (i0 > 0 ? i0 - 1 : 0) : i0;
    int64_t hi = cubic ? std::min(i1 + 1, n - 1) : i1;
    len = (int)(hi - lo + 1);
    for (int64_t a = lo; a <= hi; ++a) {
        double p = 1.0;
        for (int64_t b = lo; b <= hi; ++b)
            if (b != a) p *= (time - times[b]) / (times[a] - times[b]);
        idx[a - lo] = a;
        w[a - lo] = p;
    }
    return true;
}

struct Boundary {
    int kind = DGSWE_BC_WALL;
    double wall_h_min = 1e-6;
    // InverseBarometer (src/boundary/characteristic.rs:273-340)
    bool raise = false;
    double raise_factor = 0.0;
    int elevation_only = DGSWE_AT_REST;
    std::vector<dgswe_tide_constituent> constituents;
    double mean_elevation = 0.0, ramp_duration = 0.0;
    // BoundaryTides (src/boundary/tidal_atlas.rs:855-1070), a copy
    struct NodeTides {
        int n = 0;
        std::vector<double> omega, f_rate, positions, coefficients, mean, source_depth;
        std::vector<uint32_t> slot_of_node;
        bool velocity = false, use_mean = false;
        double max_ratio = 0.0, ramp = 0.0;
        int64_t n_slots = 0;
    } tides;
    // OceanModelState's boundary data (src/boundary/ocean_nesting.rs), a copy
    struct Parent {
        int64_t n_slots = 0, n_times = 0;
        std::vector<double> positions, times, depth;
        std::vector<float> values;  // [slot][time][3]
        std::vector<uint8_t> on_boundary;
        std::vector<uint32_t> slot_of_node;
        bool cubic = false, velocity = false;
        double reference_level = 0.0, max_ratio = 0.0, ramp = 0.0;
    } parent;

    // OceanModelState::slot_of (ocean_nesting.rs:543-562)
    int64_t parent_slot_of(int64_t node_index, double x, double y) const {
        if (!parent.slot_of_node.empty() && parent.slot_of_node[node_index] != 0xFFFFFFFFu)
            return parent.slot_of_node[node_index];
        int64_t best = -1;
        double dmin = INF;
        for (int64_t p = 0; p < parent.n_slots; ++p) {
            if (!parent.on_boundary.empty() && !parent.on_boundary[p]) continue;
            double d = std::hypot(parent.positions[2 * p] - x, parent.positions[2 * p + 1] - y);
            if (best < 0 || d < dmin) {
                dmin = d;
                best = p;
            }
        }
        return best;
    }

    // OceanModelState::external_state (ocean_nesting.rs:821-826): evaluate
    // with parent_term and parent_state (ocean_nesting.rs:833-880)
    void parent_external(int64_t slot, double t, double bed, double& eta, double& u, double& v,
                         bool& has_uv) const {
        int64_t idx[4];
        double w[4];
        int len = 0;
        if (!time_stencil(parent.times.data(), parent.n_times, t, parent.cubic, idx, w, len)) {
            eta = u = v = NAN;  // the reference panics: a configuration error
            has_uv = parent.velocity;
            return;
        }
        double sum[3] = {0.0, 0.0, 0.0};
        for (int k = 0; k < len; ++k) {
            const float* q = &parent.values[((size_t)slot * parent.n_times + idx[k]) * 3];
            sum[0] += w[k] * (double)q[0];
            sum[1] += w[k] * (double)q[1];
            sum[2] += w[k] * (double)q[2];
        }
        double ramp = tidal_ramp(t, parent.ramp);
        double zeta = ramp * sum[0];
        u = ramp * sum[1];
        v = ramp * sum[2];
        eta = zeta + ramp * parent.reference_level;
        has_uv = parent.velocity;
        if (has_uv && parent.max_ratio > 0.0 && std::isfinite(parent.depth[slot])) {
            double d_parent = zeta + parent.depth[slot], d_child = eta - bed;
            if (d_parent > 0.0 && d_child > 0.0) {
                double ratio = d_parent / d_child;
                double lo = 1.0 / parent.max_ratio;
                ratio = ratio < lo ? lo : (ratio > parent.max_ratio ? parent.max_ratio : ratio);
                u *= ratio;
                v *= ratio;
            }
        }
    }

    // BoundaryTides::slot_of (tidal_atlas.rs:1026-1045)
    int64_t slot_of(int64_t node_index, double x, double y) const {
        if (!tides.slot_of_node.empty() && tides.slot_of_node[node_index] != 0xFFFFFFFFu)
            return tides.slot_of_node[node_index];
        int64_t best = 0;
        double dmin = INF;
        for (int64_t p = 0; p < tides.n_slots; ++p) {
            double d = std::hypot(tides.positions[2 * p] - x, tides.positions[2 * p + 1] - y);
            if (d < dmin) {
                dmin = d;
                best = p;
            }
        }
        return best;
    }

    // BoundaryTides::external_state (tidal_atlas.rs:1049-1065): η and, with
    // velocity, (u, v) over the child bed `bed`
    void node_external(int64_t slot, double t, double bed, double& eta, double& u, double& v,
                       bool& has_uv) const {
        const int n = tides.n;
        double sum[3] = {0.0, 0.0, 0.0};
        for (int j = 0; j < n; ++j) {
            double f = 1.0 + tides.f_rate[j] * t;
            double x = tides.omega[j] * t;
            double sn = std::sin(x), cs = std::cos(x);
            const double* c = &tides.coefficients[((size_t)slot * n + j) * 6];
            sum[0] += f * (c[0] * cs + c[1] * sn);  // tide_term (tidal_atlas.rs:1078-1082)
            sum[1] += f * (c[2] * cs + c[3] * sn);
            sum[2] += f * (c[4] * cs + c[5] * sn);
        }
        double ramp = tidal_ramp(t, tides.ramp);
        double mean = tides.use_mean ? tides.mean[slot] : 0.0;
        eta = mean + ramp * sum[0];  // tide_level (tidal_atlas.rs:1088-1091)
        u = ramp * sum[1];
        v = ramp * sum[2];
        has_uv = tides.velocity;
        if (has_uv && tides.max_ratio > 0.0) {  // tide_state (tidal_atlas.rs:1100-1131)
            double h_source = tides.source_depth[slot];
            double d_source = h_source + eta, d_child = eta - bed;
            if (h_source > 0.0 && d_source > 0.0 && d_child > 0.0) {
                double ratio = d_source / d_child;
                double lo = 1.0 / tides.max_ratio;
                ratio = ratio < lo ? lo : (ratio > tides.max_ratio ? tides.max_ratio : ratio);
                u *= ratio;
                v *= ratio;
            }
        }
    }

    // HarmonicTide::elevation (src/boundary/harmonic_tide.rs:124-136)
    double elevation(double t) const {
        double tide = 0.0;
        for (const auto& c : constituents) {
            double f = c.f + c.f_rate * t;
            double u_deg = c.u_deg + c.u_rate_deg * t;
            double omega = 2.0 * M_PI / c.period;
            double offset = (c.v0_deg + u_deg) * (M_PI / 180.0);
            tide += f * c.amplitude * std::cos(omega * t + c.phase + offset);
        }
        return mean_elevation + tidal_ramp(t, ramp_duration) * tide;
    }
};

struct Buffer {
    std::vector<double> h, hu, hv;
    void resize(size_t n) {
        h.assign(n, 0.0);
        hu.assign(n, 0.0);
        hv.assign(n, 0.0);
    }
    State get(size_t i) const { return {h[i], hu[i], hv[i]}; }
};

// NestingRelaxation2D (src/boundary/ocean_nesting.rs:900-1065): the parent
// (a Boundary holding its series) and each slot's weight
struct Relaxation {
    bool on = false;
    Boundary parent;
    std::vector<double> weight;
    double rate = 0.0, wet_depth = 0.0;
    bool momentum_only = false;
};

// GriddedAtmosphere2D (src/source/swe_2d/gridded_atmosphere.rs:60-900) as
// the device form holds it: the snapshots regridded onto the nodes
// ([time][node][5]: u, v, ∂p/∂x, ∂p/∂y, p − p_ref, f32) and the options
struct Atmosphere {
    bool on = false, source = false, wind = false, pressure = false, level = false;
    int drag = 1;
    double cd = 0.0, rho_air = 1.225, rho_water = 1025.0, h_min = 0.01, ramp = 0.0, epoch = 0.0;
    std::vector<double> times;
    std::vector<float> values;
    size_t n_nodes = 0;

    // The weather at flat node g and simulation time t: the linear time
    // stencil at epoch + t (time_stencil), the snapshots summed in turn from
    // zero (add_snapshot, :143-150; cached, :680-688). Outside the snapshots
    // the nearest end (the reference panics there; the runs refuse it).
    void at(size_t g, double t, double out[5]) const {
        int64_t idx[4] = {0, 0, 0, 0};
        double w[4] = {1.0, 0.0, 0.0, 0.0};
        int len = 1;
        const int64_t n = (int64_t)times.size();
        if (!time_stencil(times.data(), n, epoch + t, false, idx, w, len)) {
            idx[0] = epoch + t < times[0] ? 0 : n - 1;
            w[0] = 1.0;
            len = 1;
        }
        for (int q = 0; q < 5; ++q) out[q] = 0.0;
        for (int j = 0; j < len; ++j) {
            const float* v = &values[((size_t)idx[j] * n_nodes + g) * 5];
            for (int q = 0; q < 5; ++q) out[q] += w[j] * (double)v[q];
        }
    }
    // BoundaryLevel::level by node index (:873-895)
    double level_at(size_t g, double t) const {
        if (!level) return 0.0;
        double s[5];
        at(g, t, s);
        return inverse_barometer_level(s[4], tidal_ramp(t, ramp), rho_water);
    }
};

struct Model {
    dgswe_form form;
    Ops ops;
    Mesh mesh;
    Geometry geom;
    std::vector<double> bed;  // per node (empty: no bathymetry)
    std::vector<double> g_n2;  // per node (friction)
    std::map<int32_t, Boundary> boundaries;
    Buffer buf[DGSWE_N_BUFFERS];
    std::vector<State> faces;  // face pass output: [edge][side][fi]
    int64_t clips = 0;
    std::string error;
    WetDry wd;
    bool has_bed = false;
    Relaxation relax;
    Atmosphere atm;

    explicit Model(int order) : ops(order) {}
    size_t n_values() const { return (size_t)mesh.n_elements * ops.nn; }
    double bed_at(int64_t k, int i) const { return has_bed ? bed[(size_t)k * ops.nn + i] : 0.0; }
};

// ---------------------------------------------------------------------------
// RHS: SplitFormSWE2D (src/solver/rhs/swe_2d_split_form.rs:500-1123)

struct Workspace {
    std::vector<Node> nodes;
    std::vector<State> rhs;
    std::vector<std::pair<double, double>> metric, interfaces;
    std::vector<std::pair<Side, Side>> faces;
    struct Outer {
        bool present = false;
        Node node;
        double distance = 0.0;
    };
    std::vector<Outer> outer;
    // compute_rhs_swe_2d_mass_fluxes_into's outputs of the element being
    // computed (src/solver/rhs/swe_2d.rs:1017-1075), or null: the mass
    // component of F* at its 4·n1 face nodes and the mass flux through its
    // 2·n1·(n1 − 1) subcell interfaces
    double* face_mass = nullptr;
    double* subcell_mass = nullptr;
    explicit Workspace(const Ops& ops)
        : nodes(ops.nn), rhs(ops.nn), metric(ops.n1), interfaces(ops.n1 + 1), faces(ops.n1),
          outer(4 * ops.n1) {}
};

enum class SurfaceFlux { EntropyConservative, EntropyStable, HydrostaticHll };

static SurfaceFlux surface_kind(const Model& m) {
    switch (m.form.formulation) {
        case DGSWE_ENTROPY_CONSERVATIVE: return SurfaceFlux::EntropyConservative;
        case DGSWE_ENTROPY_STABLE: return SurfaceFlux::EntropyStable;
        default: return SurfaceFlux::HydrostaticHll;
    }
}

// SplitFormSWE2D::surface_flux (src/solver/rhs/swe_2d_split_form.rs:618-651)
static void surface_flux(const Model& m, const Node& qa, const Node& qb, double nx, double ny,
                         State& fa, State& fb) {
    double g = m.form.g;
    SurfaceFlux kind = surface_kind(m);
    if (kind == SurfaceFlux::HydrostaticHll) {
        State a, b;
        hydrostatic_hll(side_of(qa), side_of(qb), nx, ny, g, m.form.h_min, a, b);
        fa = a;
        fb = -b;
        return;
    }
    State shared = wintermeyer_flux(qa, qb, nx, ny, g);
    if (kind == SurfaceFlux::EntropyStable) shared = shared + entropy_stable_dissipation(qa, qb, nx, ny, g);
    fa = shared + bed_interface_term(qa.h, qa.b, qb.b, nx, ny, g);
    fb = -shared + bed_interface_term(qb.h, qb.b, qa.b, -nx, -ny, g);
}

static Node node_at(const Model& m, const Buffer& q, int64_t k, int i) {
    size_t n = (size_t)k * m.ops.nn + i;
    return make_node(q.get(n), m.bed_at(k, i), m.form.h_min);
}

// The face normal of an element face node as the kernels read it: a
// parallelogram's face-node-0 value, else the node's own
static void face_normal(const Model& m, int64_t k, int face, int fi, double& nx, double& ny,
                        double& s_j) {
    const Geometry& g = m.geom;
    size_t fn = g.affine[k] ? g.fidx(k, face, 0) : g.fidx(k, face, fi);
    nx = g.nxv[fn];
    ny = g.nyv[fn];
    s_j = g.surface_j[fn];
}

// SplitFormSWE2D::edge_fluxes (src/solver/rhs/swe_2d_split_form.rs:580-616)
static void edge_fluxes(const Model& m, const Buffer& q, int64_t e, State* out) {
    const Edge& edge = m.mesh.edges[e];
    if (edge.right.element < 0) return;
    int n1 = m.ops.n1;
    for (int fi = 0; fi < n1; ++fi) {
        double nx, ny, sj;
        face_normal(m, edge.left.element, edge.left.face, fi, nx, ny, sj);
        int left_node = m.ops.face_nodes[edge.left.face][fi];
        int rfi = n1 - 1 - fi;
        int right_node = m.ops.face_nodes[edge.right.face][rfi];
        State fl, fr;
        surface_flux(m, node_at(m, q, edge.left.element, left_node),
                     node_at(m, q, edge.right.element, right_node), nx, ny, fl, fr);
        out[fi] = fl;
        out[n1 + rfi] = fr;
    }
}

// boundary_state (src/solver/rhs/swe_2d.rs:304-327) and
// SplitFormSWE2D::boundary_flux (src/solver/rhs/swe_2d_split_form.rs:1090-1123)
static State boundary_flux(const Model& m, int64_t k, int face, int node, const Node& q_int,
                           double nx, double ny, double time, int32_t tag) {
    double g = m.form.g, h_min = m.form.h_min;
    auto it = m.boundaries.find(tag);
    const Boundary& bc = it->second;
    State interior{q_int.h, q_int.hu, q_int.hv};
    if (bc.kind == DGSWE_BC_WALL) {
        // Reflective2D::ghost_state (src/boundary/boundary_2d.rs:271-283)
        State ghost;
        if (interior.h <= bc.wall_h_min) {
            ghost = {interior.h, 0.0, 0.0};
        } else {
            double u, v, ur, vr;
            velocity_simple(interior, h_min, u, v);  // BCContext2D::interior_velocity
            reflect_velocity(u, v, nx, ny, ur, vr);
            ghost = {interior.h, interior.h * ur, interior.h * vr};
        }
        Node q_ext = make_node(ghost, q_int.b, h_min);
        State fa, fb;
        surface_flux(m, q_int, q_ext, nx, ny, fa, fb);
        return fa;
    }
    // CharacteristicOBC: characteristic_boundary_state
    // (src/boundary/characteristic.rs:411-437) with a uniform tide or the
    // tide per boundary node
    double bathy = q_int.b;
    double eta, ue = 0.0, ve = 0.0;
    bool has_uv = false;
    if (bc.kind == DGSWE_BC_NODE_TIDES || bc.kind == DGSWE_BC_PARENT) {
        auto c = m.mesh.corners(k);
        double r = m.ops.nodes_r[node], sv = m.ops.nodes_s[node];
        double n0 = (1 - r) * (1 - sv) / 4, n1b = (1 + r) * (1 - sv) / 4;
        double n2 = (1 + r) * (1 + sv) / 4, n3 = (1 - r) * (1 + sv) / 4;
        double x = n0 * c[0][0] + n1b * c[1][0] + n2 * c[2][0] + n3 * c[3][0];
        double y = n0 * c[0][1] + n1b * c[1][1] + n2 * c[2][1] + n3 * c[3][1];
        if (bc.kind == DGSWE_BC_PARENT) {
            int64_t slot = bc.parent_slot_of(k * m.ops.nn + node, x, y);
            bc.parent_external(slot, time, bathy, eta, ue, ve, has_uv);
        } else {
            int64_t slot = bc.slot_of(k * m.ops.nn + node, x, y);
            bc.node_external(slot, time, bathy, eta, ue, ve, has_uv);
        }
    } else {
        eta = bc.elevation(time);
    }
    // InverseBarometer::external_state: raised by the weather's level at the
    // face node (GriddedAtmosphere2D's level by node index)
    if (bc.raise) eta += bc.raise_factor * m.atm.level_at((size_t)k * m.ops.nn + node, time);
    double h_e = fmax_(eta - bathy, 0.0);
    double un_e = 0.0, ut_e;
    if (has_uv) {
        un_e = ue * nx + ve * ny;
        ut_e = -ue * ny + ve * nx;
    } else {
        if (bc.elevation_only == DGSWE_INCOMING_WAVE)
            un_e = 2.0 * (std::sqrt(g * fmax_(-bathy, 0.0)) - std::sqrt(g * h_e));
        double u, v;
        velocity_simple(interior, h_min, u, v);
        ut_e = -u * ny + v * nx;
    }
    State qb = characteristic_state(interior, h_e, un_e, ut_e, nx, ny, g, h_min);
    Node nb = make_node(qb, q_int.b, h_min);
    (void)k;
    (void)face;
    (void)node;
    return wintermeyer_flux(nb, nb, nx, ny, g);  // F(q_b)·n
}

// telescoped_interfaces (src/solver/rhs/subcells.rs:63-92)
static void telescoped_interfaces(const Ops& ops, const std::vector<std::pair<double, double>>& metric,
                                  bool affine, std::vector<std::pair<double, double>>& out) {
    int n1 = ops.n1;
    if (affine) {
        for (int a = 0; a <= n1; ++a) out[a] = metric[0];
        return;
    }
    out[0] = metric[0];
    double m0 = 0.0, m1 = 0.0;
    for (int a = 0; a < n1 - 1; ++a) {
        for (int c = 0; c < n1; ++c) {
            if (c == a) continue;
            double q2 = 2.0 * ops.w1[a] * ops.d1[a * n1 + c];
            m0 += q2 * 0.5 * (metric[a].first + metric[c].first);
            m1 += q2 * 0.5 * (metric[a].second + metric[c].second);
        }
        out[a + 1] = {m0, m1};
    }
    out[n1] = metric[n1 - 1];
}

// SplitFormSWE2D::line_volume (src/solver/rhs/swe_2d_split_form.rs:843-894)
template <class Idx>
static void line_volume(const Model& m, Workspace& ws, Idx idx, bool affine,
                        std::pair<double, double> affine_metric) {
    const Ops& ops = m.ops;
    int n1 = ops.n1;
    const std::vector<double>& d1 = ops.d1;
    double g = m.form.g;
    for (int a = 0; a < n1; ++a) {
        int ia = idx(a);
        Node q_a = ws.nodes[ia];
        std::pair<double, double> m_a = affine ? affine_metric : ws.metric[a];
        State acc = (2.0 * d1[a * n1 + a]) * wintermeyer_flux(q_a, q_a, m_a.first, m_a.second, g);
        for (int c = a + 1; c < n1; ++c) {
            int ic = idx(c);
            std::pair<double, double> mm;
            if (affine) {
                mm = m_a;
            } else {
                auto m_c = ws.metric[c];
                mm = {0.5 * (m_a.first + m_c.first), 0.5 * (m_a.second + m_c.second)};
            }
            State f = wintermeyer_flux(q_a, ws.nodes[ic], mm.first, mm.second, g);
            acc = acc + (2.0 * d1[a * n1 + c]) * f;
            ws.rhs[ic] = ws.rhs[ic] - (2.0 * d1[c * n1 + a]) * f;
        }
        if (m.has_bed) {
            double db = 0.0, db_x = 0.0, db_y = 0.0;
            for (int c = 0; c < n1; ++c) {
                double d_b = d1[a * n1 + c] * ws.nodes[idx(c)].b;
                db += d_b;
                if (!affine) {
                    db_x += d_b * ws.metric[c].first;
                    db_y += d_b * ws.metric[c].second;
                }
            }
            double bx, by;
            if (affine) {
                bx = db * m_a.first;
                by = db * m_a.second;
            } else {
                bx = 0.5 * (db * m_a.first + db_x);
                by = 0.5 * (db * m_a.second + db_y);
            }
            double force = g * q_a.h;
            acc = acc + State{0.0, force * bx, force * by};
        }
        ws.rhs[ia] = ws.rhs[ia] - acc;
    }
}

// SplitFormSWE2D::line_subcells (src/solver/rhs/swe_2d_split_form.rs:938-1035)
template <class Idx>
static void line_subcells(const Model& m, Workspace& ws, Idx idx, const Workspace::Outer& end0,
                          const Workspace::Outer& end1, bool affine, double* mass) {
    const Ops& ops = m.ops;
    int n1 = ops.n1;
    const std::vector<double>& w = ops.w1;
    const std::vector<double>& xi = ops.x1;
    double g = m.form.g, h_min = m.form.h_min;
    double h_dry = m.form.subcell_h_dry;
    telescoped_interfaces(ops, ws.metric, affine, ws.interfaces);
    int first = idx(0), last = idx(n1 - 1);
    Node q_first = ws.nodes[first], q_last = ws.nodes[last];
    auto m_first = ws.metric[0], m_last = ws.metric[n1 - 1];
    ws.rhs[first] = ws.rhs[first] +
                    (1.0 / w[0]) * wintermeyer_flux(q_first, q_first, m_first.first, m_first.second, g);
    ws.rhs[last] = ws.rhs[last] -
                   (1.0 / w[n1 - 1]) * wintermeyer_flux(q_last, q_last, m_last.first, m_last.second, g);
    double x_left = -1.0;
    for (int a = 0; a < n1; ++a) {
        Side q = side_of(ws.nodes[idx(a)]);
        double x_right = x_left + w[a];
        bool have_l, have_r;
        Side l, r;
        double x_l = 0.0, x_r = 0.0;
        if (a > 0) {
            have_l = true;
            l = side_of(ws.nodes[idx(a - 1)]);
            x_l = xi[a - 1];
        } else {
            have_l = end0.present;
            if (have_l) {
                l = side_of(end0.node);
                x_l = -1.0 - end0.distance;
            }
        }
        if (a + 1 < n1) {
            have_r = true;
            r = side_of(ws.nodes[idx(a + 1)]);
            x_r = xi[a + 1];
        } else {
            have_r = end1.present;
            if (have_r) {
                r = side_of(end1.node);
                x_r = 1.0 + end1.distance;
            }
        }
        if (have_l && have_r) {
            Side nodes[3] = {l, q, r};
            double xs[3] = {x_l, xi[a], x_r};
            reconstruct_subcell(nodes, xs, x_left, x_right, h_dry, ws.faces[a].first, ws.faces[a].second);
        } else {
            ws.faces[a] = {q, q};
        }
        x_left = x_right;
    }
    for (int a = 0; a < n1 - 1; ++a) {
        int ia = idx(a), ib = idx(a + 1);
        auto mm = ws.interfaces[a + 1];
        State f_a, f_b;
        hydrostatic_hll(ws.faces[a].second, ws.faces[a + 1].first, mm.first, mm.second, g, h_min, f_a, f_b);
        if (mass) mass[a] = f_a.h;
        ws.rhs[ia] = ws.rhs[ia] - (1.0 / w[a]) * f_a;
        ws.rhs[ib] = ws.rhs[ib] + (1.0 / w[a + 1]) * f_b;
    }
    for (int a = 0; a < n1; ++a) {
        int ia = idx(a);
        const Side& left = ws.faces[a].first;
        const Side& right = ws.faces[a].second;
        double w_a = w[a];
        double bed = -0.5 * g * (left.h + right.h) * (right.b - left.b) / w_a;
        double fx, fy;
        if (affine) {
            auto m0 = ws.metric[0];
            fx = bed * m0.first;
            fy = bed * m0.second;
        } else {
            auto m_l = ws.interfaces[a], m_r = ws.interfaces[a + 1];
            double h_a = ws.nodes[ia].h, b_a = ws.nodes[ia].b;
            double metric = 0.25 * g *
                            ((right.h + h_a) * (b_a - right.b) + (left.h + h_a) * (b_a - left.b)) / w_a;
            fx = bed * 0.5 * (m_l.first + m_r.first) + metric * (m_r.first - m_l.first);
            fy = bed * 0.5 * (m_l.second + m_r.second) + metric * (m_r.second - m_l.second);
        }
        ws.rhs[ia] = ws.rhs[ia] + State{0.0, fx, fy};
    }
}

// SplitFormSWE2D::outer_node (src/solver/rhs/swe_2d_split_form.rs:1048-1085)
static Workspace::Outer outer_node(const Model& m, const Buffer& q, int64_t k, int face, int fi) {
    const Ops& ops = m.ops;
    const Geometry& g = m.geom;
    int n1 = ops.n1;
    Workspace::Outer out;
    ElementFace nb;
    if (!m.mesh.neighbor(k, face, nb)) return out;
    auto height = [&](int64_t e, int f, int fidx, int node) {
        if (g.affine[e]) return g.det_j[g.nidx(e, 0)] / g.surface_j[g.fidx(e, f, 0)];
        return g.det_j[g.nidx(e, node)] / g.surface_j[g.fidx(e, f, fidx)];
    };
    int nb_node = ops.face_nodes[nb.face][n1 - 1 - fi];
    int inner;
    switch (nb.face) {
        case 0: inner = nb_node + n1; break;
        case 1: inner = nb_node - 1; break;
        case 2: inner = nb_node - n1; break;
        default: inner = nb_node + 1; break;
    }
    int own_node = ops.face_nodes[face][fi];
    double distance = (ops.x1[1] - ops.x1[0]) * height(nb.element, nb.face, n1 - 1 - fi, nb_node) /
                      height(k, face, fi, own_node);
    out.present = true;
    out.node = node_at(m, q, nb.element, inner);
    out.distance = distance;
    return out;
}

// SplitFormSWE2D::element_rhs (src/solver/rhs/swe_2d_split_form.rs:665-820)
// then SWE2DRhsKernel::source_terms (src/solver/rhs/swe_2d.rs:929-973)
static void element_rhs(const Model& m, const Buffer& q, int64_t k, double time, Workspace& ws,
                        double* out_h, double* out_hu, double* out_hv) {
    const Ops& ops = m.ops;
    const Geometry& g = m.geom;
    int n1 = ops.n1, nn = ops.nn;
    for (int i = 0; i < nn; ++i) {
        ws.nodes[i] = node_at(m, q, k, i);
        ws.rhs[i] = State{0.0, 0.0, 0.0};
    }
    bool subcells = false;
    if (m.form.formulation == DGSWE_WET_DRY)
        for (int i = 0; i < nn; ++i) subcells = subcells || (ws.nodes[i].h < m.form.subcell_depth);
    if (subcells)
        for (int face = 0; face < 4; ++face)
            for (int fi = 0; fi < n1; ++fi) ws.outer[face * n1 + fi] = outer_node(m, q, k, face, fi);
    else if (ws.subcell_mass)
        for (int slot = 0; slot < 2 * n1 * (n1 - 1); ++slot) ws.subcell_mass[slot] = NAN;
    // subcell_slot (src/solver/rhs/subcells.rs:37-42): (dir·n1 + line)·(n1 − 1) + a
    auto line_mass = [&](int dir, int line) {
        return ws.subcell_mass ? ws.subcell_mass + (dir * n1 + line) * (n1 - 1) : nullptr;
    };
    bool affine = g.affine[k] != 0;
    double ar0, ar1, as0, as1;
    g.contravariant(k, 0, ar0, ar1, as0, as1);
    for (int line = 0; line < n1; ++line) {
        auto r_line = [&](int a) { return line * n1 + a; };
        auto s_line = [&](int j) { return j * n1 + line; };
        int rev = n1 - 1 - line, fwd = line;
        for (int a = 0; a < n1; ++a) {
            if (affine) {
                ws.metric[a] = {ar0, ar1};
            } else {
                double r0, r1, s0, s1;
                g.contravariant(k, r_line(a), r0, r1, s0, s1);
                ws.metric[a] = {r0, r1};
            }
        }
        if (subcells)
            line_subcells(m, ws, r_line, ws.outer[3 * n1 + rev], ws.outer[n1 + fwd], affine,
                          line_mass(0, line));
        else
            line_volume(m, ws, r_line, affine, {ar0, ar1});
        for (int j = 0; j < n1; ++j) {
            if (affine) {
                ws.metric[j] = {as0, as1};
            } else {
                double r0, r1, s0, s1;
                g.contravariant(k, s_line(j), r0, r1, s0, s1);
                ws.metric[j] = {s0, s1};
            }
        }
        if (subcells)
            line_subcells(m, ws, s_line, ws.outer[fwd], ws.outer[2 * n1 + rev], affine,
                          line_mass(1, line));
        else
            line_volume(m, ws, s_line, affine, {as0, as1});
    }
    // Surface terms (src/solver/rhs/swe_2d_split_form.rs:777-807)
    for (int face = 0; face < 4; ++face) {
        int64_t e = m.mesh.element_edges[k][face];
        const Edge& edge = m.mesh.edges[e];
        bool interior = edge.right.element >= 0;
        int side = (edge.left.element != k || edge.left.face != face) ? 1 : 0;
        for (int fi = 0; fi < n1; ++fi) {
            int node = ops.face_nodes[face][fi];
            double nx, ny, scale;
            face_normal(m, k, face, fi, nx, ny, scale);
            const Node& q_int = ws.nodes[node];
            State f_star = interior ? m.faces[(2 * e + side) * n1 + fi]
                                    : boundary_flux(m, k, face, node, q_int, nx, ny, time, edge.tag);
            if (ws.face_mass) ws.face_mass[face * n1 + fi] = f_star.h;
            State flux_diff = wintermeyer_flux(q_int, q_int, nx, ny, m.form.g) - f_star;
            ws.rhs[node] = ws.rhs[node] + (scale * ops.lift_at(face, node, fi)) * flux_diff;
        }
    }
    for (int i = 0; i < nn; ++i) {
        double j_inv = affine ? g.det_j_inv[g.nidx(k, 0)] : g.det_j_inv[g.nidx(k, i)];
        out_h[i] = j_inv * ws.rhs[i].h;
        out_hu[i] = j_inv * ws.rhs[i].hu;
        out_hv[i] = j_inv * ws.rhs[i].hv;
    }
    // CoriolisSource2D::add_element (src/source/swe_2d/coriolis.rs:151-175)
    if (m.form.has_coriolis) {
        auto v = m.mesh.corners(k);
        for (int i = 0; i < nn; ++i) {
            double f = m.form.coriolis_f0;
            if (m.form.coriolis_beta != 0.0) {
                // Mesh2D::bilinear (src/mesh/core/mesh2d.rs:644-660)
                double r = ops.nodes_r[i], s = ops.nodes_s[i];
                double n0 = (1.0 - r) * (1.0 - s) / 4.0, n1b = (1.0 + r) * (1.0 - s) / 4.0;
                double n2 = (1.0 + r) * (1.0 + s) / 4.0, n3 = (1.0 - r) * (1.0 + s) / 4.0;
                double y = n0 * v[0][1] + n1b * v[1][1] + n2 * v[2][1] + n3 * v[3][1];
                f = m.form.coriolis_f0 + m.form.coriolis_beta * (y - m.form.coriolis_y0);
            }
            State st = q.get((size_t)k * nn + i);
            out_hu[i] += f * st.hv;
            out_hv[i] += -f * st.hu;
        }
    }
    // NestingRelaxation2D::add_element with relaxation_source
    // (src/boundary/ocean_nesting.rs:955-1030), after Coriolis
    if (m.relax.on) {
        const Relaxation& r = m.relax;
        for (int i = 0; i < nn; ++i) {
            size_t flat = (size_t)k * nn + i;
            uint32_t slot = r.parent.parent.slot_of_node[flat];
            if (slot == 0xFFFFFFFFu) continue;
            State st = q.get(flat);
            double w = r.weight[slot];
            if (w <= 0.0 || st.h < r.wet_depth) continue;
            double bed = m.bed_at(k, i);
            double eta, u, v;
            bool has_uv;
            r.parent.parent_external(slot, time, bed, eta, u, v, has_uv);
            double h = eta - bed;
            if (h < r.wet_depth) continue;
            double gamma = w * r.rate;
            if (!has_uv) {
                u = st.hu / st.h;
                v = st.hv / st.h;
            }
            double dh = r.momentum_only ? 0.0 : h - st.h;
            double depth = r.momentum_only ? st.h : h;
            out_h[i] += gamma * dh;
            out_hu[i] += gamma * (depth * u - st.hu);
            out_hv[i] += gamma * (depth * v - st.hv);
        }
    }
    // GriddedAtmosphere2D::add_element (src/source/swe_2d/gridded_atmosphere.rs:698-729),
    // after the band
    if (m.atm.on && m.atm.source && (m.atm.wind || m.atm.pressure)) {
        const Atmosphere& a = m.atm;
        double ramp = tidal_ramp(time, a.ramp);
        double rw = a.wind ? ramp : 0.0, rp = a.pressure ? ramp : 0.0;
        for (int i = 0; i < nn; ++i) {
            size_t flat = (size_t)k * nn + i;
            double h = q.get(flat).h;
            if (h < a.h_min) continue;
            double wx[5];
            a.at(flat, time, wx);
            double su, sv;
            atmosphere_source(h, rw * wx[0], rw * wx[1], rp * wx[2], rp * wx[3], a.drag, a.cd,
                              a.rho_air, a.rho_water, a.h_min, su, sv);
            out_hu[i] += su;
            out_hv[i] += sv;
        }
    }
}

// The face pass over every interior edge (compute_rhs_swe_2d_*: face_fluxes,
// src/solver/rhs/swe_2d.rs:619-646)
static void face_pass(Model& m, const Buffer& q) {
    int64_t n_edges = (int64_t)m.mesh.edges.size();
    m.faces.assign((size_t)2 * n_edges * m.ops.n1, State{});
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < n_edges; ++e) edge_fluxes(m, q, e, &m.faces[(size_t)2 * e * m.ops.n1]);
}

// ---------------------------------------------------------------------------
// Physics: damping, wet/dry correction, stages (src/physics/builder.rs)

// damp_node (src/solver/algorithms/wetting_drying.rs:324-357); the block
// path of damp_wet_block gives the same bits (wetting_drying.rs:775-822)
static void damp_node(const Model& m, size_t node, double h, double& hu, double& hv, State from,
                      double dt) {
    if (h <= 0.0) {
        hu = 0.0;
        hv = 0.0;
        return;
    }
    double rate = 0.0;
    if (m.form.friction != DGSWE_FRICTION_NONE) {
        double u, v;
        if (m.form.has_wet_dry)
            m.wd.desingularized_velocity(from.h, from.hu, from.hv, u, v);
        else
            state_velocity(from, m.form.h_min, u, v);
        double speed = std::sqrt(u * u + v * v);
        if (speed > 0.0) rate += manning_rate(m.g_n2[node], fmax_(h, m.form.manning_h_min), speed);
    }
    if (m.form.has_wet_dry) rate += m.wd.thin_layer_rate(h);
    double factor = 1.0 / (1.0 + dt * rate);
    hu *= factor;
    hv *= factor;
}

// wet_dry_element (src/solver/algorithms/wetting_drying.rs:194-215) with
// element_mean and positivity_limit_element (src/solver/limiters/swe_2d.rs:135-203)
static bool wet_dry_element(const Model& m, int64_t k, double* h, double* hu, double* hv) {
    const Geometry& g = m.geom;
    int nn = m.ops.nn;
    const double* mass = &g.mass[g.nidx(k, 0)];
    double inv_area = 1.0 / g.area[k];
    double h_dry = m.wd.h_dry;
    bool needs = false;
    for (int i = 0; i < nn; ++i) needs = needs || (h[i] < h_dry);
    bool clipped = false;
    if (needs) {
        double sh = 0.0, shu = 0.0, shv = 0.0;
        for (int i = 0; i < nn; ++i) {
            sh += mass[i] * h[i];
            shu += mass[i] * hu[i];
            shv += mass[i] * hv[i];
        }
        double h_avg = sh * inv_area, hu_avg = shu * inv_area, hv_avg = shv * inv_area;
        if (h_avg <= 0.0) {
            for (int i = 0; i < nn; ++i) h[i] = hu[i] = hv[i] = 0.0;
            clipped = h_avg < 0.0;
        } else {
            double h_min_elem = INF;
            for (int i = 0; i < nn; ++i) h_min_elem = fmin_(h_min_elem, h[i]);
            if (h_min_elem < 0.0) {
                // compute_theta_positivity (src/solver/limiters/swe_2d.rs:98-106)
                double theta = h_avg / (h_avg - h_min_elem);
                theta = theta < 0.0 ? 0.0 : (theta > 1.0 ? 1.0 : theta);
                for (int i = 0; i < nn; ++i) {
                    h[i] = theta * (h[i] - h_avg) + h_avg;
                    hu[i] = theta * (hu[i] - hu_avg) + hu_avg;
                    hv[i] = theta * (hv[i] - hv_avg) + hv_avg;
                }
                for (int i = 0; i < nn; ++i) h[i] = fmax_(h[i], 0.0);
            }
            if (h_avg < h_dry)
                for (int i = 0; i < nn; ++i) hu[i] = hv[i] = 0.0;
        }
    }
    for (int i = 0; i < nn; ++i) m.wd.correct_node(h[i], hu[i], hv[i]);
    return clipped;
}

// SWEPhysics2D::post_process_element (src/physics/builder.rs:266-278): the
// positivity pass of a wet/dry run is the redundant one
static bool post_process_element(const Model& m, int64_t k, double* h, double* hu, double* hv) {
    if (!m.form.has_wet_dry) return false;
    return wet_dry_element(m, k, h, hu, hv);
}

static std::string check_buffer(const Model& m, int32_t b) {
    if (b < 0 || b >= DGSWE_N_BUFFERS) return "buffer id out of range";
    (void)m;
    return "";
}

// stage_where over every element (src/physics/builder.rs:652-737) with
// compute_rhs_swe_2d_subset_then (src/solver/rhs/swe_2d.rs:1759-1996)
static void stage_all(Model& m, const dgswe_stage_plan& p) {
    const Buffer& input = m.buf[p.input];
    face_pass(m, input);
    int nn = m.ops.nn;
    Buffer& out = m.buf[p.out];
    const Buffer& base = m.buf[p.base];
    Buffer* acc = p.accumulate ? &m.buf[p.acc] : nullptr;
    int64_t clips = 0;
#pragma omp parallel reduction(+ : clips)
    {
        Workspace ws(m.ops);
        std::vector<double> rh(nn), rhu(nn), rhv(nn);
#pragma omp for schedule(static)
        for (int64_t k = 0; k < m.mesh.n_elements; ++k) {
            element_rhs(m, input, k, p.time, ws, rh.data(), rhu.data(), rhv.data());
            size_t o = (size_t)k * nn;
            double* rows[3] = {rh.data(), rhu.data(), rhv.data()};
            const std::vector<double>* bases[3] = {&base.h, &base.hu, &base.hv};
            const std::vector<double>* inputs[3] = {&input.h, &input.hu, &input.hv};
            for (int var = 0; var < 3; ++var)
                for (int i = 0; i < nn; ++i) {
                    double s = (*bases[var])[o + i], x = (*inputs[var])[o + i], f = rows[var][i];
                    double v = p.a != 0.0 ? p.a * s : 0.0;
                    if (p.b != 0.0) v += p.b * x;
                    if (p.c != 0.0) v += p.c * f;
                    rows[var][i] = v;
                }
            // ImplicitDamping2D::damp_element (src/solver/algorithms/wetting_drying.rs:582-592)
            if (m.form.friction != DGSWE_FRICTION_NONE || m.form.has_wet_dry)
                for (int i = 0; i < nn; ++i)
                    damp_node(m, o + i, rh[i], rhu[i], rhv[i], input.get(o + i), p.c);
            if (p.accumulate) {
                double* sums[3] = {&acc->h[o], &acc->hu[o], &acc->hv[o]};
                for (int var = 0; var < 3; ++var)
                    for (int i = 0; i < nn; ++i)
                        sums[var][i] = p.keep != 0.0 ? p.w * rows[var][i] + p.keep * sums[var][i]
                                                     : p.w * rows[var][i];
            } else {
                clips += post_process_element(m, k, rh.data(), rhu.data(), rhv.data()) ? 1 : 0;
            }
            std::memcpy(&out.h[o], rh.data(), nn * sizeof(double));
            std::memcpy(&out.hu[o], rhu.data(), nn * sizeof(double));
            std::memcpy(&out.hv[o], rhv.data(), nn * sizeof(double));
        }
    }
    m.clips += clips;
}

// finish_where over every element (src/physics/builder.rs:739-782)
static void finish_all(Model& m, int32_t acc_id) {
    int nn = m.ops.nn;
    Buffer& s = m.buf[DGSWE_STATE];
    const Buffer& acc = m.buf[acc_id];
    int64_t clips = 0;
#pragma omp parallel for schedule(static) reduction(+ : clips)
    for (int64_t k = 0; k < m.mesh.n_elements; ++k) {
        size_t o = (size_t)k * nn;
        for (int i = 0; i < nn; ++i) {
            s.h[o + i] = acc.h[o + i];
            s.hu[o + i] = acc.hu[o + i];
            s.hv[o + i] = acc.hv[o + i];
        }
        clips += post_process_element(m, k, &s.h[o], &s.hu[o], &s.hv[o]) ? 1 : 0;
    }
    m.clips += clips;
}

// SspScheme::stages (src/time/integrator.rs:239-263): (start, input, beta, c)
struct ShuOsher {
    double start, input, beta, c;
};
static int scheme_stages(int scheme, ShuOsher* out) {
    if (scheme == DGSWE_SSP_RK43) {
        out[0] = {1.0, 0.0, 0.5, 0.0};
        out[1] = {0.0, 1.0, 0.5, 0.5};
        out[2] = {2.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0, 1.0};
        out[3] = {0.0, 1.0, 0.5, 0.5};
        return 4;
    }
    out[0] = {1.0, 0.0, 1.0, 0.0};
    out[1] = {0.75, 0.25, 0.25, 1.0};
    out[2] = {1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0, 0.5};
    return 3;
}

// MultirateStepper::step with one level (src/time/multirate.rs:1285-1315)
// and element_stage (multirate.rs:169-200): stage s reads the previous
// stage's value, the last sums into acc, then finish_where
static void step_one_level(Model& m, int scheme, double t, double dt) {
    ShuOsher st[4];
    int n = scheme_stages(scheme, st);
    // buffers: values 1..n-1, last n, acc n+1
    int last = n, acc = n + 1;
    for (int s = 0; s < n; ++s) {
        dgswe_stage_plan p{};
        p.base = DGSWE_STATE;
        p.input = s == 0 ? DGSWE_STATE : s;
        p.time = t + st[s].c * dt;
        p.a = st[s].start;
        p.b = st[s].input;
        p.c = st[s].beta * dt;
        if (s + 1 < n) {
            p.out = s + 1;
            p.accumulate = 0;
        } else {
            p.out = last;
            p.acc = acc;
            p.accumulate = 1;
            p.w = 1.0;
            p.keep = 0.0;
        }
        stage_all(m, p);
    }
    finish_all(m, acc);
}

// ---------------------------------------------------------------------------
// Time step (src/solver/rhs/swe_2d.rs:1238-1367, 2072-2258)

static double positivity_cfl(int order) {
    double n = (double)order;
    return (2.0 * n + 1.0) / (2.0 * n * (n + 1.0));
}
static double linear_cfl(int order, int scheme) {
    static const double rk3[4] = {1.6, 1.04, 0.73, 0.56}, rk43[4] = {2.2, 1.51, 1.15, 0.93};
    if (order < 1 || order > 4) return -1.0;
    return scheme == DGSWE_SSP_RK43 ? rk43[order - 1] : rk3[order - 1];
}
static double linear_cfl_subcells(int order, int scheme) {
    static const double rk3[4] = {0.94, 0.65, 0.47, 0.36}, rk43[4] = {1.5, 1.1, 0.97, 0.75};
    if (order < 1 || order > 4) return -1.0;
    return scheme == DGSWE_SSP_RK43 ? rk43[order - 1] : rk3[order - 1];
}

// PositivityBound::new (src/solver/rhs/swe_2d.rs:2194-2212)
struct PositivityBound {
    double cfl, max_cfl, max_cfl_subcells, h_dry;
};
static PositivityBound positivity_bound(int order, int scheme, double h_dry) {
    double ssp = scheme == DGSWE_SSP_RK43 ? 2.0 : 1.0;
    double cfl = ssp * positivity_cfl(order);
    auto cap = [&](double limit) { return limit < 0.0 ? cfl : fmax_(cfl, 0.9 * limit); };
    return {cfl, cap(linear_cfl(order, scheme)), cap(linear_cfl_subcells(order, scheme)), h_dry};
}

// node_reference_rate (src/solver/rhs/swe_2d.rs:1346-1357)
static double node_reference_rate(State s, double gr0, double gr1, double gs0, double gs1,
                                  double norm_r, double norm_s, double g, double h_min) {
    double u, v;
    velocity_simple(s, h_min, u, v);
    double c = std::sqrt(g * fmax_(s.h, 0.0));
    double lambda_r = std::fabs(u * gr0 + v * gr1) + c * norm_r;
    double lambda_s = std::fabs(u * gs0 + v * gs1) + c * norm_s;
    return 0.25 * (lambda_r + lambda_s);
}

// element_dt (src/solver/rhs/swe_2d.rs:2072-2115) with
// element_max_reference_rate (swe_2d.rs:1308-1341) and
// PositivityBound::element_cfl / positivity_relaxation (swe_2d.rs:2220-2258)
static double element_dt(const Model& m, const Buffer& q, int64_t k, double cfl, bool positivity,
                         const PositivityBound& bound) {
    const Ops& ops = m.ops;
    const Geometry& g = m.geom;
    int nn = ops.nn, n1 = ops.n1;
    double gg = m.form.g, h_min = m.form.h_min;
    auto norm = [](double a, double b) { return std::sqrt(a * a + b * b); };
    size_t n0 = g.nidx(k, 0);
    double rate = 0.0;
    for (int i = 0; i < nn; ++i) {
        State s = q.get(g.nidx(k, i));
        double r;
        if (s.h <= h_min) {
            r = 0.0;
        } else {
            size_t ni = g.affine[k] ? n0 : g.nidx(k, i);
            r = node_reference_rate(s, g.rx[ni], g.ry[ni], g.sx[ni], g.sy[ni], norm(g.rx[ni], g.ry[ni]),
                                    norm(g.sx[ni], g.sy[ni]), gg, h_min);
        }
        rate = fmax_(rate, r);
    }
    for (int face = 0; face < 4; ++face) {
        ElementFace nb;
        if (!m.mesh.neighbor(k, face, nb)) continue;
        for (int fi = 0; fi < n1; ++fi) {
            int i = ops.face_nodes[face][fi];
            int j = ops.face_nodes[nb.face][n1 - 1 - fi];
            State s = q.get(g.nidx(nb.element, j));
            if (s.h <= h_min) continue;
            size_t ni = g.nidx(k, i);
            rate = fmax_(rate, node_reference_rate(s, g.rx[ni], g.ry[ni], g.sx[ni], g.sy[ni],
                                                   norm(g.rx[ni], g.ry[ni]), norm(g.sx[ni], g.sy[ni]),
                                                   gg, h_min));
        }
    }
    if (positivity) {
        double shallow = 100.0 * bound.h_dry;
        double water = 0.0, water_b = 0.0, weight = 0.0, weight_b = 0.0;
        bool is_shallow = false;
        int last = n1 - 1;
        for (int i = 0; i < nn; ++i) {
            double h = q.h[g.nidx(k, i)], mm = g.mass[g.nidx(k, i)];
            is_shallow = is_shallow || (h <= shallow);
            double water_i = mm * fmax_(h, 0.0);
            water += water_i;
            weight += mm;
            int a = i % n1, j = i / n1;
            if (a == 0 || a == last || j == 0 || j == last) {
                water_b += water_i;
                weight_b += mm;
            }
        }
        double ratio = fmin_(water / water_b, weight / weight_b);
        double rho = fmax_(0.9 * ratio, 1.0);
        double cap = is_shallow ? bound.max_cfl_subcells : bound.max_cfl;
        cfl = fmin_(cfl, fmin_(bound.cfl * rho, cap));
    }
    // dt_from_reference_rate (src/solver/rhs/swe_2d.rs:1362-1367)
    if (rate < 1e-14) return INF;
    return cfl / ((2.0 * (double)ops.order + 1.0) * rate);
}

static double min_element_dt(Model& m, double cfl, int scheme, double* dt_el) {
    bool positivity = m.form.positivity_h_dry > 0.0;
    PositivityBound bound = positivity_bound(m.ops.order, scheme, m.form.positivity_h_dry);
    const Buffer& q = m.buf[DGSWE_STATE];
    double dt_min = INF;
#pragma omp parallel for schedule(static) reduction(min : dt_min)
    for (int64_t k = 0; k < m.mesh.n_elements; ++k) {
        double dt = element_dt(m, q, k, cfl, positivity, bound);
        if (dt_el) dt_el[k] = dt;
        dt_min = fmin_(dt_min, dt);
    }
    return dt_min;
}

static bool state_is_finite(const Model& m) {
    const Buffer& s = m.buf[DGSWE_STATE];
    size_t n = m.n_values();
    bool ok = true;
#pragma omp parallel for schedule(static) reduction(&& : ok)
    for (size_t i = 0; i < n; ++i)
        ok = ok && std::isfinite(s.h[i]) && std::isfinite(s.hu[i]) && std::isfinite(s.hv[i]);
    return ok;
}

// ---------------------------------------------------------------------------
// Local time stepping (src/time/multirate.rs): MultirateStepper's levels,
// stage rates and schedule, and the element subsets' stages and finishes of
// SWEPhysics2D's LocalTimeStepping (src/physics/builder.rs:546-782)

struct Multirate {
    int max_levels = 0, n_stages = 3;
    int finest = 0;
    double stable_step = INF;
    std::vector<uint8_t> level;
    std::vector<uint8_t> rate[4];
    // MultirateStats (multirate.rs:785-860)
    int64_t steps = 0, element_evaluations = 0, global_evaluations = 0;
    int finest_used = 0;
    double model_seconds = 0.0, ideal_evaluations = 0.0, level_evaluations = 0.0;
    int64_t line_local_elements = 0;
    int64_t evaluations_per_step = 0, level_evaluations_per_step = 0;
    double inverse_dt_sum = 0.0;
    int64_t n_line_local = 0;
};

// assign_levels (multirate.rs:527-568)
static double mr_assign_levels(const std::vector<double>& element_dt, int max_levels,
                               double dt_cap, std::vector<uint8_t>& level, int& finest) {
    double dt_min = INF, dt_max = 0.0;
    for (double d : element_dt)
        if (std::isfinite(d)) {
            dt_min = fmin_(dt_min, d);
            dt_max = fmax_(dt_max, d);
        }
    level.assign(element_dt.size(), 0);
    finest = 0;
    if (!std::isfinite(dt_min)) return INF;
    while (finest < max_levels) {
        double coarser = dt_min * (double)(2ull << finest);
        if (coarser > dt_max || (dt_cap > 0.0 && coarser > dt_cap)) break;
        finest += 1;
    }
    double dt = dt_min * (double)(1ull << finest);
    for (size_t k = 0; k < element_dt.size(); ++k) {
        int l = 0;
        double dt_l = dt;
        while (l < finest && dt_l > element_dt[k]) {
            dt_l *= 0.5;
            l += 1;
        }
        level[k] = (uint8_t)l;
    }
    return dt;
}

// levels_for_step (multirate.rs:570-583)
static int mr_levels_for_step(const std::vector<double>& element_dt, double dt, int max_levels,
                              std::vector<uint8_t>& level) {
    int finest = 0;
    for (size_t k = 0; k < element_dt.size(); ++k) {
        int l = 0;
        double dt_l = dt;
        while (l < max_levels && dt_l > element_dt[k]) {
            dt_l *= 0.5;
            l += 1;
        }
        level[k] = (uint8_t)l;
        finest = std::max(finest, l);
    }
    return finest;
}

// spread_to_neighbours (multirate.rs:592-615): to[k] = max(from[k],
// from[j] − drop) over the face neighbours j; whether any changed
static bool mr_spread(const Mesh& mesh, const std::vector<uint8_t>& from, std::vector<uint8_t>& to,
                      int drop) {
    bool changed = false;
    to.assign(from.size(), 0);
    for (int64_t k = 0; k < mesh.n_elements; ++k) {
        int best = from[k];
        for (int face = 0; face < 4; ++face) {
            ElementFace nb;
            if (!mesh.neighbor(k, face, nb)) continue;
            best = std::max(best, std::max((int)from[nb.element] - drop, 0));
        }
        to[k] = (uint8_t)best;
        changed = changed || to[k] != from[k];
    }
    return changed;
}

// spread_over_lines (multirate.rs:678-743) of one stage
static void mr_spread_lines(const Model& m, const std::vector<uint8_t>& line_local,
                            const std::vector<uint8_t>& from, std::vector<uint8_t>& to,
                            std::vector<uint8_t>& rate) {
    const Ops& ops = m.ops;
    const int n1 = ops.n1, nn = ops.nn;
    to.assign(from.size(), 0);
    rate.assign((size_t)m.mesh.n_elements, 0);
    auto inner = [&](int face, int node) {
        return face == 0 ? node + n1 : face == 1 ? node - 1 : face == 2 ? node - n1 : node + 1;
    };
    for (int64_t k = 0; k < m.mesh.n_elements; ++k) {
        const uint8_t* own = &from[(size_t)k * nn];
        uint8_t* t = &to[(size_t)k * nn];
        if (!line_local[k]) {
            int finest = 0;
            for (int i = 0; i < nn; ++i) finest = std::max(finest, (int)own[i]);
            for (int face = 0; face < 4; ++face) {
                ElementFace nb;
                if (!m.mesh.neighbor(k, face, nb)) continue;
                const uint8_t* other = &from[(size_t)nb.element * nn];
                for (int fi = 0; fi < n1; ++fi) {
                    int node = ops.face_nodes[nb.face][fi];
                    finest = std::max(finest, std::max((int)other[node], (int)other[inner(nb.face, node)]));
                }
            }
            for (int i = 0; i < nn; ++i) t[i] = (uint8_t)finest;
            rate[k] = (uint8_t)finest;
            continue;
        }
        for (int j = 0; j < n1; ++j) {
            int mx = 0;
            for (int i = 0; i < n1; ++i) mx = std::max(mx, (int)own[j * n1 + i]);
            for (int i = 0; i < n1; ++i) t[j * n1 + i] = (uint8_t)mx;
        }
        for (int i = 0; i < n1; ++i) {
            int mx = 0;
            for (int j = 0; j < n1; ++j) mx = std::max(mx, (int)own[j * n1 + i]);
            for (int j = 0; j < n1; ++j) t[j * n1 + i] = (uint8_t)std::max((int)t[j * n1 + i], mx);
        }
        for (int face = 0; face < 4; ++face) {
            ElementFace nb;
            if (!m.mesh.neighbor(k, face, nb)) continue;
            const uint8_t* other = &from[(size_t)nb.element * nn];
            for (int fi = 0; fi < n1; ++fi) {
                int node = ops.face_nodes[face][fi];
                int o = other[ops.face_nodes[nb.face][n1 - 1 - fi]];
                t[node] = (uint8_t)std::max((int)t[node], o);
            }
        }
        int mx = 0;
        for (int i = 0; i < nn; ++i) mx = std::max(mx, (int)t[i]);
        rate[k] = (uint8_t)mx;
    }
}

// MultirateStepper::assign (multirate.rs:1044-1157) without the kept plan
// (which gives what a fresh one gives) and the longest step (off)
static double mr_assign(const Model& m, Multirate& mr, const std::vector<double>& element_dt,
                        const std::vector<uint8_t>* line_local, double dt_cap, double landing) {
    const int64_t K = m.mesh.n_elements;
    int finest = 0;
    double dt = mr_assign_levels(element_dt, mr.max_levels, dt_cap, mr.level, finest);
    mr.stable_step = dt;
    if (finest > 0 && landing > 0.0 && std::isfinite(dt)) {
        double steps = std::ceil(landing / (dt * (1.0 + 1e-9)));
        if (steps < 1.0) steps = 1.0;
        double fitted = landing / steps;
        if (fitted < dt) {
            dt = fitted;
            finest = mr_levels_for_step(element_dt, dt, mr.max_levels, mr.level);
        }
    }
    mr.finest = finest;
    mr.inverse_dt_sum = 0.0;
    for (double d : element_dt)
        if (std::isfinite(d)) mr.inverse_dt_sum += 1.0 / d;
    // limit_level_jumps (multirate.rs:745-752)
    std::vector<uint8_t> scratch;
    while (mr_spread(m.mesh, mr.level, scratch, 1)) std::swap(mr.level, scratch);
    int64_t lev = 0;
    for (int64_t k = 0; k < K; ++k) lev += (int64_t)1 << mr.level[k];
    mr.level_evaluations_per_step = (int64_t)mr.n_stages * lev;
    mr.n_line_local = 0;
    if (line_local) {
        for (int64_t k = 0; k < K; ++k) mr.n_line_local += (*line_local)[k] ? 1 : 0;
        const int nn = m.ops.nn;
        std::vector<uint8_t> from((size_t)K * nn), to;
        for (int64_t k = 0; k < K; ++k)
            for (int i = 0; i < nn; ++i) from[(size_t)k * nn + i] = mr.level[k];
        for (int s = 0; s < mr.n_stages; ++s) {
            mr_spread_lines(m, *line_local, from, to, mr.rate[s]);
            std::swap(from, to);
        }
    } else {
        for (int s = 0; s < mr.n_stages; ++s)
            mr_spread(m.mesh, s == 0 ? mr.level : mr.rate[s - 1], mr.rate[s], 0);
    }
    mr.evaluations_per_step = 0;
    for (int s = 0; s < mr.n_stages; ++s)
        for (int64_t k = 0; k < K; ++k) mr.evaluations_per_step += (int64_t)1 << mr.rate[s][k];
    return dt;
}

// depth (multirate.rs:771-778)
static int mr_depth(int64_t p, int finest) {
    if (p == 0 || p == ((int64_t)1 << finest)) return 0;
    int tz = 0;
    while (((p >> tz) & 1) == 0) ++tz;
    return finest - tz;
}

// element_stage (multirate.rs:169-200)
struct ElementStage {
    double time, a, b, c;
    bool accumulate;
    double w, keep;
};
static ElementStage mr_element_stage(double t, double dt, int finest, int64_t substep, int depth,
                                     const ShuOsher& st, bool last, int level, int rate) {
    double dt_l = dt / (double)(1ull << level);
    int64_t q = substep >> (finest - level);
    double t_k = t + (double)q * dt_l;
    ElementStage e{};
    e.time = t_k + st.c * dt_l;
    e.a = st.start;
    e.b = st.input;
    e.c = st.beta * dt_l;
    e.accumulate = last;
    if (last) {
        uint64_t blocks = 1ull << (rate - level);
        e.w = 1.0 / (double)blocks;
        e.keep = level >= depth ? 0.0 : 1.0;
    }
    return e;
}

// stage_where (builder.rs:652-737) on the elements whose stage rate is at
// least the pass's depth
static void mr_stage(Model& m, const Multirate& mr, int s, const ShuOsher& st, bool last,
                     double t, double dt, int64_t p, int d, int32_t input_id, int32_t out_id,
                     int32_t acc_id) {
    const Buffer& input = m.buf[input_id];
    face_pass(m, input);
    const int nn = m.ops.nn;
    Buffer& out = m.buf[out_id];
    const Buffer& base = m.buf[DGSWE_STATE];
    Buffer& acc = m.buf[acc_id];
    int64_t clips = 0;
#pragma omp parallel reduction(+ : clips)
    {
        Workspace ws(m.ops);
        std::vector<double> rh(nn), rhu(nn), rhv(nn);
#pragma omp for schedule(static)
        for (int64_t k = 0; k < m.mesh.n_elements; ++k) {
            if (mr.rate[s][k] < d) continue;
            ElementStage e = mr_element_stage(t, dt, mr.finest, p, d, st, last, mr.level[k],
                                              mr.rate[s][k]);
            element_rhs(m, input, k, e.time, ws, rh.data(), rhu.data(), rhv.data());
            size_t o = (size_t)k * nn;
            double* rows[3] = {rh.data(), rhu.data(), rhv.data()};
            const std::vector<double>* bases[3] = {&base.h, &base.hu, &base.hv};
            const std::vector<double>* inputs[3] = {&input.h, &input.hu, &input.hv};
            for (int var = 0; var < 3; ++var)
                for (int i = 0; i < nn; ++i) {
                    double sv = (*bases[var])[o + i], x = (*inputs[var])[o + i], f = rows[var][i];
                    double v = e.a != 0.0 ? e.a * sv : 0.0;
                    if (e.b != 0.0) v += e.b * x;
                    if (e.c != 0.0) v += e.c * f;
                    rows[var][i] = v;
                }
            if (m.form.friction != DGSWE_FRICTION_NONE || m.form.has_wet_dry)
                for (int i = 0; i < nn; ++i)
                    damp_node(m, o + i, rh[i], rhu[i], rhv[i], input.get(o + i), e.c);
            if (e.accumulate) {
                double* sums[3] = {&acc.h[o], &acc.hu[o], &acc.hv[o]};
                for (int var = 0; var < 3; ++var)
                    for (int i = 0; i < nn; ++i)
                        sums[var][i] = e.keep != 0.0 ? e.w * rows[var][i] + e.keep * sums[var][i]
                                                     : e.w * rows[var][i];
            } else {
                clips += post_process_element(m, k, rh.data(), rhu.data(), rhv.data()) ? 1 : 0;
            }
            std::memcpy(&out.h[o], rh.data(), nn * sizeof(double));
            std::memcpy(&out.hu[o], rhu.data(), nn * sizeof(double));
            std::memcpy(&out.hv[o], rhv.data(), nn * sizeof(double));
        }
    }
    m.clips += clips;
}

// finish_where (builder.rs:739-782) on the elements whose level is at least d
static void mr_finish(Model& m, const Multirate& mr, int d, int32_t acc_id) {
    const int nn = m.ops.nn;
    Buffer& st = m.buf[DGSWE_STATE];
    const Buffer& acc = m.buf[acc_id];
    int64_t clips = 0;
#pragma omp parallel for schedule(static) reduction(+ : clips)
    for (int64_t k = 0; k < m.mesh.n_elements; ++k) {
        if (mr.level[k] < d) continue;
        size_t o = (size_t)k * nn;
        for (int i = 0; i < nn; ++i) {
            st.h[o + i] = acc.h[o + i];
            st.hu[o + i] = acc.hu[o + i];
            st.hv[o + i] = acc.hv[o + i];
        }
        clips += post_process_element(m, k, &st.h[o], &st.hu[o], &st.hv[o]) ? 1 : 0;
    }
    m.clips += clips;
}

// MultirateStepper::step (multirate.rs:1285-1315) over schedule
// (multirate.rs:1249-1283): buffers 1..n−1 the stage values, n the last
// stage's, n + 1 the substeps' sums
static void mr_step(Model& m, Multirate& mr, int scheme, double t, double dt) {
    ShuOsher st[4];
    const int n = scheme_stages(scheme, st);
    const int last = n, acc = n + 1;
    for (int64_t p = 0; p < ((int64_t)1 << mr.finest); ++p) {
        const int d = mr_depth(p, mr.finest);
        for (int s = 0; s < n; ++s)
            mr_stage(m, mr, s, st[s], s + 1 == n, t, dt, p, d, s == 0 ? DGSWE_STATE : s,
                     s + 1 < n ? s + 1 : last, acc);
        mr_finish(m, mr, mr_depth(p + 1, mr.finest), acc);
    }
    mr.steps += 1;
    mr.element_evaluations += mr.evaluations_per_step;
    mr.global_evaluations += (int64_t)n * m.mesh.n_elements * ((int64_t)1 << mr.finest);
    mr.finest_used = std::max(mr.finest_used, mr.finest);
    mr.model_seconds += dt;
    mr.ideal_evaluations += (double)n * mr.inverse_dt_sum * dt;
    mr.level_evaluations += (double)mr.level_evaluations_per_step;
    mr.line_local_elements += mr.n_line_local;
}

// SWEPhysics2D::line_local and coarse_step_bound (builder.rs:560-632) of the
// state: the line-local flags (null: none) and the bound
static double mr_flags(const Model& m, const std::vector<double>& element_dt,
                       std::vector<uint8_t>& line_local, bool& has_lines) {
    const int nn = m.ops.nn;
    const int64_t K = m.mesh.n_elements;
    const Buffer& q = m.buf[DGSWE_STATE];
    auto all_deeper = [&](int64_t k, double depth) {
        for (int i = 0; i < nn; ++i)
            if (!(q.h[(size_t)k * nn + i] > depth)) return false;
        return true;
    };
    has_lines = m.form.has_line_local != 0 && m.ops.n1 >= 2;
    if (has_lines) {
        double depth = m.form.line_local_depth;
        if (!(std::isinf(depth) && depth < 0.0)) depth += 1.0;  // LINE_LOCAL_HEADROOM
        line_local.assign(K, 0);
        for (int64_t k = 0; k < K; ++k) line_local[k] = all_deeper(k, depth) ? 1 : 0;
    }
    if (!(m.form.positivity_h_dry > 0.0)) return INF;
    const double h_dry = m.form.positivity_h_dry;
    for (double shallow : {100.0 * h_dry, h_dry}) {
        double longest = 0.0;
        for (int64_t k = 0; k < K; ++k)
            if (std::isfinite(element_dt[k]) && all_deeper(k, shallow))
                longest = fmax_(longest, element_dt[k]);
        if (longest > 0.0) return longest;
    }
    return INF;
}

}  // namespace oracle

// ---------------------------------------------------------------------------
// C API (oracle.h): the library's entry points on the CPU

using namespace oracle;

struct oracle_handle {
    Model* m;
    Multirate mr;
};

extern "C" {

int oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

int oracle_create(const dgswe_form* f, int device, oracle_handle** out) {
    (void)device;
    if (!f || !out) return DGSWE_ERR_INVALID;
    *out = nullptr;
    if (f->abi_version != DGSWE_ABI_VERSION || f->order < 1 || f->order > 4 || f->n_elements <= 0 ||
        !f->vertices || !f->elements)
        return DGSWE_ERR_INVALID;
    Model* m = new Model(f->order);
    m->form = *f;
    std::string err = build_mesh(f, m->mesh);
    if (err.empty()) err = build_geometry(m->mesh, m->ops, m->geom);
    if (!err.empty()) {
        delete m;
        return DGSWE_ERR_INVALID;
    }
    size_t nv = m->n_values();
    m->has_bed = f->bathymetry != nullptr;
    if (m->has_bed) m->bed.assign(f->bathymetry, f->bathymetry + nv);
    if (f->friction == DGSWE_FRICTION_MANNING) {
        double g_n2 = f->friction_g * f->manning_n * f->manning_n;
        m->g_n2.assign(nv, g_n2);
    } else if (f->friction == DGSWE_FRICTION_MANNING_NODES) {
        m->g_n2.resize(nv);
        for (size_t i = 0; i < nv; ++i)
            m->g_n2[i] = f->friction_g * f->manning_n_nodes[i] * f->manning_n_nodes[i];
    }
    m->wd.h_dry = f->wet_dry_h_dry;
    m->wd.relaxation_time = f->wet_dry_relaxation_time;
    m->wd.max_velocity = f->wet_dry_max_velocity;
    for (int b = 0; b < f->n_boundaries; ++b) {
        const dgswe_boundary& in = f->boundaries[b];
        Boundary bc;
        bc.kind = in.kind;
        bc.wall_h_min = in.wall_h_min;
        bc.elevation_only = in.elevation_only;
        bc.constituents.assign(in.constituents, in.constituents + in.n_constituents);
        bc.mean_elevation = in.mean_elevation;
        bc.ramp_duration = in.ramp_duration;
        bc.raise = in.kind != DGSWE_BC_WALL && in.raise != 0;
        bc.raise_factor = in.raise_factor;
        if (bc.raise && !f->atmosphere) {
            delete m;
            return DGSWE_ERR_INVALID;
        }
        if (in.kind == DGSWE_BC_NODE_TIDES) {
            const dgswe_node_tides* t = in.node_tides;
            if (!t || t->n_slots <= 0 || !t->positions || !t->coefficients) {
                delete m;
                return DGSWE_ERR_INVALID;
            }
            Boundary::NodeTides& nt = bc.tides;
            nt.n = t->n_constituents;
            nt.n_slots = t->n_slots;
            nt.omega.assign(t->omega, t->omega + nt.n);
            nt.f_rate.assign(t->f_rate, t->f_rate + nt.n);
            nt.positions.assign(t->positions, t->positions + 2 * t->n_slots);
            nt.coefficients.assign(t->coefficients, t->coefficients + (size_t)t->n_slots * nt.n * 6);
            nt.mean.assign(t->n_slots, 0.0);
            nt.source_depth.assign(t->n_slots, 0.0);
            if (t->mean) nt.mean.assign(t->mean, t->mean + t->n_slots);
            if (t->source_depth) nt.source_depth.assign(t->source_depth, t->source_depth + t->n_slots);
            if (t->slot_of_node)
                nt.slot_of_node.assign(t->slot_of_node,
                                       t->slot_of_node + (size_t)f->n_elements * m->ops.nn);
            nt.velocity = t->velocity != 0;
            nt.use_mean = t->use_mean != 0 && t->mean;
            nt.max_ratio = t->max_transport_ratio;
            nt.ramp = t->ramp_duration;
        }
        if (in.kind == DGSWE_BC_PARENT) {
            const dgswe_parent_series* p = in.parent;
            if (!p || p->n_slots <= 0 || p->n_times <= 0 || !p->positions || !p->times ||
                !p->values) {
                delete m;
                return DGSWE_ERR_INVALID;
            }
            Boundary::Parent& pp = bc.parent;
            pp.n_slots = p->n_slots;
            pp.n_times = p->n_times;
            pp.positions.assign(p->positions, p->positions + 2 * p->n_slots);
            pp.times.assign(p->times, p->times + p->n_times);
            pp.values.assign(p->values, p->values + (size_t)p->n_slots * p->n_times * 3);
            pp.depth.assign(p->n_slots, NAN);
            if (p->parent_depth) pp.depth.assign(p->parent_depth, p->parent_depth + p->n_slots);
            if (p->on_boundary) pp.on_boundary.assign(p->on_boundary, p->on_boundary + p->n_slots);
            if (p->slot_of_node)
                pp.slot_of_node.assign(p->slot_of_node,
                                       p->slot_of_node + (size_t)f->n_elements * m->ops.nn);
            pp.cubic = p->cubic != 0;
            pp.velocity = p->velocity != 0;
            pp.reference_level = p->reference_level;
            pp.max_ratio = p->max_transport_ratio;
            pp.ramp = p->ramp_duration;
        }
        m->boundaries[in.tag] = bc;
    }
    if (f->relaxation) {
        const dgswe_relaxation& r = *f->relaxation;
        const dgswe_parent_series* p = r.parent;
        if (!p || !p->slot_of_node || !r.weight || p->n_slots <= 0 || p->n_times <= 0) {
            delete m;
            return DGSWE_ERR_INVALID;
        }
        Boundary::Parent& pp = m->relax.parent.parent;
        pp.n_slots = p->n_slots;
        pp.n_times = p->n_times;
        pp.times.assign(p->times, p->times + p->n_times);
        pp.values.assign(p->values, p->values + (size_t)p->n_slots * p->n_times * 3);
        pp.depth.assign(p->n_slots, NAN);
        if (p->parent_depth) pp.depth.assign(p->parent_depth, p->parent_depth + p->n_slots);
        pp.slot_of_node.assign(p->slot_of_node, p->slot_of_node + (size_t)f->n_elements * m->ops.nn);
        pp.cubic = p->cubic != 0;
        pp.velocity = p->velocity != 0;
        pp.reference_level = p->reference_level;
        pp.max_ratio = p->max_transport_ratio;
        pp.ramp = p->ramp_duration;
        m->relax.weight.assign(r.weight, r.weight + p->n_slots);
        m->relax.rate = r.rate;
        m->relax.wet_depth = r.wet_depth;
        m->relax.momentum_only = r.momentum_only != 0;
        m->relax.on = true;
    }
    if (f->atmosphere) {
        const dgswe_atmosphere& a = *f->atmosphere;
        if (a.n_times <= 0 || !a.times || !a.values || !(a.rho_water > 0.0)) {
            delete m;
            return DGSWE_ERR_INVALID;
        }
        Atmosphere& at = m->atm;
        at.on = true;
        at.source = a.source != 0;
        at.wind = a.wind != 0;
        at.pressure = a.pressure != 0;
        at.level = a.level != 0;
        at.drag = a.drag;
        at.cd = a.drag_cd;
        at.rho_air = a.rho_air;
        at.rho_water = a.rho_water;
        at.h_min = a.h_min;
        at.ramp = a.ramp_duration;
        at.epoch = a.epoch_unix;
        at.n_nodes = (size_t)f->n_elements * m->ops.nn;
        at.times.assign(a.times, a.times + a.n_times);
        at.values.assign(a.values, a.values + (size_t)a.n_times * at.n_nodes * 5);
    }
    for (auto& e : m->mesh.edges)
        if (e.right.element < 0 && !m->boundaries.count(e.tag)) {
            delete m;
            return DGSWE_ERR_INVALID;
        }
    m->form.boundaries = nullptr;
    m->form.relaxation = nullptr;
    m->form.atmosphere = nullptr;
    m->form.bathymetry = nullptr;
    m->form.manning_n_nodes = nullptr;
    m->form.vertices = nullptr;
    m->form.elements = nullptr;
    m->form.periodic = nullptr;
    m->form.face_tags = nullptr;
    for (auto& b : m->buf) b.resize(nv);
    *out = new oracle_handle{m};
    return DGSWE_OK;
}

void oracle_destroy(oracle_handle* h) {
    if (!h) return;
    delete h->m;
    delete h;
}

int64_t oracle_n_values(const oracle_handle* h) { return (int64_t)h->m->n_values(); }

int oracle_upload(oracle_handle* h, int32_t b, const double* hh, const double* hu, const double* hv,
                  int64_t n) {
    if (!check_buffer(*h->m, b).empty() || n != (int64_t)h->m->n_values()) return DGSWE_ERR_INVALID;
    Buffer& buf = h->m->buf[b];
    std::memcpy(buf.h.data(), hh, n * 8);
    std::memcpy(buf.hu.data(), hu, n * 8);
    std::memcpy(buf.hv.data(), hv, n * 8);
    return DGSWE_OK;
}

int oracle_download(oracle_handle* h, int32_t b, double* hh, double* hu, double* hv, int64_t n) {
    if (!check_buffer(*h->m, b).empty() || n != (int64_t)h->m->n_values()) return DGSWE_ERR_INVALID;
    const Buffer& buf = h->m->buf[b];
    std::memcpy(hh, buf.h.data(), n * 8);
    std::memcpy(hu, buf.hu.data(), n * 8);
    std::memcpy(hv, buf.hv.data(), n * 8);
    return DGSWE_OK;
}

int oracle_compute_rhs(oracle_handle* h, int32_t input, double time, double* oh, double* ohu,
                       double* ohv, int64_t n) {
    Model& m = *h->m;
    if (!check_buffer(m, input).empty() || n != (int64_t)m.n_values()) return DGSWE_ERR_INVALID;
    const Buffer& q = m.buf[input];
    face_pass(m, q);
    int nn = m.ops.nn;
#pragma omp parallel
    {
        Workspace ws(m.ops);
#pragma omp for schedule(static)
        for (int64_t k = 0; k < m.mesh.n_elements; ++k) {
            size_t o = (size_t)k * nn;
            element_rhs(m, q, k, time, ws, oh + o, ohu + o, ohv + o);
        }
    }
    return DGSWE_OK;
}

// compute_rhs_swe_2d_mass_fluxes_into (src/solver/rhs/swe_2d.rs:1042-1075):
// the RHS with each element face node's F*_h and each subcell interface's
// mass flux (NaN in elements without subcells); either may be null
int oracle_compute_rhs_mass_fluxes(oracle_handle* h, int32_t input, double time, double* oh,
                                   double* ohu, double* ohv, int64_t n, double* face_mass,
                                   int64_t n_face, double* subcell_mass, int64_t n_sub) {
    Model& m = *h->m;
    const int n1 = m.ops.n1, nn = m.ops.nn;
    const int64_t K = m.mesh.n_elements;
    if (!check_buffer(m, input).empty() || n != (int64_t)m.n_values()) return DGSWE_ERR_INVALID;
    if ((face_mass && n_face != K * 4 * n1) || (subcell_mass && n_sub != K * 2 * n1 * (n1 - 1)))
        return DGSWE_ERR_INVALID;
    const Buffer& q = m.buf[input];
    face_pass(m, q);
#pragma omp parallel
    {
        Workspace ws(m.ops);
#pragma omp for schedule(static)
        for (int64_t k = 0; k < K; ++k) {
            size_t o = (size_t)k * nn;
            ws.face_mass = face_mass ? face_mass + k * 4 * n1 : nullptr;
            ws.subcell_mass = subcell_mass ? subcell_mass + k * 2 * n1 * (n1 - 1) : nullptr;
            element_rhs(m, q, k, time, ws, oh + o, ohu + o, ohv + o);
        }
    }
    return DGSWE_OK;
}

// subcell_divergence_element (src/solver/rhs/transport_3d.rs:253-330): the
// divergence of a transport (hu, hv) on element k's GLL subcells from its
// interface fluxes (subcell_slot order) and its faces' F*, with the line
// ends' own m·(hu, hv) replaced by F* through the lift; with the RHS's mass
// fluxes it is −dh/dt node by node in a subcell element. Test helper.
int oracle_subcell_divergence(oracle_handle* h, int64_t k, const double* hu, const double* hv,
                              const double* interfaces, const double* face, double* div) {
    const Model& m = *h->m;
    const Ops& ops = m.ops;
    const Geometry& g = m.geom;
    const int n1 = ops.n1, nn = ops.nn;
    if (k < 0 || k >= m.mesh.n_elements) return DGSWE_ERR_INVALID;
    const bool affine = g.affine[k] != 0;
    auto node_of = [&](int dir, int line, int a) { return dir == 0 ? line * n1 + a : a * n1 + line; };
    for (int i = 0; i < nn; ++i) div[i] = 0.0;
    for (int dir = 0; dir < 2; ++dir)
        for (int line = 0; line < n1; ++line) {
            std::vector<std::pair<double, double>> metric(n1);
            for (int a = 0; a < n1; ++a) {  // line_metric (src/solver/rhs/subcells.rs:94-114)
                double r0, r1, s0, s1;
                g.contravariant(k, affine ? 0 : node_of(dir, line, a), r0, r1, s0, s1);
                metric[a] = dir == 0 ? std::make_pair(r0, r1) : std::make_pair(s0, s1);
            }
            auto end_flux = [&](int a) {
                int node = node_of(dir, line, a);
                return metric[a].first * hu[node] + metric[a].second * hv[node];
            };
            for (int a = 0; a < n1; ++a) {
                double right = a + 1 < n1 ? interfaces[(dir * n1 + line) * (n1 - 1) + a] : end_flux(a);
                double left = a > 0 ? interfaces[(dir * n1 + line) * (n1 - 1) + a - 1] : end_flux(a);
                div[node_of(dir, line, a)] += (right - left) / ops.w1[a];
            }
        }
    for (int i = 0; i < nn; ++i) div[i] *= g.det_j_inv[g.nidx(k, i)];
    for (int f = 0; f < 4; ++f)  // subtract_face_lift
        for (int fi = 0; fi < n1; ++fi) {
            int node = ops.face_nodes[f][fi];
            size_t fn = g.fidx(k, f, fi);
            double scale = g.surface_j[fn] * g.det_j_inv[g.nidx(k, node)];
            double jump = g.nxv[fn] * hu[node] + g.nyv[fn] * hv[node] - face[f * n1 + fi];
            for (int i = 0; i < nn; ++i) div[i] -= scale * ops.lift_at(f, i, fi) * jump;
        }
    return DGSWE_OK;
}

int oracle_stage(oracle_handle* h, const dgswe_stage_plan* p) {
    Model& m = *h->m;
    if (!p) return DGSWE_ERR_INVALID;
    for (int32_t b : {p->base, p->input, p->out})
        if (!check_buffer(m, b).empty()) return DGSWE_ERR_INVALID;
    if (p->accumulate && !check_buffer(m, p->acc).empty()) return DGSWE_ERR_INVALID;
    stage_all(m, *p);
    return DGSWE_OK;
}

int oracle_finish(oracle_handle* h, int32_t acc) {
    if (!check_buffer(*h->m, acc).empty()) return DGSWE_ERR_INVALID;
    finish_all(*h->m, acc);
    return DGSWE_OK;
}

// PhysicsModule::implicit_damping (src/physics/builder.rs:501-504;
// apply_implicit_damping_2d, src/solver/algorithms/wetting_drying.rs:376-389):
// damp_node at every node of buffer `stage`, the rates frozen at `from`
int oracle_implicit_damping(oracle_handle* h, int32_t stage, int32_t from, double dt) {
    Model& m = *h->m;
    if (!check_buffer(m, stage).empty() || !check_buffer(m, from).empty()) return DGSWE_ERR_INVALID;
    if (m.form.friction == DGSWE_FRICTION_NONE && !m.form.has_wet_dry) return DGSWE_OK;
    Buffer& s = m.buf[stage];
    const Buffer& f = m.buf[from];
    const int64_t n = (int64_t)m.n_values();
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) damp_node(m, (size_t)i, s.h[i], s.hu[i], s.hv[i], f.get(i), dt);
    return DGSWE_OK;
}

// PhysicsModule::post_process (src/physics/builder.rs:488-499) of a buffer in
// place, element by element, the clipped elements counted
int oracle_post_process(oracle_handle* h, int32_t buffer) {
    Model& m = *h->m;
    if (!check_buffer(m, buffer).empty()) return DGSWE_ERR_INVALID;
    Buffer& b = m.buf[buffer];
    const int nn = m.ops.nn;
    int64_t clips = 0;
#pragma omp parallel for schedule(static) reduction(+ : clips)
    for (int64_t k = 0; k < m.mesh.n_elements; ++k) {
        const size_t o = (size_t)k * nn;
        clips += post_process_element(m, k, &b.h[o], &b.hu[o], &b.hv[o]) ? 1 : 0;
    }
    m.clips += clips;
    return DGSWE_OK;
}

int oracle_element_dt(oracle_handle* h, double cfl, int32_t scheme, double* dt_el, double* dt_min) {
    double d = min_element_dt(*h->m, cfl, scheme, dt_el);
    if (dt_min) *dt_min = d;
    return DGSWE_OK;
}

int oracle_step(oracle_handle* h, int32_t scheme, double t, double dt) {
    step_one_level(*h->m, scheme, t, dt);
    return DGSWE_OK;
}

int64_t oracle_negative_depth_clips(const oracle_handle* h) { return h->m->clips; }

// Simulation::run_with_callback (src/simulation/runner.rs:264-500) with
// fused one-level stages
int oracle_run(oracle_handle* h, const dgswe_run_config* run, dgswe_callback cb, void* user,
               dgswe_report* report) {
    Model& m = *h->m;
    if (!run || !report) return DGSWE_ERR_INVALID;
    std::memset(report, 0, sizeof(*report));
    std::snprintf(report->device, sizeof(report->device), "cpu (oracle)");
    auto start = std::chrono::steady_clock::now();
    const double LANDING_SLACK = 1e-9;
    double t_start = run->t_start, t_end = run->t_end, t = t_start;
    int64_t n_steps = 0;
    double dt_min_used = INF, dt_max_used = 0.0;
    uint64_t callbacks_done = 0;
    bool has_interval = run->interval > 0.0;
    auto next_callback = [&](uint64_t k) { return t_start + (double)(k + 1) * run->interval; };
    size_t n = m.n_values();
    const Buffer& s = m.buf[DGSWE_STATE];
    auto call = [&](double time) {
        if (cb) cb(user, time, s.h.data(), s.hu.data(), s.hv.data(), (int64_t)n);
    };
    auto finish = [&](int status, const char* msg) {
        report->success = status == DGSWE_OK;
        report->final_time = t;
        report->n_steps = n_steps;
        report->dt_min_used = dt_min_used;
        report->dt_max_used = dt_max_used;
        report->wall_time =
            std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
        report->negative_depth_clips = m.clips;
        std::snprintf(report->message, sizeof(report->message), "%s", msg);
        return status;
    };
    const bool multirate = run->levels > 0;
    if (run->levels < 0 || run->levels > DGSWE_MAX_LEVELS) return DGSWE_ERR_INVALID;
    if (multirate) {
        h->mr = Multirate{};
        h->mr.max_levels = run->levels;
        ShuOsher st[4];
        h->mr.n_stages = scheme_stages(run->scheme, st);
        // the stage values, the last stage's and the sums start as the state
        // (MultirateStepper::step, src/time/multirate.rs:1287-1293)
        for (int b = 1; b <= h->mr.n_stages + 1; ++b) m.buf[b] = m.buf[DGSWE_STATE];
    }
    std::vector<double> element_dt(multirate ? (size_t)m.mesh.n_elements : 0);
    std::vector<uint8_t> line_local;
    call(t);
    char msg[200];
    while (t < t_end) {
        if (run->max_steps > 0 && n_steps >= run->max_steps) {
            std::snprintf(msg, sizeof msg, "Maximum step limit (%lld) reached", (long long)run->max_steps);
            return finish(DGSWE_ERR_MAX_STEPS, msg);
        }
        if (run->stop && *run->stop) {
            std::snprintf(msg, sizeof msg, "Stopped at t = %.1f s", t);
            return finish(DGSWE_ERR_STOPPED, msg);
        }
        double target = has_interval ? fmin_(next_callback(callbacks_done), t_end) : t_end;
        double dt, fitted = INF;
        if (multirate) {
            // Simulation::run_with_callback with a multirate integrator
            // (src/simulation/runner.rs:370-382)
            min_element_dt(m, run->cfl, run->scheme, element_dt.data());
            bool has_lines = false;
            double bound = mr_flags(m, element_dt, line_local, has_lines);
            double cap = run->dt_max > 0.0 ? fmin_(run->dt_max, bound) : bound;
            if (!std::isfinite(cap)) cap = 0.0;
            fitted = mr_assign(m, h->mr, element_dt, has_lines ? &line_local : nullptr, cap,
                               target - t);
            dt = h->mr.stable_step;
        } else {
            dt = min_element_dt(m, run->cfl, run->scheme, nullptr);
        }
        if (run->dt_max > 0.0) dt = fmin_(dt, run->dt_max);
        if (run->dt_min > 0.0 && dt < run->dt_min) {
            std::snprintf(msg, sizeof msg, "Time step (%.2e) below minimum (%.2e)", dt, run->dt_min);
            return finish(DGSWE_ERR_DT_MIN, msg);
        }
        dt_min_used = fmin_(dt_min_used, dt);
        dt_max_used = fmax_(dt_max_used, dt);
        if (multirate) dt = fmin_(dt, fitted);
        bool landed = t + dt * (1.0 + LANDING_SLACK) >= target;
        if (landed) dt = target - t;
        if (multirate)
            mr_step(m, h->mr, run->scheme, t, dt);
        else
            step_one_level(m, run->scheme, t, dt);
        t = landed ? target : t + dt;
        n_steps += 1;
        if (!state_is_finite(m)) {
            std::snprintf(msg, sizeof msg, "The state is not finite at t = %.1f s: it has blown up", t);
            return finish(DGSWE_ERR_NONFINITE, msg);
        }
        if (has_interval) {
            if (t >= next_callback(callbacks_done)) {
                call(t);
                callbacks_done += 1;
            }
        } else {
            call(t);
        }
    }
    return finish(DGSWE_OK, "");
}

int oracle_multirate_stats_get(const oracle_handle* h, dgswe_multirate_stats* out) {
    if (!h || !out) return DGSWE_ERR_INVALID;
    const Multirate& mr = h->mr;
    out->steps = mr.steps;
    out->element_evaluations = mr.element_evaluations;
    out->global_evaluations = mr.global_evaluations;
    out->finest_level = mr.finest_used;
    out->model_seconds = mr.model_seconds;
    out->ideal_evaluations = mr.ideal_evaluations;
    out->level_evaluations = mr.level_evaluations;
    out->line_local_elements = mr.line_local_elements;
    out->plans = 0;
    out->plan_seconds = 0.0;
    out->device_seconds = 0.0;
    return DGSWE_OK;
}

// ---- pointwise entry points for the known-answer tests -------------------

int oracle_time_stencil(const double* times, int64_t n, double t, int cubic, int64_t* idx,
                        double* w) {
    int len = 0;
    if (!time_stencil(times, n, t, cubic != 0, idx, w, len)) return 0;
    return len;
}

double oracle_manning_cbrt(double x) { return manning_cbrt(x); }
double oracle_tidal_ramp(double t, double duration) { return tidal_ramp(t, duration); }
double oracle_hypot(double x, double y) { return ref_hypot(x, y); }
double oracle_drag_coefficient(int kind, double cd, double speed) {
    return drag_coefficient(kind, cd, speed);
}
void oracle_atmosphere_source(double h, double u, double v, double px, double py, int drag,
                              double cd, double rho_air, double rho_water, double h_min,
                              double out[2]) {
    atmosphere_source(h, u, v, px, py, drag, cd, rho_air, rho_water, h_min, out[0], out[1]);
}
double oracle_inverse_barometer_level(double p, double ramp, double rho_water) {
    return inverse_barometer_level(p, ramp, rho_water);
}

void oracle_characteristic_state(const double interior[3], double h_e, double un_e, double ut_e,
                                 double nx, double ny, double g, double h_min, double out[3]) {
    State s = characteristic_state({interior[0], interior[1], interior[2]}, h_e, un_e, ut_e, nx, ny, g,
                                   h_min);
    out[0] = s.h;
    out[1] = s.hu;
    out[2] = s.hv;
}

void oracle_desingularized_velocity(double h_dry, double h, double hu, double hv, double out[2]) {
    WetDry wd;
    wd.h_dry = h_dry;
    wd.desingularized_velocity(h, hu, hv, out[0], out[1]);
}

double oracle_thin_layer_rate(double h_dry, double relaxation_time, double h) {
    WetDry wd;
    wd.h_dry = h_dry;
    wd.relaxation_time = relaxation_time;
    return wd.thin_layer_rate(h);
}

void oracle_correct_node(double h_dry, double max_velocity, double h, double io[2]) {
    WetDry wd;
    wd.h_dry = h_dry;
    wd.max_velocity = max_velocity;
    wd.correct_node(fmax_(h, 0.0), io[0], io[1]);
}

void oracle_wintermeyer_flux(const double l[6], const double r[6], double m0, double m1, double g,
                             double out[3]) {
    Node a{l[0], l[1], l[2], l[3], l[4], l[5]}, b{r[0], r[1], r[2], r[3], r[4], r[5]};
    State f = wintermeyer_flux(a, b, m0, m1, g);
    out[0] = f.h;
    out[1] = f.hu;
    out[2] = f.hv;
}

void oracle_hydrostatic_hll(const double a[4], const double b[4], double m0, double m1, double g,
                            double h_min, double fa[3], double fb[3]) {
    State x, y;
    hydrostatic_hll({a[0], a[1], a[2], a[3]}, {b[0], b[1], b[2], b[3]}, m0, m1, g, h_min, x, y);
    fa[0] = x.h;
    fa[1] = x.hu;
    fa[2] = x.hv;
    fb[0] = y.h;
    fb[1] = y.hu;
    fb[2] = y.hv;
}

void oracle_gll(int order, double* nodes, double* weights, double* d) {
    Ops ops(order);
    for (int i = 0; i < ops.n1; ++i) {
        nodes[i] = ops.x1[i];
        weights[i] = ops.w1[i];
    }
    for (int i = 0; i < ops.n1 * ops.n1; ++i) d[i] = ops.d1[i];
}

double oracle_positivity_cfl(int order) { return positivity_cfl(order); }

void oracle_positivity_bound(int order, int scheme, double out[3]) {
    PositivityBound b = positivity_bound(order, scheme, 1e-3);
    out[0] = b.cfl;
    out[1] = b.max_cfl;
    out[2] = b.max_cfl_subcells;
}

// The element-wise wet/dry correction of one element with nodal masses
// `mass` (wet_dry_element, src/solver/algorithms/wetting_drying.rs:194-215)
int oracle_wet_dry_element(int nn, double* h, double* hu, double* hv, const double* mass,
                           double h_dry, double max_velocity) {
    Model m(1);
    m.form.has_wet_dry = 1;
    m.wd.h_dry = h_dry;
    m.wd.max_velocity = max_velocity;
    m.ops.nn = nn;
    m.geom.nn = nn;
    m.geom.mass.assign(mass, mass + nn);
    double area = 0.0;
    for (int i = 0; i < nn; ++i) area += mass[i];
    m.geom.area.assign(1, area);
    return wet_dry_element(m, 0, h, hu, hv) ? 1 : 0;
}

// The point-implicit damping of nodes (damp_node,
// src/solver/algorithms/wetting_drying.rs:324-357) under uniform Manning
// `manning_n` (≤ 0: none) and the wet/dry thin layer (h_dry ≤ 0: none)
void oracle_damp_nodes(int64_t n, const double* h, double* hu, double* hv, const double* fh,
                       const double* fhu, const double* fhv, double dt, double g, double manning_n,
                       double h_dry, double relaxation_time) {
    Model m(1);
    m.form.friction = manning_n > 0.0 ? DGSWE_FRICTION_MANNING : DGSWE_FRICTION_NONE;
    m.form.manning_h_min = 1e-6;
    m.form.h_min = 1e-6;
    m.form.has_wet_dry = h_dry > 0.0;
    m.wd.h_dry = h_dry;
    m.wd.relaxation_time = relaxation_time;
    m.g_n2.assign(n, g * manning_n * manning_n);
    for (int64_t i = 0; i < n; ++i) damp_node(m, i, h[i], hu[i], hv[i], {fh[i], fhu[i], fhv[i]}, dt);
}

double oracle_tide_elevation(const dgswe_boundary* b, double t) {
    Boundary bc;
    bc.constituents.assign(b->constituents, b->constituents + b->n_constituents);
    bc.mean_elevation = b->mean_elevation;
    bc.ramp_duration = b->ramp_duration;
    return bc.elevation(t);
}


// The Standard-kernel helpers (src/solver/simd/kernels.rs), one element
// each, as the reference's scalar forms compute them

// apply_diff_matrix_scalar (src/solver/simd/kernels.rs:31-61)
void oracle_apply_diff_matrix(const double* d, const double* fh, const double* fhu,
                              const double* fhv, double* oh, double* ohu, double* ohv, int64_t n) {
    for (int64_t i = 0; i < n; ++i) {
        double sh = 0.0, shu = 0.0, shv = 0.0;
        for (int64_t j = 0; j < n; ++j) {
            const double dij = d[i * n + j];
            sh += dij * fh[j];
            shu += dij * fhu[j];
            shv += dij * fhv[j];
        }
        oh[i] = sh;
        ohu[i] = shu;
        ohv[i] = shv;
    }
}

// apply_lift_scalar (src/solver/simd/kernels.rs:74-104)
void oracle_apply_lift(const double* lift, const double* dh, const double* dhu, const double* dhv,
                       double* oh, double* ohu, double* ohv, int64_t n, int64_t nf, double scale) {
    for (int64_t i = 0; i < n; ++i) {
        double sh = 0.0, shu = 0.0, shv = 0.0;
        for (int64_t fi = 0; fi < nf; ++fi) {
            const double l = lift[i * nf + fi];
            sh += l * dh[fi];
            shu += l * dhu[fi];
            shv += l * dhv[fi];
        }
        oh[i] += scale * sh;
        ohu[i] += scale * shu;
        ohv[i] += scale * shv;
    }
}

// coriolis_source_scalar (src/solver/simd/kernels.rs:117-131)
void oracle_coriolis_source(const double* hu, const double* hv, double* ohu, double* ohv, double f,
                            int64_t n) {
    for (int64_t i = 0; i < n; ++i) {
        ohu[i] += f * hv[i];
        ohv[i] += -f * hu[i];
    }
}

// combine_derivatives_scalar (src/solver/simd/kernels.rs:184-224)
void oracle_combine_derivatives(const double* const in[12], double* oh, double* ohu, double* ohv,
                                double rx, double sx, double ry, double sy, int64_t n) {
    double* out[3] = {oh, ohu, ohv};
    for (int64_t i = 0; i < n; ++i)
        for (int v = 0; v < 3; ++v) {
            const double div = in[v][i] * rx + in[3 + v][i] * sx + in[6 + v][i] * ry + in[9 + v][i] * sy;
            out[v][i] = -div;
        }
}

}  // extern "C"
