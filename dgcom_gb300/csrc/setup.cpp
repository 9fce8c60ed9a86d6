// Host-side set-up of a dgswe handle (see setup.hpp).

#include "setup.hpp"

#include "fp64_bits.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <unordered_map>

namespace dgswe {

// ---------------------------------------------------------------------------
// Operators

static void legendre_pd(int n, double x, double& p, double& dp) {
    // Three-term recurrence and P'_n from P_n, P_{n−1}
    // (src/polynomial/legendre.rs:62-94)
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
    double pm = 1.0, pc = x;
    for (int k = 1; k < n; ++k) {
        double pn = ((double)(2 * k + 1) * x * pc - (double)k * pm) / (double)(k + 1);
        pm = pc;
        pc = pn;
    }
    p = pc;
    if (std::fabs(x - 1.0) < 1e-14) {
        dp = (double)(n * (n + 1)) / 2.0;
    } else if (std::fabs(x + 1.0) < 1e-14) {
        dp = ((n & 1) ? 1.0 : -1.0) * (double)(n * (n + 1)) / 2.0;
    } else {
        dp = (double)n * (x * pc - pm) / (x * x - 1.0);
    }
}

Operators::Operators(int order_) : order(order_), n1(order_ + 1), nn((order_ + 1) * (order_ + 1)) {
    const int n = order;
    // GLL nodes: Newton on (1−x²)P'_N from the Chebyshev–Lobatto points
    // (src/polynomial/nodes.rs:17-77)
    x.assign(n1, 0.0);
    for (int j = 0; j <= n; ++j) x[j] = -std::cos(M_PI * (double)j / (double)n);
    x[0] = -1.0;
    x[n] = 1.0;
    for (int j = 1; j < n; ++j) {
        double xj = x[j];
        for (int it = 0; it < 100; ++it) {
            double p, dp;
            legendre_pd(n, xj, p, dp);
            double step = (1.0 - xj * xj) * dp / ((double)n * (double)(n + 1) * p);
            if (std::fabs(step) < 1e-15) break;
            xj += step;
        }
        x[j] = xj;
    }
    // w_j = 2/(N(N+1) P_N(x_j)²) (src/polynomial/nodes.rs:82-103)
    w.assign(n1, 0.0);
    for (int j = 0; j < n1; ++j) {
        double p, dp;
        legendre_pd(n, x[j], p, dp);
        w[j] = 2.0 / ((double)(n * (n + 1)) * p * p);
    }
    // D_ij = ℓ_j'(x_i) at these nodes: barycentric weights in long double;
    // the diagonal from the row sums, exactly 0 where it vanishes
    d.assign(n1 * n1, 0.0);
    long double bw[kMaxN1];
    for (int j = 0; j < n1; ++j) {
        long double prod = 1.0L;
        for (int k = 0; k < n1; ++k)
            if (k != j) prod *= (long double)x[j] - (long double)x[k];
        bw[j] = 1.0L / prod;
    }
    for (int i = 0; i < n1; ++i) {
        long double row = 0.0L;
        for (int j = 0; j < n1; ++j) {
            if (j == i) continue;
            long double v = (bw[j] / bw[i]) / ((long double)x[i] - (long double)x[j]);
            d[i * n1 + j] = (double)v;
            row += v;
        }
        double diag = (double)(-row);
        d[i * n1 + i] = std::fabs(diag) < 1e-14 ? 0.0 : diag;
    }
    r.assign(nn, 0.0);
    s.assign(nn, 0.0);
    w2.assign(nn, 0.0);
    for (int j = 0; j < n1; ++j)
        for (int a = 0; a < n1; ++a) {
            r[j * n1 + a] = x[a];
            s[j * n1 + a] = x[j];
            w2[j * n1 + a] = w[a] * w[j];
        }
    // Faces counter-clockwise; faces 2 and 3 list their nodes in reverse
    // (src/operators/operators_2d.rs:388-412)
    for (int q = 0; q < n1; ++q) {
        face_node[0][q] = q;
        face_node[1][q] = q * n1 + n1 - 1;
        face_node[2][q] = (n1 - 1) * n1 + (n1 - 1 - q);
        face_node[3][q] = (n1 - 1 - q) * n1;
    }
}

double Operators::lift(int face, int node, int fi) const {
    double e = face_node[face][fi] == node ? 1.0 : 0.0;
    return (1.0 / w2[node]) * (e * w[fi]);
}

// ---------------------------------------------------------------------------
// Topology: faces with the same two vertices are one edge, its left side
// the first to appear; periodic pairs are edges of their own

std::string build_topology(const dgswe_form& f, Topology& topo) {
    const int64_t K = f.n_elements;
    topo.n_elements = K;
    topo.link.assign(K, {});
    topo.tag.assign(K, {0, 0, 0, 0});
    topo.corners.assign(K, {});
    for (int64_t k = 0; k < K; ++k)
        for (int c = 0; c < 4; ++c) {
            int64_t v = f.elements[4 * k + c];
            if (v < 0 || v >= f.n_vertices) return "an element uses a vertex that does not exist";
            topo.corners[k][2 * c] = f.vertices[2 * v];
            topo.corners[k][2 * c + 1] = f.vertices[2 * v + 1];
        }
    auto verts = [&](int64_t k, int face) {
        return std::make_pair(f.elements[4 * k + face], f.elements[4 * k + (face + 1) % 4]);
    };
    // periodic faces → pair index
    std::vector<int64_t> periodic_of(K * 4, -1);
    for (int64_t p = 0; p < f.n_periodic; ++p)
        for (int side = 0; side < 2; ++side) {
            int64_t k = f.periodic[4 * p + 2 * side];
            int64_t fc = f.periodic[4 * p + 2 * side + 1];
            if (k < 0 || k >= K || fc < 0 || fc > 3) return "a periodic face does not exist";
            if (periodic_of[k * 4 + fc] >= 0) return "a periodic face is paired twice";
            periodic_of[k * 4 + fc] = p;
        }
    struct Key {
        size_t operator()(uint64_t x) const { return std::hash<uint64_t>()(x * 0x9E3779B97F4A7C15ull); }
    };
    std::unordered_map<uint64_t, int64_t, Key> first_face;  // vertex pair → k·4 + face
    first_face.reserve((size_t)(2 * K + 16));
    std::vector<uint8_t> matched(K * 4, 0);
    for (int64_t k = 0; k < K; ++k)
        for (int fc = 0; fc < 4; ++fc) {
            if (periodic_of[k * 4 + fc] >= 0) continue;
            auto ab = verts(k, fc);
            uint64_t lo = (uint64_t)std::min(ab.first, ab.second);
            uint64_t hi = (uint64_t)std::max(ab.first, ab.second);
            uint64_t key = lo * (uint64_t)(f.n_vertices + 1) + hi;
            auto it = first_face.find(key);
            if (it == first_face.end()) {
                first_face.emplace(key, k * 4 + fc);
                continue;
            }
            int64_t other = it->second;
            if (other < 0) return "an edge is shared by more than two elements";
            int64_t ok = other / 4;
            int of = (int)(other % 4);
            auto lv = verts(ok, of);
            if (!(lv.first == ab.second && lv.second == ab.first))
                return "two faces traverse their shared edge in the same direction";
            topo.link[ok][of] = {k, fc, true, true};
            topo.link[k][fc] = {ok, of, false, true};
            matched[ok * 4 + of] = matched[k * 4 + fc] = 1;
            it->second = -1;
        }
    for (int64_t p = 0; p < f.n_periodic; ++p) {
        int64_t ka = f.periodic[4 * p], kb = f.periodic[4 * p + 2];
        int fa = (int)f.periodic[4 * p + 1], fb = (int)f.periodic[4 * p + 3];
        for (auto [kk, ff] : {std::make_pair(ka, fa), std::make_pair(kb, fb)}) {
            auto ab = verts(kk, ff);
            uint64_t lo = (uint64_t)std::min(ab.first, ab.second);
            uint64_t hi = (uint64_t)std::max(ab.first, ab.second);
            if (first_face.count(lo * (uint64_t)(f.n_vertices + 1) + hi))
                return "a periodic face shares its vertices with another face";
        }
        // The left side of a periodic edge is its pair's first face
        auto shared_v = verts(kb, fb) == std::make_pair(verts(ka, fa).second, verts(ka, fa).first);
        topo.link[ka][fa] = {kb, fb, true, shared_v};
        topo.link[kb][fb] = {ka, fa, false, shared_v};
        matched[ka * 4 + fa] = matched[kb * 4 + fb] = 1;
    }
    for (int64_t k = 0; k < K; ++k)
        for (int fc = 0; fc < 4; ++fc)
            if (!matched[k * 4 + fc]) {
                topo.link[k][fc] = Link{};
                topo.tag[k][fc] = f.face_tags ? f.face_tags[4 * k + fc] : 0;
            }
    return "";
}

// ---------------------------------------------------------------------------
// Geometry: the bilinear map's derivatives at (r, s)
// (src/operators/geometric.rs:704-718)

struct Jac {
    double x_r, x_s, y_r, y_s, det;
};

static Jac jacobian(const std::array<double, 8>& c, double r, double s) {
    const double x0 = c[0], y0 = c[1], x1 = c[2], y1 = c[3];
    const double x2 = c[4], y2 = c[5], x3 = c[6], y3 = c[7];
    Jac m;
    m.x_r = 0.25 * ((1.0 - s) * (x1 - x0) + (1.0 + s) * (x2 - x3));
    m.y_r = 0.25 * ((1.0 - s) * (y1 - y0) + (1.0 + s) * (y2 - y3));
    m.x_s = 0.25 * ((1.0 - r) * (x3 - x0) + (1.0 + r) * (x2 - x1));
    m.y_s = 0.25 * ((1.0 - r) * (y3 - y0) + (1.0 + r) * (y2 - y1));
    m.det = m.x_r * m.y_s - m.x_s * m.y_r;
    return m;
}

std::string element_geometry(const Operators& ops, const std::array<double, 8>& c,
                             ElementGeometry& g) {
    // a parallelogram has no bilinear term (src/operators/geometric.rs:722-733)
    double bx = c[0] - c[2] + c[4] - c[6], by = c[1] - c[3] + c[5] - c[7];
    double scale = 0.0;
    for (int i = 0; i < 4; ++i) {
        int j = (i + 1) % 4;
        scale = std::fmax(scale, std::hypot(c[2 * j] - c[2 * i], c[2 * j + 1] - c[2 * i + 1]));
    }
    g.affine = std::hypot(bx, by) <= 1.0e-12 * scale;
    g.area = 0.0;
    for (int i = 0; i < ops.nn; ++i) {
        Jac m = jacobian(c, ops.r[i], ops.s[i]);
        if (!(std::isfinite(m.det) && m.det > 0.0))
            return "an element has a Jacobian that is not positive and finite "
                   "(degenerate, non-convex or clockwise)";
        g.rx[i] = m.y_s / m.det;
        g.ry[i] = -m.x_s / m.det;
        g.sx[i] = -m.y_r / m.det;
        g.sy[i] = m.x_r / m.det;
        g.det[i] = m.det;
        g.det_inv[i] = 1.0 / m.det;
        g.mass[i] = ops.w2[i] * m.det;
        g.area += g.mass[i];
    }
    for (int face = 0; face < 4; ++face) {
        int node = ops.face_node[face][0];
        Jac m = jacobian(c, ops.r[node], ops.s[node]);
        double vx, vy;
        if (face == 0) {
            vx = m.y_r;
            vy = -m.x_r;
        } else if (face == 1) {
            vx = m.y_s;
            vy = -m.x_s;
        } else if (face == 2) {
            vx = -m.y_r;
            vy = m.x_r;
        } else {
            vx = -m.y_s;
            vy = m.x_s;
        }
        double sj = std::sqrt(vx * vx + vy * vy);
        g.sj[face] = sj;
        g.nx[face] = vx / sj;
        g.ny[face] = vy / sj;
    }
    for (int i = 0; i < ops.nn; ++i) {
        int src = g.affine ? 0 : i;
        double j = g.det[src];
        g.mr0[i] = j * g.rx[src];
        g.mr1[i] = j * g.ry[src];
        g.ms0[i] = j * g.sx[src];
        g.ms1[i] = j * g.sy[src];
    }
    return "";
}

// ---------------------------------------------------------------------------
// Pair schedule: orient the pair graph (every node paired with the other
// nodes of its two GLL lines, degree 2(n1−1)) along an Euler circuit, so
// every node owns exactly n1−1 pairs

static int line_node(int n1, int dir, int line, int pos) {
    return dir == 0 ? line * n1 + pos : pos * n1 + line;
}

PairSchedule::PairSchedule(const Operators& ops) : n1(ops.n1), nn(ops.nn) {
    struct E {
        int u, v, dir, pu, pv;
        bool used;
    };
    std::vector<E> edges;
    std::vector<std::vector<int>> adj(nn);
    for (int dir = 0; dir < 2; ++dir)
        for (int line = 0; line < n1; ++line)
            for (int pa = 0; pa < n1; ++pa)
                for (int pc = pa + 1; pc < n1; ++pc) {
                    int a = line_node(n1, dir, line, pa), c = line_node(n1, dir, line, pc);
                    adj[a].push_back((int)edges.size());
                    adj[c].push_back((int)edges.size());
                    edges.push_back({a, c, dir, pa, pc, false});
                }
    // Hierholzer: walk unused edges, each traversed u → v is owned by u
    std::vector<std::vector<PairSlot>> own(nn);
    std::vector<size_t> next(nn, 0);
    std::vector<int> stack{0};
    std::vector<int> via{-1};
    while (!stack.empty()) {
        int u = stack.back();
        while (next[u] < adj[u].size() && edges[adj[u][next[u]]].used) ++next[u];
        if (next[u] == adj[u].size()) {
            int e = via.back();
            stack.pop_back();
            via.pop_back();
            (void)e;
            continue;
        }
        int e = adj[u][next[u]];
        edges[e].used = true;
        E& ed = edges[e];
        int v = ed.u == u ? ed.v : ed.u;
        PairSlot ps;
        ps.dir = (int8_t)ed.dir;
        // a before c along the line
        ps.a = (int8_t)ed.u;
        ps.c = (int8_t)ed.v;
        ps.pa = (int8_t)ed.pu;
        ps.pc = (int8_t)ed.pv;
        own[u].push_back(ps);
        stack.push_back(v);
        via.push_back(e);
    }
    owned.resize(nn * (n1 - 1));
    for (int i = 0; i < nn; ++i)
        for (int j = 0; j < n1 - 1; ++j) owned[i * (n1 - 1) + j] = own[i].at(j);
    accum_slot.assign(nn * 2 * (n1 - 1), -1);
    accum_coef.assign(nn * 2 * (n1 - 1), 0.0);
    std::vector<int> filled(nn, 0);
    for (int o = 0; o < nn; ++o)
        for (int j = 0; j < n1 - 1; ++j) {
            const PairSlot& ps = owned[o * (n1 - 1) + j];
            int slot = o * (n1 - 1) + j;
            // rhs_x −= 2 D(pos_x, pos_y) F at both ends
            int ends[2] = {ps.a, ps.c};
            int pos[2] = {ps.pa, ps.pc};
            for (int e = 0; e < 2; ++e) {
                int x = ends[e];
                int q = filled[x]++;
                accum_slot[x * 2 * (n1 - 1) + q] = slot;
                accum_coef[x * 2 * (n1 - 1) + q] = 2.0 * ops.d[pos[e] * n1 + pos[1 - e]];
            }
        }
}

// ---------------------------------------------------------------------------
// Tables

std::string build_tables(const dgswe_form& f, const Operators& ops, const Topology& topo,
                         const std::vector<int32_t>& tags, const std::vector<int32_t>& cond_index,
                         Tables& t) {
    const int n1 = ops.n1, nn = ops.nn;
    const int64_t K = topo.n_elements;
    t.n1 = n1;
    t.nn = nn;
    t.K = K;
    t.npair = n1 - 1;
    const size_t NV = (size_t)K * nn, NF = (size_t)K * 4 * n1;
    PairSchedule sched(ops);
    t.bed.assign(NV, 0.0);
    if (f.bathymetry) std::memcpy(t.bed.data(), f.bathymetry, NV * 8);
    t.jinv.assign(NV, 0.0);
    t.pair_hm.assign(NV * (n1 - 1) * 2, 0.0);
    t.gdb.assign(NV * 2, 0.0);
    t.contra.assign(NV * 4, 0.0);
    t.affine.assign(K, 0);
    t.lift_scale.assign(NF, 0.0);
    t.outer_idx.assign(NF, -1);
    t.outer_dist.assign(NF, 0.0);
    t.mass.assign(NV, 0.0);
    t.inv_area.assign(K, 0.0);
    t.weight_ratio.assign(K, 0.0);
    t.dtm_own.assign(NV * 6, 0.0);
    t.dtm_face.assign(NF * 6, 0.0);
    t.nb_face_node.assign(NF, -1);
    if (f.has_coriolis && f.coriolis_beta != 0.0) t.fcor.assign(NV, 0.0);
    if (f.friction == DGSWE_FRICTION_MANNING_NODES) {
        t.g_n2.assign(NV, 0.0);
        for (size_t i = 0; i < NV; ++i)
            t.g_n2[i] = f.friction_g * f.manning_n_nodes[i] * f.manning_n_nodes[i];
    }
    const double g = f.g;
    const bool has_bed = f.bathymetry != nullptr;
    std::vector<ElementGeometry> geo(K);
    std::string err;
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < K; ++k) {
        std::string e = element_geometry(ops, topo.corners[k], geo[k]);
        if (!e.empty()) {
#pragma omp critical
            err = e;
        }
    }
    if (!err.empty()) return err;
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < K; ++k) {
        const ElementGeometry& G = geo[k];
        const size_t o = (size_t)k * nn;
        t.affine[k] = G.affine ? 1 : 0;
        t.inv_area[k] = 1.0 / G.area;
        double weight = 0.0, weight_b = 0.0;
        for (int i = 0; i < nn; ++i) {
            t.jinv[o + i] = G.affine ? G.det_inv[0] : G.det_inv[i];
            t.mass[o + i] = G.mass[i];
            t.contra[(o + i) * 4 + 0] = G.mr0[i];
            t.contra[(o + i) * 4 + 1] = G.mr1[i];
            t.contra[(o + i) * 4 + 2] = G.ms0[i];
            t.contra[(o + i) * 4 + 3] = G.ms1[i];
            weight += G.mass[i];
            int a = i % n1, j = i / n1;
            if (a == 0 || a == n1 - 1 || j == 0 || j == n1 - 1) weight_b += G.mass[i];
            // time-step metric: a parallelogram's node-0 ∇r, ∇s for its own
            // nodes (src/solver/rhs/swe_2d.rs:1308-1341)
            int src = G.affine ? 0 : i;
            double* m = &t.dtm_own[(o + i) * 6];
            m[0] = G.rx[src];
            m[1] = G.ry[src];
            m[2] = G.sx[src];
            m[3] = G.sy[src];
            m[4] = std::sqrt(m[0] * m[0] + m[1] * m[1]);
            m[5] = std::sqrt(m[2] * m[2] + m[3] * m[3]);
            for (int c = 0; c < 6; ++c) m[c] *= 0.25;  // the rate's ¼, exact
            if (!t.fcor.empty()) {
                double r = ops.r[i], s = ops.s[i];
                const auto& c = topo.corners[k];
                double n0 = (1.0 - r) * (1.0 - s) / 4.0, nb1 = (1.0 + r) * (1.0 - s) / 4.0;
                double n2 = (1.0 + r) * (1.0 + s) / 4.0, n3 = (1.0 - r) * (1.0 + s) / 4.0;
                double y = n0 * c[1] + nb1 * c[3] + n2 * c[5] + n3 * c[7];
                t.fcor[o + i] = f.coriolis_f0 + f.coriolis_beta * (y - f.coriolis_y0);
            }
        }
        t.weight_ratio[k] = weight / weight_b;
        // pair metrics, in owner order
        for (int i = 0; i < nn; ++i)
            for (int j = 0; j < n1 - 1; ++j) {
                const PairSlot& ps = sched.owned[i * (n1 - 1) + j];
                double m0, m1;
                if (G.affine) {
                    m0 = ps.dir == 0 ? G.mr0[0] : G.ms0[0];
                    m1 = ps.dir == 0 ? G.mr1[0] : G.ms1[0];
                } else if (ps.dir == 0) {
                    m0 = 0.5 * (G.mr0[ps.a] + G.mr0[ps.c]);
                    m1 = 0.5 * (G.mr1[ps.a] + G.mr1[ps.c]);
                } else {
                    m0 = 0.5 * (G.ms0[ps.a] + G.ms0[ps.c]);
                    m1 = 0.5 * (G.ms1[ps.a] + G.ms1[ps.c]);
                }
                size_t q = ((o + i) * (n1 - 1) + j) * 2;
                t.pair_hm[q] = 0.5 * m0;
                t.pair_hm[q + 1] = 0.5 * m1;
            }
        // bed slope, both directions (src/solver/rhs/swe_2d_split_form.rs:876-890)
        if (has_bed) {
            for (int i = 0; i < nn; ++i) {
                double gx = 0.0, gy = 0.0;
                for (int dir = 0; dir < 2; ++dir) {
                    int line = dir == 0 ? i / n1 : i % n1;
                    int pa = dir == 0 ? i % n1 : i / n1;
                    const double* M0 = dir == 0 ? G.mr0 : G.ms0;
                    const double* M1 = dir == 0 ? G.mr1 : G.ms1;
                    double db = 0.0, dbx = 0.0, dby = 0.0;
                    for (int pc = 0; pc < n1; ++pc) {
                        int c = line_node(n1, dir, line, pc);
                        double d_b = ops.d[pa * n1 + pc] * t.bed[o + c];
                        db += d_b;
                        dbx += d_b * M0[c];
                        dby += d_b * M1[c];
                    }
                    double bx, by;
                    if (G.affine) {
                        bx = db * M0[i];
                        by = db * M1[i];
                    } else {
                        bx = 0.5 * (db * M0[i] + dbx);
                        by = 0.5 * (db * M1[i] + dby);
                    }
                    gx += g * bx;
                    gy += g * by;
                }
                t.gdb[(o + i) * 2] = gx;
                t.gdb[(o + i) * 2 + 1] = gy;
            }
        }
        for (int face = 0; face < 4; ++face) {
            const Link& L = topo.link[k][face];
            for (int fi = 0; fi < n1; ++fi) {
                int node = ops.face_node[face][fi];
                size_t q = ((size_t)k * 4 + face) * n1 + fi;
                t.lift_scale[q] = G.sj[face] * ops.lift(face, node, fi);
                // the own node's stored ∇r, ∇s for the neighbour's face node
                // (src/solver/rhs/swe_2d.rs:2090-2104)
                double* m = &t.dtm_face[q * 6];
                m[0] = G.rx[node];
                m[1] = G.ry[node];
                m[2] = G.sx[node];
                m[3] = G.sy[node];
                m[4] = std::sqrt(m[0] * m[0] + m[1] * m[1]);
                m[5] = std::sqrt(m[2] * m[2] + m[3] * m[3]);
                for (int c = 0; c < 6; ++c) m[c] *= 0.25;  // the rate's ¼, exact
                if (L.element < 0) continue;
                const ElementGeometry& NB = geo[L.element];
                int nb_node = ops.face_node[L.face][n1 - 1 - fi];
                t.nb_face_node[q] = L.element * nn + nb_node;
                // the neighbour's first interior node on the GLL line
                // through the face node, and its distance in this element's
                // reference coordinate (src/solver/rhs/swe_2d_split_form.rs:1048-1085)
                int inner = L.face == 0 ? nb_node + n1
                            : L.face == 1 ? nb_node - 1
                            : L.face == 2 ? nb_node - n1
                                          : nb_node + 1;
                double h_nb = NB.affine ? NB.det[0] / NB.sj[L.face] : NB.det[nb_node] / NB.sj[L.face];
                double h_own = G.affine ? G.det[0] / G.sj[face] : G.det[node] / G.sj[face];
                t.outer_idx[q] = L.element * nn + inner;
                t.outer_dist[q] = (ops.x[1] - ops.x[0]) * h_nb / h_own;
            }
        }
    }
    // faces: every interior edge once, from its left side with that side's
    // normal (src/solver/rhs/swe_2d_split_form.rs:580-616); boundary faces
    auto geo5 = [](double nx, double ny, double* out) {
        double norm = std::sqrt(nx * nx + ny * ny);
        double inv = 1.0 / norm;
        out[0] = nx;
        out[1] = ny;
        out[2] = norm;
        out[3] = nx * inv;
        out[4] = ny * inv;
    };
    for (int64_t k = 0; k < K; ++k)
        for (int face = 0; face < 4; ++face) {
            const Link& L = topo.link[k][face];
            if (L.element >= 0) {
                if (!L.left) continue;
                t.edge_left.push_back(k * 4 + face);
                t.edge_right.push_back(L.element * 4 + L.face);
                double g5[5];
                geo5(geo[k].nx[face], geo[k].ny[face], g5);
                t.edge_geo.insert(t.edge_geo.end(), g5, g5 + 5);
            } else {
                int32_t tag = topo.tag[k][face];
                auto it = std::find(tags.begin(), tags.end(), tag);
                if (it == tags.end())
                    return "no boundary condition for the faces tagged " + std::to_string(tag);
                t.bface.push_back(k * 4 + face);
                t.bface_cond.push_back(cond_index[it - tags.begin()]);
                double g5[5];
                geo5(geo[k].nx[face], geo[k].ny[face], g5);
                t.bface_geo.insert(t.bface_geo.end(), g5, g5 + 5);
            }
        }
    t.dtm32_own.resize(t.dtm_own.size());
    t.dtm32_face.resize(t.dtm_face.size());
    for (size_t i = 0; i < t.dtm_own.size(); ++i) t.dtm32_own[i] = fp::f32_trunc(t.dtm_own[i]);
    for (size_t i = 0; i < t.dtm_face.size(); ++i) t.dtm32_face[i] = fp::f32_trunc(t.dtm_face[i]);
    return "";
}

}  // namespace dgswe
