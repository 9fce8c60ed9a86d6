// The multirate level planner (multirate.hpp); host code, OpenMP over
// elements.
#include "multirate.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <utility>

#include <omp.h>

namespace dgswe {

namespace {

const double kLandingSlack = 1e-9;  // LANDING_SLACK (src/time/multirate.rs:589)

inline bool finite(double x) { return std::isfinite(x); }

// items 0..n by key, largest first, index order within a key; at_least[d]
// for d in 0..=finest. A counting sort: each thread counts its contiguous
// chunk, the chunks' offsets follow from the counts, each thread scatters
// its chunk in index order, so the order is the serial one.
template <class Key>
void order_by_key(int64_t n, int finest, Key key, std::vector<int32_t>& order,
                  std::vector<int64_t>& at_least) {
    const int V = finest + 1;
    const int max_threads = omp_get_max_threads();
    std::vector<int64_t> hist((size_t)max_threads * V, 0), off((size_t)max_threads * V, 0);
    at_least.assign(V + 1, 0);
    order.assign(n, 0);
#pragma omp parallel num_threads(max_threads)
    {
        const int t = omp_get_thread_num(), nt = omp_get_num_threads();
        const int64_t lo = n * t / nt, hi = n * (t + 1) / nt;
        int64_t* h = &hist[(size_t)t * V];
        for (int64_t i = lo; i < hi; ++i) h[key(i)] += 1;
#pragma omp barrier
#pragma omp single
        {
            std::vector<int64_t> count(V, 0);
            for (int u = 0; u < nt; ++u)
                for (int v = 0; v < V; ++v) count[v] += hist[(size_t)u * V + v];
            for (int d = V - 1; d >= 0; --d) at_least[d] = at_least[d + 1] + count[d];
            for (int v = 0; v < V; ++v) {
                int64_t o = at_least[v + 1];  // key v starts after the larger keys
                for (int u = 0; u < nt; ++u) {
                    off[(size_t)u * V + v] = o;
                    o += hist[(size_t)u * V + v];
                }
            }
        }
        int64_t* o = &off[(size_t)t * V];
        for (int64_t i = lo; i < hi; ++i) order[o[key(i)]++] = (int32_t)i;
    }
    at_least.resize(V);
}

}  // namespace

MultiratePlanner::MultiratePlanner(std::vector<std::array<int64_t, 4>> neighbour,
                                   std::vector<std::array<int8_t, 4>> nb_face,
                                   const int (*face_node)[5], int n1, int max_levels,
                                   int n_stages)
    : nb_(std::move(neighbour)),
      nb_face_(std::move(nb_face)),
      n1_(n1),
      nn_(n1 * n1),
      max_levels_(std::min(max_levels, kMaxLevels)),
      n_stages_(n_stages),
      K_((int64_t)nb_.size()) {
    for (int f = 0; f < 4; ++f)
        for (int i = 0; i < 5; ++i) face_node_[f][i] = i < n1 ? face_node[f][i] : 0;
    level_.assign(K_, 0);
    for (int s = 0; s < n_stages_; ++s) rate_[s].assign(K_, 0);
}

int MultiratePlanner::depth(int64_t p, int finest) {
    if (p == 0 || p == (int64_t)1 << finest) return 0;
    int tz = 0;
    while (((p >> tz) & 1) == 0) ++tz;
    return finest - tz;
}

double MultiratePlanner::assign_levels(const double* element_dt, int64_t n, int max_levels,
                                       double dt_cap, std::vector<uint8_t>& level, int& finest) {
    double lo = std::numeric_limits<double>::infinity(), hi = 0.0;
#pragma omp parallel for schedule(static) reduction(min : lo) reduction(max : hi)
    for (int64_t k = 0; k < n; ++k) {
        const double d = element_dt[k];
        if (!finite(d)) continue;
        lo = std::min(lo, d);
        hi = std::max(hi, d);
    }
    level.assign(n, 0);
    finest = 0;
    if (!finite(lo)) return std::numeric_limits<double>::infinity();
    const bool capped = dt_cap > 0.0 && finite(dt_cap);
    while (finest < max_levels) {
        // powers of two scale exactly: level L steps exactly dt_min
        const double coarser = lo * (double)(2ull << finest);
        if (coarser > hi || (capped && coarser > dt_cap)) break;
        finest += 1;
    }
    const double dt = lo * (double)(1ull << finest);
    const int L = finest;
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < n; ++k) {
        int l = 0;
        double dl = dt;
        while (l < L && dl > element_dt[k]) {
            dl *= 0.5;
            l += 1;
        }
        level[k] = (uint8_t)l;
    }
    return dt;
}

int MultiratePlanner::levels_for_step(const double* element_dt, int64_t n, double dt,
                                      int max_levels, std::vector<uint8_t>& level) {
    int finest = 0;
#pragma omp parallel for schedule(static) reduction(max : finest)
    for (int64_t k = 0; k < n; ++k) {
        int l = 0;
        double dl = dt;
        while (l < max_levels && dl > element_dt[k]) {
            dl *= 0.5;
            l += 1;
        }
        level[k] = (uint8_t)l;
        finest = std::max(finest, l);
    }
    return finest;
}

// to[k] = max(from[k], from[j] − 1) over the face neighbours j, until no
// element changes (limit_level_jumps, multirate.rs:745-752)
void MultiratePlanner::limit_level_jumps(std::vector<uint8_t>& level) {
    scratch_.assign(K_, 0);
    for (;;) {
        int changed = 0;
#pragma omp parallel for schedule(static) reduction(| : changed)
        for (int64_t k = 0; k < K_; ++k) {
            uint8_t m = level[k];
            for (int f = 0; f < 4; ++f) {
                const int64_t j = nb_[k][f];
                if (j < 0) continue;
                const uint8_t v = level[j];
                const uint8_t dropped = v > 0 ? (uint8_t)(v - 1) : 0;
                m = std::max(m, dropped);
            }
            scratch_[k] = m;
            changed |= m != level[k] ? 1 : 0;
        }
        if (!changed) break;
        std::swap(level, scratch_);
    }
}

// to[k] = the largest `from` over k and its face neighbours
void MultiratePlanner::spread_faces(const std::vector<uint8_t>& from,
                                    std::vector<uint8_t>& to) const {
    to.assign(K_, 0);
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < K_; ++k) {
        uint8_t m = from[k];
        for (int f = 0; f < 4; ++f) {
            const int64_t j = nb_[k][f];
            if (j >= 0) m = std::max(m, from[j]);
        }
        to[k] = m;
    }
}

// One stage of node rates (spread_over_lines, multirate.rs:678-743): a
// line-local element's node follows its two GLL lines and, on a face, the
// neighbour's coincident node; any other element follows all of its own
// nodes and its neighbours' shared-face nodes and the nodes one in from them
void MultiratePlanner::spread_lines(const uint8_t* line_local, const std::vector<uint8_t>& from,
                                    std::vector<uint8_t>& to, std::vector<uint8_t>& rate) const {
    const int n1 = n1_, nn = nn_;
    to.assign((size_t)K_ * nn, 0);
    rate.assign(K_, 0);
    auto inner = [n1](int face, int node) {
        switch (face) {
            case 0: return node + n1;
            case 1: return node - 1;
            case 2: return node - n1;
            default: return node + 1;
        }
    };
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < K_; ++k) {
        const uint8_t* own = &from[(size_t)k * nn];
        uint8_t* out = &to[(size_t)k * nn];
        if (!line_local || !line_local[k]) {
            uint8_t m = 0;
            for (int i = 0; i < nn; ++i) m = std::max(m, own[i]);
            for (int f = 0; f < 4; ++f) {
                const int64_t j = nb_[k][f];
                if (j < 0) continue;
                const uint8_t* other = &from[(size_t)j * nn];
                const int of = nb_face_[k][f];
                for (int fi = 0; fi < n1; ++fi) {
                    const int node = face_node_[of][fi];
                    m = std::max(m, std::max(other[node], other[inner(of, node)]));
                }
            }
            for (int i = 0; i < nn; ++i) out[i] = m;
            rate[k] = m;
            continue;
        }
        // r-lines (rows), then s-lines (columns)
        for (int r = 0; r < n1; ++r) {
            uint8_t m = 0;
            for (int i = 0; i < n1; ++i) m = std::max(m, own[r * n1 + i]);
            for (int i = 0; i < n1; ++i) out[r * n1 + i] = m;
        }
        for (int c = 0; c < n1; ++c) {
            uint8_t m = 0;
            for (int r = 0; r < n1; ++r) m = std::max(m, own[r * n1 + c]);
            for (int r = 0; r < n1; ++r) out[r * n1 + c] = std::max(out[r * n1 + c], m);
        }
        for (int f = 0; f < 4; ++f) {
            const int64_t j = nb_[k][f];
            if (j < 0) continue;
            const uint8_t* other = &from[(size_t)j * nn];
            const int of = nb_face_[k][f];
            for (int fi = 0; fi < n1; ++fi) {
                const int node = face_node_[f][fi];
                out[node] = std::max(out[node], other[face_node_[of][n1 - 1 - fi]]);
            }
        }
        uint8_t m = 0;
        for (int i = 0; i < nn; ++i) m = std::max(m, out[i]);
        rate[k] = m;
    }
}

void MultiratePlanner::make_lists() {
    const int L = finest_;
    int64_t ev = 0;
    for (int s = 0; s < n_stages_; ++s)
        for (int64_t k = 0; k < K_; ++k) ev += (int64_t)1 << rate_[s][k];
    evaluations_ = ev;
    for (int j = 0; j <= n_stages_; ++j) {
        const std::vector<uint8_t>& key = j < n_stages_ ? rate_[j] : level_;
        order_by_key(K_, L, [&](int64_t i) { return (int)key[i]; }, order_[j], count_[j]);
    }
    for (int s = 0; s < n_stages_; ++s) {
        edge_order_[s].clear();
        bface_order_[s].clear();
        edge_count_[s].clear();
        bface_count_[s].clear();
    }
    version_ += 1;
}

void MultiratePlanner::edge_lists(const std::vector<int64_t>& edge_left,
                                  const std::vector<int64_t>& edge_right,
                                  const std::vector<int64_t>& bface) {
    const int L = finest_;
    for (int s = 0; s < n_stages_; ++s) {
        if (!edge_count_[s].empty()) continue;  // made for this plan already
        const std::vector<uint8_t>& r = rate_[s];
        order_by_key(
            (int64_t)edge_left.size(), L,
            [&](int64_t e) { return (int)std::max(r[edge_left[e] >> 2], r[edge_right[e] >> 2]); },
            edge_order_[s], edge_count_[s]);
        order_by_key(
            (int64_t)bface.size(), L, [&](int64_t b) { return (int)r[bface[b] >> 2]; },
            bface_order_[s], bface_count_[s]);
    }
}

void MultiratePlanner::set_plan(const uint8_t* levels, const uint8_t* rates) {
    memo_ = false;
    level_.assign(levels, levels + K_);
    int finest = 0;
    for (int64_t k = 0; k < K_; ++k) finest = std::max(finest, (int)level_[k]);
    for (int s = 0; s < n_stages_; ++s) rate_[s].assign(rates + s * K_, rates + (s + 1) * K_);
    finest_ = finest;
    int64_t lev = 0;
    for (int64_t k = 0; k < K_; ++k) lev += (int64_t)1 << level_[k];
    level_evaluations_ = (int64_t)n_stages_ * lev;
    inverse_dt_sum_ = 0.0;
    n_line_local_ = 0;
    make_lists();
}

void MultiratePlanner::set_device_plan(int finest, int n_stages, int V, const int64_t* counts,
                                       const int64_t* edge_counts, const int64_t* bface_counts,
                                       int stride, int64_t evaluations,
                                       int64_t level_evaluations) {
    memo_ = false;
    finest_ = finest;
    for (int j = 0; j <= n_stages; ++j) {
        count_[j].assign(counts + j * stride, counts + j * stride + V);
        order_[j].clear();
    }
    for (int s = 0; s < n_stages; ++s) {
        edge_count_[s].assign(edge_counts + s * stride, edge_counts + s * stride + V);
        bface_count_[s].assign(bface_counts + s * stride, bface_counts + s * stride + V);
        edge_order_[s].clear();
        bface_order_[s].clear();
        rate_[s].clear();
    }
    level_.clear();
    evaluations_ = evaluations;
    level_evaluations_ = level_evaluations;
    version_ += 1;
}

void MultiratePlanner::assign_one_level() {
    memo_ = false;
    finest_ = 0;
    level_.assign(K_, 0);
    for (int s = 0; s < n_stages_; ++s) rate_[s].assign(K_, 0);
    level_evaluations_ = (int64_t)n_stages_ * K_;
    inverse_dt_sum_ = 0.0;
    n_line_local_ = 0;
    make_lists();
}

double MultiratePlanner::assign(const double* element_dt, const uint8_t* line_local,
                                double dt_cap, double landing) {
    int finest = 0;
    double dt = assign_levels(element_dt, K_, max_levels_, dt_cap, level_, finest);
    stable_step_ = dt;
    // equal steps to the time to land on, each with its own levels (one
    // level has nothing to gain: its steps cost what they span)
    if (finest > 0 && landing > 0.0 && finite(landing) && finite(dt)) {
        const double steps = std::max(std::ceil(landing / (dt * (1.0 + kLandingSlack))), 1.0);
        const double fitted = landing / steps;
        if (fitted < dt) {
            dt = fitted;
            finest = levels_for_step(element_dt, K_, dt, max_levels_, level_);
        }
    }
    finest_ = finest;
    double inv = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : inv)
    for (int64_t k = 0; k < K_; ++k)
        if (finite(element_dt[k])) inv += 1.0 / element_dt[k];
    inverse_dt_sum_ = inv;
    int64_t n_ll = 0;
    if (line_local)
        for (int64_t k = 0; k < K_; ++k) n_ll += line_local[k] ? 1 : 0;
    n_line_local_ = n_ll;

    // the last plan stands while its inputs do
    const bool has_line = line_local != nullptr;
    if (memo_ && memo_finest_ == finest && memo_has_line_ == has_line && memo_level_ == level_ &&
        (!has_line || std::memcmp(memo_line_.data(), line_local, (size_t)K_) == 0)) {
        level_ = memo_limited_;
        return dt;
    }
    memo_level_ = level_;
    limit_level_jumps(level_);
    int64_t lev = 0;
    for (int64_t k = 0; k < K_; ++k) lev += (int64_t)1 << level_[k];
    level_evaluations_ = (int64_t)n_stages_ * lev;
    if (has_line) {
        node_from_.assign((size_t)K_ * nn_, 0);
        for (int64_t k = 0; k < K_; ++k)
            std::fill(&node_from_[(size_t)k * nn_], &node_from_[(size_t)(k + 1) * nn_], level_[k]);
        for (int s = 0; s < n_stages_; ++s) {
            spread_lines(line_local, node_from_, node_to_, rate_[s]);
            std::swap(node_from_, node_to_);
        }
    } else {
        for (int s = 0; s < n_stages_; ++s) spread_faces(s == 0 ? level_ : rate_[s - 1], rate_[s]);
    }
    make_lists();
    memo_ = true;
    memo_finest_ = finest;
    memo_has_line_ = has_line;
    if (has_line) memo_line_.assign(line_local, line_local + K_);
    memo_limited_ = level_;
    return dt;
}

}  // namespace dgswe
