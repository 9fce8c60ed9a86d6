// The level planner of multirate (local) time stepping, on the host: from
// every element's stable step, the coarse step, each element's level (it
// takes 2^level substeps of dt/2^level), each stage's rate (the finest
// level whose substeps that stage's RHS follows), and the order of the
// passes' elements and faces on the device. The reference plans on the host
// too (MultirateStepper, src/time/multirate.rs:880-1320); the device runs
// the passes (kernels.cuh's listed stage, face and finish kernels).
//
// What it computes is the reference's, rule for rule:
//  - assign_levels (multirate.rs:527-568): dt = 2^L·min(element dt) with L
//    the most levels (≤ max_levels) keeping dt ≤ max(element dt) and ≤ the
//    cap; level k = the smallest ℓ with dt/2^ℓ ≤ element_dt[k];
//  - a landing (multirate.rs:1088-1096): the time left over the fewest
//    equal steps, each with the levels of its own length (levels_for_step,
//    multirate.rs:570-583);
//  - the jump limit (multirate.rs:745-752): face neighbours' levels differ
//    by at most one, the coarser side refined;
//  - the stage rates: node by node over the GLL lines for line-local
//    elements (spread_over_lines, multirate.rs:678-743), else one face
//    stencil per stage (spread_over_stencil, multirate.rs:617-676);
//  - the kept plan (multirate.rs:1104-1113): unchanged inputs keep the
//    last levels, rates and lists.
#pragma once

#include <array>
#include <cstdint>
#include <vector>

namespace dgswe {

constexpr int kMaxLevels = 8;   // finest level the device takes (2^8 substeps)
constexpr int kPlanStages = 4;  // SSP-RK(4,3)

class MultiratePlanner {
public:
    // `neighbour[k][f]`: the element across face f of element k (−1 on the
    // boundary) and `nb_face[k][f]` its face there; `face_node[f][fi]`: the
    // volume node of face node fi (the reference's face order); n1 nodes
    // per GLL line
    MultiratePlanner(std::vector<std::array<int64_t, 4>> neighbour,
                     std::vector<std::array<int8_t, 4>> nb_face, const int (*face_node)[5], int n1,
                     int max_levels, int n_stages);

    // Levels and rates from the element steps (∞ where nothing limits an
    // element). `line_local` (one flag per element, or null: none) marks
    // the elements whose stage reads only its GLL lines; `dt_cap` ≤ 0 or
    // ∞: none; `landing` ≤ 0 or ∞: none. Returns the coarse step, fitted to
    // the landing; stable_step() is the step before the fit.
    double assign(const double* element_dt, const uint8_t* line_local, double dt_cap,
                  double landing);
    // Every element on level 0 (global steps)
    void assign_one_level();
    // Given levels and rates (rates[s] for each stage, each between the
    // element's level and the finest): a host that plans itself
    // (LocalTimeStepping::begin_coarse_step)
    void set_plan(const uint8_t* levels, const uint8_t* rates);
    // A plan the device made (multirate_plan.cu): its finest level and the
    // counts of its passes (counts[j·stride + d], edge and boundary-face
    // counts alike, d < V = finest + 1), and the evaluations; the device
    // holds its levels, rates and orders, which this object does not keep
    void set_device_plan(int finest, int n_stages, int V, const int64_t* counts,
                         const int64_t* edge_counts, const int64_t* bface_counts, int stride,
                         int64_t evaluations, int64_t level_evaluations);
    // The step's figures of a device plan, kept plan or not
    void set_step_figures(double stable_step, double inverse_dt_sum, int64_t n_line_local) {
        stable_step_ = stable_step;
        inverse_dt_sum_ = inverse_dt_sum;
        n_line_local_ = n_line_local;
    }

    int finest() const { return finest_; }
    int nn() const { return nn_; }
    double stable_step() const { return stable_step_; }
    const std::vector<uint8_t>& level() const { return level_; }
    const std::vector<uint8_t>& rate(int s) const { return rate_[s]; }
    // Element RHS evaluations per coarse step, and the same with every
    // stage at the element's level
    int64_t evaluations_per_step() const { return evaluations_; }
    int64_t level_evaluations_per_step() const { return level_evaluations_; }
    double inverse_dt_sum() const { return inverse_dt_sum_; }
    int64_t n_line_local() const { return n_line_local_; }
    // Bumped whenever the levels, rates and lists change
    uint64_t version() const { return version_; }

    // The device's pass order: for key j (the stage rates 0..n_stages−1,
    // then the levels) the elements by key, largest first (index order
    // within a key), and count(j, d) = how many have a key ≥ d, so a pass
    // at depth d is a prefix
    const std::vector<int32_t>& order(int j) const { return order_[j]; }
    int64_t count(int j, int d) const { return count_[j][d]; }
    // For stage s: the interior edges by the larger rate of their two
    // elements, the boundary faces by their element's rate (edge and
    // boundary-face indices of the device tables)
    void edge_lists(const std::vector<int64_t>& edge_left, const std::vector<int64_t>& edge_right,
                    const std::vector<int64_t>& bface);
    const std::vector<int32_t>& edge_order(int s) const { return edge_order_[s]; }
    const std::vector<int32_t>& bface_order(int s) const { return bface_order_[s]; }
    int64_t edge_count(int s, int d) const { return edge_count_[s][d]; }
    int64_t bface_count(int s, int d) const { return bface_count_[s][d]; }

    // Level of finest substep p's alignment: the coarsest level whose
    // substeps start at p (multirate.rs:771-778)
    static int depth(int64_t p, int finest);

    // Pieces of the plan, public for the known-answer tests
    static double assign_levels(const double* element_dt, int64_t n, int max_levels,
                                double dt_cap, std::vector<uint8_t>& level, int& finest);
    static int levels_for_step(const double* element_dt, int64_t n, double dt, int max_levels,
                               std::vector<uint8_t>& level);
    void limit_level_jumps(std::vector<uint8_t>& level);
    void spread_faces(const std::vector<uint8_t>& from, std::vector<uint8_t>& to) const;
    void spread_lines(const uint8_t* line_local, const std::vector<uint8_t>& from,
                      std::vector<uint8_t>& to, std::vector<uint8_t>& rate) const;

private:
    void make_lists();

    std::vector<std::array<int64_t, 4>> nb_;
    std::vector<std::array<int8_t, 4>> nb_face_;
    int face_node_[4][5];
    int n1_, nn_, max_levels_, n_stages_;
    int64_t K_;
    int finest_ = 0;
    double stable_step_ = 0.0;
    std::vector<uint8_t> level_, scratch_;
    std::vector<uint8_t> rate_[kPlanStages];
    std::vector<uint8_t> node_from_, node_to_;
    int64_t evaluations_ = 0, level_evaluations_ = 0, n_line_local_ = 0;
    double inverse_dt_sum_ = 0.0;
    std::vector<int32_t> order_[kPlanStages + 1];
    std::vector<int64_t> count_[kPlanStages + 1];
    std::vector<int32_t> edge_order_[kPlanStages], bface_order_[kPlanStages];
    std::vector<int64_t> edge_count_[kPlanStages], bface_count_[kPlanStages];
    uint64_t version_ = 0;
    // the kept plan's inputs
    bool memo_ = false;
    std::vector<uint8_t> memo_level_, memo_line_, memo_limited_;
    int memo_finest_ = -1;
    bool memo_has_line_ = false;
};

}  // namespace dgswe
