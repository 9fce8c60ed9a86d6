// Host-side set-up of a dgswe handle: the DG operators, the mesh
// connectivity, the bilinear geometry and every static table the kernels
// read, built once from a dgswe_form and copied to the device.
//
// The kernels are FP64-bound on GB300 (the path does ≈ 5 flop per byte
// against a machine balance near 0.2), so the set-up trades bytes for
// flops: everything that depends only on the mesh and the bed (pair-averaged
// contravariant metrics, the bed-slope coefficients, lift scales,
// normalised face normals, time-step metrics, neighbour indices) is
// computed here, with the reference's own arithmetic, and read by the
// kernels instead of being recomputed every stage.
#pragma once

#include <array>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/dgswe.h"

namespace dgswe {

constexpr int kMaxN1 = 5;

// GLL operators of order N (src/operators/operators_2d.rs:114-190)
struct Operators {
    int order = 0, n1 = 0, nn = 0;
    std::vector<double> x, w;  // GLL nodes and weights
    std::vector<double> d;     // 1D derivative, row-major n1×n1
    std::vector<double> r, s, w2;
    int face_node[4][kMaxN1];  // volume node of face node fi
    // lift[face][node][fi] = (1/w2[node])·(δ·w[fi])
    double lift(int face, int node, int fi) const;
    explicit Operators(int order);
};

struct Link {
    int64_t element = -1;  // neighbour element, -1 on the boundary
    int face = 0;          // its face
    bool left = false;     // this face is the left side of the edge
    bool shared = false;   // the two faces share their vertices
};

// Mesh2D::from_quads connectivity (src/mesh/core/mesh2d.rs:456-620)
struct Topology {
    int64_t n_elements = 0;
    std::vector<std::array<Link, 4>> link;
    std::vector<std::array<int32_t, 4>> tag;  // boundary faces' tags
    std::vector<std::array<double, 8>> corners;
};

std::string build_topology(const dgswe_form& f, Topology& topo);

// Per-element geometry at the nodes (src/operators/geometric.rs:126-221)
struct ElementGeometry {
    bool affine = false;
    double rx[25], ry[25], sx[25], sy[25], det[25], det_inv[25], mass[25];
    double area = 0.0;
    // per face (constant along a straight face): outward unit normal, sJ
    double nx[4], ny[4], sj[4];
    // contravariant vectors as the split form reads them (a
    // parallelogram's node-0 values at every node)
    double mr0[25], mr1[25], ms0[25], ms1[25];
};

std::string element_geometry(const Operators& ops, const std::array<double, 8>& c,
                             ElementGeometry& g);

// One unknown pair of a GLL line and its owner thread (node)
struct PairSlot {
    int8_t a, c;     // element-local nodes, a before c along the line
    int8_t dir;      // 0: r-line, 1: s-line
    int8_t pa, pc;   // positions along the line
};

// The kernel's static schedule of flux-differencing pairs for order N:
// node i computes pairs owned[i][0..n1-2]; every node then sums the
// 2(n1−1) pairs it belongs to (accum[i][..], with the pair's owner slot).
struct PairSchedule {
    int n1 = 0, nn = 0;
    std::vector<PairSlot> owned;     // [nn][n1-1]
    std::vector<int32_t> accum_slot; // [nn][2(n1-1)] global slot = owner*(n1-1)+j
    std::vector<double> accum_coef;  // [nn][2(n1-1)] 2·D(own position, other)
    explicit PairSchedule(const Operators& ops);
};

// All static device data, host copies
struct Tables {
    int n1 = 0, nn = 0, npair = 0;
    int64_t K = 0;
    // volume
    std::vector<double> bed;        // [K·nn]
    std::vector<double> jinv;       // [K·nn]
    std::vector<double> pair_hm;    // [K·nn·(n1−1)·2] half pair metric ½{{Ja}}
    std::vector<double> gdb;        // [K·nn·2] g·(bed-slope coefficient), both directions
    std::vector<double> contra;     // [K·nn·4] J∇r, J∇s (subcells)
    std::vector<uint8_t> affine;    // [K]
    std::vector<double> lift_scale; // [K·4·n1] sJ·LIFT
    std::vector<int64_t> outer_idx; // [K·4·n1] neighbour's inner node (global) or −1
    std::vector<double> outer_dist; // [K·4·n1]
    std::vector<double> fcor;       // [K·nn] β-plane Coriolis parameter (empty: f-plane)
    std::vector<double> g_n2;       // [K·nn] Manning g·n² per node (empty: uniform)
    // wet/dry and dt
    std::vector<double> mass;       // [K·nn]
    std::vector<double> inv_area;   // [K]
    std::vector<double> weight_ratio; // [K] W/W∂
    std::vector<double> dtm_own;    // [K·nn·6] ¼ of ∇r, ∇s, |∇r|, |∇s| of own nodes
    std::vector<double> dtm_face;   // [K·4·n1·6] the same at face nodes (own node's stored)
    // the same two tables as floats truncated toward zero (f32_trunc), read
    // by the dt pass's single-precision filter
    std::vector<float> dtm32_own, dtm32_face;
    std::vector<int64_t> nb_face_node; // [K·4·n1] neighbour's coincident node (global) or −1
    // faces
    std::vector<int64_t> edge_left, edge_right; // [E] k·4 + face
    std::vector<double> edge_geo;   // [E·5] nx, ny, |n|, n̂x, n̂y of the left side
    std::vector<int64_t> bface;     // [B] k·4 + face
    std::vector<int32_t> bface_cond;// [B] condition index
    std::vector<double> bface_geo;  // [B·5]
};

std::string build_tables(const dgswe_form& f, const Operators& ops, const Topology& topo,
                         const std::vector<int32_t>& cond_of_tag_sorted_tags,
                         const std::vector<int32_t>& cond_index, Tables& t);

}  // namespace dgswe
