"""The Gmsh reader and writer (dgcom_gb300/gmsh.py) against the behaviour
the reference's own tests pin for its reader (src/mesh/io/gmsh.rs:1088-1614,
tests/gmsh_mesh_test.rs): formats, orientation, tags, every error, and the
round trip. The fixtures are small meshes written here: an L of three unit
squares with sparse node tags, one clockwise element, named and unnamed
physical groups, a parametric node block and a point element."""

import numpy as np
import pytest

from dgcom_gb300 import gmsh
from dgcom_gb300.mesh import (TAG_DIRICHLET, TAG_NEUMANN, TAG_OPEN, TAG_RIVER, TAG_TIDAL, TAG_WALL,
                              custom_tag, graded_jittered_box, in_hilbert_order)

# (tag, x, y): sparse tags, not in order
NODES = [(7, 0.0, 0.0), (3, 1.0, 0.0), (50, 2.0, 0.0), (9, 0.0, 1.0), (44, 1.0, 1.0),
         (12, 2.0, 1.0), (100, 0.0, 2.0), (101, 1.0, 2.0)]
# A, then B clockwise, then C
QUADS = [(1, 7, 3, 44, 9), (2, 3, 44, 12, 50), (3, 9, 44, 101, 100)]
# (tag, curve, node a, node b): A's south side, B's east side, C's north side
LINES = [(20, 11, 7, 3), (21, 12, 50, 12), (22, 13, 101, 100)]
CURVES = {11: [5], 12: [6], 13: [21]}
NAMES = [(1, 5, "Coast"), (1, 6, "sea"), (2, 30, "domain")]


def l_v41(nodes=NODES, quads=QUADS, lines=LINES, curves=CURVES, names=NAMES, header="4.1 0 8",
          triangles=()):
    """The L mesh as MSH 4.1 ASCII: the first six nodes in a surface block,
    the last two in a parametric curve block; a point element."""
    out = ["$MeshFormat", header, "$EndMeshFormat", "$PhysicalNames", str(len(names))]
    out += [f'{d} {t} "{n}"' for d, t, n in names]
    out += ["$EndPhysicalNames", "$Entities", f"0 {len(curves)} 1 0"]
    for c, groups in sorted(curves.items()):
        out.append(f"{c} 0 0 0 2 2 0 {len(groups)} {' '.join(map(str, groups))} 0")
    out += ["1 0 0 0 2 2 0 1 30 0", "$EndEntities", "$Nodes"]
    first, second = nodes[:6], nodes[6:]
    tags = [t for t, _, _ in nodes]
    out.append(f"2 {len(nodes)} {min(tags)} {max(tags)}")
    out.append(f"2 1 0 {len(first)}")
    out += [str(t) for t, _, _ in first]
    out += [f"{x} {y} 0" for _, x, y in first]
    out.append(f"1 13 1 {len(second)}")
    out += [str(t) for t, _, _ in second]
    out += [f"{x} {y} 0 0.5" for _, x, y in second]
    out += ["$EndNodes", "$Elements"]
    by_curve = {c: [ln for ln in lines if ln[1] == c] for c in sorted(curves)}
    blocks = [("2 1 3", [" ".join(map(str, q)) for q in quads])] if quads else []
    if triangles:
        blocks.insert(0, ("2 1 2", [" ".join(map(str, t)) for t in triangles]))
    for c, lns in by_curve.items():
        if lns:
            blocks.append((f"1 {c} 1", [f"{t} {a} {b}" for t, _, a, b in lns]))
    blocks.append(("0 1 15", ["40 7"]))
    n = sum(len(rows) for _, rows in blocks)
    out.append(f"{len(blocks)} {n} 1 40")
    for head, rows in blocks:
        out.append(f"{head} {len(rows)}")
        out += rows
    out.append("$EndElements")
    return "\n".join(out) + "\n"


def l_v2():
    """The L mesh as MSH 2.2: the lines' first tag is their physical group."""
    out = ["$MeshFormat", "2.2 0 8", "$EndMeshFormat", "$PhysicalNames", "2",
           '1 5 "Coast"', '1 6 "sea"', "$EndPhysicalNames", "$Nodes", str(len(NODES))]
    out += [f"{t} {x} {y} 0" for t, x, y in NODES]
    out += ["$EndNodes", "$Elements", str(len(QUADS) + len(LINES))]
    for t, c, a, b in LINES:
        g = CURVES[c][0]
        out.append(f"{t} 1 2 {g} {c} {a} {b}")
    out += [f"{q[0]} 3 2 30 1 {' '.join(map(str, q[1:]))}" for q in QUADS]
    out.append("$EndElements")
    return "\n".join(out) + "\n"


def l_binary(big_endian=False, size_bytes=8):
    return gmsh.binary_msh41(NODES, QUADS, LINES, CURVES, NAMES, big_endian, size_bytes)


def centroid_key(mesh):
    c = mesh.corners().mean(axis=1)
    return {(round(x, 9), round(y, 9)): k for k, (x, y) in enumerate(c)}


def signed_areas(mesh):
    p = mesh.corners()
    s = sum(p[:, i, 0] * p[:, (i + 1) % 4, 1] - p[:, (i + 1) % 4, 0] * p[:, i, 1] for i in range(4))
    return 0.5 * s


def boundary_tags(mesh):
    """{((x0, y0), (x1, y1)) sorted: tag} of the boundary faces."""
    out = {}
    for k, f, a, b, t in gmsh.boundary_edges(mesh):
        ends = sorted([tuple(mesh.vertices[a]), tuple(mesh.vertices[b])])
        out[tuple(ends)] = int(t)
    return out


def test_msh41_ascii():
    mesh = gmsh.parse_gmsh_mesh(l_v41().encode())
    assert mesh.n_elements == 3 and mesh.vertices.shape == (8, 2)
    assert np.allclose(signed_areas(mesh), 1.0, atol=1e-14)  # B turned counter-clockwise
    tags = boundary_tags(mesh)
    assert len(tags) == 8
    assert tags[((2.0, 0.0), (2.0, 1.0))] == TAG_OPEN  # "sea"
    assert tags[((0.0, 2.0), (1.0, 2.0))] == custom_tag(21)  # unnamed group 21
    assert tags[((0.0, 0.0), (1.0, 0.0))] == TAG_WALL  # "Coast"
    assert sum(t == TAG_WALL for t in tags.values()) == 6
    # neighbours traverse each shared edge in opposite directions
    a = mesh.elements.reshape(-1)
    b = mesh.elements[:, [1, 2, 3, 0]].reshape(-1)
    directed = set(zip(a.tolist(), b.tolist()))
    shared = [(u, v) for u, v in directed if (v, u) in directed]
    assert len(shared) == 4  # two interior edges, each both ways
    # vertices are numbered by first use in the element order
    first_use = list(dict.fromkeys(mesh.elements.reshape(-1).tolist()))
    assert first_use == list(range(8))


@pytest.mark.parametrize("big_endian", [False, True])
@pytest.mark.parametrize("size_bytes", [4, 8])
def test_msh41_binary_is_the_ascii_mesh(big_endian, size_bytes):
    a = gmsh.parse_gmsh_mesh(l_v41().encode())
    b = gmsh.parse_gmsh_mesh(l_binary(big_endian, size_bytes))
    assert np.array_equal(a.vertices, b.vertices)
    assert np.array_equal(a.elements, b.elements)
    assert np.array_equal(a.face_tags, b.face_tags)


def test_msh22_is_the_same_mesh():
    a = gmsh.parse_gmsh_mesh(l_v41().encode())
    b = gmsh.parse_gmsh_mesh(l_v2().encode())
    assert np.array_equal(a.vertices, b.vertices)
    assert np.array_equal(a.elements, b.elements)
    assert boundary_tags(a) == boundary_tags(b)


def test_cut_files_are_errors_never_crashes():
    binary = l_binary()
    for n in range(len(binary) - 1):
        with pytest.raises(gmsh.GmshError):
            gmsh.parse_gmsh_mesh(binary[:n])
    text = l_v41().encode()
    for n in range(len(text)):
        try:
            gmsh.parse_gmsh_mesh(text[:n])
        except gmsh.GmshError:
            pass


def test_triangles_are_counted_with_advice():
    tris = [(1, 7, 3, 44), (4, 7, 44, 9)]  # A split in two
    text = l_v41(quads=QUADS[1:], triangles=tris)
    with pytest.raises(gmsh.UnsupportedElements) as err:
        gmsh.parse_gmsh_mesh(text.encode())
    assert err.value.counts == [(2, 2)]
    assert "2 × 3-node triangle (type 2)" in str(err.value)
    assert "Mesh.SubdivisionAlgorithm = 1" in str(err.value)


def test_unsupported_versions():
    for header, expected in [("4 0 8", "MSH 4.1"), ("4.0 0 8", "MSH 4.1"), ("3.0 0 8", "3.0")]:
        with pytest.raises(gmsh.UnsupportedVersion, match=expected.replace(".", r"\.")):
            gmsh.parse_gmsh_mesh(l_v41(header=header).encode())
    with pytest.raises(gmsh.UnsupportedVersion):
        gmsh.parse_gmsh_mesh(b"$MeshFormat\n2.2 1 8\n")
    with pytest.raises(gmsh.MissingSection):
        gmsh.parse_gmsh_mesh(b"$Nodes\n0\n$EndNodes\n")


def test_a_bad_number_names_its_line():
    text = l_v41().replace("\n1.0 1.0 0\n", "\n1.0 q 0\n")
    line = text.split("\n").index("1.0 q 0") + 1
    with pytest.raises(gmsh.GmshParseError) as err:
        gmsh.parse_gmsh_mesh(text.encode())
    assert 'invalid node y: "q"' in str(err.value)
    assert f"line {line}," in str(err.value)


def test_undefined_and_duplicate_nodes():
    text = l_v41().replace("\n1 7 3 44 9\n", "\n1 7 3 44 8\n")
    with pytest.raises(gmsh.InvalidMesh, match="element 1 uses undefined node 8"):
        gmsh.parse_gmsh_mesh(text.encode())
    nodes = NODES[:6] + [(12, 0.0, 2.0), NODES[7]]  # tag 12 twice
    with pytest.raises(gmsh.InvalidMesh, match="node 12 is defined twice"):
        gmsh.parse_gmsh_mesh(l_v41(nodes=nodes).encode())


def test_non_convex_and_degenerate_elements():
    nodes = [(t, 0.3, 0.3) if t == 44 else (t, x, y) for t, x, y in NODES]  # a dart in A
    with pytest.raises(gmsh.InvalidMesh, match="element 1 is degenerate or non-convex at node 44"):
        gmsh.parse_gmsh_mesh(l_v41(nodes=nodes).encode())
    quads = [(1, 7, 3, 3, 9)] + QUADS[1:]  # a repeated node
    with pytest.raises(gmsh.InvalidMesh):
        gmsh.parse_gmsh_mesh(l_v41(quads=quads).encode())


def test_non_manifold_and_overlapping_elements():
    # a fourth element on A–B's edge 3–44, folded back over B
    nodes = NODES + [(60, 1.5, 0.0), (61, 1.5, 1.0)]
    quads = QUADS + [(4, 44, 3, 60, 61)]
    with pytest.raises(gmsh.InvalidMesh, match="shared by more than two elements"):
        gmsh.parse_gmsh_mesh(l_v41(nodes=nodes, quads=quads).encode())
    # B moved onto A: both traverse 3–44 the same way
    moved = [(t, 0.5, y) if t in (50, 12) else (t, x, y) for t, x, y in NODES]
    with pytest.raises(gmsh.InvalidMesh, match="overlap"):
        gmsh.parse_gmsh_mesh(l_v41(nodes=moved).encode())


def test_conflicting_tags():
    curves = {**CURVES, 12: [6, 5]}  # one curve in "sea" and "Coast"
    with pytest.raises(gmsh.InvalidMesh, match="different boundary tags"):
        gmsh.parse_gmsh_mesh(l_v41(curves=curves).encode())
    lines = LINES + [(23, 11, 50, 12)]  # B's east edge also on the shore curve
    with pytest.raises(gmsh.InvalidMesh, match="has two boundary tags"):
        gmsh.parse_gmsh_mesh(l_v41(lines=lines).encode())


def test_lines_off_and_inside_the_mesh():
    lines = [(20, 11, 7, 44)] + LINES[1:]  # a diagonal of A
    with pytest.raises(gmsh.InvalidMesh, match="line element 20"):
        gmsh.parse_gmsh_mesh(l_v41(lines=lines).encode())
    lines = LINES + [(24, 12, 3, 44)]  # on the interior edge A–B: ignored
    mesh = gmsh.parse_gmsh_mesh(l_v41(lines=lines).encode())
    assert sum(t == TAG_OPEN for t in boundary_tags(mesh).values()) == 1


def test_no_quadrilaterals_advises_a_physical_surface():
    with pytest.raises(gmsh.InvalidMesh, match="physical surface"):
        gmsh.parse_gmsh_mesh(l_v41(quads=[]).encode())


def test_sections_skipped_and_refused():
    extra = "$Comments\nnot $Nodes here\n$EndComments\n$NodeData\n1\n\"eta\"\n$EndNodeData\n"
    assert gmsh.parse_gmsh_mesh((l_v41() + extra).encode()).n_elements == 3
    with pytest.raises(gmsh.GmshUnsupported):
        gmsh.parse_gmsh_mesh((l_v41() + "$Periodic\n0\n$EndPeriodic\n").encode())
    with pytest.raises(gmsh.GmshUnsupported):
        gmsh.parse_gmsh_mesh((l_v41() + "$PartitionedEntities\n$EndPartitionedEntities\n").encode())
    with pytest.raises(gmsh.GmshParseError):
        gmsh.parse_gmsh_mesh(l_v41().replace("$EndNodes", "$EndNode").encode())


def test_crlf_line_ends():
    mesh = gmsh.parse_gmsh_mesh(l_v41().replace("\n", "\r\n").encode())
    assert mesh.n_elements == 3
    assert sum(t == TAG_OPEN for t in boundary_tags(mesh).values()) == 1


def test_physical_group_tags():
    for name in ("wall", "Walls", "LAND", "coast", "CoastLine", "shore", "Shoreline", "closed"):
        assert gmsh.group_boundary_tag(99, name) == TAG_WALL
    assert gmsh.group_boundary_tag(99, "shore-line") == custom_tag(99)  # read as shore_line
    for name in ("open", "Ocean", "sea", "open boundary"):
        assert gmsh.group_boundary_tag(99, name) == TAG_OPEN
    for name in ("tidal", "tide", "Tides", "tidal-forcing"):
        assert gmsh.group_boundary_tag(99, name) == TAG_TIDAL
    assert gmsh.group_boundary_tag(99, "rivers") == TAG_RIVER
    assert gmsh.group_boundary_tag(13, "outflow") == custom_tag(13)
    numbered = [TAG_WALL, TAG_OPEN, TAG_TIDAL, TAG_RIVER, TAG_DIRICHLET, TAG_NEUMANN]
    for number, tag in enumerate(numbered, start=1):
        assert gmsh.group_boundary_tag(number, None) == tag
        assert gmsh.tag_to_physical(tag) == number
    assert gmsh.group_boundary_tag(42, None) == custom_tag(42)
    assert gmsh.tag_to_physical(custom_tag(42)) == 42
    with pytest.raises(gmsh.InvalidMesh):
        gmsh.group_boundary_tag(-1, None)


def test_write_then_read_is_the_mesh(tmp_path):
    m = graded_jittered_box(3000.0, 2000.0, 9, 7, size_range=(200.0, 500.0), seed=4,
                            sides=(TAG_WALL, TAG_OPEN, TAG_TIDAL, custom_tag(13)))
    m, _ = in_hilbert_order(m)
    path = tmp_path / "box.msh"
    gmsh.write_gmsh_mesh(m, path)
    back = gmsh.read_gmsh_mesh(path)
    assert np.array_equal(back.vertices, m.vertices)  # shortest round-trip decimals
    assert np.array_equal(back.elements, m.elements)
    assert boundary_tags(back) == boundary_tags(m)
