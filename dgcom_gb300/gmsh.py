"""Gmsh mesh files: how real coastline-fitted domains reach the device path.

Reads MSH 4.1 (ASCII and binary, either byte order) and MSH 2.2 (ASCII);
writes MSH 2.2 (ASCII). The behaviour is the reference reader's
(src/mesh/io/gmsh.rs):

- the mesh is first-order quadrilaterals (Gmsh type 3). Any other element
  type is an error that counts them by type, with the Gmsh options that
  give an all-quad first-order 2D mesh; points (type 15) are ignored and
  2-node lines (type 1) carry boundary tags;
- node tags may be sparse and in any order; the vertices are the nodes the
  quadrilaterals use, in file order; clockwise quadrilaterals are turned
  counter-clockwise; a degenerate or non-convex one (a non-positive
  bilinear Jacobian at a corner), an edge of more than two elements and
  two elements traversing their shared edge the same way are errors;
- a boundary edge takes the tag of the physical groups of the line on it
  (MSH 4.1: the groups of the line's curve entity; MSH 2.2: the line's
  first tag): a named group by its name (``group_boundary_tag``), an
  unnamed one by its number (1 wall, 2 open, 3 tidal, 4 river,
  5 Dirichlet, 6 Neumann, other n custom). Untagged boundary edges are
  walls; groups of one line that map to different tags, an edge with two
  different tags, and a line that is not an edge of the mesh are errors;
  lines on interior edges are ignored;
- MSH 4.0, binary MSH 2, ``$Periodic`` and ``$PartitionedEntities`` are
  errors; other sections are skipped; CRLF line ends are read;
- the mesh comes back in Hilbert order (``mesh.in_hilbert_order``).

Errors are ``GmshError`` subclasses named after the reference's variants.
Tags are the ABI's face tags (``mesh.TAG_*``, ``mesh.custom_tag``)."""

from __future__ import annotations

import itertools
import re
import struct
from pathlib import Path

import numpy as np

from .mesh import (CUSTOM_TAG_BASE, TAG_DIRICHLET, TAG_NEUMANN, TAG_OPEN, TAG_RIVER, TAG_TIDAL,
                   TAG_WALL, QuadMesh, custom_tag, in_hilbert_order)


class GmshError(ValueError):
    """A Gmsh file the device path cannot take (GmshError, gmsh.rs:82-111)."""


class GmshParseError(GmshError):
    """Malformed file: a bad number, a truncated section, a missing end marker."""


class UnsupportedVersion(GmshError):
    pass


class UnsupportedElements(GmshError):
    """Element types the solver cannot use; ``counts`` = [(type, count)]."""

    def __init__(self, counts):
        self.counts = [(int(t), int(n)) for t, n in counts]
        parts = []
        for t, n in self.counts:
            name = ELEMENT_TYPES.get(t, (0, "unknown element"))[1]
            parts.append(f"{n} × {name} (type {t})")
        super().__init__(
            f"unsupported Gmsh elements: {', '.join(parts)}. The device path takes 2D meshes of "
            "first-order quadrilaterals; in Gmsh, mesh in 2D with Mesh.ElementOrder = 1 and "
            "recombine and subdivide to all quads (Mesh.RecombineAll = 1; "
            "Mesh.SubdivisionAlgorithm = 1)")


class GmshUnsupported(GmshError):
    """A file feature the reader does not take (periodic, partitioned)."""


class MissingSection(GmshError):
    pass


class InvalidMesh(GmshError):
    """The file parses but is not a valid quadrilateral mesh."""


# Gmsh's fixed-order element types: node count and name
ELEMENT_TYPES = {
    1: (2, "2-node line"), 2: (3, "3-node triangle"), 3: (4, "4-node quadrangle"),
    4: (4, "4-node tetrahedron"), 5: (8, "8-node hexahedron"), 6: (6, "6-node prism"),
    7: (5, "5-node pyramid"), 8: (3, "3-node line"), 9: (6, "6-node triangle"),
    10: (9, "9-node quadrangle"), 11: (10, "10-node tetrahedron"),
    12: (27, "27-node hexahedron"), 13: (18, "18-node prism"), 14: (14, "14-node pyramid"),
    15: (1, "1-node point"), 16: (8, "8-node quadrangle"), 17: (20, "20-node hexahedron"),
    18: (15, "15-node prism"), 19: (13, "13-node pyramid"), 20: (9, "9-node triangle"),
    21: (10, "10-node triangle"), 22: (12, "12-node triangle"), 23: (15, "15-node triangle"),
    24: (15, "15-node incomplete triangle"), 25: (21, "21-node triangle"),
    26: (4, "4-node line"), 27: (5, "5-node line"), 28: (6, "6-node line"),
    29: (20, "20-node tetrahedron"), 30: (35, "35-node tetrahedron"),
    31: (56, "56-node tetrahedron"), 36: (16, "16-node quadrangle"),
    37: (25, "25-node quadrangle"), 38: (36, "36-node quadrangle"),
}
LINE, QUAD, POINT = 1, 3, 15

_NAMED = {}
for _tag, _names in ((TAG_WALL, "wall walls land coast coastline shore shoreline closed"),
                     (TAG_OPEN, "open ocean sea open_boundary"),
                     (TAG_TIDAL, "tidal tide tides tidal_forcing"),
                     (TAG_RIVER, "river rivers")):
    for _n in _names.split():
        _NAMED[_n] = _tag
_NUMBERED = {1: TAG_WALL, 2: TAG_OPEN, 3: TAG_TIDAL, 4: TAG_RIVER, 5: TAG_DIRICHLET,
             6: TAG_NEUMANN}


def group_boundary_tag(number: int, name: str | None) -> int:
    """The face tag of a physical group: by its name (case-insensitive,
    spaces and dashes read as ``_``) if it has one, else by its number."""
    if number < 0:
        raise InvalidMesh(f"negative physical group tag {number}")
    if name is None:
        return _NUMBERED.get(number, custom_tag(number))
    key = name.lower().replace(" ", "_").replace("-", "_")
    return _NAMED.get(key, custom_tag(number))


def tag_to_physical(tag: int) -> int:
    """The physical group number a face tag is written with."""
    for number, t in _NUMBERED.items():
        if t == tag:
            return number
    if tag >= CUSTOM_TAG_BASE:
        return tag - CUSTOM_TAG_BASE
    raise ValueError(f"face tag {tag} has no Gmsh physical group")


def tag_name(tag: int) -> str:
    names = {TAG_WALL: "Wall", TAG_OPEN: "Open", TAG_TIDAL: "TidalForcing", TAG_RIVER: "River",
             TAG_DIRICHLET: "Dirichlet", TAG_NEUMANN: "Neumann"}
    return names.get(tag, f"Custom({tag - CUSTOM_TAG_BASE})")


# ---------------------------------------------------------------------------
# Reading tokens and binary values
# ---------------------------------------------------------------------------

_TOKEN = re.compile(rb"\S+")
_INT_OK = re.compile(rb"[+-]?[0-9]+\Z")
_FLOAT_OK = re.compile(rb"[+-]?(?:[0-9]+\.?[0-9]*(?:[eE][+-]?[0-9]+)?|\.[0-9]+(?:[eE][+-]?[0-9]+)?"
                       rb"|inf|infinity|nan)\Z", re.IGNORECASE)


class _Reader:
    def __init__(self, buf: bytes):
        self.buf = buf
        self.pos = 0
        self.binary = False
        self.big_endian = False
        self.size_bytes = 8

    def error(self, msg: str) -> GmshParseError:
        line = 1 + self.buf.count(b"\n", 0, self.pos)
        return GmshParseError(f"{msg} (line {line}, byte {self.pos})")

    def at_end(self) -> bool:
        m = _TOKEN.search(self.buf, self.pos)
        if m is None:
            self.pos = len(self.buf)
            return True
        self.pos = m.start()
        return False

    def token(self, what: str) -> bytes:
        m = _TOKEN.search(self.buf, self.pos)
        if m is None:
            self.pos = len(self.buf)
            raise self.error(f"unexpected end of file, expected {what}")
        self.pos = m.end()
        return m.group()

    def _bad(self, what: str, tok: bytes) -> GmshParseError:
        return self.error(f'invalid {what}: "{tok.decode("ascii", "replace")}"')

    def ascii_int(self, what: str, unsigned: bool = False) -> int:
        tok = self.token(what)
        if not _INT_OK.match(tok) or (unsigned and tok.startswith(b"-")):
            raise self._bad(what, tok)
        return int(tok)

    def ascii_float(self, what: str) -> float:
        tok = self.token(what)
        if not _FLOAT_OK.match(tok):
            raise self._bad(what, tok)
        return float(tok)

    def line(self) -> str:
        end = self.buf.find(b"\n", self.pos)
        if end < 0:
            end = len(self.buf)
        text = self.buf[self.pos:end]
        self.pos = min(end + 1, len(self.buf))
        try:
            return text.decode("utf-8").rstrip("\r")
        except UnicodeDecodeError:
            raise self.error("invalid text: not UTF-8") from None

    def expect(self, expected: str):
        tok = self.token(expected)
        if tok != expected.encode():
            raise self.error(f'expected {expected}, found "{tok.decode("ascii", "replace")}"')

    def skip_section(self, name: str):
        end = f"$End{name}".encode()
        at = self.buf.find(end, self.pos)
        if at < 0:
            raise self.error(f"missing $End{name}")
        self.pos = at + len(end)

    def raw(self, n: int, what: str) -> bytes:
        if self.pos + n > len(self.buf):
            raise self.error(f"unexpected end of file, expected {what}")
        out = self.buf[self.pos:self.pos + n]
        self.pos += n
        return out

    def _array(self, n: int, code: str, what: str) -> np.ndarray:
        dtype = np.dtype(code).newbyteorder(">" if self.big_endian else "<")
        data = self.raw(n * dtype.itemsize, what)
        return np.frombuffer(data, dtype=dtype).astype(np.dtype(code).newbyteorder("="))

    # int: 4-byte binary or a token; size: size_t (4 or 8 bytes) or a token
    def int(self, what: str) -> int:
        if self.binary:
            return int(self._array(1, "i4", what)[0])
        return self.ascii_int(what)

    def size(self, what: str) -> int:
        if self.binary:
            return int(self._array(1, "u4" if self.size_bytes == 4 else "u8", what)[0])
        return self.ascii_int(what, unsigned=True)

    def count(self, what: str, min_bytes: int) -> int:
        """A count bounded by what the rest of the file can hold, so that a
        corrupt count cannot ask for a huge allocation."""
        n = self.size(what)
        room = (len(self.buf) - self.pos) // max(min_bytes, 1) + 1
        if n > room:
            raise self.error(f"{what} {n} exceeds the file size")
        return n

    def double(self, what: str) -> float:
        if self.binary:
            return float(self._array(1, "f8", what)[0])
        return self.ascii_float(what)

    def sizes(self, n: int, what: str) -> np.ndarray:
        if self.binary:
            return self._array(n, "u4" if self.size_bytes == 4 else "u8", what).astype(np.int64)
        return self._ascii_many(n, (what,), True)

    def doubles(self, n: int, whats: tuple[str, ...]) -> np.ndarray:
        if self.binary:
            return self._array(n, "f8", whats[0])
        return self._ascii_many(n, whats, False)

    def _ascii_many(self, n: int, whats: tuple[str, ...], integer: bool) -> np.ndarray:
        """n tokens, the k-th named whats[k % len(whats)] in messages."""
        matches = list(itertools.islice(_TOKEN.finditer(self.buf, self.pos), n))
        if len(matches) < n:
            self.pos = len(self.buf)
            raise self.error(f"unexpected end of file, expected {whats[len(matches) % len(whats)]}")
        toks = [m.group() for m in matches]
        ok = _INT_OK if integer else _FLOAT_OK
        try:
            arr = np.array(toks).astype(np.int64 if integer else np.float64)
            bad = (not all(ok.match(t) for t in toks)) or (integer and bool((arr < 0).any()))
        except (ValueError, OverflowError):
            bad = True
        if bad:
            for k, (m, t) in enumerate(zip(matches, toks)):
                if not ok.match(t) or (integer and t.startswith(b"-")):
                    self.pos = m.end()
                    raise self._bad(whats[k % len(whats)], t)
        self.pos = matches[-1].end() if matches else self.pos
        return arr if n else np.zeros(0, np.int64 if integer else np.float64)


# ---------------------------------------------------------------------------
# Sections
# ---------------------------------------------------------------------------

class _Raw:
    def __init__(self):
        self.node_tags: list[np.ndarray] = []
        self.node_xy: list[np.ndarray] = []
        self.quads: list[tuple[int, list[int]]] = []        # (element tag, node tags)
        self.lines: list[tuple[int, list[int], tuple]] = []  # (tag, nodes, groups)
        self.names: dict[tuple[int, int], str] = {}
        self.curve_groups: dict[int, list[int]] = {}
        self.unsupported: dict[int, int] = {}

    def add_block(self, etype: int, tags: np.ndarray, nodes: np.ndarray, groups):
        if etype == QUAD:
            self.quads.extend(zip(tags.tolist(), nodes.tolist()))
        elif etype == LINE:
            self.lines.extend((t, n, groups) for t, n in zip(tags.tolist(), nodes.tolist()))
        elif etype != POINT:
            self.unsupported[etype] = self.unsupported.get(etype, 0) + len(tags)

    def push_nodes(self, r: _Reader, tags: np.ndarray, xy: np.ndarray):
        finite = np.isfinite(xy).all(axis=1)
        if not finite.all():
            k = int(np.argmin(finite))
            raise r.error(f"node {int(tags[k])} has non-finite coordinates "
                          f"({xy[k, 0]}, {xy[k, 1]})")
        self.node_tags.append(tags)
        self.node_xy.append(xy)


def _parse_msh(buf: bytes) -> _Raw:
    r = _Reader(buf)
    raw = _Raw()
    version = None
    while not r.at_end():
        header = r.line().strip()
        if not header.startswith("$"):
            raise r.error(f'expected a section header, found "{header}"')
        name = header[1:]

        def need_format():
            if version is None:
                raise MissingSection(f"MeshFormat (before ${name})")
            return version

        if name == "MeshFormat":
            version = _mesh_format(r)
        elif name == "PhysicalNames":
            _physical_names(r, raw)
        elif name == "Entities":
            if need_format() != "4.1":
                raise r.error("$Entities in an MSH 2 file")
            _entities(r, raw)
        elif name == "Nodes":
            (_nodes_v41 if need_format() == "4.1" else _nodes_v2)(r, raw)
        elif name == "Elements":
            (_elements_v41 if need_format() == "4.1" else _elements_v2)(r, raw)
        elif name == "Periodic":
            raise GmshUnsupported("periodic meshes ($Periodic)")
        elif name == "PartitionedEntities":
            raise GmshUnsupported("partitioned meshes ($PartitionedEntities): save the mesh "
                                  "unpartitioned")
        else:
            r.skip_section(name)
            continue
        r.expect(f"$End{name}")
    if version is None:
        raise MissingSection("MeshFormat")
    return raw


def _mesh_format(r: _Reader) -> str:
    v = r.token("format version").decode("ascii", "replace")
    file_type = r.ascii_int("file type")
    data_size = r.ascii_int("data size", unsigned=True)
    if v == "4.1":
        version = "4.1"
    elif v.startswith("2."):
        version = "2"
    elif v.startswith("4"):
        raise UnsupportedVersion(f"{v}: save as MSH 4.1 (Mesh.MshFileVersion = 4.1) or 2.2")
    else:
        raise UnsupportedVersion(v)
    if file_type == 0:
        return version
    if file_type == 1 and version == "4.1":
        if data_size not in (4, 8):
            raise r.error(f"unsupported data size {data_size}")
        r.line()  # the rest of the header line
        r.binary = True
        r.size_bytes = data_size
        mark = r.raw(4, "byte-order mark")
        if mark == b"\x01\x00\x00\x00":
            r.big_endian = False
        elif mark == b"\x00\x00\x00\x01":
            r.big_endian = True
        else:
            raise r.error(f"invalid byte-order mark {list(mark)}")
        return version
    if file_type == 1:
        raise UnsupportedVersion("binary MSH 2: save as ASCII or as MSH 4.1")
    raise r.error(f"invalid file type {file_type}")


def _physical_names(r: _Reader, raw: _Raw):
    binary, r.binary = r.binary, False  # always ASCII
    n = r.ascii_int("physical name count", unsigned=True)
    for _ in range(n):
        dim = r.ascii_int("physical group dimension")
        tag = r.ascii_int("physical group tag")
        name = r.line().strip()
        if len(name) >= 2 and name.startswith('"') and name.endswith('"'):
            name = name[1:-1]
        raw.names[(dim, tag)] = name
    r.binary = binary


def _entities(r: _Reader, raw: _Raw):
    counts = [r.count("entity count", 1) for _ in range(4)]
    for dim, n in enumerate(counts):
        for _ in range(n):
            tag = r.int("entity tag")
            for _ in range(3 if dim == 0 else 6):  # a point's coordinates, else a box
                r.double("entity coordinate")
            groups = [r.int("physical tag") for _ in range(r.count("physical tag count", 1))]
            if dim > 0:
                for _ in range(r.count("bounding entity count", 1)):
                    r.int("bounding entity tag")
            if dim == 1:
                raw.curve_groups[tag] = groups


def _nodes_v41(r: _Reader, raw: _Raw):
    n_blocks = r.count("node block count", 4)
    n_nodes = r.count("node count", 4)
    r.size("minimum node tag")
    r.size("maximum node tag")
    read = 0
    for _ in range(n_blocks):
        dim = r.int("entity dimension")
        r.int("entity tag")
        parametric = r.int("parametric flag")
        n = r.count("nodes in block", 4)
        if parametric == 0:
            n_param = 0
        elif parametric == 1 and 0 <= dim <= 3:
            n_param = dim
        else:
            raise r.error(f"invalid node block ({dim}, {parametric})")
        tags = r.sizes(n, "node tag")
        per = 3 + n_param
        names = ("node x", "node y") + ("node coordinate",) * (1 + n_param)
        coords = r.doubles(n * per, names).reshape(n, per)
        raw.push_nodes(r, tags, coords[:, :2].copy())
        read += n
    if read != n_nodes:
        raise r.error(f"$Nodes declares {n_nodes} nodes, found {read}")


def _nodes_v2(r: _Reader, raw: _Raw):
    n = r.count("node count", 4)
    vals = r.doubles(4 * n, ("node tag", "node x", "node y", "node z")).reshape(n, 4)
    tags = vals[:, 0]
    if not (np.all(tags == np.floor(tags)) and np.all(tags >= 0)):
        k = int(np.argmax((tags != np.floor(tags)) | (tags < 0)))
        raise r.error(f'invalid node tag: "{tags[k]}"')
    raw.push_nodes(r, tags.astype(np.int64), vals[:, 1:3].copy())


def _elements_v41(r: _Reader, raw: _Raw):
    n_blocks = r.count("element block count", 4)
    n_elements = r.count("element count", 4)
    r.size("minimum element tag")
    r.size("maximum element tag")
    read = 0
    for _ in range(n_blocks):
        r.int("entity dimension")
        entity = r.int("entity tag")
        etype = r.int("element type")
        n = r.count("elements in block", 4)
        if etype not in ELEMENT_TYPES:
            raise UnsupportedElements([(etype, n)])
        nn = ELEMENT_TYPES[etype][0]
        vals = r.sizes(n * (1 + nn), "element node tag").reshape(n, 1 + nn)
        raw.add_block(etype, vals[:, 0], vals[:, 1:], ("curve", entity))
        read += n
    if read != n_elements:
        raise r.error(f"$Elements declares {n_elements} elements, found {read}")


def _elements_v2(r: _Reader, raw: _Raw):
    n = r.count("element count", 4)
    for _ in range(n):
        tag = r.ascii_int("element tag", unsigned=True)
        etype = r.ascii_int("element type")
        n_tags = r.ascii_int("element tag count", unsigned=True)
        physical = 0
        for i in range(n_tags):
            t = r.ascii_int("element tag")
            if i == 0:
                physical = t
        if etype not in ELEMENT_TYPES:
            raise UnsupportedElements([(etype, 1)])
        nodes = [r.ascii_int("element node tag", unsigned=True)
                 for _ in range(ELEMENT_TYPES[etype][0])]
        raw.add_block(etype, np.array([tag]), np.array([nodes]), ("physical", physical))


# ---------------------------------------------------------------------------
# The mesh
# ---------------------------------------------------------------------------

def _line_tag(raw: _Raw, groups) -> int | None:
    kind, value = groups
    if kind == "curve":
        physical = raw.curve_groups.get(value, [])
    else:
        physical = [] if value == 0 else [value]
    tag = None
    for p in physical:
        t = group_boundary_tag(p, raw.names.get((1, p)))
        if tag is not None and tag != t:
            raise InvalidMesh("a curve is in physical groups that map to different boundary "
                              f"tags ({tag_name(tag)} and {tag_name(t)})")
        tag = t
    return tag


def _fmt(x: float) -> str:
    return repr(float(x))


def _build(raw: _Raw) -> QuadMesh:
    if raw.unsupported:
        raise UnsupportedElements(sorted(raw.unsupported.items()))
    if not raw.node_tags:
        raise MissingSection("Nodes")
    if not raw.quads:
        raise InvalidMesh("no quadrilateral elements: once a model has physical groups, Gmsh "
                          "saves only the elements in them, so give the domain a physical "
                          "surface (or set Mesh.SaveAll = 1)")
    node_tags = np.concatenate(raw.node_tags)
    node_xy = np.concatenate(raw.node_xy)
    order = np.argsort(node_tags, kind="stable")
    sorted_tags = node_tags[order]
    dup = np.nonzero(sorted_tags[1:] == sorted_tags[:-1])[0]
    if dup.size:
        raise InvalidMesh(f"node {int(sorted_tags[dup[0] + 1])} is defined twice")

    def lookup(tags: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
        at = np.clip(np.searchsorted(sorted_tags, tags), 0, sorted_tags.size - 1)
        found = sorted_tags[at] == tags
        return np.where(found, order[at], -1), found

    qtags = np.array([t for t, _ in raw.quads], dtype=np.int64)
    qnodes = np.array([n for _, n in raw.quads], dtype=np.int64).reshape(-1, 4)
    qidx, found = lookup(qnodes)
    if not found.all():
        k, c = divmod(int(np.argmin(found.reshape(-1))), 4)
        raise InvalidMesh(f"element {int(qtags[k])} uses undefined node {int(qnodes[k, c])}")
    # vertices: the nodes the quadrilaterals use, in file order
    used = np.zeros(node_tags.size, bool)
    used[qidx.reshape(-1)] = True
    vertex_of_node = np.full(node_tags.size, -1, np.int64)
    vertex_of_node[used] = np.arange(int(used.sum()))
    vertices = node_xy[used]
    quads = vertex_of_node[qidx]

    # counter-clockwise, then a positive Jacobian at every corner
    p = vertices[quads]
    twice_area = np.zeros(len(quads))
    for i in range(4):
        j = (i + 1) % 4
        twice_area = twice_area + (p[:, i, 0] * p[:, j, 1] - p[:, j, 0] * p[:, i, 1])
    flip = twice_area < 0.0
    quads[flip] = quads[flip][:, [0, 3, 2, 1]]
    p = vertices[quads]
    bad = np.zeros((len(quads), 4), bool)
    for i in range(4):
        a, b, c = p[:, (i + 3) % 4], p[:, i], p[:, (i + 1) % 4]
        e0, e1 = b - a, c - b
        cross = e0[:, 0] * e1[:, 1] - e0[:, 1] * e1[:, 0]
        scale = np.hypot(e0[:, 0], e0[:, 1]) * np.hypot(e1[:, 0], e1[:, 1])
        bad[:, i] = np.isnan(cross) | (cross <= 1e-12 * scale)
    if bad.any():
        k, i = divmod(int(np.argmax(bad.reshape(-1))), 4)
        corner = (4 - i) % 4 if flip[k] else i
        x, y = p[k, i]
        raise InvalidMesh(f"element {int(qtags[k])} is degenerate or non-convex at node "
                          f"{int(qnodes[k, corner])} ({_fmt(x)}, {_fmt(y)}): its bilinear map "
                          "has a non-positive Jacobian")

    # edges: at most two faces each, traversed in opposite directions
    K = len(quads)
    a = quads.reshape(-1)
    b = quads[:, [1, 2, 3, 0]].reshape(-1)
    lo, hi = np.minimum(a, b), np.maximum(a, b)
    key = lo * vertices.shape[0] + hi
    ek, inverse, counts = np.unique(key, return_inverse=True, return_counts=True)

    def segment(e: int) -> str:
        (x0, y0), (x1, y1) = vertices[lo[e]], vertices[hi[e]]
        return f"({_fmt(x0)}, {_fmt(y0)})–({_fmt(x1)}, {_fmt(y1)})"

    faces_of = np.argsort(inverse, kind="stable")
    starts = np.concatenate([[0], np.cumsum(counts)])
    many = np.nonzero(counts > 2)[0]
    if many.size:
        e = int(many[0])
        f = faces_of[starts[e]:starts[e] + 3]
        raise InvalidMesh(f"the edge {segment(int(f[0]))} is shared by more than two elements "
                          f"(elements {int(qtags[f[0] // 4])}, {int(qtags[f[1] // 4])} and "
                          f"{int(qtags[f[2] // 4])})")
    pairs = np.nonzero(counts == 2)[0]
    f0 = faces_of[starts[pairs]]
    f1 = faces_of[starts[pairs] + 1]
    same = a[f0] == a[f1]
    if same.any():
        i = int(np.argmax(same))
        raise InvalidMesh(f"elements {int(qtags[f0[i] // 4])} and {int(qtags[f1[i] // 4])} "
                          f"overlap: they traverse their shared edge {segment(int(f0[i]))} in "
                          "the same direction")

    # boundary tags from the line elements; untagged boundary edges are walls
    boundary = counts[inverse] == 1
    edge_tag: dict[int, int] = {}
    for etag, nodes, groups in raw.lines:
        idx, ok = lookup(np.array(nodes, dtype=np.int64))
        v = np.where(ok, vertex_of_node[np.maximum(idx, 0)], -1)
        e = -1
        if (v >= 0).all():
            k = min(v) * vertices.shape[0] + max(v)
            at = int(np.searchsorted(ek, k))
            e = at if at < ek.size and ek[at] == k else -1
        if e < 0:
            raise InvalidMesh(f"line element {etag} (nodes {nodes[0]} and {nodes[1]}) is not an "
                              "edge of the quadrilateral mesh")
        if counts[e] != 1:
            continue
        t = _line_tag(raw, groups)
        if t is None:
            continue
        if e in edge_tag and edge_tag[e] != t:
            f = int(faces_of[starts[e]])
            raise InvalidMesh(f"the boundary edge {segment(f)} has two boundary tags, "
                              f"{tag_name(edge_tag[e])} and {tag_name(t)}")
        edge_tag[e] = t
    face_tags = np.full(K * 4, TAG_WALL, np.int32)
    for e, t in edge_tag.items():
        face_tags[faces_of[starts[e]]] = t
    face_tags[~boundary] = TAG_WALL
    mesh = QuadMesh(vertices, quads, np.zeros((0, 4), np.int64), face_tags.reshape(K, 4))
    return in_hilbert_order(mesh)[0]


def parse_gmsh_mesh(data: bytes) -> QuadMesh:
    """The quadrilateral mesh of a Gmsh file's contents (MSH 4.1 ASCII or
    binary, MSH 2.2 ASCII)."""
    return _build(_parse_msh(bytes(data)))


def read_gmsh_mesh(path) -> QuadMesh:
    return parse_gmsh_mesh(Path(path).read_bytes())


def boundary_edges(mesh: QuadMesh):
    """The boundary faces of a mesh as (element, face, vertex a, vertex b,
    tag) rows, element by element (periodic pairs are interior)."""
    K = mesh.n_elements
    a = mesh.elements.reshape(-1)
    b = mesh.elements[:, [1, 2, 3, 0]].reshape(-1)
    key = np.minimum(a, b) * mesh.vertices.shape[0] + np.maximum(a, b)
    _, inverse, counts = np.unique(key, return_inverse=True, return_counts=True)
    on = counts[inverse] == 1
    if mesh.periodic.size:
        for k0, f0, k1, f1 in mesh.periodic:
            on[4 * k0 + f0] = on[4 * k1 + f1] = False
    tags = (mesh.face_tags.reshape(-1) if mesh.face_tags is not None
            else np.zeros(4 * K, np.int32))
    faces = np.nonzero(on)[0]
    return np.stack([faces // 4, faces % 4, a[faces], b[faces], tags[faces]], axis=1)


def write_gmsh_mesh(mesh: QuadMesh, path) -> None:
    """MSH 2.2 ASCII: the vertices, each boundary face as a line in the
    physical group of its tag (so the tags survive a round trip), then the
    quadrilaterals (write_gmsh_mesh, gmsh.rs:950-1015)."""
    if mesh.periodic.size:
        raise GmshUnsupported("periodic meshes cannot be written to MSH 2.2")
    out = ["$MeshFormat", "2.2 0 8", "$EndMeshFormat", "$Nodes", str(mesh.vertices.shape[0])]
    out += [f"{i + 1} {_fmt(x)} {_fmt(y)} 0" for i, (x, y) in enumerate(mesh.vertices)]
    out += ["$EndNodes", "$Elements"]
    edges = boundary_edges(mesh)
    out.append(str(len(edges) + mesh.n_elements))
    eid = 1
    for _, _, va, vb, tag in edges:
        phys = tag_to_physical(int(tag))
        lo, hi = min(va, vb), max(va, vb)
        out.append(f"{eid} 1 2 {phys} {phys} {lo + 1} {hi + 1}")
        eid += 1
    for q in mesh.elements:
        out.append(f"{eid} 3 2 0 0 {q[0] + 1} {q[1] + 1} {q[2] + 1} {q[3] + 1}")
        eid += 1
    out.append("$EndElements")
    Path(path).write_text("\n".join(out) + "\n")


def binary_msh41(mesh_nodes, quads, lines, curve_groups, names=(), big_endian=False,
                 size_bytes=8) -> bytes:
    """A binary MSH 4.1 file (for tests and converters): nodes [(tag, x, y)],
    quads [(tag, n0..n3)] on surface 1, lines [(tag, curve, na, nb)] on
    their curves, curve_groups {curve: [physical groups]}, names
    [(dim, tag, name)]."""
    e = ">" if big_endian else "<"
    st = "I" if size_bytes == 4 else "Q"

    def pack(fmt, *v):
        return struct.pack(e + fmt, *v)

    b = bytearray(f"$MeshFormat\n4.1 1 {size_bytes}\n".encode())
    b += pack("i", 1) + b"\n$EndMeshFormat\n"
    if names:
        b += f"$PhysicalNames\n{len(names)}\n".encode()
        for dim, tag, name in names:
            b += f'{dim} {tag} "{name}"\n'.encode()
        b += b"$EndPhysicalNames\n"
    curves = sorted(curve_groups)
    b += b"$Entities\n" + pack(st * 4, 0, len(curves), 1, 0)
    for c in curves:
        g = curve_groups[c]
        b += pack("i", c) + pack("6d", *([0.0] * 6)) + pack(st, len(g))
        b += pack(f"{len(g)}i", *g) + pack(st, 0)
    b += pack("i", 1) + pack("6d", *([0.0] * 6)) + pack(st, 0) + pack(st, 0)
    b += b"\n$EndEntities\n$Nodes\n"
    tags = [t for t, _, _ in mesh_nodes]
    b += pack(st * 4, 1, len(mesh_nodes), min(tags), max(tags))
    b += pack("iii", 2, 1, 0) + pack(st, len(mesh_nodes))
    b += pack(st * len(tags), *tags)
    for _, x, y in mesh_nodes:
        b += pack("3d", x, y, 0.0)
    b += b"\n$EndNodes\n$Elements\n"
    blocks = [(2, 1, QUAD, [(q[0], *q[1:]) for q in quads])]
    for c in curves:
        blocks.append((1, c, LINE, [(t, na, nb) for t, cc, na, nb in lines if cc == c]))
    blocks = [blk for blk in blocks if blk[3]]
    n = sum(len(blk[3]) for blk in blocks)
    all_tags = [row[0] for blk in blocks for row in blk[3]]
    b += pack(st * 4, len(blocks), n, min(all_tags), max(all_tags))
    for dim, ent, etype, rows in blocks:
        b += pack("iii", dim, ent, etype) + pack(st, len(rows))
        for row in rows:
            b += pack(st * len(row), *row)
    b += b"\n$EndElements\n"
    return bytes(b)
