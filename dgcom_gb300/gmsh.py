"""Gmsh meshes for the device path: how coastline-fitted domains made in
Gmsh reach the C ABI.

The reader takes the MSH 4.1 format (text, or binary in either byte order
with 4- or 8-byte sizes) and the MSH 2.2 text format, following Gmsh's
published file-format description; the writer writes MSH 2.2 text. What it
accepts and refuses is what the reference's reader does
(src/mesh/io/gmsh.rs), as the reference's tests pin it:

- the domain is first-order quadrilaterals (Gmsh type 3); points (type 15)
  are ignored, 2-node lines (type 1) carry boundary tags, and any other
  element type is refused with a count per type and the Gmsh settings that
  give an all-quad first-order mesh;
- node tags may be sparse and unordered; the vertices are the nodes the
  quadrilaterals use, in the order the file gives them; a clockwise
  quadrilateral is turned round; a corner with a non-positive bilinear
  Jacobian, an edge of three or more elements and two elements running the
  same way along their common edge are refused;
- a boundary edge takes the tag of the physical groups of the line element
  on it (MSH 4.1: the groups of the line's curve entity; MSH 2.2: the
  line's first integer tag), by group name where the group has one, else by
  number (1 wall, 2 open, 3 tidal, 4 river, 5 Dirichlet, 6 Neumann, n
  custom); untagged boundary edges are walls; lines on interior edges are
  ignored; a line that is no edge of the mesh, a curve whose groups give two
  tags and an edge given two tags are refused;
- MSH 4.0, binary MSH 2, periodic and partitioned meshes are refused; other
  sections are skipped; CRLF line ends are read;
- the mesh is returned in Hilbert order (``mesh.in_hilbert_order``).

How it reads. The file is cut into its ``$Name … $EndName`` sections
first. Each section that matters is decoded from one stream of numbers: a
text section is split into tokens once and converted in bulk, a binary
section is read through a byte cursor with ``numpy.frombuffer``; node and
element blocks come out as arrays, never one number at a time. Mesh checks
then run on whole arrays. Tags are the ABI's face tags (``mesh.TAG_*``,
``mesh.custom_tag``)."""

from __future__ import annotations

import re
import struct
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from .mesh import (CUSTOM_TAG_BASE, TAG_DIRICHLET, TAG_NEUMANN, TAG_OPEN, TAG_RIVER, TAG_TIDAL,
                   TAG_WALL, QuadMesh, custom_tag, in_hilbert_order)


# -- errors -------------------------------------------------------------------

class GmshError(ValueError):
    """Any Gmsh file the device path cannot take."""


class GmshParseError(GmshError):
    """The bytes do not follow the format (a bad number, a short section)."""


class UnsupportedVersion(GmshError):
    """A format version other than MSH 4.1 and MSH 2.x text."""


class MissingSection(GmshError):
    """A section the mesh needs is absent."""


class GmshUnsupported(GmshError):
    """A feature of the format the device path has no use for."""


class InvalidMesh(GmshError):
    """The file reads, but its elements do not form a usable quad mesh."""


class UnsupportedElements(GmshError):
    """Elements other than quadrilaterals, lines and points; ``counts``
    holds (Gmsh type, how many) in type order."""

    def __init__(self, counts):
        self.counts = sorted((int(t), int(n)) for t, n in counts)
        listed = ", ".join(f"{n} × {_type_name(t)} (type {t})" for t, n in self.counts)
        super().__init__(
            f"the mesh holds {listed}, and the device path takes first-order "
            "quadrilaterals only. In Gmsh: Mesh.ElementOrder = 1, Mesh.RecombineAll = 1 "
            "and Mesh.SubdivisionAlgorithm = 1 give an all-quad 2D mesh")


# -- element types and physical groups -------------------------------------------

# Nodes per element of Gmsh's fixed-order element types (the format's table)
NODES_PER_TYPE = {
    1: 2, 2: 3, 3: 4, 4: 4, 5: 8, 6: 6, 7: 5, 8: 3, 9: 6, 10: 9, 11: 10, 12: 27, 13: 18,
    14: 14, 15: 1, 16: 8, 17: 20, 18: 15, 19: 13, 20: 9, 21: 10, 22: 12, 23: 15, 24: 15,
    25: 21, 26: 4, 27: 5, 28: 6, 29: 20, 30: 35, 31: 56, 36: 16, 37: 25, 38: 36,
}
_SHAPES = {1: "line", 8: "line", 26: "line", 27: "line", 28: "line", 15: "point",
           2: "triangle", 9: "triangle", 20: "triangle", 21: "triangle", 22: "triangle",
           23: "triangle", 24: "incomplete triangle", 25: "triangle",
           3: "quadrangle", 10: "quadrangle", 16: "quadrangle", 36: "quadrangle",
           37: "quadrangle", 38: "quadrangle", 4: "tetrahedron", 11: "tetrahedron",
           29: "tetrahedron", 30: "tetrahedron", 31: "tetrahedron", 5: "hexahedron",
           12: "hexahedron", 17: "hexahedron", 6: "prism", 13: "prism", 18: "prism",
           7: "pyramid", 14: "pyramid", 19: "pyramid"}
T_LINE, T_QUAD, T_POINT = 1, 3, 15


def _type_name(t: int) -> str:
    if t not in NODES_PER_TYPE:
        return "element of an unknown type"
    return f"{NODES_PER_TYPE[t]}-node {_SHAPES[t]}"


# group names, compared lower-case with spaces and dashes read as "_"
_BY_NAME = {
    **dict.fromkeys(("wall", "walls", "land", "coast", "coastline", "shore", "shoreline",
                     "closed"), TAG_WALL),
    **dict.fromkeys(("open", "ocean", "sea", "open_boundary"), TAG_OPEN),
    **dict.fromkeys(("tidal", "tide", "tides", "tidal_forcing"), TAG_TIDAL),
    **dict.fromkeys(("river", "rivers"), TAG_RIVER),
}
_BY_NUMBER = (TAG_WALL, TAG_OPEN, TAG_TIDAL, TAG_RIVER, TAG_DIRICHLET, TAG_NEUMANN)  # 1..6
_TAG_NAMES = {TAG_WALL: "Wall", TAG_OPEN: "Open", TAG_TIDAL: "TidalForcing", TAG_RIVER: "River",
              TAG_DIRICHLET: "Dirichlet", TAG_NEUMANN: "Neumann"}


def group_boundary_tag(number: int, name: str | None) -> int:
    """The face tag a physical group stands for: by its name where it has
    one that means something, else by its number."""
    if number < 0:
        raise InvalidMesh(f"physical group {number}: group numbers are not negative")
    if name is not None:
        key = re.sub(r"[ \-]", "_", name.lower())
        if key in _BY_NAME:
            return _BY_NAME[key]
    if 1 <= number <= len(_BY_NUMBER):
        return _BY_NUMBER[number - 1]
    return custom_tag(number)


def tag_to_physical(tag: int) -> int:
    """The physical group number a face tag is written under (the inverse of
    :func:`group_boundary_tag` for unnamed groups)."""
    if tag in _BY_NUMBER:
        return _BY_NUMBER.index(tag) + 1
    if tag >= CUSTOM_TAG_BASE:
        return tag - CUSTOM_TAG_BASE
    raise ValueError(f"face tag {tag} has no physical group number")


def tag_name(tag: int) -> str:
    return _TAG_NAMES.get(tag, f"Custom({tag - CUSTOM_TAG_BASE})")


# -- cutting the file into sections ---------------------------------------------------

@dataclass
class _Section:
    name: str
    start: int   # first byte of the payload (after the header line)
    stop: int    # first byte of "$End<name>"


_BINARY_SECTIONS = ("Entities", "Nodes", "Elements")


def _line_of(data: bytes, pos: int) -> int:
    return 1 + data.count(b"\n", 0, pos)


def _header_at(data: bytes, pos: int) -> tuple[str, int]:
    """The section name of the header line at ``pos`` and where its payload
    starts."""
    end = data.find(b"\n", pos)
    end = len(data) if end < 0 else end
    text = data[pos:end].strip()
    if not text.startswith(b"$") or len(text) < 2:
        shown = text[:40].decode("ascii", "replace")
        raise GmshParseError(f"line {_line_of(data, pos)}: a section header ($Name) was due, "
                             f'not "{shown}"')
    return text[1:].decode("ascii", "replace"), min(end + 1, len(data))


def _skip_space(data: bytes, pos: int) -> int:
    while pos < len(data) and data[pos] in b" \t\r\n":
        pos += 1
    return pos


class _Layout:
    """What the format line said: text or binary, byte order, size width."""

    def __init__(self):
        self.version: str | None = None  # "4.1" or "2"
        self.binary = False
        self.order = "<"
        self.size_bytes = 8


def _cut(data: bytes, layout: _Layout, decode) -> None:
    """Walk the sections in file order, handing each to ``decode(section,
    stream)``. A text section ends at its ``$End`` line; a binary 4.1
    section ends where its decoder stops reading."""
    pos = _skip_space(data, 0)
    while pos < len(data):
        name, start = _header_at(data, pos)
        marker = f"$End{name}".encode()
        if layout.binary and name in _BINARY_SECTIONS:
            stream = _BinaryStream(data, start, layout)
            decode(_Section(name, start, -1), stream)
            stop = _skip_space(data, stream.pos)
        else:
            if name == "MeshFormat":  # the version decides before anything else
                _read_format(data, start, layout)
            stop = _find_marker(data, start, marker)
            if stop < 0:
                raise GmshParseError(f"line {_line_of(data, start)}: ${name} has no {marker.decode()}")
            if name != "MeshFormat":
                decode(_Section(name, start, stop), _TextStream(data, start, stop))
        if not data.startswith(marker, stop) or (len(data) > stop + len(marker)
                                                 and data[stop + len(marker)] not in b" \t\r\n"):
            raise GmshParseError(f"line {_line_of(data, stop)}: {marker.decode()} was due")
        pos = _skip_space(data, stop + len(marker))


def _find_marker(data: bytes, start: int, marker: bytes) -> int:
    """The first line holding ``marker`` alone at or after ``start``."""
    at = start
    while True:
        at = data.find(marker, at)
        if at < 0:
            return -1
        before_ok = at == 0 or data[at - 1] in b"\r\n"
        end = at + len(marker)
        after_ok = end == len(data) or data[end] in b" \t\r\n"
        if before_ok and after_ok:
            return at
        at += 1


def _read_format(data: bytes, start: int, layout: _Layout) -> None:
    eol = data.find(b"\n", start)
    words = data[start:len(data) if eol < 0 else eol].split()
    if len(words) < 3:
        raise GmshParseError(f"line {_line_of(data, start)}: the format line needs a version, "
                             "a file type and a data size")
    version = words[0].decode("ascii", "replace")
    try:
        file_type, size = int(words[1]), int(words[2])
    except ValueError:
        raise GmshParseError(f"line {_line_of(data, start)}: the format line's file type and "
                             "data size are integers") from None
    if version == "4.1":
        layout.version = "4.1"
    elif version.startswith("2."):
        layout.version = "2"
    elif version.startswith("4"):
        raise UnsupportedVersion(f"MSH {version} is not read: save the mesh as MSH 4.1 "
                                 "(Mesh.MshFileVersion = 4.1) or MSH 2.2")
    else:
        raise UnsupportedVersion(f"MSH {version} is not read (MSH 4.1 and 2.2 are)")
    if file_type == 0:
        return
    if file_type != 1:
        raise GmshParseError(f"line {_line_of(data, start)}: file type {file_type} is neither "
                             "text (0) nor binary (1)")
    if layout.version != "4.1":
        raise UnsupportedVersion("binary MSH 2 is not read: save the mesh as text or as MSH 4.1")
    if size not in (4, 8):
        raise GmshParseError(f"line {_line_of(data, start)}: sizes of {size} bytes (4 or 8 are "
                             "written by Gmsh)")
    # the binary marker: the integer 1 in the file's byte order, after the line
    eol = data.find(b"\n", start)
    mark = data[eol + 1:eol + 5] if eol >= 0 else b""
    if mark == struct.pack("<i", 1):
        layout.order = "<"
    elif mark == struct.pack(">i", 1):
        layout.order = ">"
    else:
        raise GmshParseError(f"line {_line_of(data, start)}: the binary marker (the integer 1) "
                             "is missing")
    layout.binary = True
    layout.size_bytes = size


# -- number streams ----------------------------------------------------------------------

_INT = re.compile(rb"[+-]?\d+\Z")


class _TextStream:
    """The numbers of one text section, split into tokens once; ``ints``,
    ``sizes`` and ``reals`` convert the next n in bulk and name the first
    bad one (with its line) when a conversion fails."""

    def __init__(self, data: bytes, start: int, stop: int):
        self.data, self.start = data, start
        self.tokens = data[start:stop].split()
        self.at = 0

    def _take(self, n: int, what) -> list:
        if n < 0 or self.at + n > len(self.tokens):
            name = what if isinstance(what, str) else what[0]
            raise GmshParseError(f"line {_line_of(self.data, self.start)}: the section ends "
                                 f"before its {name} values")
        toks = self.tokens[self.at:self.at + n]
        self.at += n
        return toks

    def _bad(self, index: int, what) -> GmshParseError:
        names = (what,) if isinstance(what, str) else what
        k = 0
        for k, m in enumerate(re.finditer(rb"\S+", self.data[self.start:])):
            if k == index:
                line = _line_of(self.data, self.start + m.start())
                name = names[(index - self._first) % len(names)]
                return GmshParseError(f'invalid {name}: "{m.group().decode("ascii", "replace")}" '
                                      f"(line {line}, token {index + 1} of the section)")
        return GmshParseError(f"invalid {names[0]}")

    def ints(self, n: int, what, nonnegative: bool = False) -> np.ndarray:
        self._first = self.at
        toks = self._take(n, what)
        try:
            out = np.array(toks, dtype=object).astype(np.int64) if n else np.zeros(0, np.int64)
        except (ValueError, OverflowError):
            out = None
        if out is None or not all(_INT.match(t) for t in toks) or (nonnegative and (out < 0).any()):
            for i, t in enumerate(toks):
                if not _INT.match(t) or (nonnegative and t.startswith(b"-")):
                    raise self._bad(self._first + i, what)
        return out

    sizes = ints

    def reals(self, n: int, what) -> np.ndarray:
        self._first = self.at
        toks = self._take(n, what)
        try:
            return np.array(toks, dtype=np.bytes_).astype(np.float64) if n else np.zeros(0)
        except ValueError:
            for i, t in enumerate(toks):
                try:
                    float(t)
                except ValueError:
                    raise self._bad(self._first + i, what) from None
            raise GmshParseError(f"invalid {what}") from None

    def rest_text(self) -> str:
        return self.data[self.start:].decode("utf-8", "replace")


class _BinaryStream:
    """A byte cursor over a binary MSH 4.1 section: int32 values, size_t
    values of the file's width, float64 values, all in its byte order."""

    def __init__(self, data: bytes, start: int, layout: _Layout):
        self.data, self.pos = data, start
        self.order = layout.order
        self.size_code = "u4" if layout.size_bytes == 4 else "u8"

    def _array(self, n: int, code: str, what) -> np.ndarray:
        dtype = np.dtype(self.order + code)
        need = n * dtype.itemsize
        if n < 0 or self.pos + need > len(self.data):
            name = what if isinstance(what, str) else what[0]
            raise GmshParseError(f"byte {self.pos}: the file ends before its {name} values")
        out = np.frombuffer(self.data, dtype=dtype, count=n, offset=self.pos)
        self.pos += need
        return out.astype(dtype.newbyteorder("="))

    def ints(self, n: int, what, nonnegative: bool = False) -> np.ndarray:
        return self._array(n, "i4", what).astype(np.int64)

    def sizes(self, n: int, what, nonnegative: bool = False) -> np.ndarray:
        out = self._array(n, self.size_code, what)
        if (out > np.iinfo(np.int64).max).any():
            raise GmshParseError(f"byte {self.pos}: a {what} beyond any file's reach")
        return out.astype(np.int64)

    def reals(self, n: int, what) -> np.ndarray:
        return self._array(n, "f8", what)


def _count(stream, what: str, per_item_tokens: int = 1) -> int:
    """A count that the rest of the section can hold (so a corrupt count
    cannot ask for a huge array)."""
    n = int(stream.sizes(1, what)[0])
    if isinstance(stream, _TextStream):
        room = len(stream.tokens) - stream.at
    else:
        room = len(stream.data) - stream.pos
    if n * max(per_item_tokens, 1) > room + 1:
        raise GmshParseError(f"a {what} of {n} is more than the rest of the file holds")
    return n


# -- the file's tables ----------------------------------------------------------------------

@dataclass
class _Tables:
    node_tags: list = field(default_factory=list)     # arrays of node tags
    node_xy: list = field(default_factory=list)       # arrays (n, 2)
    quad_tags: list = field(default_factory=list)
    quad_nodes: list = field(default_factory=list)    # arrays (n, 4)
    line_tags: list = field(default_factory=list)
    line_nodes: list = field(default_factory=list)    # arrays (n, 2)
    line_groups: list = field(default_factory=list)   # per line block: tuple of physical groups
    other: dict = field(default_factory=dict)         # element type → count
    names: dict = field(default_factory=dict)         # (dim, number) → name
    curve_groups: dict = field(default_factory=dict)  # curve entity → physical groups


def _decoder(tables: _Tables, layout: _Layout):
    def decode(section: _Section, stream):
        name = section.name
        if name in ("Nodes", "Elements", "Entities") and layout.version is None:
            raise MissingSection(f"the file has no $MeshFormat before its ${name}")
        if name == "PhysicalNames":
            _physical_names(stream, tables)
        elif name == "Entities":
            if layout.version != "4.1":
                raise GmshParseError("$Entities belongs to MSH 4 files, not to an MSH 2 file")
            _entities(stream, tables)
        elif name == "Nodes":
            (_nodes_41 if layout.version == "4.1" else _nodes_22)(stream, tables)
        elif name == "Elements":
            (_elements_41 if layout.version == "4.1" else _elements_22)(stream, tables)
        elif name == "Periodic":
            raise GmshUnsupported("the mesh is periodic; periodic Gmsh meshes are not read")
        elif name == "PartitionedEntities":
            raise GmshUnsupported("the mesh is partitioned: save it whole "
                                  "(Mesh.PartitionSplitMeshFiles = 0, no partitions)")
        # any other section is skipped
    return decode


def _physical_names(stream: _TextStream, t: _Tables) -> None:
    n = _count(stream, "physical name count", 3)
    # names may hold spaces: read them from the lines, not from the tokens
    lines = stream.rest_text().splitlines()[1:1 + n]
    if len(lines) < n:
        raise GmshParseError("$PhysicalNames ends before its names")
    for row in lines:
        parts = row.strip().split(None, 2)
        if len(parts) < 3 or not _INT.match(parts[0].encode()) or not _INT.match(parts[1].encode()):
            raise GmshParseError(f'a physical name row reads "dim number name", not "{row.strip()}"')
        label = parts[2].strip()
        if len(label) >= 2 and label[0] == label[-1] == '"':
            label = label[1:-1]
        t.names[(int(parts[0]), int(parts[1]))] = label


def _entities(stream, t: _Tables) -> None:
    counts = [_count(stream, "entity count") for _ in range(4)]
    for dim, n in enumerate(counts):
        for _ in range(n):
            tag = int(stream.ints(1, "entity tag")[0])
            stream.reals(3 if dim == 0 else 6, "entity coordinate")
            groups = stream.ints(_count(stream, "physical tag count"), "physical tag")
            if dim > 0:
                stream.ints(_count(stream, "bounding entity count"), "bounding entity tag")
            if dim == 1:
                t.curve_groups[tag] = tuple(int(g) for g in groups)


def _add_nodes(t: _Tables, tags: np.ndarray, xy: np.ndarray) -> None:
    bad = ~np.isfinite(xy).all(axis=1)
    if bad.any():
        k = int(np.argmax(bad))
        raise GmshParseError(f"node {int(tags[k])} sits at ({xy[k, 0]}, {xy[k, 1]}), not a "
                             "finite point")
    t.node_tags.append(tags)
    t.node_xy.append(xy)


def _nodes_41(stream, t: _Tables) -> None:
    n_blocks = _count(stream, "node block count", 4)
    n_total = _count(stream, "node count")
    stream.sizes(2, "node tag range")
    seen = 0
    for _ in range(n_blocks):
        dim, _entity, parametric = (int(v) for v in stream.ints(3, "node block header"))
        n = _count(stream, "node count of a block")
        if parametric not in (0, 1) or not 0 <= dim <= 3:
            raise GmshParseError(f"a node block of dimension {dim} with parametric flag "
                                 f"{parametric}")
        per = 3 + (dim if parametric else 0)
        tags = stream.sizes(n, "node tag", nonnegative=True)
        coords = stream.reals(n * per, ("node x", "node y", "node z") + ("node parameter",) * (per - 3))
        coords = coords.reshape(n, per)
        _add_nodes(t, tags, np.ascontiguousarray(coords[:, :2]))
        seen += n
    if seen != n_total:
        raise GmshParseError(f"$Nodes announces {n_total} nodes and holds {seen}")


def _nodes_22(stream: _TextStream, t: _Tables) -> None:
    n = _count(stream, "node count", 4)
    rows = stream.reals(4 * n, ("node tag", "node x", "node y", "node z")).reshape(n, 4)
    tags = rows[:, 0]
    whole = (tags == np.floor(tags)) & (tags >= 0)
    if not whole.all():
        k = int(np.argmin(whole))
        raise GmshParseError(f'invalid node tag: "{tags[k]}" (node {k + 1} of $Nodes)')
    _add_nodes(t, tags.astype(np.int64), np.ascontiguousarray(rows[:, 1:3]))


def _keep(t: _Tables, etype: int, tags: np.ndarray, nodes: np.ndarray, groups: tuple) -> None:
    if etype == T_QUAD:
        t.quad_tags.append(tags)
        t.quad_nodes.append(nodes)
    elif etype == T_LINE:
        t.line_tags.append(tags)
        t.line_nodes.append(nodes)
        t.line_groups.extend([groups] * len(tags))
    elif etype != T_POINT:
        t.other[etype] = t.other.get(etype, 0) + len(tags)


def _elements_41(stream, t: _Tables) -> None:
    n_blocks = _count(stream, "element block count", 4)
    n_total = _count(stream, "element count")
    stream.sizes(2, "element tag range")
    seen = 0
    for _ in range(n_blocks):
        _dim, entity, etype = (int(v) for v in stream.ints(3, "element block header"))
        n = _count(stream, "element count of a block")
        if etype not in NODES_PER_TYPE:
            raise UnsupportedElements([(etype, n)])
        width = 1 + NODES_PER_TYPE[etype]
        rows = stream.sizes(n * width, "element node tag", nonnegative=True).reshape(n, width)
        groups = t.curve_groups.get(entity, ()) if etype == T_LINE else ()
        _keep(t, etype, rows[:, 0], rows[:, 1:], groups)
        seen += n
    if seen != n_total:
        raise GmshParseError(f"$Elements announces {n_total} elements and holds {seen}")


def _elements_22(stream: _TextStream, t: _Tables) -> None:
    n = _count(stream, "element count", 4)
    # every value of an MSH 2.2 element row is an integer: convert the
    # section once, then walk the rows (their lengths vary with the type)
    values = stream.ints(len(stream.tokens) - stream.at, "element value")
    stream.at -= len(values)
    by_type: dict = {}
    at = 0
    for _ in range(n):
        if at + 3 > len(values):
            raise GmshParseError("$Elements ends inside an element row")
        tag, etype, n_tags = (int(v) for v in values[at:at + 3])
        if etype not in NODES_PER_TYPE:
            raise UnsupportedElements([(etype, 1)])
        if n_tags < 0 or tag < 0:
            raise GmshParseError(f"element {tag}: a negative count or tag")
        first = int(values[at + 3]) if n_tags > 0 and at + 3 < len(values) else 0
        nodes_at = at + 3 + n_tags
        nodes_to = nodes_at + NODES_PER_TYPE[etype]
        if nodes_to > len(values):
            raise GmshParseError("$Elements ends inside an element row")
        by_type.setdefault(etype, []).append((tag, first, values[nodes_at:nodes_to]))
        at = nodes_to
    stream.at += at
    for etype, rows in by_type.items():
        tags = np.array([r[0] for r in rows], np.int64)
        nodes = np.array([r[2] for r in rows], np.int64).reshape(len(rows), -1)
        if etype == T_LINE:
            for tag, first, nd in rows:
                _keep(t, etype, np.array([tag]), nd.reshape(1, -1), (first,) if first else ())
        else:
            _keep(t, etype, tags, nodes, ())


# -- from the tables to the mesh ----------------------------------------------------------

def _xy(x: float, y: float) -> str:
    return f"({float(x)!r}, {float(y)!r})"


class _NodeIndex:
    """Node tag → row of the concatenated node table, by binary search."""

    def __init__(self, tags: np.ndarray):
        self.order = np.argsort(tags, kind="stable")
        self.sorted = tags[self.order]
        twice = np.nonzero(self.sorted[1:] == self.sorted[:-1])[0]
        if twice.size:
            raise InvalidMesh(f"node {int(self.sorted[twice[0]])} is defined twice")

    def rows(self, tags: np.ndarray) -> np.ndarray:
        """Rows of ``tags``, −1 where a tag is not defined."""
        if self.sorted.size == 0:
            return np.full(tags.shape, -1, np.int64)
        at = np.clip(np.searchsorted(self.sorted, tags), 0, self.sorted.size - 1)
        return np.where(self.sorted[at] == tags, self.order[at], -1)


def _quads(t: _Tables, index: _NodeIndex, xy: np.ndarray):
    """Vertices (the used nodes, in file order), the quads on them turned
    counter-clockwise, the quads' file tags and file node tags."""
    tags = np.concatenate(t.quad_tags)
    nodes = np.concatenate(t.quad_nodes).astype(np.int64)
    rows = index.rows(nodes)
    missing = np.argwhere(rows < 0)
    if missing.size:
        k, c = missing[0]
        raise InvalidMesh(f"element {int(tags[k])} uses undefined node {int(nodes[k, c])}")
    used = np.zeros(xy.shape[0], bool)
    used[rows.reshape(-1)] = True
    renumber = np.cumsum(used) - 1
    vertices = xy[used]
    quads = renumber[rows]
    p = vertices[quads]
    shoelace = (p[:, :, 0] * np.roll(p[:, :, 1], -1, axis=1)
                - np.roll(p[:, :, 0], -1, axis=1) * p[:, :, 1]).sum(axis=1)
    # a clockwise quad is read backwards from its first corner
    clockwise = shoelace < 0.0
    quads[clockwise] = np.roll(quads[clockwise][:, ::-1], 1, axis=1)
    nodes = nodes.copy()
    nodes[clockwise] = np.roll(nodes[clockwise][:, ::-1], 1, axis=1)
    return vertices, quads, tags, nodes, np.where(used, renumber, -1)


def _check_corners(vertices, quads, tags, nodes) -> None:
    """Every corner turns left by more than round-off: the bilinear map's
    Jacobian is positive there (and so everywhere)."""
    p = vertices[quads]
    into = p - np.roll(p, 1, axis=1)      # edge arriving at each corner
    out = np.roll(p, -1, axis=1) - p      # edge leaving it
    turn = into[..., 0] * out[..., 1] - into[..., 1] * out[..., 0]
    size = np.hypot(into[..., 0], into[..., 1]) * np.hypot(out[..., 0], out[..., 1])
    bad = ~(turn > 1e-12 * size)
    if bad.any():
        k, c = np.argwhere(bad)[0]
        raise InvalidMesh(f"element {int(tags[k])} is degenerate or non-convex at node "
                          f"{int(nodes[k, c])} {_xy(*p[k, c])}: the Jacobian of its bilinear "
                          "map is not positive there")


def _edges(vertices, quads, tags):
    """The mesh's edges: for every face (4·k + f) its edge number, and per
    edge how many faces it has; refuses an edge of three or more faces and
    two faces running the same way along one."""
    nv = vertices.shape[0]
    a = quads.reshape(-1)
    b = np.roll(quads, -1, axis=1).reshape(-1)
    key = np.minimum(a, b) * nv + np.maximum(a, b)
    keys, edge_of_face, faces = np.unique(key, return_inverse=True, return_counts=True)
    by_edge = np.argsort(edge_of_face, kind="stable")
    first = np.concatenate([[0], np.cumsum(faces)[:-1]])

    def where(f):
        return f"{_xy(*vertices[a[f]])}–{_xy(*vertices[b[f]])}"

    crowded = np.nonzero(faces > 2)[0]
    if crowded.size:
        f = by_edge[first[crowded[0]]:first[crowded[0]] + faces[crowded[0]]]
        owners = ", ".join(str(int(tags[i // 4])) for i in f)
        raise InvalidMesh(f"the edge {where(f[0])} is shared by more than two elements "
                          f"({owners})")
    pairs = np.nonzero(faces == 2)[0]
    f0, f1 = by_edge[first[pairs]], by_edge[first[pairs] + 1]
    same_way = a[f0] == a[f1]
    if same_way.any():
        i = int(np.argmax(same_way))
        raise InvalidMesh(f"elements {int(tags[f0[i] // 4])} and {int(tags[f1[i] // 4])} overlap "
                          f"along {where(f0[i])}: both run along it the same way")
    return keys, edge_of_face, faces, by_edge, first, where


def _line_tag(t: _Tables, groups: tuple) -> int | None:
    tag = None
    for g in groups:
        this = group_boundary_tag(int(g), t.names.get((1, int(g))))
        if tag is not None and this != tag:
            raise InvalidMesh(f"a boundary curve lies in physical groups that give it different "
                              f"boundary tags, {tag_name(tag)} and {tag_name(this)}")
        tag = this
    return tag


def _face_tags(t: _Tables, index: _NodeIndex, used_row_to_vertex, nv, quads, edges):
    keys, edge_of_face, faces, by_edge, first, where = edges
    K = quads.shape[0]
    tags = np.full(4 * K, TAG_WALL, np.int32)
    if not t.line_tags:
        return tags.reshape(K, 4)
    line_tags = np.concatenate(t.line_tags)
    line_nodes = np.concatenate(t.line_nodes).astype(np.int64)
    rows = index.rows(line_nodes)
    verts = np.where(rows >= 0, used_row_to_vertex[np.maximum(rows, 0)], -1)
    key = np.minimum(verts[:, 0], verts[:, 1]) * nv + np.maximum(verts[:, 0], verts[:, 1])
    at = np.clip(np.searchsorted(keys, key), 0, keys.size - 1)
    on_mesh = (verts >= 0).all(axis=1) & (keys[at] == key)
    if not on_mesh.all():
        i = int(np.argmin(on_mesh))
        raise InvalidMesh(f"line element {int(line_tags[i])} (nodes {int(line_nodes[i, 0])} and "
                          f"{int(line_nodes[i, 1])}) is not an edge of the quadrilateral mesh")
    given: dict = {}
    for i in np.nonzero(faces[at] == 1)[0]:  # lines on interior edges carry nothing
        tag = _line_tag(t, t.line_groups[i])
        if tag is None:
            continue
        e = int(at[i])
        if given.setdefault(e, tag) != tag:
            raise InvalidMesh(f"the boundary edge {where(by_edge[first[e]])} has two boundary "
                              f"tags, {tag_name(given[e])} and {tag_name(tag)}")
    for e, tag in given.items():
        tags[by_edge[first[e]]] = tag
    return tags.reshape(K, 4)


def _assemble(t: _Tables) -> QuadMesh:
    if t.other:
        raise UnsupportedElements(t.other.items())
    if not t.node_tags:
        raise MissingSection("the file has no $Nodes")
    if not t.quad_tags or sum(len(x) for x in t.quad_tags) == 0:
        raise InvalidMesh("the file holds no quadrilaterals. Gmsh saves only the elements of "
                          "physical groups once there are any: put the domain in a physical "
                          "surface, or set Mesh.SaveAll = 1")
    node_tags = np.concatenate(t.node_tags)
    xy = np.concatenate(t.node_xy)
    index = _NodeIndex(node_tags)
    vertices, quads, qtags, qnodes, row_to_vertex = _quads(t, index, xy)
    _check_corners(vertices, quads, qtags, qnodes)
    edges = _edges(vertices, quads, qtags)
    face_tags = _face_tags(t, index, row_to_vertex, vertices.shape[0], quads, edges)
    mesh = QuadMesh(vertices, quads, np.zeros((0, 4), np.int64), face_tags)
    return in_hilbert_order(mesh)[0]


# -- public entry points ----------------------------------------------------------------------

def parse_gmsh_mesh(data: bytes) -> QuadMesh:
    """The quadrilateral mesh in the bytes of a Gmsh file (MSH 4.1 text or
    binary, MSH 2.2 text)."""
    data = bytes(data)
    layout = _Layout()
    tables = _Tables()
    try:
        _cut(data, layout, _decoder(tables, layout))
    except (IndexError, struct.error, OverflowError) as err:  # a cut file, whatever byte it ends on
        raise GmshParseError(f"the file ends or breaks off inside a section ({err})") from None
    if layout.version is None:
        raise MissingSection("the file has no $MeshFormat")
    return _assemble(tables)


def read_gmsh_mesh(path) -> QuadMesh:
    return parse_gmsh_mesh(Path(path).read_bytes())


def boundary_edges(mesh: QuadMesh) -> np.ndarray:
    """The mesh's boundary faces, one row each in element order: (element,
    face, first vertex, second vertex, tag). Periodic pairs are not
    boundary."""
    a = mesh.elements.reshape(-1)
    b = np.roll(mesh.elements, -1, axis=1).reshape(-1)
    key = np.minimum(a, b) * mesh.vertices.shape[0] + np.maximum(a, b)
    _, edge_of_face, faces = np.unique(key, return_inverse=True, return_counts=True)
    alone = faces[edge_of_face] == 1
    for k0, f0, k1, f1 in mesh.periodic:
        alone[4 * k0 + f0] = alone[4 * k1 + f1] = False
    tags = (np.zeros(a.size, np.int32) if mesh.face_tags is None
            else mesh.face_tags.reshape(-1))
    f = np.nonzero(alone)[0]
    return np.stack([f // 4, f % 4, a[f], b[f], tags[f]], axis=1)


def write_gmsh_mesh(mesh: QuadMesh, path) -> None:
    """The mesh as MSH 2.2 text: its vertices (shortest round-trip
    decimals), every boundary face as a line element whose physical and
    elementary tags are its tag's group number (so the tags read back), then
    the quadrilaterals."""
    if mesh.periodic.size:
        raise GmshUnsupported("a periodic mesh has no MSH 2.2 form here")
    rows = boundary_edges(mesh)
    nv = mesh.vertices.shape[0]
    text = ["$MeshFormat", "2.2 0 8", "$EndMeshFormat", "$Nodes", str(nv)]
    text += [f"{i} {x!r} {y!r} 0" for i, (x, y) in enumerate(mesh.vertices.tolist(), start=1)]
    text += ["$EndNodes", "$Elements", str(len(rows) + mesh.n_elements)]
    number = 0
    for _, _, va, vb, tag in rows.tolist():
        number += 1
        group = tag_to_physical(int(tag))
        text.append(f"{number} {T_LINE} 2 {group} {group} {min(va, vb) + 1} {max(va, vb) + 1}")
    for quad in (mesh.elements + 1).tolist():
        number += 1
        text.append(f"{number} {T_QUAD} 2 0 0 " + " ".join(map(str, quad)))
    text.append("$EndElements")
    Path(path).write_text("\n".join(text) + "\n")


def binary_msh41(nodes, quads, lines, curve_groups, names=(), big_endian=False,
                 size_bytes=8) -> bytes:
    """A binary MSH 4.1 file of ``nodes`` [(tag, x, y)] on surface 1,
    ``quads`` [(tag, n0, n1, n2, n3)] on surface 1, ``lines`` [(tag, curve,
    na, nb)] on their curves, ``curve_groups`` {curve: [physical group]}
    and ``names`` [(dim, group, name)] (for tests and converters)."""
    end = ">" if big_endian else "<"
    size = "I" if size_bytes == 4 else "Q"
    out = bytearray()

    def put(fmt: str, *values):
        out.extend(struct.pack(end + fmt, *values))

    def text(s: str):
        out.extend(s.encode())

    text(f"$MeshFormat\n4.1 1 {size_bytes}\n")
    put("i", 1)
    text("\n$EndMeshFormat\n")
    if names:
        text(f"$PhysicalNames\n{len(names)}\n")
        for dim, group, label in names:
            text(f'{dim} {group} "{label}"\n')
        text("$EndPhysicalNames\n")
    curves = sorted(curve_groups)
    text("$Entities\n")
    put(size * 4, 0, len(curves), 1, 0)
    for c in curves:
        groups = list(curve_groups[c])
        put("i6d", c, *([0.0] * 6))
        put(size, len(groups))
        put("i" * len(groups), *groups)
        put(size, 0)
    put("i6d", 1, *([0.0] * 6))
    put(size * 2, 0, 0)
    text("\n$EndEntities\n$Nodes\n")
    tags = [n[0] for n in nodes]
    put(size * 4, 1, len(nodes), min(tags), max(tags))
    put("iii", 2, 1, 0)
    put(size, len(nodes))
    put(size * len(tags), *tags)
    for _, x, y in nodes:
        put("3d", x, y, 0.0)
    text("\n$EndNodes\n$Elements\n")
    blocks = [(2, 1, T_QUAD, [tuple(q) for q in quads])] if quads else []
    for c in curves:
        rows = [(tag, a, b) for tag, cc, a, b in lines if cc == c]
        if rows:
            blocks.append((1, c, T_LINE, rows))
    every = [row[0] for _, _, _, rows in blocks for row in rows]
    put(size * 4, len(blocks), len(every), min(every, default=0), max(every, default=0))
    for dim, entity, etype, rows in blocks:
        put("iii", dim, entity, etype)
        put(size, len(rows))
        for row in rows:
            put(size * len(row), *row)
    text("\n$EndElements\n")
    return bytes(out)
