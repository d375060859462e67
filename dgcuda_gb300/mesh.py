"""Triangle meshes in the reference's array layout.

A mesh is the set of arrays the reference's driver builds from a ``.pmsh`` file
(``read_mesh``, src/2d/conservation/conserv.cu:118-192):

* ``V1x, V1y, V2x, V2y, V3x, V3y`` -- the three vertices of each element,
  counter-clockwise (positive Jacobian), float64 ``[num_elem]``;
* ``elem_s1, elem_s2, elem_s3`` -- the side index of the element's local sides
  0 (V1->V2), 1 (V2->V3) and 2 (V3->V1), int32 ``[num_elem]``;
* ``left_elem, right_elem`` -- the two elements of each side; ``right_elem < 0``
  marks a boundary side (-1 reflecting, -2 outflow, -3 inflow,
  conserv_kernels.cu:657-679), int32 ``[num_sides]``;
* ``left_side, right_side`` -- the local side number of the side in the left
  and right element, int32 ``[num_sides]``.

Periodic meshes pair the sides on opposite boundaries as ordinary interior
sides, so they carry no boundary tags.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

__all__ = ["Mesh", "periodic_square", "scramble", "dirichlet_square", "unit_draws", "write_pmsh",
           "read_pmsh", "read_gmsh", "gmsh_to_pmsh", "tag_boundary", "from_triangles", "annulus"]


def _splitmix64(x: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        x = x + np.uint64(0x9E3779B97F4A7C15)
        x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return x ^ (x >> np.uint64(31))


def unit_draws(seed: int, k: np.ndarray) -> np.ndarray:
    """Uniform [0,1) draws of a counter-based generator: draw k of stream `seed`
    is splitmix64(seed * golden + k) >> 11, scaled by 2^-53.  The native mesh
    generator (dgx_meshgen.cpp) uses the same draws."""
    with np.errstate(over="ignore"):
        base = np.array([seed], dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15)
        v = _splitmix64(base + np.asarray(k, dtype=np.uint64))
    return (v >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


@dataclass
class Mesh:
    V1x: np.ndarray
    V1y: np.ndarray
    V2x: np.ndarray
    V2y: np.ndarray
    V3x: np.ndarray
    V3y: np.ndarray
    elem_s1: np.ndarray
    elem_s2: np.ndarray
    elem_s3: np.ndarray
    left_elem: np.ndarray
    right_elem: np.ndarray
    left_side: np.ndarray
    right_side: np.ndarray
    meta: dict = field(default_factory=dict)

    def __post_init__(self):
        for k in ("V1x", "V1y", "V2x", "V2y", "V3x", "V3y"):
            setattr(self, k, np.ascontiguousarray(getattr(self, k), dtype=np.float64))
        for k in ("elem_s1", "elem_s2", "elem_s3", "left_elem", "right_elem",
                  "left_side", "right_side"):
            setattr(self, k, np.ascontiguousarray(getattr(self, k), dtype=np.int32))

    @property
    def num_elem(self) -> int:
        return int(self.V1x.shape[0])

    @property
    def num_sides(self) -> int:
        return int(self.left_elem.shape[0])

    def vertices(self):
        return (self.V1x, self.V1y, self.V2x, self.V2y, self.V3x, self.V3y)

    def elem_sides(self):
        return (self.elem_s1, self.elem_s2, self.elem_s3)

    def side_arrays(self):
        return (self.left_elem, self.right_elem, self.left_side, self.right_side)

    def jacobian(self) -> np.ndarray:
        return ((self.V2x - self.V1x) * (self.V3y - self.V1y)
                - (self.V3x - self.V1x) * (self.V2y - self.V1y))

    def centroids(self):
        return ((self.V1x + self.V2x + self.V3x) / 3.0,
                (self.V1y + self.V2y + self.V3y) / 3.0)

    def check(self) -> None:
        """Raise ValueError if the connectivity is inconsistent."""
        E, S = self.num_elem, self.num_sides
        es = np.stack(self.elem_sides(), axis=1)
        if es.min() < 0 or es.max() >= S:
            raise ValueError("elem_s out of range")
        if self.left_elem.min() < 0 or self.left_elem.max() >= E:
            raise ValueError("left_elem out of range")
        if self.right_elem.max() >= E:
            raise ValueError("right_elem out of range")
        if np.any(self.jacobian() <= 0):
            raise ValueError("elements must be counter-clockwise")
        for s_arr, e_arr, name in ((self.left_side, self.left_elem, "left"),
                                   (self.right_side, self.right_elem, "right")):
            interior = e_arr >= 0
            if np.any((s_arr[interior] < 0) | (s_arr[interior] > 2)):
                raise ValueError(f"{name}_side out of range")
            ok = es[e_arr[interior], s_arr[interior]] == np.nonzero(interior)[0]
            if not np.all(ok):
                raise ValueError(f"{name} side numbers disagree with elem_s")


def periodic_square(n: int, lx: float = 1.0, ly: float = 1.0, x0: float = 0.0,
                    y0: float = 0.0, jitter: float = 0.0, seed: int = 0) -> Mesh:
    """Structured periodic triangulation of [x0,x0+lx] x [y0,y0+ly].

    ``n x n`` squares, each split along its SW-NE diagonal into a lower
    triangle (SW, SE, NE) and an upper triangle (SW, NE, NW): ``2 n^2``
    elements and ``3 n^2`` sides.  Interior vertices move by independent
    uniform offsets ``jitter h (2u - 1)`` (u from :func:`unit_draws` of the
    seed and the vertex index j*(n+1)+i); boundary vertices stay put so that
    periodic images coincide.  Bit-identical to the native generator
    ``dgx_periodic_square_arrays``.  Element ``2q`` and ``2q+1``
    belong to square ``q = j n + i``; sides ``3q``, ``3q+1``, ``3q+2`` are its
    bottom, left and diagonal sides, so neighbouring elements have nearby
    indices.
    """
    if n < 1:
        raise ValueError("n must be >= 1")
    hx, hy = lx / n, ly / n
    ii, jj = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="ij")
    X = x0 + ii * hx
    Y = y0 + jj * hy
    if jitter > 0 and n > 1:
        v = (jj[1:n, 1:n] * (n + 1) + ii[1:n, 1:n]).astype(np.uint64)
        dx = (jitter * hx) * (2.0 * unit_draws(seed, 2 * v) - 1.0)
        dy = (jitter * hy) * (2.0 * unit_draws(seed, 2 * v + 1) - 1.0)
        X = X.copy(); Y = Y.copy()
        X[1:n, 1:n] += dx
        Y[1:n, 1:n] += dy
    i, j = np.meshgrid(np.arange(n), np.arange(n), indexing="xy")
    i = i.ravel(); j = j.ravel()            # square q = j*n + i, i fastest
    q = j * n + i
    E = 2 * n * n
    S = 3 * n * n
    swx, swy = X[i, j], Y[i, j]
    sex, sey = X[i + 1, j], Y[i + 1, j]
    nex, ney = X[i + 1, j + 1], Y[i + 1, j + 1]
    nwx, nwy = X[i, j + 1], Y[i, j + 1]
    V = np.empty((6, E))
    V[:, 0::2] = (swx, swy, sex, sey, nex, ney)      # lower (SW, SE, NE)
    V[:, 1::2] = (swx, swy, nex, ney, nwx, nwy)      # upper (SW, NE, NW)
    qr = j * n + (i + 1) % n                          # square to the right
    qu = ((j + 1) % n) * n + i                        # square above
    ql = j * n + (i - 1) % n                          # square to the left
    qd = ((j - 1) % n) * n + i                        # square below
    es = np.empty((3, E), dtype=np.int64)
    es[:, 0::2] = (3 * q, 3 * qr + 1, 3 * q + 2)
    es[:, 1::2] = (3 * q + 2, 3 * qu, 3 * q + 1)
    le = np.empty(S, dtype=np.int64); re = np.empty(S, dtype=np.int64)
    ls = np.empty(S, dtype=np.int64); rs = np.empty(S, dtype=np.int64)
    le[0::3], ls[0::3], re[0::3], rs[0::3] = 2 * q, 0, 2 * qd + 1, 1      # bottom
    le[1::3], ls[1::3], re[1::3], rs[1::3] = 2 * q + 1, 2, 2 * ql, 1      # left
    le[2::3], ls[2::3], re[2::3], rs[2::3] = 2 * q, 2, 2 * q + 1, 0       # diagonal
    m = Mesh(*V, *es, le, re, ls, rs,
             meta=dict(kind="periodic_square", n=n, lx=lx, ly=ly, x0=x0, y0=y0,
                       jitter=jitter, seed=seed, h=min(hx, hy)))
    return m


def dirichlet_square(n: int, lx: float = 1.0, ly: float = 1.0, x0: float = 0.0,
                     y0: float = 0.0, jitter: float = 0.0, seed: int = 0,
                     tag: int = -1) -> Mesh:
    """Same triangulation as :func:`periodic_square` but with the outer sides
    as boundary sides tagged ``tag`` (-1 is the advection solver's exact
    Dirichlet boundary, 2dadvec_kernels.cu:492-517).  Boundary sides are sorted
    first, as the reference's mesh converter does (genmesh.py:244-284)."""
    m = periodic_square(n, lx, ly, x0, y0, jitter, seed)
    i = np.arange(n * n) % n
    j = np.arange(n * n) // n
    bottom = 3 * np.arange(n * n)
    left = bottom + 1
    re = m.right_elem.astype(np.int64).copy()
    rs = m.right_side.astype(np.int64).copy()
    re[bottom[j == 0]] = tag; rs[bottom[j == 0]] = -1
    re[left[i == 0]] = tag; rs[left[i == 0]] = -1
    # sides on the top and right boundary are owned (as left element) by the
    # elements at the top / right; they currently point across the periodic
    # seam, so rebuild them as boundary sides of the top/right elements.
    E = m.num_elem
    es = np.stack([m.elem_s1, m.elem_s2, m.elem_s3], axis=1).astype(np.int64)
    le = m.left_elem.astype(np.int64).copy()
    ls = m.left_side.astype(np.int64).copy()
    V = [a.copy() for a in m.vertices()]
    extra_le, extra_ls = [], []
    S0 = m.num_sides
    # top row upper triangles: local side 1 (NE->NW) was the bottom side of row 0
    for q in np.nonzero(j == n - 1)[0]:
        e = 2 * q + 1
        es[e, 1] = S0 + len(extra_le)
        extra_le.append(e); extra_ls.append(1)
    # right column lower triangles: local side 1 (SE->NE) was the left side of column 0
    for q in np.nonzero(i == n - 1)[0]:
        e = 2 * q
        es[e, 1] = S0 + len(extra_le)
        extra_le.append(e); extra_ls.append(1)
    le = np.concatenate([le, np.array(extra_le, dtype=np.int64)])
    ls = np.concatenate([ls, np.array(extra_ls, dtype=np.int64)])
    re = np.concatenate([re, np.full(len(extra_le), tag, dtype=np.int64)])
    rs = np.concatenate([rs, np.full(len(extra_le), -1, dtype=np.int64)])
    # boundary sides first (stable), then interior
    order = np.concatenate([np.nonzero(re < 0)[0], np.nonzero(re >= 0)[0]])
    inv = np.empty_like(order); inv[order] = np.arange(order.size)
    es = inv[es]
    out = Mesh(*V, es[:, 0], es[:, 1], es[:, 2], le[order], re[order], ls[order], rs[order],
               meta=dict(m.meta, kind="dirichlet_square", tag=tag))
    out.check()
    return out


def scramble(m: Mesh, seed: int = 0, rotate: bool = True, swap: bool = True,
             permute: bool = True) -> Mesh:
    """Return an equivalent mesh with shuffled element and side numbering,
    cyclically rotated vertex order and swapped left/right roles, so that
    every combination of local side numbers occurs (tests only)."""
    rng = np.random.default_rng(seed)
    E, S = m.num_elem, m.num_sides
    V = np.stack(m.vertices()).reshape(6, E)
    es = np.stack(m.elem_sides(), axis=1).astype(np.int64)
    le, re = m.left_elem.astype(np.int64).copy(), m.right_elem.astype(np.int64).copy()
    ls, rs = m.left_side.astype(np.int64).copy(), m.right_side.astype(np.int64).copy()
    if rotate:
        r = rng.integers(0, 3, size=E)
        P = V.reshape(3, 2, E)
        idx = (np.arange(3)[:, None] + r[None, :]) % 3           # new k <- old (k+r)
        P = np.take_along_axis(P, idx[:, None, :].repeat(2, axis=1), axis=0)
        V = P.reshape(6, E)
        es = np.take_along_axis(es, (np.arange(3)[None, :] + r[:, None]) % 3, axis=1)
        ls = (ls - r[le]) % 3
        inter = re >= 0
        rs[inter] = (rs[inter] - r[re[inter]]) % 3
    if swap:
        sw = (rng.random(S) < 0.5) & (re >= 0)
        le[sw], re[sw] = re[sw].copy(), le[sw].copy()
        ls[sw], rs[sw] = rs[sw].copy(), ls[sw].copy()
    if permute:
        pe = rng.permutation(E)          # new element index of old element
        ps = rng.permutation(S)          # new side index of old side
        inv_e = np.empty(E, dtype=np.int64); inv_e[pe] = np.arange(E)
        inv_s = np.empty(S, dtype=np.int64); inv_s[ps] = np.arange(S)
        V = V[:, inv_e]
        es = ps[es[inv_e]]
        le, ls = pe[le[inv_s]], ls[inv_s]
        re_old, rs = re[inv_s], rs[inv_s]
        re = np.where(re_old >= 0, pe[np.maximum(re_old, 0)], re_old)
    out = Mesh(*V, es[:, 0], es[:, 1], es[:, 2], le, re, ls, rs,
               meta=dict(m.meta, scrambled=seed))
    out.check()
    return out


# ---------------------------------------------------------------------------
# File formats
# ---------------------------------------------------------------------------

def _pmsh_text(E, S, V, es, side_xy, le, re, ls, rs, fixed6: bool) -> str:
    """The .pmsh text (src/2d/genmesh.py:290-308): E, then per element its six
    vertex coordinates and three side indices; S, then per side its two end
    points, left and right element and side numbers.  fixed6 writes the
    coordinates as the reference's converter does ("%lf": six decimals,
    correctly rounded), else full precision (shortest round-trip form)."""
    num = (lambda x: "%f" % x) if fixed6 else (lambda x: repr(float(x)))
    out = [f"{E}"]
    for e in range(E):
        out.append(" ".join(num(x) for x in V[:, e]) + f" {es[0, e]} {es[1, e]} {es[2, e]}")
    out.append(f"{S}")
    for s in range(S):
        out.append(" ".join(num(x) for x in side_xy[:, s]) + f" {le[s]} {re[s]} {ls[s]} {rs[s]}")
    return "\n".join(out) + "\n"


def write_pmsh(mesh: Mesh, path: str, fixed6: bool = False) -> None:
    """Write the reference's .pmsh text format (src/2d/genmesh.py:290-308); side
    end points are the left element's.  Coordinates at full precision, or with
    fixed6 at the reference converter's six decimals ("%lf")."""
    E, S = mesh.num_elem, mesh.num_sides
    V = np.stack(mesh.vertices())
    es = np.stack(mesh.elem_sides())
    P = V.reshape(3, 2, E)
    le, ls = mesh.left_elem.astype(np.int64), mesh.left_side.astype(np.int64)
    side_xy = np.concatenate([P[ls, :, le].T, P[(ls + 1) % 3, :, le].T]) if S else np.zeros((4, 0))
    with open(path, "w") as f:
        f.write(_pmsh_text(E, S, V, es, side_xy, mesh.left_elem, mesh.right_elem, mesh.left_side,
                           mesh.right_side, fixed6))


def read_pmsh(path: str) -> Mesh:
    """Read a .pmsh file (the reference's read_mesh, src/2d/conservation/conserv.cu:118-192)."""
    with open(path) as f:
        lines = [ln for ln in f.read().splitlines() if ln.strip()]
    E = int(lines[0].split()[0])
    el = np.array([ln.split()[:9] for ln in lines[1:1 + E]], dtype=np.float64)
    S = int(lines[1 + E].split()[0])
    sd = np.array([ln.split()[:8] for ln in lines[2 + E:2 + E + S]], dtype=np.float64)
    return Mesh(*el[:, :6].T, *el[:, 6:9].T.astype(np.int64), *sd[:, 4:8].T.astype(np.int64),
                meta=dict(kind="pmsh", path=path))


BOUNDARY_TAGS = {10000: -1, 20000: -2, 30000: -3}   # physical tags of genmesh.py:170-180


def _parse_gmsh(path_or_text: str):
    """Gmsh v2.2 ASCII: node coordinates (n, 2), triangles as node-index triples
    and lines as (node pair, physical tag), both in file order.  Nodes are
    addressed by their file order; element lines are read by type and tag
    count (the reference's converter reads lines of 7 and 8 fields, the same
    elements for the two-tag files Gmsh writes, src/2d/genmesh.py:36-58)."""
    text = path_or_text
    if "\n" not in path_or_text:
        with open(path_or_text) as f:
            text = f.read()
    lines = [ln.strip() for ln in text.splitlines()]
    if "$Nodes" not in lines:
        raise ValueError("not a Gmsh v2 file (no $Nodes section)")
    i = lines.index("$Nodes")
    n_nodes = int(lines[i + 1])
    node_id, xy = {}, []
    for k in range(n_nodes):
        parts = lines[i + 2 + k].split()
        node_id[int(parts[0])] = k
        xy.append((float(parts[1]), float(parts[2])))
    i = lines.index("$Elements")
    n_el = int(lines[i + 1])
    tris, segs = [], []
    for k in range(n_el):
        parts = [int(x) for x in lines[i + 2 + k].split()]
        etype, ntags = parts[1], parts[2]
        phys = parts[3] if ntags > 0 else 0
        nodes = [node_id[x] for x in parts[3 + ntags:]]
        if etype == 2:
            tris.append(tuple(nodes[:3]))
        elif etype == 1:
            segs.append(((nodes[0], nodes[1]), phys))
    return np.array(xy, dtype=np.float64).reshape(-1, 2), tris, segs


def _number_sides(tris, tag_of, unmatched):
    """Sides of a triangulation in the reference converter's numbering
    (src/2d/genmesh.py:84-241).  Elements are visited in order; a side of
    element i that an earlier element created (its vertex pair in either
    direction) gets i as its right element and k as its right side number;
    then each of the element's new sides k = 0, 1, 2 (V1V2, V2V3, V3V1) is
    appended with i as its left element.  tag_of(a, b) is the boundary tag of a
    new side (or None); a side that no second element meets and that has no
    tag gets `unmatched` as its right element.  Returns es[E][3], le, re, ls,
    rs (lists)."""
    E = len(tris)
    es = [[0, 0, 0] for _ in range(E)]
    le, re, ls, rs = [], [], [], []
    created = {}
    for i, t in enumerate(tris):
        edges = ((t[0], t[1]), (t[1], t[2]), (t[2], t[0]))
        new = [True, True, True]
        for k, (a, b) in enumerate(edges):
            for key in ((a, b), (b, a)):
                q = created.get(key)
                if q is not None:
                    new[k] = False
                    re[q], rs[q], es[i][k] = i, k, q
        for k, (a, b) in enumerate(edges):
            if new[k]:
                q = len(le)
                created[(a, b)] = q
                tag = tag_of(a, b)
                le.append(i); ls.append(k); re.append(unmatched if tag is None else tag); rs.append(0)
                es[i][k] = q
    return es, le, re, ls, rs


def _boundary_first(es, le, re, ls, rs, order=(-1, -2, -3)):
    """Move the boundary sides to the front, all of tag -1, then -2, then -3,
    by the reference converter's exchanges (src/2d/genmesh.py:244-284): a
    running slot j starts at 0; for each side i with the tag (in index order)
    the sides at i and j trade places -- the elements of the side at j are
    pointed at i, the left element of the side at i at j -- and j advances.
    The reference also points "the right element" of the side at j at i when
    that side is a boundary side, which Python's negative indexing turns into
    a write into the side lists of the mesh's last elements; that write is
    left out here (on every .msh/.pmsh pair the reference ships, later
    exchanges overwrite those entries and the files agree byte for byte).
    Modifies the lists in place."""
    j = 0
    for tag in order:
        for i in range(len(le)):
            if re[i] != tag:
                continue
            es[le[j]][ls[j]] = i
            if re[j] >= 0:
                es[re[j]][rs[j]] = i
            es[le[i]][ls[i]] = j
            for arr in (le, re, ls, rs):
                arr[i], arr[j] = arr[j], arr[i]
            j += 1


def _tagger(segs, tags):
    """tag_of(a, b) for the sides of a triangulation: the tag of the physical
    group of a line element on the side (either direction), the last such
    line with a known group winning (genmesh.py:170-180); None without one."""
    on_side = {}
    for (a, b), phys in segs:
        if phys in tags:
            on_side[(a, b)] = on_side[(b, a)] = tags[phys]
    return lambda a, b: on_side.get((a, b))


def read_gmsh(path_or_text: str, boundary_tags=None) -> Mesh:
    """Gmsh v2.2 ASCII .msh -> Mesh, the job of the reference's Python-2
    converter (src/2d/genmesh.py:11-310) restated for Python 3, for solving.
    Triangles become elements in file order; sides are numbered as the
    reference numbers them (``_number_sides``) and its boundary sides sorted
    first, -1, -2, -3, by its exchanges (``_boundary_first``); line elements
    tag boundary sides by their physical group (10000 reflecting -> -1, 20000
    outflow -> -2, 30000 inflow -> -3).  For counter-clockwise triangles and
    tagged boundaries the arrays equal those of the reference's .pmsh (see
    ``gmsh_to_pmsh``) at full precision.  Two cases differ, where the
    reference's file would not be a valid mesh: a clockwise triangle has its
    first two vertices exchanged in that element only (the reference exchanges
    the two vertices' coordinates for the whole mesh), and a boundary side
    without a known tag becomes reflecting (-1) (the reference leaves element 0
    as its right element)."""
    tags = dict(BOUNDARY_TAGS if boundary_tags is None else boundary_tags)
    xy, tris, segs = _parse_gmsh(path_or_text)
    ccw = []
    for a, b, c in tris:
        J = (xy[b, 0] - xy[a, 0]) * (xy[c, 1] - xy[a, 1]) - (xy[c, 0] - xy[a, 0]) * (xy[b, 1] - xy[a, 1])
        ccw.append((b, a, c) if J < 0 else (a, b, c))
    tag_of = _tagger(segs, tags)
    return from_triangles(xy, ccw, lambda a, b: tag_of(a, b) or -1, kind="gmsh")


def gmsh_to_pmsh(msh_path_or_text: str, pmsh_path: str | None = None, boundary_tags=None) -> str:
    """The reference's mesh converter (src/2d/genmesh.py:11-310, Python 2) as a
    Python 3 function: Gmsh v2.2 .msh -> the .pmsh text its solvers read,
    byte for byte what the reference's converter writes, written to pmsh_path
    when given and returned.  Kept alike on purpose, for files that must
    match the reference's: the six-decimal coordinates ("%lf"); a triangle
    with a negative Jacobian (computed from the coordinates as they stand when
    it is visited) exchanges the coordinates of its first two vertices in the
    shared vertex list, which moves them for every element that uses them
    (genmesh.py:95-100); a side that no second element meets and no tagged line
    lies on keeps element 0 and side 0 as its right neighbour (genmesh.py:
    69-75).  ``read_gmsh`` gives the solvable mesh instead."""
    tags = dict(BOUNDARY_TAGS if boundary_tags is None else boundary_tags)
    xy, tris, segs = _parse_gmsh(msh_path_or_text)
    xy = xy.copy()
    for a, b, c in tris:
        J = (xy[b, 0] - xy[a, 0]) * (xy[c, 1] - xy[a, 1]) - (xy[c, 0] - xy[a, 0]) * (xy[b, 1] - xy[a, 1])
        if J < 0:
            xy[[a, b]] = xy[[b, a]]
    es, le, re, ls, rs = _number_sides(tris, _tagger(segs, tags), unmatched=0)
    _boundary_first(es, le, re, ls, rs)
    T = np.array(tris, dtype=np.int64).reshape(-1, 3)
    E, S = T.shape[0], len(le)
    V = np.stack([xy[T[:, 0], 0], xy[T[:, 0], 1], xy[T[:, 1], 0], xy[T[:, 1], 1],
                  xy[T[:, 2], 0], xy[T[:, 2], 1]]) if E else np.zeros((6, 0))
    ends = [(T[le[s], ls[s]], T[le[s], (ls[s] + 1) % 3]) for s in range(S)]
    side_xy = np.array([[xy[a, 0], xy[a, 1], xy[b, 0], xy[b, 1]] for a, b in ends]).T.reshape(4, S)
    text = _pmsh_text(E, S, V, np.array(es, dtype=np.int64).reshape(-1, 3).T, side_xy, le, re, ls, rs,
                      fixed6=True)
    if pmsh_path:
        with open(pmsh_path, "w") as f:
            f.write(text)
    return text


def tag_boundary(mesh: Mesh, fn) -> Mesh:
    """Re-tag boundary sides by position: fn(x_mid, y_mid) -> tag in {-1, -2, -3}
    for each boundary side's midpoint.  Returns a new Mesh."""
    V = np.stack(mesh.vertices()).reshape(3, 2, -1)
    re = mesh.right_elem.astype(np.int64).copy()
    for s in np.nonzero(re < 0)[0]:
        L, ls = mesh.left_elem[s], mesh.left_side[s]
        a, b = V[ls, :, L], V[(ls + 1) % 3, :, L]
        re[s] = int(fn(0.5 * (a[0] + b[0]), 0.5 * (a[1] + b[1])))
    return Mesh(*mesh.vertices(), *mesh.elem_sides(), mesh.left_elem, re, mesh.left_side,
                mesh.right_side, meta=dict(mesh.meta, tagged=True))


def from_triangles(xy, tris, boundary_tag, kind: str = "triangles") -> Mesh:
    """Vertices ``xy[n, 2]`` and counter-clockwise triangles ``tris[E, 3]`` (vertex
    indices) -> Mesh, with the sides numbered as the reference's converter
    numbers them (``_number_sides``: matched by their vertex pair, the first
    element to meet a side is its left element).  A side that no second
    element meets is a boundary side tagged ``boundary_tag(a, b)`` (its vertex
    indices, in the left element's order), with right side number 0 as in the
    reference's files.  Boundary sides come first, -1, -2, -3, moved there by
    the reference's exchanges (``_boundary_first``, genmesh.py:244-284)."""
    xy = np.asarray(xy, dtype=np.float64)
    T = np.asarray(tris, dtype=np.int64).reshape(-1, 3)
    open_side = -(1 << 30)
    es, le, re, ls, rs = _number_sides([tuple(int(v) for v in t) for t in T], lambda a, b: None, open_side)
    for q in range(len(le)):
        if re[q] == open_side:   # sides met once: boundary sides
            tag = int(boundary_tag(int(T[le[q], ls[q]]), int(T[le[q], (ls[q] + 1) % 3])))
            if tag not in (-1, -2, -3):
                raise ValueError("boundary tags must be -1, -2 or -3")
            re[q] = tag
    _boundary_first(es, le, re, ls, rs)
    es = np.array(es, dtype=np.int64).reshape(-1, 3)
    V = [xy[T[:, 0], 0], xy[T[:, 0], 1], xy[T[:, 1], 0], xy[T[:, 1], 1], xy[T[:, 2], 0], xy[T[:, 2], 1]]
    m = Mesh(*V, es[:, 0], es[:, 1], es[:, 2], le, re, ls, rs, meta=dict(kind=kind))
    m.check()
    return m


def annulus(nr: int, nt: int, r0: float, r1: float, theta0: float = 0.0,
            theta1: float = 2.0 * np.pi, cx: float = 0.0, cy: float = 0.0,
            tag=None) -> Mesh:
    """Structured triangulation of the ring sector r0 <= r <= r1,
    theta0 <= theta <= theta1 about (cx, cy): nr x nt cells, each split into
    two counter-clockwise triangles.  A full ring (theta1 - theta0 = 2 pi)
    closes on itself.  ``tag(x_mid, y_mid, where)`` gives each boundary side's
    tag, ``where`` one of "inner", "outer", "start", "end"; the default tags
    the arcs -1 (reflecting walls), the start ray -3 (inflow) and the end ray -2
    (outflow).  The meshes of the reference's cylinder and supersonic-vortex
    problems are of this kind."""
    full = abs((theta1 - theta0) - 2.0 * np.pi) < 1e-12
    ntv = nt if full else nt + 1
    r = np.linspace(r0, r1, nr + 1)
    th = theta0 + (theta1 - theta0) * np.arange(ntv) / nt
    R, TH = np.meshgrid(r, th, indexing="ij")
    xy = np.stack([cx + R * np.cos(TH), cy + R * np.sin(TH)], axis=-1).reshape(-1, 2)

    def vid(i, j):
        return i * ntv + (j % ntv if full else j)

    tris = []
    for i in range(nr):
        for j in range(nt):
            a, b, c, d = vid(i, j), vid(i + 1, j), vid(i + 1, j + 1), vid(i, j + 1)
            tris.append((a, b, c))
            tris.append((a, c, d))
    tris = np.array(tris)
    J = ((xy[tris[:, 1], 0] - xy[tris[:, 0], 0]) * (xy[tris[:, 2], 1] - xy[tris[:, 0], 1])
         - (xy[tris[:, 2], 0] - xy[tris[:, 0], 0]) * (xy[tris[:, 1], 1] - xy[tris[:, 0], 1]))
    flip = J < 0
    tris[flip] = tris[flip][:, [0, 2, 1]]

    def where(a, b):
        ia, ja = divmod(a, ntv)
        ib, jb = divmod(b, ntv)
        if ia == ib == 0:
            return "inner"
        if ia == ib == nr:
            return "outer"
        return "start" if ja == jb == 0 else "end"

    default = {"inner": -1, "outer": -1, "start": -3, "end": -2}

    def btag(a, b):
        w = where(a, b)
        if tag is None:
            return default[w]
        xm, ym = 0.5 * (xy[a] + xy[b])
        return tag(xm, ym, w)

    m = from_triangles(xy, tris, btag, kind="annulus")
    m.meta.update(nr=nr, nt=nt, r0=r0, r1=r1, theta0=theta0, theta1=theta1, cx=cx, cy=cy)
    return m
