"""Deterministic structured quadrilateral meshes of a rectangle, and an SU2 writer.

The meshes use the reference's local node order for each element type:

* bilinear (SU2/VTK type 9): 0:(-1,-1) 1:(1,-1) 2:(1,1) 3:(-1,1)
  (libraries/metamath/finite_elements/finite_elements_2d/element/basis/serendipity_2d.hpp:155-164)
* 8-node serendipity (type 23): 0:(-1,-1) 1:(0,-1) 2:(1,-1) 3:(1,0) 4:(1,1)
  5:(0,1) 6:(-1,1) 7:(-1,0)  (serendipity_2d.hpp:192-207)

Boundary edges are 2-node (type 3) or 3-node (type 21, local order end, middle,
end) line elements in four groups named ``left``, ``right``, ``down``, ``up``.

The SU2 writer emits the file order that the reference parser maps back to the
local order (libraries/mesh/mesh_2d/su2_parser.hpp:57-66): corners first, then
mid-sides for type 23; both ends, then the middle node for type 21.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

BILINEAR = "bilinear"
SERENDIPITY = "serendipity"

_SU2_TYPE_2D = {BILINEAR: 9, SERENDIPITY: 23}
_SU2_TYPE_1D = {BILINEAR: 3, SERENDIPITY: 21}
# local index of each SU2 file position (inverse of su2_parser.hpp:63-66)
_FILE_ORDER_2D = {BILINEAR: [0, 1, 2, 3], SERENDIPITY: [0, 2, 4, 6, 1, 3, 5, 7]}
_FILE_ORDER_1D = {BILINEAR: [0, 1], SERENDIPITY: [0, 2, 1]}


@dataclass
class QuadMesh:
    """Nodes, 2D elements and boundary line elements of a quadrilateral mesh."""

    element: str
    nodes: np.ndarray                 # (n_nodes, 2) float64
    elements: np.ndarray              # (n_elements, nen) int64, local node order
    boundaries: dict[str, np.ndarray] = field(default_factory=dict)  # name -> (n_edges, 2|3)

    @property
    def nodes_per_element(self) -> int:
        return int(self.elements.shape[1])

    @property
    def n_nodes(self) -> int:
        return int(self.nodes.shape[0])

    @property
    def n_elements(self) -> int:
        return int(self.elements.shape[0])


def relabel_nodes(mesh: QuadMesh, new_of_old: np.ndarray) -> QuadMesh:
    """The same mesh with node i renamed new_of_old[i] (element and edge order kept)."""
    p = np.asarray(new_of_old, dtype=np.int64)
    nodes = np.empty_like(mesh.nodes)
    nodes[p] = mesh.nodes
    return QuadMesh(mesh.element, nodes, p[mesh.elements], {k: p[v] for k, v in mesh.boundaries.items()})


def structured_quad_mesh(nx: int, ny: int, element: str = BILINEAR, *, width: float = 1.0,
                         height: float = 1.0, jitter: float = 0.0, seed: int = 0,
                         shuffle_seed: int | None = None) -> QuadMesh:
    """Uniform nx-by-ny quadrilateral mesh of [0,width]x[0,height].

    ``jitter`` moves every interior corner node by U(-jitter*h, +jitter*h) in
    each direction (numpy ``default_rng(seed)``); mid-side nodes of 8-node
    elements are then put back at the midpoints of their edges.  With
    ``shuffle_seed`` the nodes are numbered by a random permutation
    (``default_rng(shuffle_seed)``) instead of row by row, as an unstructured
    mesher might number them.
    """
    if shuffle_seed is not None:
        m = structured_quad_mesh(nx, ny, element, width=width, height=height, jitter=jitter, seed=seed)
        return relabel_nodes(m, np.random.default_rng(shuffle_seed).permutation(m.n_nodes))
    if element not in (BILINEAR, SERENDIPITY):
        raise ValueError(f"unknown element type {element!r}")
    hx, hy = width / nx, height / ny
    rng = np.random.default_rng(seed)
    cx = np.linspace(0.0, width, nx + 1)
    cy = np.linspace(0.0, height, ny + 1)
    corner_x, corner_y = np.meshgrid(cx, cy)          # (ny+1, nx+1)
    if jitter > 0.0:
        dx = rng.uniform(-jitter * hx, jitter * hx, size=corner_x.shape)
        dy = rng.uniform(-jitter * hy, jitter * hy, size=corner_y.shape)
        interior = np.zeros(corner_x.shape, dtype=bool)
        interior[1:-1, 1:-1] = True
        corner_x = np.where(interior, corner_x + dx, corner_x)
        corner_y = np.where(interior, corner_y + dy, corner_y)

    if element == BILINEAR:
        nodes = np.stack([corner_x.ravel(), corner_y.ravel()], axis=1)
        nid = np.arange((nx + 1) * (ny + 1)).reshape(ny + 1, nx + 1)
        el = np.stack([nid[:-1, :-1], nid[:-1, 1:], nid[1:, 1:], nid[1:, :-1]], axis=-1).reshape(-1, 4)
        bnd = {
            "down": np.stack([nid[0, :-1], nid[0, 1:]], axis=1),
            "right": np.stack([nid[:-1, -1], nid[1:, -1]], axis=1),
            "up": np.stack([nid[-1, 1:], nid[-1, :-1]], axis=1),
            "left": np.stack([nid[1:, 0], nid[:-1, 0]], axis=1),
        }
        return QuadMesh(element, nodes, el.astype(np.int64), {k: v.astype(np.int64) for k, v in bnd.items()})

    # 8-node serendipity: points of the (2nx+1) x (2ny+1) grid without cell centres.
    na, nb = 2 * nx + 1, 2 * ny + 1
    gid = -np.ones((nb, na), dtype=np.int64)
    keep = ~((np.arange(nb)[:, None] % 2 == 1) & (np.arange(na)[None, :] % 2 == 1))
    gid[keep] = np.arange(int(keep.sum()))
    gx = np.zeros((nb, na))
    gy = np.zeros((nb, na))
    gx[0::2, 0::2], gy[0::2, 0::2] = corner_x, corner_y
    gx[0::2, 1::2] = 0.5 * (corner_x[:, :-1] + corner_x[:, 1:])   # horizontal edge midpoints
    gy[0::2, 1::2] = 0.5 * (corner_y[:, :-1] + corner_y[:, 1:])
    gx[1::2, 0::2] = 0.5 * (corner_x[:-1, :] + corner_x[1:, :])   # vertical edge midpoints
    gy[1::2, 0::2] = 0.5 * (corner_y[:-1, :] + corner_y[1:, :])
    nodes = np.stack([gx[keep], gy[keep]], axis=1)
    a = 2 * np.arange(nx)[None, :]
    b = 2 * np.arange(ny)[:, None]
    el = np.stack([gid[b, a], gid[b, a + 1], gid[b, a + 2], gid[b + 1, a + 2],
                   gid[b + 2, a + 2], gid[b + 2, a + 1], gid[b + 2, a], gid[b + 1, a]], axis=-1).reshape(-1, 8)
    i = 2 * np.arange(nx)
    j = 2 * np.arange(ny)
    bnd = {
        "down": np.stack([gid[0, i], gid[0, i + 1], gid[0, i + 2]], axis=1),
        "right": np.stack([gid[j, -1], gid[j + 1, -1], gid[j + 2, -1]], axis=1),
        "up": np.stack([gid[-1, i + 2], gid[-1, i + 1], gid[-1, i]], axis=1),
        "left": np.stack([gid[j + 2, 0], gid[j + 1, 0], gid[j, 0]], axis=1),
    }
    return QuadMesh(element, nodes, el.astype(np.int64), {k: v.astype(np.int64) for k, v in bnd.items()})


def write_su2(mesh: QuadMesh, path: str, groups_2d: dict[str, list[int]] | None = None) -> None:
    """Write ``mesh`` as an SU2 text file the reference parser reads back.

    ``groups_2d`` adds markers of 2D elements (name -> element indices); the
    reference puts the 2D elements no marker names into its default group.
    """
    t2 = _SU2_TYPE_2D[mesh.element]
    t1 = _SU2_TYPE_1D[mesh.element]
    o2 = _FILE_ORDER_2D[mesh.element]
    o1 = _FILE_ORDER_1D[mesh.element]
    groups_2d = groups_2d or {}

    def element_line(e):
        return f"{t2} " + " ".join(str(int(e[i])) for i in o2)

    lines = ["NDIME= 2", f"NELEM= {mesh.n_elements}"]
    for k, e in enumerate(mesh.elements):
        lines.append(element_line(e) + f" {k}")
    lines.append(f"NPOIN= {mesh.n_nodes}")
    for k, (x, y) in enumerate(mesh.nodes):
        lines.append(f"{float(x)!r} {float(y)!r} {k}")
    lines.append(f"NMARK= {len(mesh.boundaries) + len(groups_2d)}")
    for name, edges in mesh.boundaries.items():
        lines.append(f"MARKER_TAG= {name}")
        lines.append(f"MARKER_ELEMS= {len(edges)}")
        for e in edges:
            lines.append(f"{t1} " + " ".join(str(int(e[i])) for i in o1))
    for name, members in groups_2d.items():
        lines.append(f"MARKER_TAG= {name}")
        lines.append(f"MARKER_ELEMS= {len(members)}")
        for k in members:
            lines.append(element_line(mesh.elements[k]))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def read_su2(path: str) -> QuadMesh:
    """Read an SU2 file of one quadrilateral element type (file order of elements kept)."""
    with open(path) as f:
        tokens = [ln.split() for ln in f if ln.strip()]
    pos = 0

    def take():
        nonlocal pos
        pos += 1
        return tokens[pos - 1]

    take()                                           # NDIME= 2
    n_el = int(take()[1])
    rows = [take() for _ in range(n_el)]
    types = {int(r[0]) for r in rows}
    if types == {9}:
        element = BILINEAR
    elif types == {23}:
        element = SERENDIPITY
    else:
        raise ValueError(f"unsupported element types {sorted(types)}")
    o2 = _FILE_ORDER_2D[element]
    els = np.zeros((n_el, len(o2)), dtype=np.int64)
    for k, r in enumerate(rows):
        vals = [int(v) for v in r[1:1 + len(o2)]]
        for fpos, local in enumerate(o2):
            els[k, local] = vals[fpos]
    n_nodes = int(take()[1])
    nodes = np.array([[float(v) for v in take()[:2]] for _ in range(n_nodes)])
    bnd = {}
    n_mark = int(take()[1]) if pos < len(tokens) else 0
    o1 = _FILE_ORDER_1D[element]
    for _ in range(n_mark):
        name = take()[1]
        cnt = int(take()[1])
        edges = np.zeros((cnt, len(o1)), dtype=np.int64)
        for k in range(cnt):
            vals = [int(v) for v in take()[1:1 + len(o1)]]
            for fpos, local in enumerate(o1):
                edges[k, local] = vals[fpos]
        bnd[name] = edges
    return QuadMesh(element, nodes, els, bnd)
