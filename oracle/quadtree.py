"""ORACLE — test infrastructure only.

NumPy restatement of the quadtree mesh generation of the reference:
  * MeshSetUp.m (func/MeshSetUp.m): the uniform mesh of the search grid;
  * funMarkEdge.m / funMarkInside.m (func_quadtree/): the mask tests over
    each element's bounding box;
  * QrefineR.m + provideGeometricData.m (func_quadtree/refinement/): red
    refinement of the marked quadrilaterals with the one-hanging-node-per-edge
    closure, new nodes numbered in the order of the sorted edge list;
  * GenerateQuadtreeMesh.m:18-133: refinement until no element is marked,
    corner reordering, the hanging-node columns 5-8, removal of the elements
    inside the mask, and the Dirichlet set markCoordHoleEdge.
Indices are 1-based like MATLAB's; coordinates are (N, 2), elements (E, 4) or
(E, 8), irregular (nI, 3) = [node_a node_b midnode].  Only the tests use this
module, as the checker of the library's mesh generation; the product never
imports it.
"""
import numpy as np


def mesh_setup(x0, y0):
    """MeshSetUp.m: x0, y0 are the N x M grids of the search as MeshSetUp
    receives them (row = y; the DICmesh.x0 it stores is the transpose).
    Returns coordinatesFEM (M N x 2) and elementsFEM ((M-1)(N-1) x 4)."""
    x0 = np.asarray(x0, dtype=np.float64)
    y0 = np.asarray(y0, dtype=np.float64)
    N, M = x0.shape
    xt, yt = x0.T, y0.T
    coords = np.stack([xt.ravel(order="F"), yt.ravel(order="F")], 1)
    els = []
    for j in range(1, N):
        for i in range(1, M):
            els.append([(j - 1) * M + i, (j - 1) * M + i + 1, j * M + i + 1, j * M + i])
    return coords, np.asarray(els, dtype=np.int64).reshape(-1, 4)


def _boxes(coords, elems4):
    c = coords[elems4[:, :4] - 1]  # E x 4 x 2
    return (c[:, :, 0].min(1), c[:, :, 0].max(1), c[:, :, 1].min(1), c[:, :, 1].max(1))


def mark_edge(coords, elems4, mask, element_min_size):
    """funMarkEdge.m: elements whose bounding box holds both mask values and
    whose smaller side exceeds elementMinSize."""
    if elems4.shape[0] == 0:
        return np.zeros(0, dtype=bool)
    x0, x1, y0, y1 = _boxes(coords, elems4)
    out = np.zeros(elems4.shape[0], dtype=bool)
    for e in range(elems4.shape[0]):
        box = mask[int(x0[e]) - 1:int(x1[e]), int(y0[e]) - 1:int(y1[e])]
        rng = float(box.max()) - float(box.min())
        size = min(abs(x1[e] - x0[e]), abs(y1[e] - y0[e]))
        out[e] = rng > 0 and size > element_min_size
    return out


def mark_outside(coords, elems4, mask):
    """funMarkInside.m: indices (0-based) of the elements kept, those whose
    box holds at least half of (xmax - xmin)(ymax - ymin) mask ones."""
    if elems4.shape[0] == 0:
        return np.zeros(0, dtype=np.int64)
    x0, x1, y0, y1 = _boxes(coords, elems4)
    keep = []
    for e in range(elems4.shape[0]):
        s = float(mask[int(x0[e]) - 1:int(x1[e]), int(y0[e]) - 1:int(y1[e])].sum())
        if not (s < 0.5 * (x1[e] - x0[e]) * (y1[e] - y0[e])):
            keep.append(e)
    return np.asarray(keep, dtype=np.int64)


def geometric_data(irregular, elems4):
    """provideGeometricData.m with the irregular list as its 'triangles':
    the sorted unique edge list and each row's edges (0-based edge ids)."""
    nI, nE = irregular.shape[0], elems4.shape[0]
    e3 = [np.stack([irregular[:, k], irregular[:, (k + 1) % 3]], 1) for k in range(3)]
    e4 = [np.stack([elems4[:, k], elems4[:, (k + 1) % 4]], 1) for k in range(4)]
    edges = np.concatenate(e3 + e4, 0) if (nI + nE) else np.zeros((0, 2), np.int64)
    edges = np.sort(edges, 1)
    edge2nodes, ie = np.unique(edges, axis=0, return_inverse=True)
    ie = ie.ravel()
    irr2edges = ie[:3 * nI].reshape(3, nI).T if nI else np.zeros((0, 3), np.int64)
    el2edges = ie[3 * nI:].reshape(4, nE).T
    return edge2nodes, irr2edges, el2edges


def qrefine_r(coords, elems4, irregular, marked):
    """QrefineR.m: red refinement of the marked elements (0-based indices)
    with the closure that keeps at most one hanging node per edge."""
    coords = np.array(coords, dtype=np.float64)
    nE = elems4.shape[0]
    edge2nodes, irr2edges, el2edges = geometric_data(irregular, elems4)
    e2n = np.zeros(edge2nodes.shape[0], dtype=np.int64)
    if len(marked):
        e2n[el2edges[marked].ravel()] = 1
    if irregular.shape[0]:
        e2n[irr2edges[:, 0]] = 1
    while True:
        me = e2n[el2edges]
        s = np.abs(me).sum(1)
        kdx = np.nonzero((s < 4) & ((s > 2) | (me.min(1) < 0)))[0]
        if kdx.size:
            sub = el2edges[kdx]
            e2n[sub[me[kdx] == 0]] = 1
        if irregular.shape[0]:
            mi = e2n[irr2edges]
            flag = irr2edges[np.any(mi[:, 1:] != 0, 1), 0]
            swap = flag[e2n[flag] != -1]
            e2n[swap] = -1
        else:
            swap = np.zeros(0, np.int64)
        if kdx.size == 0 and swap.size == 0:
            break
    if irregular.shape[0]:
        e2n[irr2edges[:, 0]] = -1
    idx = e2n > 0
    nC = coords.shape[0]
    e2n[idx] = nC + np.arange(1, int(idx.sum()) + 1)
    newc = 0.5 * (coords[edge2nodes[idx, 0] - 1] + coords[edge2nodes[idx, 1] - 1])
    coords = np.concatenate([coords, newc], 0)
    if irregular.shape[0]:
        e2n[irr2edges[:, 0]] = irregular[:, 2]
    newNodes = e2n[el2edges]  # nE x 4
    reftyp = (newNodes != 0).astype(np.int64) @ np.array([1, 2, 4, 8])
    none = reftyp < 15
    red = np.nonzero(reftyp == 15)[0]
    mid = np.zeros(nE, dtype=np.int64)
    mid[red] = coords.shape[0] + np.arange(1, red.size + 1)
    cen = 0.25 * (coords[elems4[red, 0] - 1] + coords[elems4[red, 1] - 1] + coords[elems4[red, 2] - 1]
                  + coords[elems4[red, 3] - 1])
    coords = np.concatenate([coords, cen], 0)
    cnt = np.where(none, 1, 4)
    start = np.concatenate([[0], np.cumsum(cnt)])[:-1]
    newEl = np.zeros((int(cnt.sum()), 4), dtype=np.int64)
    newEl[start[none]] = elems4[none]
    e, n = elems4[red], newNodes[red]
    m = mid[red]
    newEl[start[red]] = np.stack([e[:, 0], n[:, 0], m, n[:, 3]], 1)
    newEl[start[red] + 1] = np.stack([e[:, 1], n[:, 1], m, n[:, 0]], 1)
    newEl[start[red] + 2] = np.stack([e[:, 2], n[:, 2], m, n[:, 1]], 1)
    newEl[start[red] + 3] = np.stack([e[:, 3], n[:, 3], m, n[:, 2]], 1)
    # hanging nodes of the elements kept whole, edge by edge (MATLAB's
    # column-major find over newNodes(kdx, :))
    rows = []
    kdx = np.nonzero((reftyp > 0) & (reftyp < 15))[0]
    for j in range(4):
        for k in kdx:
            if newNodes[k, j] != 0:
                ed = el2edges[k, j]
                rows.append([edge2nodes[ed, 0], edge2nodes[ed, 1], newNodes[k, j]])
    if irregular.shape[0]:
        nn = e2n[irr2edges[:, 1:3]]
        kd = np.nonzero(nn.sum(1) != 0)[0]
        for j in range(2):
            for k in kd:
                if nn[k, j] != 0:
                    ed = irr2edges[k, 1 + j]
                    rows.append([edge2nodes[ed, 0], edge2nodes[ed, 1], nn[k, j]])
    newIrr = np.asarray(rows, dtype=np.int64).reshape(-1, 3)
    return coords, newEl, newIrr


def _reorder_corners(coords, els):
    """GenerateQuadtreeMesh.m:45-54: each element's corners from the one at
    (min x, min y), by (x - xmin)^2 + 2 (y - ymin)^2 with the order [1 2 4 3]
    of that ranking (MATLAB's stable sort)."""
    out = els.copy()
    for k in range(els.shape[0]):
        c = coords[els[k, :4] - 1]
        xs, ys = np.sort(c[:, 0]), np.sort(c[:, 1])
        t = (c[:, 0] - xs[0]) ** 2 + 2 * (c[:, 1] - ys[0]) ** 2
        r = np.argsort(t, kind="stable")
        out[k, :4] = els[k, r[[0, 1, 3, 2]]]
    return out


def _hanging_columns(els4, irregular):
    """GenerateQuadtreeMesh.m:57-75: the midnode of each irregular edge goes
    into column 5 (edge 2-3), 6 (3-4), 7 (4-1) or 8 (1-2) of the first element
    holding that edge, in either orientation, in the reference's order of
    checks."""
    E = els4.shape[0]
    out = np.zeros((E, 8), dtype=np.int64)
    out[:, :4] = els4[:, :4]
    checks = (((0, 1), 7), ((1, 2), 4), ((2, 3), 5), ((3, 0), 6), ((1, 0), 7), ((2, 1), 4), ((3, 2), 5),
              ((0, 3), 6))
    # ismember(..., 'rows') returns the first element whose columns (a, b)
    # hold (n1, n2): one first-occurrence table per column pair
    first = {}
    for (a, b), _ in checks:
        t = {}
        for k in range(E):
            t.setdefault((int(els4[k, a]), int(els4[k, b])), k)
        first[(a, b)] = t
    for n1, n2, m in irregular:
        for (a, b), col in checks:
            hit = first[(a, b)].get((int(n1), int(n2)), -1)
            if hit >= 0:
                out[hit, col] = m
    return out


def generate_quadtree_mesh(x0, y0, mask, winstepsize, element_min_size):
    """GenerateQuadtreeMesh.m:18-133 (without its plots and the U0 RBF
    interpolation onto the new nodes).  Returns coordinatesFEM (N x 2),
    elementsFEM (E x 8), irregular (nI x 3) and markCoordHoleEdge (sorted,
    1-based), all as the reference builds them."""
    mask = np.asarray(mask)
    coords0, els0 = mesh_setup(x0, y0)
    coords, els = coords0.copy(), els0.copy()
    irregular = np.zeros((0, 3), dtype=np.int64)
    while True:
        marked = np.nonzero(mark_edge(coords, els, mask, element_min_size))[0]
        coords, els, irregular = qrefine_r(coords, els, irregular, marked)
        if marked.size == 0:
            break
    els = _reorder_corners(coords, els)
    els = _hanging_columns(els, irregular)
    els = els[mark_outside(coords, els, mask)]
    # markCoordHoleEdge: refined elements and the border band, grown twice
    diag = np.hypot(coords[els[:, 0] - 1, 0] - coords[els[:, 2] - 1, 0],
                    coords[els[:, 0] - 1, 1] - coords[els[:, 2] - 1, 1])
    step = float(np.max(np.atleast_1d(winstepsize)))
    xmin, xmax = coords0[:, 0].min(), coords0[:, 0].max()
    ymin, ymax = coords0[:, 1].min(), coords0[:, 1].max()
    c1, c3 = coords[els[:, 0] - 1], coords[els[:, 2] - 1]
    sel = ((diag < 0.99 * np.sqrt(2) * step) | (c1[:, 0] < xmin + 1.01 * step) | (c3[:, 0] > xmax - 1.01 * step)
           | (c1[:, 1] < ymin + 1.01 * step) | (c3[:, 1] > ymax - 1.01 * step))
    edge = np.unique(els[sel])
    edge = edge[edge > 0]
    for _ in range(2):
        hit = np.isin(els, edge).any(1)
        edge = np.unique(els[hit])
        edge = edge[edge > 0]
    return coords, els, irregular, edge
