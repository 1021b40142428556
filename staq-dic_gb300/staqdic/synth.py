"""Seeded synthetic speckle pairs for the STAQ-DIC hot path.

Arrays follow MATLAB's index order (see ``staqdic.api``): an image is a (W, H)
array ``Img[x-1, y-1]`` stored Fortran-contiguous; node coordinates are 1-based
pixel positions.

A reference image is a sum of isotropic Gaussian speckles plus white noise.  The
deformed image is the same speckle field rendered at the reference positions of
each deformed pixel, ``g(x) = f(X)`` with ``x = X + u(X)``, so it is exact for
any displacement field (the inverse map is found by fixed-point iteration).

Deformation fields used by the workloads:
  * affine: translation + small strain about the image centre;
  * Kirsch: plate with a circular hole under far-field uniaxial strain (plane
    stress), the classical Kirsch displacement solution;
  * bumps: a sum of Gaussian displacement bumps;
  * rotation about the centre composed with a straight crack opening.
"""
import math
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np


# ---------------------------------------------------------------------------
# speckle rendering
# ---------------------------------------------------------------------------
class Speckles:
    def __init__(self, W, H, n, rng, sigma=(1.5, 3.0), amp=(0.5, 1.0)):
        self.W, self.H = W, H
        self.cx = rng.uniform(1, W, n)
        self.cy = rng.uniform(1, H, n)
        self.sig = rng.uniform(sigma[0], sigma[1], n)
        self.amp = rng.uniform(amp[0], amp[1], n)


def _render(sp, W, H, X, Y, fwd_x, fwd_y, grow=1.0):
    """Sum the speckles at reference positions (X, Y) of every deformed pixel.

    fwd_x/fwd_y are the deformed-image positions of the speckle centres; each
    speckle is evaluated in a window around that position.
    """
    R = int(math.ceil(4.0 * sp.sig.max() * grow)) + 1
    img = np.zeros(W * H)
    px = np.rint(fwd_x).astype(np.int64) - 1  # 0-based
    py = np.rint(fwd_y).astype(np.int64) - 1
    keep = (px > -R) & (px < W + R) & (py > -R) & (py < H + R)
    px, py = px[keep], py[keep]
    cx, cy = sp.cx[keep], sp.cy[keep]
    inv2s2 = 1.0 / (2.0 * sp.sig[keep] ** 2)
    amp = sp.amp[keep]
    Xf = X.ravel(order="F")
    Yf = Y.ravel(order="F")
    offs = [(dx, dy) for dy in range(-R, R + 1) for dx in range(-R, R + 1)]

    def part(chunk):
        # one bincount per group of window offsets (the full-image pass of a
        # bincount dominates), summed into this worker's own image
        out = np.zeros(W * H)
        group = 8
        for g0 in range(0, len(chunk), group):
            lins, wts = [], []
            for dx, dy in chunk[g0:g0 + group]:
                yi = py + dy
                xi = px + dx
                ok = (yi >= 0) & (yi < H) & (xi >= 0) & (xi < W)
                if not ok.any():
                    continue
                lin = xi[ok] + yi[ok] * W
                d2 = (Xf[lin] - cx[ok]) ** 2 + (Yf[lin] - cy[ok]) ** 2
                lins.append(lin)
                wts.append(amp[ok] * np.exp(-d2 * inv2s2[ok]))
            if lins:
                out += np.bincount(np.concatenate(lins), weights=np.concatenate(wts), minlength=W * H)
        return out

    # numpy releases the GIL in these loops: split the offsets over host threads
    nw = max(1, min(_threads(), len(offs) // 16))
    chunks = [offs[k::nw] for k in range(nw)]
    if nw == 1:
        img = part(offs)
    else:
        with ThreadPoolExecutor(nw) as ex:
            for p in ex.map(part, chunks):
                img += p
    return img.reshape((W, H), order="F")


def _threads():
    return min(16, os.cpu_count() or 1)


def pixel_grid(W, H):
    x = np.arange(1, W + 1, dtype=np.float64)
    y = np.arange(1, H + 1, dtype=np.float64)
    return np.meshgrid(x, y, indexing="ij")  # (W, H)


def invert_map(ufun, xs, ys, iters=30):
    """Solve X + u(X) = x by fixed-point iteration (|grad u| << 1), in row
    blocks over host threads (each pixel iterates independently)."""
    W = xs.shape[0]
    nw = max(1, min(_threads(), W // 64))
    bounds = np.linspace(0, W, nw + 1).astype(int)

    def block(k):
        a, b = bounds[k], bounds[k + 1]
        x0, y0 = xs[a:b], ys[a:b]
        X, Y = x0.copy(), y0.copy()
        for _ in range(iters):
            ux, uy = ufun(X, Y)
            X = x0 - ux
            Y = y0 - uy
        return X, Y

    if nw == 1:
        return block(0)
    with ThreadPoolExecutor(nw) as ex:
        parts = list(ex.map(block, range(nw)))
    return np.concatenate([p[0] for p in parts], 0), np.concatenate([p[1] for p in parts], 0)


def render_pair(W, H, sp, ufun, noise=0.01, rng=None, inv=None, want_f=True):
    """Reference and deformed images for displacement field ufun(X, Y)
    (f is None when want_f is false)."""
    xs, ys = pixel_grid(W, H)
    f = _render(sp, W, H, xs, ys, sp.cx, sp.cy) if want_f else None
    if inv is None:
        X, Y = invert_map(ufun, xs, ys)
    else:
        X, Y = inv(xs, ys)
    ux, uy = ufun(sp.cx, sp.cy)
    g = _render(sp, W, H, X, Y, sp.cx + ux, sp.cy + uy, grow=1.2)
    if noise and rng is not None:
        if f is not None:
            f = f + rng.normal(0.0, noise, f.shape)
        g = g + rng.normal(0.0, noise, g.shape)
    return (np.asfortranarray(f) if f is not None else None), np.asfortranarray(g), X, Y


def normalize(img, roi=None):
    """funNormalizeImg.m:33-38: (I - mean) / std over the ROI (std with n-1)."""
    a = np.asarray(img, dtype=np.float64)
    t = a if roi is None else a[roi[0][0] - 1:roi[0][1], roi[1][0] - 1:roi[1][1]]
    return np.asfortranarray((a - t.mean()) / t.std(ddof=1))


# ---------------------------------------------------------------------------
# displacement fields
# ---------------------------------------------------------------------------
def affine_field(t, exx, eyy, exy, centre):
    cx, cy = centre

    def u(X, Y):
        dx, dy = X - cx, Y - cy
        return t[0] + exx * dx + exy * dy, t[1] + exy * dx + eyy * dy

    return u


def kirsch_field(a, eps, nu, centre):
    """Plane-stress Kirsch displacement for a hole of radius a, far-field strain
    eps along x."""
    cx, cy = centre
    kappa = (3.0 - nu) / (1.0 + nu)
    c = eps * (1.0 + nu) / 2.0  # sigma / (4 mu) with sigma = E eps

    def u(X, Y):
        dx, dy = X - cx, Y - cy
        r = np.maximum(np.hypot(dx, dy), 1e-9)
        th = np.arctan2(dy, dx)
        c2, s2 = np.cos(2 * th), np.sin(2 * th)
        a2r, a4r3 = a * a / r, a ** 4 / r ** 3
        ur = c * (r * ((kappa - 1) / 2 + c2) + a2r * (1 + (1 + kappa) * c2) - a4r3 * c2)
        ut = c * ((1 - kappa) * a2r - r - a4r3) * s2
        ct, st = np.cos(th), np.sin(th)
        return ur * ct - ut * st, ur * st + ut * ct

    return u


def bumps_field(rng, W, H, k=8, amp=(0.0, 5.0), width=(200.0, 800.0)):
    cx = rng.uniform(1, W, k)
    cy = rng.uniform(1, H, k)
    A = rng.uniform(amp[0], amp[1], k)
    w = rng.uniform(width[0], width[1], k)
    ph = rng.uniform(0, 2 * np.pi, k)

    def u(X, Y):
        ux = np.zeros_like(X, dtype=np.float64)
        uy = np.zeros_like(X, dtype=np.float64)
        for i in range(k):
            e = A[i] * np.exp(-((X - cx[i]) ** 2 + (Y - cy[i]) ** 2) / (2 * w[i] ** 2))
            ux = ux + e * np.cos(ph[i])
            uy = uy + e * np.sin(ph[i])
        return ux, uy

    return u


def crack_rotation_field(theta_deg, centre, crack_y, crack_xmax, jump, taper=100.0):
    """Rigid rotation about centre composed with a straight crack along
    y = crack_y for x < crack_xmax whose opening is `jump` px, tapering as a
    square root over the last `taper` px before the tip."""
    th = math.radians(theta_deg)
    cth, sth = math.cos(th), math.sin(th)
    cx, cy = centre

    def crack(X, Y):
        d = np.clip((crack_xmax - X) / taper, 0.0, 1.0)
        return 0.0 * X, 0.5 * jump * np.sign(Y - crack_y) * np.sqrt(d)

    def u(X, Y):
        cux, cuy = crack(X, Y)
        Xc, Yc = X + cux - cx, Y + cuy - cy
        return cth * Xc - sth * Yc + cx - X, sth * Xc + cth * Yc + cy - Y

    def inv(xs, ys):
        xr, yr = xs - cx, ys - cy
        Xp = cth * xr + sth * yr + cx
        Yp = -sth * xr + cth * yr + cy
        X, Y = Xp.copy(), Yp.copy()
        for _ in range(30):
            cux, cuy = crack(X, Y)
            X, Y = Xp - cux, Yp - cuy
        return X, Y

    return u, inv


# ---------------------------------------------------------------------------
# meshes
# ---------------------------------------------------------------------------
def uniform_nodes(W, H, winsize, winstepsize, gridx=None, gridy=None):
    """Node lists of main_ALDIC_Quadtree_v2.m:108-111."""
    gridx = gridx or (1, W)
    gridy = gridy or (1, H)
    xn = np.arange(max(4 + 0.5 * winsize, gridx[0]), min(W - 0.5 * winsize - 3, gridx[1]) + 1e-9,
                   winstepsize)
    yn = np.arange(max(4 + 0.5 * winsize, gridy[0]), min(H - 0.5 * winsize - 3, gridy[1]) + 1e-9,
                   winstepsize)
    return xn, yn


def uniform_mesh(xn, yn):
    """MeshSetUp.m: coordinatesFEM (N x 2, x fastest) and Q4 elementsFEM (E x 8)."""
    M, Nn = len(xn), len(yn)
    X, Y = np.meshgrid(xn, yn, indexing="xy")  # rows = y
    coords = np.stack([X.ravel(), Y.ravel()], axis=1).astype(np.float64)
    el = []
    for j in range(Nn - 1):
        for i in range(M - 1):
            a = j * M + i + 1
            el.append([a, a + 1, a + M + 1, a + M, 0, 0, 0, 0])
    return coords, np.asarray(el, dtype=np.int32).reshape(-1, 8)


def quadtree_mesh(W, H, winsize, winstepsize, size_fn, min_size, hole_fn=None):
    """A 2:1-balanced quadtree refinement of the uniform Q4 grid.

    size_fn(x, y) gives the wanted element size at a point; cells larger than
    it (and larger than min_size) are split.  hole_fn(x, y) -> True inside the
    material hole; elements with all four corners in the hole are dropped (the
    nodes stay, as in GenerateQuadtreeMesh.m).  Returns coordinatesFEM (N x 2),
    elementsFEM (E x 8, hanging mid-side nodes in columns 5..8: 5 on the x-max
    edge, 6 on the y-max edge, 7 on the x-min edge, 8 on the y-min edge) and the
    Dirichlet node list built like markCoordHoleEdge (GenerateQuadtreeMesh.m:
    76-111).
    """
    xn, yn = uniform_nodes(W, H, winsize, winstepsize)
    h0 = float(winstepsize)
    cells = {}  # (x0, y0, h) leaves

    def split_needed(x0, y0, h):
        if h / 2 < min_size:
            return False
        pts = [(x0 + a * h, y0 + b * h) for a in (0, 0.5, 1) for b in (0, 0.5, 1)]
        return min(size_fn(px, py) for px, py in pts) < h

    leaves = set()
    stack = [(float(x), float(y), h0) for x in xn[:-1] for y in yn[:-1]]
    while stack:
        x0, y0, h = stack.pop()
        if split_needed(x0, y0, h):
            hh = h / 2
            stack += [(x0, y0, hh), (x0 + hh, y0, hh), (x0, y0 + hh, hh), (x0 + hh, y0 + hh, hh)]
        else:
            leaves.add((x0, y0, h))
    # 2:1 balance: split any leaf with an edge neighbour smaller than half its size
    def leaf_at(px, py):
        return None

    changed = True
    while changed:
        changed = False
        corner_min = {}
        for (x0, y0, h) in leaves:
            for px, py in ((x0, y0), (x0 + h, y0), (x0, y0 + h), (x0 + h, y0 + h)):
                k = (px, py)
                corner_min[k] = min(corner_min.get(k, 1e30), h)
        new = set()
        for (x0, y0, h) in leaves:
            # points along the edges at quarter spacing reveal small neighbours
            q = h / 4
            small = False
            if h / 2 >= min_size:
                for t in (1, 2, 3):
                    for px, py in ((x0 + t * q, y0), (x0 + t * q, y0 + h), (x0, y0 + t * q), (x0 + h, y0 + t * q)):
                        if corner_min.get((px, py), 1e30) < h / 2:
                            small = True
                            break
                    if small:
                        break
            if small:
                hh = h / 2
                new |= {(x0, y0, hh), (x0 + hh, y0, hh), (x0, y0 + hh, hh), (x0 + hh, y0 + hh, hh)}
                changed = True
            else:
                new.add((x0, y0, h))
        leaves = new
    # nodes
    idx = {}
    coords = []

    def node(px, py):
        k = (px, py)
        if k not in idx:
            idx[k] = len(coords) + 1
            coords.append(k)
        return idx[k]

    order = sorted(leaves, key=lambda c: (c[1], c[0], c[2]))
    for (x0, y0, h) in order:
        node(x0, y0); node(x0 + h, y0); node(x0 + h, y0 + h); node(x0, y0 + h)
    elems = []
    sizes = []
    for (x0, y0, h) in order:
        n1, n2 = idx[(x0, y0)], idx[(x0 + h, y0)]
        n3, n4 = idx[(x0 + h, y0 + h)], idx[(x0, y0 + h)]
        hn = [idx.get((x0 + h, y0 + h / 2), 0), idx.get((x0 + h / 2, y0 + h), 0),
              idx.get((x0, y0 + h / 2), 0), idx.get((x0 + h / 2, y0), 0)]
        if hole_fn is not None and all(hole_fn(px, py) for px, py in
                                       ((x0, y0), (x0 + h, y0), (x0, y0 + h), (x0 + h, y0 + h))):
            continue
        elems.append([n1, n2, n3, n4] + hn)
        sizes.append(h)
    coords = np.asarray(coords, dtype=np.float64)
    elems = np.asarray(elems, dtype=np.int32)
    sizes = np.asarray(sizes)
    return coords, elems, dirichlet_nodes(coords, elems, winstepsize), sizes


def dirichlet_nodes(coords, elems, winstepsize, refined=True):
    """markCoordHoleEdge (GenerateQuadtreeMesh.m:90-133): the nodes of the
    elements on the ROI border and, with refined=True, of every element finer
    than winstepsize, grown twice by element adjacency.  refined=False keeps
    only the border band (the mesh then has free nodes in its refined part)."""
    xmin, xmax = coords[:, 0].min(), coords[:, 0].max()
    ymin, ymax = coords[:, 1].min(), coords[:, 1].max()
    c1 = coords[elems[:, 0] - 1]
    c3 = coords[elems[:, 2] - 1]
    mark_e = (c1[:, 0] < xmin + 1.01 * winstepsize) | (c3[:, 0] > xmax - 1.01 * winstepsize) | \
             (c1[:, 1] < ymin + 1.01 * winstepsize) | (c3[:, 1] > ymax - 1.01 * winstepsize)
    if refined:
        diag = np.hypot(c1[:, 0] - c3[:, 0], c1[:, 1] - c3[:, 1])
        mark_e |= diag < 0.99 * math.sqrt(2) * winstepsize
    marked = np.unique(elems[mark_e])
    marked = marked[marked > 0]
    for _ in range(2):
        hit = np.isin(elems, marked).any(axis=1)
        marked = np.unique(elems[hit])
        marked = marked[marked > 0]
    return marked.astype(np.int32)


def node_sizes(coords, elems, sizes):
    """Smallest incident element size per node; nodes that no element touches
    (inside a hole) get the smallest element size of the mesh."""
    N = coords.shape[0]
    big = sizes.max() if sizes.size else 0.0
    out = np.full(N, np.inf)
    for k in range(4):
        np.minimum.at(out, elems[:, k] - 1, sizes)
    out[~np.isfinite(out)] = sizes.min() if sizes.size else big
    return out
