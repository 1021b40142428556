"""The five seeded synthetic workloads of this path (numpy ``default_rng``).

  uniform256   256^2 uint8 speckle, affine map, ws 32 / step 16 -> 14x14 = 196
               nodes; integer search + FP64 local IC-GN + one Subpb2.
  hole1024     1024^2 float32, circular hole r=150 at the centre, Kirsch field
               at 1 % far-field uniaxial strain (nu 0.3), quadtree 4..32 px,
               subset size 2 x element size clipped to 8..64.
  hole2048     2048^2, hole r=300, Kirsch at 2 %, same quadtree rule; three
               ADMM iterations (mu 1e-3, beta in {1e-3,1e-2,1e-1}*step^2*mu).
  bumps4096    4096^2, 8 Gaussian displacement bumps, ws 32 on a 16 px grid.
  series1024   16 pairs of 1024^2: rotation 2k degrees about the centre plus a
               straight crack along y=512 for x<600 with a 5 px opening.

The public benchmark the reference itself uses is a real image sequence; these
synthetic pairs stand in for it with its shapes and value distributions.
Every workload carries the analytic displacement at the nodes (``Utrue``) and an
integer-rounded seed ``U0 = round(Utrue)`` standing in for the integer search.
Each generator takes a ``scale`` to make a geometrically similar, smaller case
for tests.
"""
import math

import numpy as np

from . import synth


def _speckle_count(W, H):
    return int(round(3000 * W * H / (256 * 256)))


def _pack(name, f, g, maskf, maskg, coords, elems, dirichlet, Utrue, ws_list, winstepsize,
          ufun, extra=None):
    d = dict(name=name, f=f, g=g, maskf=maskf, maskg=maskg, coordinatesFEM=coords,
             elementsFEM=elems, dirichlet=dirichlet, Utrue=Utrue, U0=np.round(Utrue),
             winsize_list=ws_list, winstepsize=winstepsize, ufun=ufun)
    if extra:
        d.update(extra)
    return d


def uniform256(seed=0, size=256):
    rng = np.random.default_rng(seed)
    W = H = size
    sp = synth.Speckles(W, H, _speckle_count(W, H), rng)
    centre = ((W + 1) / 2, (H + 1) / 2)
    ufun = synth.affine_field((3.4, -1.7), 0.01, -0.005, 0.002, centre)
    f, g, _, _ = synth.render_pair(W, H, sp, ufun, noise=0.01, rng=rng)
    # 8-bit quantisation of the speckle intensity
    scale = 80.0
    f8 = np.clip(np.rint(f * scale), 0, 255).astype(np.uint8)
    g8 = np.clip(np.rint(g * scale), 0, 255).astype(np.uint8)
    fN = synth.normalize(f8.astype(np.float64))
    gN = synth.normalize(g8.astype(np.float64))
    ws, st = 32, 16
    xn, yn = synth.uniform_nodes(W, H, ws, st)
    coords, elems = synth.uniform_mesh(xn, yn)
    ux, uy = ufun(coords[:, 0], coords[:, 1])
    Utrue = np.stack([ux, uy], 1).ravel()
    ones = np.ones((W, H), dtype=np.uint8, order="F")
    return _pack("uniform256", fN, gN, ones, ones, coords, elems, np.zeros(0, np.int32), Utrue,
                 np.full(coords.shape[0], ws, np.int32), st, ufun,
                 dict(f_u8=f8, g_u8=g8, winsize=ws))


def _hole_case(name, seed, W, a, eps, scale_sizes=1.0):
    rng = np.random.default_rng(seed)
    H = W
    sp = synth.Speckles(W, H, _speckle_count(W, H), rng)
    centre = ((W + 1) / 2, (H + 1) / 2)
    ufun = synth.kirsch_field(a, eps, 0.3, centre)
    f, g, X, Y = synth.render_pair(W, H, sp, ufun, noise=0.01, rng=rng)
    xs, ys = synth.pixel_grid(W, H)
    maskf = (np.hypot(xs - centre[0], ys - centre[1]) >= a).astype(np.uint8)
    maskg = (np.hypot(X - centre[0], Y - centre[1]) >= a).astype(np.uint8)
    f = np.asfortranarray((synth.normalize(f) * maskf).astype(np.float32))
    g = np.asfortranarray((synth.normalize(g) * maskg).astype(np.float32))
    s = scale_sizes
    hmin = 4.0

    # element size by distance from the hole edge: 4 px in a band of 75 px per
    # 1024 px of image, 8 px to 0.35 W, 16 px to 0.46 W, 32 px beyond (about
    # 20k nodes at 1024^2 and 80k at 2048^2, subsets of 8-64 px)
    def size_fn(x, y):
        d = abs(math.hypot(x - centre[0], y - centre[1]) - a)
        if d < 75 * s:
            return 4.0
        if d < 0.35 * W:
            return 8.0
        if d < 0.46 * W:
            return 16.0
        return 32.0

    def hole_fn(x, y):
        return math.hypot(x - centre[0], y - centre[1]) < a

    st = 32
    coords, elems, dirichlet, sizes = synth.quadtree_mesh(W, H, 64, st, size_fn, hmin, hole_fn)
    hn = synth.node_sizes(coords, elems, sizes)
    ws_list = np.clip(2 * hn, 8, 64).astype(np.int32)
    ux, uy = ufun(coords[:, 0], coords[:, 1])
    Utrue = np.stack([ux, uy], 1).ravel()
    inside = np.hypot(coords[:, 0] - centre[0], coords[:, 1] - centre[1]) < a
    Utrue[2 * np.nonzero(inside)[0]] = 0.0
    Utrue[2 * np.nonzero(inside)[0] + 1] = 0.0
    return _pack(name, f, g, maskf, maskg, coords, elems, dirichlet, Utrue, ws_list, st, ufun,
                 dict(hole_radius=a, centre=centre, eps=eps))


def hole1024(seed=1, size=1024):
    return _hole_case("hole1024", seed, size, 150.0 * size / 1024, 0.01, size / 1024)


def hole2048(seed=2, size=2048):
    return _hole_case("hole2048", seed, size, 300.0 * size / 2048, 0.02, size / 1024)


def bumps4096(seed=3, size=4096):
    rng = np.random.default_rng(seed)
    W = H = size
    sp = synth.Speckles(W, H, _speckle_count(W, H), rng)
    ufun = synth.bumps_field(rng, W, H)
    f, g, _, _ = synth.render_pair(W, H, sp, ufun, noise=0.01, rng=rng)
    f = np.asfortranarray(synth.normalize(f).astype(np.float32))
    g = np.asfortranarray(synth.normalize(g).astype(np.float32))
    ws, st = 32, 16
    xn, yn = synth.uniform_nodes(W, H, ws, st)
    coords, elems = synth.uniform_mesh(xn, yn)
    ux, uy = ufun(coords[:, 0], coords[:, 1])
    Utrue = np.stack([ux, uy], 1).ravel()
    ones = np.ones((W, H), dtype=np.uint8, order="F")
    return _pack("bumps4096", f, g, ones, ones, coords, elems, np.zeros(0, np.int32), Utrue,
                 np.full(coords.shape[0], ws, np.int32), st, ufun, dict(winsize=ws))


def ramp1024(seed=5, size=1024, frames=10, deps=0.002):
    """A loading sequence: frame k (k = 1..frames) of the 1024^2 plate with a
    hole under a Kirsch field at far-field strain k deps, all against one
    reference image and one quadtree mesh.  Frame-to-frame increments stay
    below about 1.5 px, the small steps the reference's sequence
    initialisation (previous result, then a POD/GPR prediction) assumes."""
    rng = np.random.default_rng(seed)
    W = H = size
    a = 150.0 * size / 1024
    sp = synth.Speckles(W, H, _speckle_count(W, H), rng)
    centre = ((W + 1) / 2, (H + 1) / 2)
    xs, ys = synth.pixel_grid(W, H)
    f = synth._render(sp, W, H, xs, ys, sp.cx, sp.cy) + rng.normal(0, 0.01, (W, H))
    maskf = (np.hypot(xs - centre[0], ys - centre[1]) >= a).astype(np.uint8)
    fN = np.asfortranarray((synth.normalize(f) * maskf).astype(np.float32))
    s = size / 1024

    def size_fn(x, y):
        d = abs(math.hypot(x - centre[0], y - centre[1]) - a)
        return 4.0 if d < 75 * s else (8.0 if d < 0.35 * W else (16.0 if d < 0.46 * W else 32.0))

    def hole_fn(x, y):
        return math.hypot(x - centre[0], y - centre[1]) < a

    coords, elems, dirichlet, sizes = synth.quadtree_mesh(W, H, 64, 32, size_fn, 4.0, hole_fn)
    hn = synth.node_sizes(coords, elems, sizes)
    ws_list = np.clip(2 * hn, 8, 64).astype(np.int32)
    inside = np.hypot(coords[:, 0] - centre[0], coords[:, 1] - centre[1]) < a
    gs, Us, ufuns = [], [], []
    for k in range(1, frames + 1):
        ufun = synth.kirsch_field(a, deps * k, 0.3, centre)
        _, g, X, Y = synth.render_pair(W, H, sp, ufun, noise=0.0, want_f=False)
        g = g + rng.normal(0, 0.01, (W, H))
        maskg = (np.hypot(X - centre[0], Y - centre[1]) >= a)
        gs.append(np.asfortranarray((synth.normalize(g) * maskg).astype(np.float32)))
        ux, uy = ufun(coords[:, 0], coords[:, 1])
        U = np.stack([ux, uy], 1)
        U[inside] = 0.0
        Us.append(U.ravel())
        ufuns.append(ufun)
    d = _pack("ramp1024", fN, gs[0], maskf, None, coords, elems, dirichlet, Us[0], ws_list, 32, ufuns[0],
              dict(hole_radius=a, centre=centre))
    d.update(g_list=gs, Utrue_list=Us, U0_first=np.round(Us[0]), ufun_list=ufuns)
    return d


def series1024(seed=4, size=1024, pairs=16):
    """16 frame pairs sharing one reference image and one quadtree mesh."""
    rng = np.random.default_rng(seed)
    W = H = size
    sp = synth.Speckles(W, H, _speckle_count(W, H), rng)
    centre = ((W + 1) / 2, (H + 1) / 2)
    cy, cxm = 512.0 * size / 1024, 600.0 * size / 1024
    xs, ys = synth.pixel_grid(W, H)
    f = synth._render(sp, W, H, xs, ys, sp.cx, sp.cy) + rng.normal(0, 0.01, (W, H))
    maskf = ~((np.abs(ys - cy) <= 3) & (xs < cxm))
    maskf = maskf.astype(np.uint8)
    fN = np.asfortranarray((synth.normalize(f) * maskf).astype(np.float32))
    gs, Us, ufuns = [], [], []

    # element size by distance from the crack: 4 px within 170 px, 8 px to
    # 500 px, 16 px to 640 px, 32 px beyond (per 1024 px; about 25k nodes)
    def size_fn(x, y):
        d = (abs(y - cy) if x < cxm + 40 else math.hypot(x - cxm, y - cy)) * 1024.0 / W
        return 4.0 if d < 170 else (8.0 if d < 500 else (16.0 if d < 640 else 32.0))

    st = 32
    coords, elems, dirichlet, sizes = synth.quadtree_mesh(W, H, 64, st, size_fn, 4.0, None)
    hn = synth.node_sizes(coords, elems, sizes)
    ws_list = np.clip(2 * hn, 8, 64).astype(np.int32)
    for k in range(pairs):
        ufun, inv = synth.crack_rotation_field(2.0 * k, centre, cy, cxm, 5.0 * size / 1024)
        _, g, X, Y = synth.render_pair(W, H, sp, ufun, noise=0.0, inv=inv, want_f=False)
        g = g + rng.normal(0, 0.01, (W, H))
        maskg = (~((np.abs(Y - cy) <= 3) & (X < cxm)) & (X >= 1) & (X <= W) & (Y >= 1) & (Y <= H))
        gs.append(np.asfortranarray((synth.normalize(g) * maskg).astype(np.float32)))
        ux, uy = ufun(coords[:, 0], coords[:, 1])
        Us.append(np.stack([ux, uy], 1).ravel())
        ufuns.append(ufun)
    d = _pack("series1024", fN, gs[0], maskf, None, coords, elems, dirichlet, Us[0], ws_list, st,
              ufuns[0])
    d.update(g_list=gs, Utrue_list=Us, U0_list=[np.round(u) for u in Us], ufun_list=ufuns)
    return d


WORKLOADS = {"uniform256": uniform256, "hole1024": hole1024, "hole2048": hole2048,
             "bumps4096": bumps4096, "series1024": series1024, "ramp1024": ramp1024}
