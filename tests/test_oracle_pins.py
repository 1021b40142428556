"""The oracle pinned against the reference (CPU only).

* ba_interp2: bit-exact against golden vectors produced by the reference's own
  ba_interp2.cpp (tests/golden/ba_interp2_golden.npz) and, when it is built
  here, against that compiled reference on fresh inputs.
* The whole IC-GN restatement against the reference's shipped result file for
  the 400x400 plate-with-hole pair: LocalICGNBadPtNum and U.
* Analytic checks on seeded synthetic pairs (affine field) and Subpb2 on a
  linear field, which the FEM system reproduces exactly.
"""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")


def test_interp_matches_reference_golden(oracle):
    d = np.load(os.path.join(GOLD, "ba_interp2_golden.npz"))
    Z = oracle.ba_interp2(d["F"], d["X"], d["Y"])
    assert np.array_equal(Z, d["Z64"])
    Z32 = oracle.ba_interp2(d["F"].astype(np.float32), d["X"].astype(np.float32),
                            d["Y"].astype(np.float32))
    assert np.array_equal(Z32, d["Z32"])


def test_interp_matches_compiled_reference(oracle):
    if oracle.ref_lib() is None:
        pytest.skip("reference ba_interp2.cpp not built here")
    rng = np.random.default_rng(5)
    F = np.asfortranarray(rng.normal(size=(61, 47)))
    X = rng.uniform(-5, 52, 5000)
    Y = rng.uniform(-5, 66, 5000)
    assert np.array_equal(oracle.ba_interp2(F, X, Y), oracle.ref_ba_interp2(F, X, Y))


def _golden_pair(oracle):
    d = np.load(os.path.join(GOLD, "circular_hole_pair.npz"))

    def norm(I):
        I = I.astype(np.float64)
        return (I - I.mean()) / I.std(ddof=1)

    f = np.asfortranarray(norm(d["f"]) * d["maskf"])
    g = np.asfortranarray(norm(d["g"]) * d["maskg"])
    Df = oracle.funImgGradient(f, d["maskf"])
    return d, f, g, Df


def test_golden_pair_pins_local_icgn(oracle):
    """The reference's result file (created Nov 2023) comes from the masked-g
    branch as it stood before Feb 2024; with that branch restored the
    restatement reproduces LocalICGNBadPtNum = 22 exactly and the converged U."""
    d, f, g, Df = _golden_pair(oracle)
    U, F, Hp, conv, mark = oracle.icgn6(d["U"], d["coordinatesFEM"], Df, f, g,
                                         int(d["winsize"]), 1e-2, variant=1)
    bad, badnum = oracle.bad_points_local(conv)
    assert badnum == int(d["ALSub1BadPtNum"][0]) == 22
    ok = (conv >= 1) & (conv <= 100)
    du = np.abs(U - d["U"]).reshape(-1, 2).max(axis=1)
    # U of the file is the end of three ADMM iterations (RBF strain, Subpb2,
    # Subpb1); the first local pass started from it agrees to 1e-3 px at the
    # median, and within 0.01 px at every converged node more than 30 px from
    # the hole edge (hole radius 50 px, from the 7860 masked pixels).
    assert np.median(du[ok]) < 1e-3
    c = d["coordinatesFEM"]
    r = np.hypot(c[:, 0] - 200.5, c[:, 1] - 200.5)
    far = ok & (r >= 80)
    assert far.sum() > 400
    assert np.all(du[far] < 0.01)


def test_current_source_minus_one_only_on_masked_subsets(oracle):
    d, f, g, Df = _golden_pair(oracle)
    U, F, Hp, conv, mark = oracle.icgn6(d["U"], d["coordinatesFEM"], Df, f, g, 32, 1e-2)
    neg = conv == -1
    assert neg.any()
    assert np.all(mark[neg] == 1)
    assert np.all(np.isnan(U.reshape(-1, 2)[neg]))
    # everything the 2023 form did not flag keeps the same code
    _, _, _, conv1, _ = oracle.icgn6(d["U"], d["coordinatesFEM"], Df, f, g, 32, 1e-2, variant=1)
    assert np.array_equal(conv[~neg & (mark == 0)], conv1[~neg & (mark == 0)])


@pytest.fixture(scope="module")
def affine_case():
    from staqdic import workloads
    return workloads.uniform256(seed=0)


def test_oracle_icgn_recovers_affine_field(oracle, affine_case):
    w = affine_case
    Df = oracle.funImgGradient(w["f"], w["maskf"])
    U, F, Hp, conv, mark = oracle.icgn6(w["U0"], w["coordinatesFEM"], Df, w["f"], w["g"], 32, 1e-2)
    ok = (conv >= 1) & (conv <= 100)
    assert ok.sum() > 150
    err = np.abs(U - w["Utrue"]).reshape(-1, 2)[ok]
    assert err.max() < 0.05
    Fm = F.reshape(-1, 4)[ok].mean(axis=0)
    assert np.allclose(Fm, [0.01, 0.002, 0.002, -0.005], atol=5e-4)


def test_oracle_integer_search_finds_translation(oracle, affine_case):
    w = affine_case
    # the driver searches g-subsets in f (IntegerSearch(g, f)), so u = -displacement
    x, y, u, v, cc, peak = oracle.funIntegerSearch(w["g"], w["f"], 6, (1, 256), (1, 256), 32, 16)
    assert u.shape == (11, 11)
    assert np.all((peak[..., 0] >= 1) & (peak[..., 0] <= 15))
    ux, uy = w["ufun"](x, y)
    assert np.nanmax(np.abs(u + ux)) < 0.5
    assert np.nanmax(np.abs(v + uy)) < 0.5
    assert np.nanmin(cc) > 0.9


def test_oracle_subpb2_reproduces_linear_field(oracle):
    from staqdic import synth
    xn, yn = synth.uniform_nodes(256, 256, 32, 16)
    coords, elems = synth.uniform_mesh(xn, yn)
    A = np.array([[0.01, 0.003], [-0.002, -0.006]])
    t = np.array([1.5, -0.7])
    U = (coords @ A.T + t).ravel()
    F = np.tile([A[0, 0], A[1, 0], A[0, 1], A[1, 1]], coords.shape[0])
    # Dirichlet on the outer ring only
    ring = np.nonzero((coords[:, 0] == xn[0]) | (coords[:, 0] == xn[-1]) |
                      (coords[:, 1] == yn[0]) | (coords[:, 1] == yn[-1]))[0] + 1
    Uh = oracle.Subpb2Quadtree(coords, elems, ring, None, 2, 2.56e-3, 1e-3, U, F, 0.0, 16)
    assert np.max(np.abs(Uh - U)) < 1e-9


def test_bad_point_rules(oracle):
    conv = np.array([3, 3, 4, -1, 101, 102, 103, 3, 12, 5])
    bad, badnum = oracle.bad_points_local(conv)
    # bad: -1, 101, 102, 103 and codes above max(mean + std, 6) of the good ones
    assert badnum == 3
    assert set(bad.tolist()) >= {3, 4, 5, 6, 8}
    bad2, badnum2 = oracle.bad_points_subpb1(conv)
    assert badnum2 == 3 and 8 in bad2.tolist()


def test_oracle_adjoint_matches_finite_differences(oracle):
    """The oracle's adjoint (no reference counterpart) is pinned by central
    differences of its own cost: h = 1e-4 px keeps the O(h^2) error of the
    piecewise-cubic interpolant well below 1e-4 relative (norm-wise)."""
    from staqdic import workloads
    w = workloads.bumps4096(seed=3, size=128)
    f = w["f"].astype(np.float64)
    g = w["g"].astype(np.float64)
    c = w["coordinatesFEM"]
    N = c.shape[0]
    rng = np.random.default_rng(1)
    U = w["Utrue"] + rng.normal(0, 0.3, 2 * N)
    F = rng.normal(0, 0.01, 4 * N)
    cost, dU, dF, dg = oracle.icgn_adjoint(f, g, None, c, 32, U, F)
    h = 1e-4
    G = np.zeros((N, 6))
    for k in range(6):
        if k < 4:
            Fp, Fm = F.copy(), F.copy()
            Fp[k::4] += h
            Fm[k::4] -= h
            G[:, k] = (oracle.icgn_adjoint(f, g, None, c, 32, U, Fp, False)[0] -
                       oracle.icgn_adjoint(f, g, None, c, 32, U, Fm, False)[0]) / (2 * h)
        else:
            Up, Um = U.copy(), U.copy()
            Up[k - 4::2] += h
            Um[k - 4::2] -= h
            G[:, k] = (oracle.icgn_adjoint(f, g, None, c, 32, Up, F, False)[0] -
                       oracle.icgn_adjoint(f, g, None, c, 32, Um, F, False)[0]) / (2 * h)
    A = np.concatenate([dF.reshape(-1, 4), dU.reshape(-1, 2)], 1)
    assert np.linalg.norm(G - A) / np.linalg.norm(A) < 1e-4
    for x, y in ((40, 40), (60, 90), (100, 30)):
        gp, gm = g.copy(), g.copy()
        gp[x, y] += h
        gm[x, y] -= h
        fd = (np.nansum(oracle.icgn_adjoint(f, gp, None, c, 32, U, F, False)[0]) -
              np.nansum(oracle.icgn_adjoint(f, gm, None, c, 32, U, F, False)[0])) / (2 * h)
        assert abs(fd - dg[x, y]) <= 1e-4 * max(abs(fd), 1e-8)


def test_oracle_nodal_strain_of_linear_field_on_quadtree(oracle):
    """The strain step (a replacement of the reference's, so pinned
    analytically): on a quadtree mesh with hanging nodes, an affine
    displacement field gives its constant gradient [du/dx dv/dx du/dy dv/dy]
    at every node that lies in an element, and NaN elsewhere; the Gauss order
    does not change it."""
    from staqdic import workloads
    w = workloads.hole1024(seed=1, size=256)
    c, el = w["coordinatesFEM"], w["elementsFEM"]
    A = np.array([[0.012, -0.004], [0.003, -0.007]])
    U = (c @ A.T + np.array([2.0, -1.0])).ravel()
    inel = np.zeros(c.shape[0], bool)
    e = el[:, :8]
    inel[e[e > 0] - 1] = True
    for order in (2, 3):
        F = oracle.nodal_strain(c, el, U, order).reshape(-1, 4)
        assert np.all(np.isnan(F[~inel])) and not np.any(np.isnan(F[inel]))
        assert np.max(np.abs(F[inel] - [A[0, 0], A[1, 0], A[0, 1], A[1, 1]])) < 1e-12


def test_oracle_fill_nans_rules(oracle):
    """The NaN fill (a replacement of the reference's RBF fill): a NaN node
    takes the mean of its finite mesh neighbours; a NaN region fills from its
    edge inwards sweep by sweep; a node in no element stays NaN."""
    from staqdic import synth
    xn, yn = synth.uniform_nodes(160, 160, 32, 16)
    c, el = synth.uniform_mesh(xn, yn)
    N = c.shape[0]
    nx = len(xn)
    rng = np.random.default_rng(5)
    U = rng.normal(0, 1, 2 * N)
    k = 2 * nx + 2  # an interior node
    U[2 * k] = U[2 * k + 1] = np.nan
    out = oracle.fill_nans(c, el, U)
    # the neighbours of an interior Q4 node: the 8 surrounding grid nodes
    nb = [k + d for d in (-nx - 1, -nx, -nx + 1, -1, 1, nx - 1, nx, nx + 1)]
    assert np.isclose(out[2 * k], np.mean(U[2 * np.array(nb)]), rtol=0, atol=1e-15)
    assert np.isclose(out[2 * k + 1], np.mean(U[2 * np.array(nb) + 1]), rtol=0, atol=1e-15)
    keep = np.ones(2 * N, bool)
    keep[[2 * k, 2 * k + 1]] = False
    assert np.array_equal(out[keep], U[keep])
    # a block of NaN nodes fills completely
    V = U.copy()
    blk = [r * nx + q for r in range(1, 5) for q in range(1, 5)]
    for b in blk:
        V[2 * b] = V[2 * b + 1] = np.nan
    assert not np.any(np.isnan(oracle.fill_nans(c, el, V)))
    # a node that no element contains keeps its NaN
    c2 = np.vstack([c, [[500.0, 500.0]]])
    V2 = np.concatenate([U, [np.nan, np.nan]])
    out2 = oracle.fill_nans(c2, el, V2)
    assert np.all(np.isnan(out2[-2:]))


def test_quadtree_mesh_restatement_reproduces_reference_mesh():
    """GenerateQuadtreeMesh.m restated (oracle/quadtree.py) on the uniform grid,
    mask, step and elementMinSize stored in the reference's shipped result file
    gives that file's quadtree mesh exactly: the coordinates (node numbering
    included), elementsFEM with its hanging-node columns, the irregular list
    and the Dirichlet set markCoordHoleEdge."""
    from oracle import quadtree as q
    d = np.load(os.path.join(GOLD, "circular_hole_pair.npz"))
    # DICmesh.x0/y0 are stored transposed by MeshSetUp.m
    coords, els, irr, dirichlet = q.generate_quadtree_mesh(d["x0"].T, d["y0"].T, d["ImgRefMask"],
                                                           int(d["winstepsize"]), float(d["elementMinSize"]))
    assert np.array_equal(coords, d["coordinatesFEM"])
    assert np.array_equal(els, d["elementsFEM"])
    assert np.array_equal(irr, d["irregular"])
    assert np.array_equal(dirichlet, d["dirichlet"])
