"""GPU parity of the CUDA path (through the C ABI) against the oracle.

Tolerances:
  * ba_interp2, funImgGradient (FP64): bit-exact.
  * integer search: integer peaks bit-exact; u, v, cc.max to 1e-9.
  * plain FP64 IC-GN / Subpb1: identical result codes and NaN pattern, U and F
    within 1e-6 px (only the order of the block-wide sums differs).
  * batched FP32 IC-GN / Subpb1: |U - U_oracle| <= 0.01 px and strain
    |F - F_oracle| <= 1e-4 on subsets with the same code (same number of
    Gauss-Newton steps); >= 99 % of the subsets converged in both within
    0.01 px; result codes identical on >= 99 %.
  * Subpb2 (Jacobi-PCG, tol 1e-10) against the direct sparse solve: 1e-6 px.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")


@pytest.fixture(scope="module")
def sd():
    import staqdic
    return staqdic


@pytest.fixture(scope="module")
def golden(oracle):
    d = np.load(os.path.join(GOLD, "circular_hole_pair.npz"))

    def norm(I):
        I = I.astype(np.float64)
        return (I - I.mean()) / I.std(ddof=1)

    f = np.asfortranarray(norm(d["f"]) * d["maskf"])
    g = np.asfortranarray(norm(d["g"]) * d["maskg"])
    return d, f, g, oracle.funImgGradient(f, d["maskf"])


@pytest.fixture(scope="module")
def affine():
    from staqdic import workloads
    return workloads.uniform256(seed=0)


@pytest.fixture(scope="module")
def hole():
    from staqdic import workloads
    return workloads.hole1024(seed=1, size=256)


# ---------------------------------------------------------------- ba_interp2
def test_interp_bit_exact_golden(sd, ctx):
    d = np.load(os.path.join(GOLD, "ba_interp2_golden.npz"))
    assert np.array_equal(sd.ba_interp2(d["F"], d["X"], d["Y"], ctx=ctx), d["Z64"])
    Z32 = sd.ba_interp2(d["F"].astype(np.float32), d["X"].astype(np.float32),
                        d["Y"].astype(np.float32), ctx=ctx)
    assert np.array_equal(Z32, d["Z32"])


def test_interp_bit_exact_large(sd, ctx, oracle):
    rng = np.random.default_rng(9)
    F = np.asfortranarray(rng.normal(size=(500, 300)))
    X = rng.uniform(-4, 305, 200000)
    Y = rng.uniform(-4, 505, 200000)
    assert np.array_equal(sd.ba_interp2(F, X, Y, ctx=ctx), oracle.ba_interp2(F, X, Y))


def test_interp_layers_and_empty(sd, ctx, oracle):
    rng = np.random.default_rng(2)
    F = np.asfortranarray(rng.normal(size=(40, 30, 3)))
    X = rng.uniform(1, 30, 77)
    Y = rng.uniform(1, 40, 77)
    Z = sd.ba_interp2(F, X, Y, ctx=ctx)
    for k in range(3):
        assert np.array_equal(Z[:, k], oracle.ba_interp2(F[:, :, k], X, Y))
    assert sd.ba_interp2(F[:, :, 0], X[:0], Y[:0], ctx=ctx).size == 0


# ----------------------------------------------------------- funImgGradient
def test_gradient_bit_exact(sd, ctx, oracle, golden):
    d, f, g, Dref = golden
    Df = sd.funImgGradient(f, f, d["maskf"], ctx=ctx)
    assert np.array_equal(Df["DfDx"], Dref["DfDx"])
    assert np.array_equal(Df["DfDy"], Dref["DfDy"])
    Df32 = sd.funImgGradient(f.astype(np.float32), None, d["maskf"], ctx=ctx)
    assert np.allclose(Df32["DfDx"], Dref["DfDx"], atol=1e-5)


# ----------------------------------------------------------- integer search
@pytest.mark.parametrize("S", [6, 11])
def test_integer_search_peaks_bit_exact(sd, ctx, oracle, affine, S):
    w = affine
    x, y, u, v, cc = sd.funIntegerSearch(w["g"], w["f"], S, (1, 256), (1, 256), 32, 16, ctx=ctx)
    xo, yo, uo, vo, cco, pko = oracle.funIntegerSearch(w["g"], w["f"], S, (1, 256), (1, 256), 32, 16)
    assert np.array_equal(cc["peak"], pko)
    assert np.array_equal(x, xo) and np.array_equal(y, yo)
    assert np.allclose(u, uo, atol=1e-9, equal_nan=True)
    assert np.allclose(v, vo, atol=1e-9, equal_nan=True)
    assert np.allclose(cc["max"], cco, atol=1e-9, equal_nan=True)


def test_integer_search_masked_and_constant(sd, ctx, oracle, golden):
    d, f, g, _ = golden
    x, y, u, v, cc = sd.funIntegerSearch(g, f, 6, (1, 400), (1, 400), 32, 16, ctx=ctx)
    xo, yo, uo, vo, cco, pko = oracle.funIntegerSearch(g, f, 6, (1, 400), (1, 400), 32, 16)
    assert np.array_equal(cc["peak"], pko)
    assert np.array_equal(np.isnan(u), np.isnan(uo))
    # a constant template makes normxcorr2 throw: NaN output, peak 0
    z = np.zeros((120, 120), order="F")
    x, y, u, v, cc = sd.funIntegerSearch(z, z, 6, (1, 120), (1, 120), 32, 16, ctx=ctx)
    assert np.all(np.isnan(u)) and np.all(cc["peak"] == 0)


# ------------------------------------------------------------- IC-GN 6-DOF
def _cmp_plain(conv, co, U, Uo, F=None, Fo=None):
    assert np.array_equal(conv, co)
    assert np.array_equal(np.isnan(U), np.isnan(Uo))
    m = ~np.isnan(Uo)
    assert np.max(np.abs(U[m] - Uo[m]), initial=0) <= 1e-6
    if F is not None:
        m = ~np.isnan(Fo)
        assert np.max(np.abs(F[m] - Fo[m]), initial=0) <= 1e-6


def test_icgn_plain_affine(sd, ctx, oracle, affine):
    w = affine
    Dref = oracle.funImgGradient(w["f"], w["maskf"])
    Uo, Fo, Ho, co, _ = oracle.icgn6(w["U0"], w["coordinatesFEM"], Dref, w["f"], w["g"], 32, 1e-2)
    U, F, H, conv = sd.icgn_subsets(w["U0"], w["coordinatesFEM"], Dref, w["f"], w["g"], 32, 1e-2,
                                    precision="plain", ctx=ctx)
    _cmp_plain(conv, co, U, Uo, F, Fo)
    assert np.allclose(H, Ho, rtol=1e-10, atol=1e-6)


def test_icgn_plain_golden_pair_with_mask_quirks(sd, ctx, oracle, golden):
    d, f, g, Dref = golden
    Uo, Fo, Ho, co, mo = oracle.icgn6(d["U"], d["coordinatesFEM"], Dref, f, g, 32, 1e-2)
    assert (co == -1).sum() > 50 and (co == 102).sum() > 100
    U, F, H, conv = sd.icgn_subsets(d["U"], d["coordinatesFEM"], Dref, f, g, 32, 1e-2,
                                    precision="plain", ctx=ctx)
    _cmp_plain(conv, co, U, Uo, F, Fo)


def test_local_icgn_filter_and_marks(sd, ctx, oracle, golden):
    d, f, g, Dref = golden
    Uo, Fo, Ho, co, badnum_o, marko = oracle.LocalICGNQuadtree(d["U"], d["coordinatesFEM"], Dref, f, g,
                                                                 32, 1e-2)
    U, F, H, t, conv, badnum, mark = sd.LocalICGNQuadtree(d["U"], d["coordinatesFEM"], Dref, f, g,
                                                          {"winsize": 32}, "GaussNewton", 1e-2,
                                                          precision="plain", ctx=ctx)
    assert badnum == badnum_o
    assert np.array_equal(mark, marko)
    _cmp_plain(conv, co, U, Uo, F, Fo)


def _cmp_batched(conv, co, U, Uo, F=None, Fo=None):
    """FP32 batched vs FP64: on subsets that take the same number of Gauss-Newton
    steps (equal codes) |dU| <= 0.01 px and |dF| <= 1e-4; a subset that stops one
    step apart (its ||b||/||b0|| sits on the reference's 1e-2 tolerance) may
    differ by up to that step, so over all subsets converged in both at least
    99 % are within 0.01 px, and at least 99 % of the codes are identical."""
    both = (conv >= 1) & (conv <= 100) & (co >= 1) & (co <= 100)
    same = both & (conv == co)
    assert both.sum() > 0
    assert np.mean(conv == co) >= 0.99
    dU = np.abs(U - Uo).reshape(-1, 2).max(axis=1)
    assert dU[same].max() <= 0.01, dU[same].max()
    assert np.mean(dU[both] <= 0.01) >= 0.99
    if F is not None:
        dF = np.abs(F - Fo).reshape(-1, 4).max(axis=1)
        assert dF[same].max() <= 1e-4, dF[same].max()


def test_icgn_batched_affine(sd, ctx, oracle, affine):
    w = affine
    Dref = oracle.funImgGradient(w["f"], w["maskf"])
    Uo, Fo, Ho, co, _ = oracle.icgn6(w["U0"], w["coordinatesFEM"], Dref, w["f"], w["g"], 32, 1e-2)
    U, F, H, conv = sd.icgn_subsets(w["U0"], w["coordinatesFEM"], Dref, w["f"], w["g"], 32, 1e-2,
                                    precision="batched", ctx=ctx)
    _cmp_batched(conv, co, U, Uo, F, Fo)


def test_icgn_batched_golden_pair(sd, ctx, oracle, golden):
    d, f, g, Dref = golden
    Uo, Fo, Ho, co, mo = oracle.icgn6(d["U"], d["coordinatesFEM"], Dref, f, g, 32, 1e-2)
    U, F, H, conv = sd.icgn_subsets(d["U"], d["coordinatesFEM"], Dref, f, g, 32, 1e-2,
                                    precision="batched", ctx=ctx)
    _cmp_batched(conv, co, U, Uo, F, Fo)


def test_icgn_uneven_quadtree_batched_and_plain(sd, ctx, oracle, hole):
    w = hole
    f64 = w["f"].astype(np.float64)
    g64 = w["g"].astype(np.float64)
    Dref = oracle.funImgGradient(f64, w["maskf"])
    wl = w["winsize_list"]
    Uo, Fo, Ho, co, _ = oracle.icgn6(w["U0"], w["coordinatesFEM"], Dref, f64, g64, wl, 1e-2)
    U, F, H, conv = sd.icgn_subsets(w["U0"], w["coordinatesFEM"], Dref, f64, g64, int(wl.max()), 1e-2,
                                    precision="plain", ws_list=wl, ctx=ctx)
    _cmp_plain(conv, co, U, Uo, F, Fo)
    Df32 = {k: (v.astype(np.float32) if k in ("DfDx", "DfDy") else v) for k, v in Dref.items()}
    U, F, H, conv = sd.icgn_subsets(w["U0"], w["coordinatesFEM"], Df32, f64.astype(np.float32),
                                    g64.astype(np.float32), int(wl.max()), 1e-2, precision="batched",
                                    ws_list=wl, ctx=ctx)
    _cmp_batched(conv, co, U, Uo)


def test_multi_frame_batch_matches_each_frame(sd, ctx, oracle):
    """Several deformed frames (rotation 2k degrees plus a crack opening) in one
    batched launch give each frame's single-frame results: identical codes,
    and U within 0.01 px and F within 1e-4 on subsets with equal codes (only
    the FP32 summation order of the launch shape may differ); the FP64 oracle
    bounds every frame as for a single frame."""
    from staqdic import workloads
    w = workloads.series1024(seed=4, size=256, pairs=4)
    f = w["f"]
    wl = np.asarray(w["winsize_list"], np.int32)
    c = w["coordinatesFEM"]
    f64 = f.astype(np.float64)
    Dref = oracle.funImgGradient(f64, w["maskf"])
    Df32 = {k: (v.astype(np.float32) if k in ("DfDx", "DfDy") else v) for k, v in Dref.items()}
    Ul, Fl, cl = sd.icgn_subsets_frames(w["U0_list"], c, Df32, f, w["g_list"], int(wl.max()), 1e-2,
                                        ws_list=wl, ctx=ctx)
    for k, g in enumerate(w["g_list"]):
        U1, F1, H1, c1 = sd.icgn_subsets(w["U0_list"][k], c, Df32, f, g, int(wl.max()), 1e-2,
                                         precision="batched", ws_list=wl, ctx=ctx)
        assert np.mean(cl[k] == c1) >= 0.99
        same = (cl[k] == c1) & (c1 >= 1) & (c1 <= 100)
        assert same.sum() > 0.5 * c1.size
        dU = np.abs(Ul[k] - U1).reshape(-1, 2).max(axis=1)
        dF = np.abs(Fl[k] - F1).reshape(-1, 4).max(axis=1)
        assert dU[same].max() <= 0.01 and dF[same].max() <= 1e-4
        Uo, Fo, Ho, co, _ = oracle.icgn6(w["U0_list"][k], c, Dref, f64, g.astype(np.float64), wl, 1e-2)
        _cmp_batched(cl[k], co, Ul[k], Uo, Fl[k], Fo)


# ------------------------------------------------------------------ Subpb1
def _subpb1_inputs(oracle, golden):
    d, f, g, Dref = golden
    N = d["coordinatesFEM"].shape[0]
    Uo, Fo, Ho, co, _ = oracle.icgn6(d["U"], d["coordinatesFEM"], Dref, f, g, 32, 1e-2, variant=1)
    FOld = np.where(np.isnan(d["F"]), 0.0, d["F"])
    UOld = d["U"].copy()
    rng = np.random.default_rng(3)
    vdual = rng.normal(0, 0.01, 2 * N)
    wl = np.full((N, 2), 32, dtype=np.int32, order="F")
    return d, f, g, Dref, UOld, FOld, vdual, wl


def test_subpb1_plain(sd, ctx, oracle, golden):
    d, f, g, Dref, UOld, FOld, vdual, wl = _subpb1_inputs(oracle, golden)
    Uo, co = oracle.icgn2(UOld, FOld, vdual, d["coordinatesFEM"], Dref, f, g, wl, 1e-3, 1e-2)
    U, conv = sd.subpb1_subsets(UOld, FOld, vdual, d["coordinatesFEM"], Dref, f, g, wl, 1e-3, 1e-2,
                                precision="plain", ctx=ctx)
    _cmp_plain(conv, co, U, Uo)


def test_subpb1_batched(sd, ctx, oracle, golden):
    d, f, g, Dref, UOld, FOld, vdual, wl = _subpb1_inputs(oracle, golden)
    Uo, co = oracle.icgn2(UOld, FOld, vdual, d["coordinatesFEM"], Dref, f, g, wl, 1e-3, 1e-2)
    U, conv = sd.subpb1_subsets(UOld, FOld, vdual, d["coordinatesFEM"], Dref, f, g, wl, 1e-3, 1e-2,
                                precision="batched", ctx=ctx)
    _cmp_batched(conv, co, U, Uo)


def test_subpb1_quadtree_filter(sd, ctx, oracle, golden):
    d, f, g, Dref, UOld, FOld, vdual, wl = _subpb1_inputs(oracle, golden)
    Uo, co = oracle.icgn2(UOld, FOld, vdual, d["coordinatesFEM"], Dref, f, g, wl, 1e-3, 1e-2)
    bad, badnum_o = oracle.bad_points_subpb1(co)
    U, HPar, t, conv, badnum = sd.Subpb1Quadtree(UOld, FOld, None, vdual, d["coordinatesFEM"], Dref, f, g,
                                                 1e-3, 0.0, None, 2, {"winsize_List": wl},
                                                 "GaussNewton", 1e-2, precision="plain", ctx=ctx)
    assert badnum == badnum_o
    Uo2 = Uo.copy()
    Uo2[2 * bad] = np.nan
    Uo2[2 * bad + 1] = np.nan
    assert np.array_equal(np.isnan(U), np.isnan(Uo2))


# ------------------------------------------------------------------ Subpb2
def test_subpb2_golden_mesh(sd, ctx, oracle, golden):
    d, f, g, Dref = golden
    mesh = {"coordinatesFEM": d["coordinatesFEM"], "elementsFEM": d["elementsFEM"],
            "dirichlet": d["dirichlet"], "neumann": None}
    U = d["U"]
    F = np.where(np.isnan(d["F"]), 0.0, d["F"])
    for beta in (2.56e-4, 2.56e-3, 2.56e-2):
        Uo = oracle.Subpb2Quadtree(d["coordinatesFEM"], d["elementsFEM"], d["dirichlet"], None, 2, beta,
                                   1e-3, U, F, 0.0, 16)
        Uh, it = sd.Subpb2Quadtree(mesh, 2, beta, 1e-3, U, F, None, None, 0.0, 16, ctx=ctx,
                                   return_iters=True)
        assert it > 0
        assert np.max(np.abs(Uh - Uo)) < 1e-6


def test_subpb2_quadtree_free_nodes(sd, ctx, oracle, hole):
    w = hole
    # few Dirichlet nodes: most of the system is solved
    dirichlet = w["dirichlet"][::7]
    N = w["coordinatesFEM"].shape[0]
    rng = np.random.default_rng(4)
    U = w["Utrue"] + rng.normal(0, 0.05, 2 * N)
    F = rng.normal(0, 0.01, 4 * N)
    mesh = {"coordinatesFEM": w["coordinatesFEM"], "elementsFEM": w["elementsFEM"],
            "dirichlet": dirichlet, "neumann": None}
    Uo = oracle.Subpb2Quadtree(w["coordinatesFEM"], w["elementsFEM"], dirichlet, None, 2, 2.56e-3, 1e-3,
                               U, F, 0.0, 32)
    Uh = sd.Subpb2Quadtree(mesh, 2, 2.56e-3, 1e-3, U, F, None, None, 0.0, 32, ctx=ctx)
    assert np.max(np.abs(Uh - Uo)) < 1e-6


def test_subpb2_neumann_and_alpha(sd, ctx, oracle, affine):
    w = affine
    coords, elems = w["coordinatesFEM"], w["elementsFEM"]
    N = coords.shape[0]
    rng = np.random.default_rng(8)
    U = rng.normal(0, 0.5, 2 * N)
    F = rng.normal(0, 0.01, 4 * N)
    neumann = np.array([[1, 2, 0.0, -1.0], [2, 3, 0.0, -1.0], [15, 29, -1.0, 0.0]])
    dirichlet = np.array([100, 101], dtype=np.int32)
    Uo = oracle.Subpb2Quadtree(coords, elems, dirichlet, neumann, 3, 1e-2, 1e-3, U, F, 1e-3, 16)
    mesh = {"coordinatesFEM": coords, "elementsFEM": elems, "dirichlet": dirichlet,
            "neumann": np.asfortranarray(neumann)}
    Uh = sd.Subpb2Quadtree(mesh, 3, 1e-2, 1e-3, U, F, None, None, 1e-3, 16, ctx=ctx)
    assert np.max(np.abs(Uh - Uo)) < 1e-6


# ------------------------------------------------------------- boundary & misc
def test_errors_and_empty(sd, ctx, affine):
    from staqdic import StdicError
    w = affine
    Df = sd.funImgGradient(w["f"], None, w["maskf"], ctx=ctx)
    with pytest.raises(StdicError):
        sd.icgn_subsets(w["U0"], w["coordinatesFEM"], Df, w["f"], w["g"], 31, 1e-2, ctx=ctx)
    U, F, H, conv = sd.icgn_subsets(np.zeros(0), np.zeros((0, 2)), Df, w["f"], w["g"], 32, 1e-2, ctx=ctx)
    assert U.size == 0 and conv.size == 0


def test_device_resident_buffers_match_host(sd, ctx, affine):
    import torch
    w = affine
    Df = sd.funImgGradient(w["f"], None, w["maskf"], ctx=ctx)
    Uh, Fh, Hh, ch = sd.icgn_subsets(w["U0"], w["coordinatesFEM"], Df, w["f"], w["g"], 32, 1e-2,
                                     precision="plain", ctx=ctx)
    dev = lambda a: torch.as_tensor(np.asfortranarray(a).ravel(order="F")).cuda()
    Dd = {k: (dev(v) if k in ("DfDx", "DfDy", "ImgRefMask") else v) for k, v in Df.items()}
    U, F, H, conv = sd.icgn_subsets(dev(w["U0"]), dev(w["coordinatesFEM"]), Dd, dev(w["f"]), dev(w["g"]),
                                    32, 1e-2, precision="plain", ctx=ctx)
    torch.cuda.synchronize()
    assert np.array_equal(U.cpu().numpy(), Uh)
    assert np.array_equal(conv.cpu().numpy(), ch)


def test_plain_is_deterministic(sd, ctx, golden):
    d, f, g, Dref = golden
    a = sd.icgn_subsets(d["U"], d["coordinatesFEM"], Dref, f, g, 32, 1e-2, precision="plain", ctx=ctx)
    b = sd.icgn_subsets(d["U"], d["coordinatesFEM"], Dref, f, g, 32, 1e-2, precision="plain", ctx=ctx)
    for x, y in zip(a, b):
        assert np.array_equal(x, y, equal_nan=True)


# ------------------------------------------------------- quadtree mesh generation
def test_quadtree_mesh_reproduces_reference_mesh(sd, ctx):
    """stdic_quadtree_mesh on the uniform grid, mask and step stored in the
    reference's shipped result file gives that file's DICmesh exactly:
    coordinatesFEM (numbering included), elementsFEM with its hanging-node
    columns, irregular and the Dirichlet set."""
    d = np.load(os.path.join(GOLD, "circular_hole_pair.npz"))
    mesh = sd.GenerateQuadtreeMesh(d["x0"].T, d["y0"].T, d["ImgRefMask"], int(d["winstepsize"]),
                                   float(d["elementMinSize"]), ctx=ctx)
    assert np.array_equal(mesh["coordinatesFEM"], d["coordinatesFEM"])
    assert np.array_equal(mesh["elementsFEM"], d["elementsFEM"])
    assert np.array_equal(mesh["irregular"], d["irregular"])
    assert np.array_equal(mesh["dirichlet"], d["dirichlet"])


def test_quadtree_mesh_matches_oracle_on_synthetic_hole(sd, ctx):
    """The 2048^2 plate with a hole on a 16 px grid against the oracle's
    restatement (oracle/quadtree.py): identical mesh, hanging nodes and
    Dirichlet set; every element at least elementMinSize on its smaller side."""
    from oracle import quadtree as q
    from staqdic import workloads
    w = workloads.hole2048(size=1024)
    mask = w["maskf"]
    W, H = mask.shape
    xs = np.arange(20, W - 20 + 1, 16, dtype=np.float64)
    ys = np.arange(20, H - 20 + 1, 16, dtype=np.float64)
    x0, y0 = np.meshgrid(xs, ys)  # N x M, row = y
    mesh = sd.GenerateQuadtreeMesh(x0, y0, mask, 16, 2, ctx=ctx)
    co, eo, io, do = q.generate_quadtree_mesh(x0, y0, mask, 16, 2)
    assert mesh["elementsFEM"].shape[0] > 4000
    assert np.array_equal(mesh["coordinatesFEM"], co)
    assert np.array_equal(mesh["elementsFEM"], eo)
    assert np.array_equal(mesh["irregular"], io)
    assert np.array_equal(mesh["dirichlet"], do)
