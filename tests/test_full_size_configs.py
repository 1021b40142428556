"""Parity at the full sizes of the benchmark configs, against the FP64 oracle.

  * hole2048 (2048^2 plate with a hole, Kirsch 2 %, 80,695 quadtree nodes):
    the plain FP64 pass against the oracle on EVERY node (identical codes and
    NaN pattern, U and F within 1e-6 on every subset with code 1..100); the batched FP32 pass against the
    oracle on every node (codes identical on >= 99 %, |dU| <= 0.01 px and
    |dF| <= 1e-4 where the codes agree, >= 99 % of the subsets converged in
    both within 0.01 px); the LocalICGNQuadtree bad-subset count of both
    passes equal to the oracle's rule (LocalICGNQuadtree.m:153-169).
  * three ADMM iterations on the hole2048 mesh with the border band held
    (the Jacobi-PCG solves the 61,912-node refined region): the plain loop
    against the same iterations driven by the oracle (oracle Subpb1, filter,
    fill, direct Subpb2 solve, strain): bad counts identical, U within 1e-5
    px, F within 1e-6; the batched loop close to the plain loop.
  * bumps4096 (4096^2, 64,516 subsets of 32 px): the adjoint, FP64 and FP32,
    against the FP64 oracle on a seeded sample of 1,000 subsets (per-subset
    cost and gradients), and dg of the sample subsets alone against the
    oracle's dg.
  * series1024 (16 frames of 1024^2, 399,984 subsets in one launch): every
    frame's batched results against the oracle on every 25th node of that
    frame (the batched bar).
  * integer search on the hole1024 pair (1024^2) with S = 6 and a widened
    S = 16: integer peaks bit-exact, u, v, cc.max to 1e-9.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sd():
    import staqdic
    return staqdic


@pytest.fixture(scope="module")
def c3():
    from staqdic import workloads
    return workloads.hole2048()


def _batched_bar(Ub, Fb, cb, Uo, Fo, co, codes_frac=0.99):
    assert np.mean(cb == co) >= codes_frac, float(np.mean(cb == co))
    same = (cb == co) & (co >= 1) & (co <= 100) & ~np.isnan(Uo[0::2]) & ~np.isnan(Ub[0::2])
    dU = np.abs(Ub - Uo).reshape(-1, 2).max(axis=1)
    dF = np.abs(Fb - Fo).reshape(-1, 4).max(axis=1)
    assert dU[same].max() <= 0.01, float(dU[same].max())
    assert dF[same].max() <= 1e-4, float(dF[same].max())
    both = (cb >= 1) & (cb <= 100) & (co >= 1) & (co <= 100) & ~np.isnan(Uo[0::2]) & ~np.isnan(Ub[0::2])
    assert np.mean(dU[both] <= 0.01) >= 0.99
    return same


def test_c3_pass_every_node_against_oracle(sd, ctx, oracle, c3):
    w = c3
    c = w["coordinatesFEM"]
    N = c.shape[0]
    assert N > 80000
    wl = np.asarray(w["winsize_list"], np.int32)
    f32, g32 = w["f"], w["g"]
    f64, g64 = f32.astype(np.float64), g32.astype(np.float64)
    Do = oracle.funImgGradient(f64, w["maskf"])
    Uo, Fo, Ho, co, _ = oracle.icgn6(w["U0"], c, Do, f64, g64, wl, 1e-2)
    Dref = sd.funImgGradient(f64, ImgRefMask=w["maskf"], ctx=ctx)
    assert np.array_equal(Dref["DfDx"], Do["DfDx"]) and np.array_equal(Dref["DfDy"], Do["DfDy"])
    Up, Fp, Hp, cp = sd.icgn_subsets(w["U0"], c, Dref, f64, g64, int(wl.max()), 1e-2, precision="plain",
                                     ws_list=wl, ctx=ctx)
    # plain FP64: the oracle on every node.  Codes and the NaN pattern are
    # identical everywhere; U and F agree to 1e-6 on every subset the
    # bad-subset filter keeps (code 1..100).  A subset that runs all 100
    # iterations without converging (code 101, always removed by the filter)
    # follows a trajectory that rounding-level differences of the sums can
    # move further.
    assert np.array_equal(cp, co)
    assert np.array_equal(np.isnan(Up), np.isnan(Uo))
    kept = (co >= 1) & (co <= 100)
    m = np.repeat(kept, 2) & ~np.isnan(Uo)
    assert np.max(np.abs(Up[m] - Uo[m])) <= 1e-6
    m = np.repeat(kept, 4) & ~np.isnan(Fo)
    assert np.max(np.abs(Fp[m] - Fo[m])) <= 1e-6
    # batched FP32: the batched bar on every node
    Df32 = sd.funImgGradient(f32, ImgRefMask=w["maskf"], ctx=ctx, dtype=np.float32)
    Ub, Fb, Hb, cb = sd.icgn_subsets(w["U0"], c, Df32, f32, g32, int(wl.max()), 1e-2, precision="batched",
                                     ws_list=wl, ctx=ctx)
    same = _batched_bar(Ub, Fb, cb, Uo, Fo, co)
    assert same.sum() > 0.7 * N
    # the bad-subset filter of LocalICGNQuadtree: both passes against the oracle's rule
    _, badnum = oracle.bad_points_local(co)
    for prec in ("plain", "batched"):
        D = Dref if prec == "plain" else Df32
        ff, gg = (f64, g64) if prec == "plain" else (f32, g32)
        out = sd.LocalICGNQuadtree(w["U0"], c, D, ff, gg, {"winsize": int(wl.max()), "winsize_per_node": wl},
                                   "GaussNewton", 1e-2, precision=prec, ctx=ctx)
        if prec == "plain":
            assert int(out[5]) == int(badnum)
        else:
            _, bad_b = oracle.bad_points_local(out[4])
            assert int(out[5]) == int(bad_b)
            assert abs(int(out[5]) - int(badnum)) <= max(3, 0.01 * badnum)


def _oracle_admm(oracle, c, el, dirichlet, Dref, f, g, U2, F2, vdual, wl, mu, beta, steps, step_size):
    bads = []
    for _ in range(steps):
        U1, conv = oracle.icgn2(U2, F2, vdual, c, Dref, f, g, wl, mu, 1e-2)
        bad, badnum = oracle.bad_points_subpb1(conv)
        U1 = U1.copy()
        U1[2 * bad] = np.nan
        U1[2 * bad + 1] = np.nan
        U1 = oracle.fill_nans(c, el, U1)
        F1 = F2.copy()
        U2 = oracle.Subpb2Quadtree(c, el, dirichlet, None, 2, beta, mu, U1, F1, 0.0, step_size)
        F2 = oracle.nodal_strain(c, el, U2)
        vdual = U2 - U1
        bads.append(badnum)
    return U1, U2, F2, vdual, bads


def test_c3_admm_three_iterations_against_oracle(sd, ctx, oracle, c3):
    from staqdic import synth
    w = c3
    c, el = w["coordinatesFEM"], w["elementsFEM"]
    N = c.shape[0]
    wl1 = np.asarray(w["winsize_list"], np.int32)
    f64, g64 = w["f"].astype(np.float64), w["g"].astype(np.float64)
    Dref = oracle.funImgGradient(f64, w["maskf"])
    # initial state: the oracle's local pass, filtered, filled, and its strain
    U, F, _, _, _, _ = oracle.LocalICGNQuadtree(w["U0"], c, Dref, f64, g64, wl1, 1e-2)
    U2 = oracle.fill_nans(c, el, U)
    F2 = np.nan_to_num(oracle.nodal_strain(c, el, U2))
    dirichlet = synth.dirichlet_nodes(c, el, w["winstepsize"], False)
    wl = np.asfortranarray(np.stack([wl1, wl1], 1))
    mu = 1e-3
    beta = 1e-3 * float(w["winstepsize"]) ** 2 * mu
    mesh = {"coordinatesFEM": c, "elementsFEM": el, "dirichlet": dirichlet}
    args = (mesh, Dref, f64, g64, wl, U2, F2, np.zeros(4 * N), np.zeros(2 * N), mu, beta)
    op = sd.admm(*args, steps=3, precision="plain", use_graph=True, ctx=ctx)
    assert op["graph_used"] and np.all(np.asarray(op["pcg_iters"]) > 0)
    U1o, U2o, F2o, vdo, bads = _oracle_admm(oracle, c, el, dirichlet, Dref, f64, g64, U2, F2, np.zeros(2 * N),
                                            wl, mu, beta, 3, float(w["winstepsize"]))
    assert list(op["badnum"]) == bads
    ok = ~np.isnan(U2o)
    assert not np.isnan(op["U2"][ok]).any()
    assert np.max(np.abs(op["U2"][ok] - U2o[ok])) < 1e-5
    okf = ~np.isnan(F2o)
    assert np.max(np.abs(op["F2"][okf] - F2o[okf])) < 1e-6
    # the batched FP32 Subpb1 inside the same loop: close to the plain loop
    f32, g32 = w["f"], w["g"]
    D32 = sd.funImgGradient(f32, ImgRefMask=w["maskf"], ctx=ctx, dtype=np.float32)
    ob = sd.admm(mesh, D32, f32, g32, wl, U2, F2, np.zeros(4 * N), np.zeros(2 * N), mu, beta, steps=3,
                 precision="batched", use_graph=True, ctx=ctx)
    assert np.all(np.abs(np.asarray(ob["badnum"]) - np.asarray(op["badnum"])) <= max(3, 0.01 * N))
    for k in ("U1", "U2"):
        a, b = ob[k], op[k]
        both = ~np.isnan(a) & ~np.isnan(b)
        assert both.sum() >= 0.99 * (~np.isnan(b)).sum()
        dev = np.abs(a[both] - b[both])
        assert np.mean(dev <= 0.01) >= 0.99 and np.percentile(dev, 90) <= 1e-3, k


@pytest.fixture(scope="module")
def c4():
    from staqdic import workloads
    w = workloads.bumps4096()
    N = w["coordinatesFEM"].shape[0]
    rng = np.random.default_rng(44)
    U = w["Utrue"] + rng.normal(0, 0.2, 2 * N)
    F = rng.normal(0, 0.005, 4 * N)
    return w, U, F


def _rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def test_c4_adjoint_sample_against_oracle(sd, ctx, oracle, c4):
    import torch
    w, U, F = c4
    c = w["coordinatesFEM"]
    N = c.shape[0]
    assert N > 60000
    W, H = w["f"].shape
    idx = np.sort(np.random.default_rng(45).choice(N, 1000, replace=False))
    cs = c[idx]
    Us, Fs = U.reshape(-1, 2)[idx].ravel(), F.reshape(-1, 4)[idx].ravel()
    f64, g64 = w["f"].astype(np.float64), w["g"].astype(np.float64)
    co, dUo, dFo, dgo = oracle.icgn_adjoint(f64, g64, None, cs, 32, Us, Fs)
    ok = np.isfinite(co)
    assert ok.sum() > 900
    dev = lambda a, dt: torch.as_tensor(np.ascontiguousarray(np.asarray(a, dt).ravel(order="F"))).cuda()
    for prec, dt, tol in (("plain", np.float64, 1e-9), ("batched", np.float32, 1e-3)):
        f, g = dev(w["f"], dt), dev(w["g"], dt)
        # every subset of the full mesh in one call; the sample's outputs
        cost, cn, dU, dF, _ = sd.icgn_adjoint(dev(U, np.float64), dev(F, np.float64), dev(c, np.float64), f, g,
                                              32, precision=prec, want_dg=False, size=(W, H), ctx=ctx)
        cn = cn.cpu().numpy()[idx]
        dU = dU.cpu().numpy().reshape(-1, 2)[idx]
        dF = dF.cpu().numpy().reshape(-1, 4)[idx]
        assert np.array_equal(np.isfinite(cn), ok)
        assert np.max(np.abs(cn[ok] - co[ok]) / np.abs(co[ok])) < (1e-10 if prec == "plain" else 1e-3)
        gref = np.concatenate([dUo.reshape(-1, 2), dFo.reshape(-1, 4)], 1)[ok]
        gout = np.concatenate([dU, dF], 1)[ok]
        nrm = np.linalg.norm(gref, axis=1)
        assert np.max(np.linalg.norm(gout - gref, axis=1) / nrm) < tol, prec
        # dg of the sample subsets alone against the oracle's dg of the same subsets
        _, _, _, _, dg = sd.icgn_adjoint(dev(Us, np.float64), dev(Fs, np.float64), dev(cs, np.float64), f, g, 32,
                                         precision=prec, want_dg=True, size=(W, H), ctx=ctx)
        dg = dg.cpu().numpy().astype(np.float64).reshape(H, W).T
        if prec == "plain":
            assert _rel(dg, dgo) < 1e-9
        else:
            assert np.linalg.norm(dg - dgo) / np.linalg.norm(dgo) < 1e-3


def test_c5_sixteen_frames_against_oracle_sample(sd, ctx, oracle):
    from staqdic import workloads
    w = workloads.series1024()
    c = w["coordinatesFEM"]
    N = c.shape[0]
    P = len(w["g_list"])
    assert P == 16 and N > 24000
    wl = np.asarray(w["winsize_list"], np.int32)
    f32 = w["f"]
    D32 = sd.funImgGradient(f32, ImgRefMask=w["maskf"], ctx=ctx, dtype=np.float32)
    res = sd.icgn_subsets_frames(w["U0_list"], c, D32, f32, w["g_list"], int(wl.max()), 1e-2, ws_list=wl,
                                 ctx=ctx)
    U, F, conv = res[0], res[1], res[-1]
    U = np.asarray(U).reshape(P, 2 * N)
    F = np.asarray(F).reshape(P, 4 * N)
    conv = np.asarray(conv).reshape(P, N)
    f64 = f32.astype(np.float64)
    Do = oracle.funImgGradient(f64, w["maskf"])
    idx = np.arange(0, N, 25)
    n_both = 0
    for k in range(P):
        U0 = w["U0_list"][k].reshape(-1, 2)[idx].ravel()
        Uo, Fo, _, co, _ = oracle.icgn6(U0, c[idx], Do, f64, w["g_list"][k].astype(np.float64), wl[idx], 1e-2)
        Ub = U[k].reshape(-1, 2)[idx].ravel()
        Fb = F[k].reshape(-1, 4)[idx].ravel()
        same = _batched_bar(Ub, Fb, conv[k][idx], Uo, Fo, co)
        n_both += int(same.sum())
    assert n_both > 0.5 * P * idx.size


@pytest.mark.parametrize("S", [6, 16])
def test_integer_search_c2_bit_exact(sd, ctx, oracle, S):
    from staqdic import workloads
    w = workloads.hole1024()
    f, g = w["f"].astype(np.float64), w["g"].astype(np.float64)
    W, H = f.shape
    x, y, u, v, cc = sd.funIntegerSearch(g, f, S, (1, W), (1, H), 32, 32, ctx=ctx)
    xo, yo, uo, vo, cco, pko = oracle.funIntegerSearch(g, f, S, (1, W), (1, H), 32, 32)
    assert x.size > 700
    assert np.array_equal(cc["peak"], pko)
    assert np.array_equal(x, xo) and np.array_equal(y, yo)
    assert np.array_equal(np.isnan(u), np.isnan(uo))
    assert np.allclose(u, uo, atol=1e-9, equal_nan=True)
    assert np.allclose(v, vo, atol=1e-9, equal_nan=True)
    assert np.allclose(cc["max"], cco, atol=1e-9, equal_nan=True)
