"""The oracle's restatement of the multigrid integer search
(funIntegerSearchMg.m) and its parts, checked on the CPU: the full normxcorr2
against a direct evaluation and against the whole-field search's own
restatement, findpeak on an exact quadratic, gridfit's springs fit, and the
multigrid search recovering a translation far beyond the whole-field search's
+-6 px region."""
import math

import numpy as np
import pytest


@pytest.fixture(scope="module")
def mg():
    from oracle import mg as m
    return m


def _direct_ncc(T, A):
    m, n = T.shape
    M, N = A.shape
    Tz = T - T.mean()
    denT = math.sqrt(float((Tz ** 2).sum()))
    P = np.zeros((M + 2 * m, N + 2 * n))
    P[m:m + M, n:n + N] = A
    out = np.zeros((M + m - 1, N + n - 1))
    den = np.zeros_like(out)
    num = np.zeros_like(out)
    for r in range(out.shape[0]):
        for c in range(out.shape[1]):
            win = P[r + 1:r + 1 + m, c + 1:c + 1 + n]
            num[r, c] = (Tz * win).sum()
            den[r, c] = denT * math.sqrt(max(float((win ** 2).sum() - win.sum() ** 2 / (m * n)), 0.0))
    tol = math.sqrt(np.spacing(np.abs(den).max()))
    ok = den > tol
    out[ok] = num[ok] / den[ok]
    return out


def test_normxcorr2_full_matches_direct_sums(mg):
    rng = np.random.default_rng(0)
    T = rng.normal(size=(7, 5))
    A = rng.normal(size=(15, 12))
    A[:3, :4] = 0.0  # a flat corner: lags there have no variance
    X = mg.normxcorr2_full(T, A)
    Y = _direct_ncc(T, A)
    assert X.shape == (21, 16)
    assert np.max(np.abs(X - Y)) < 1e-12
    assert np.all(np.abs(X) <= 1 + 1e-12)
    with pytest.raises(ValueError):
        mg.normxcorr2_full(np.ones((3, 3)), A)


def test_whole_field_search_agrees_with_its_restatement(mg, oracle):
    """The cropped full map plus findpeak gives the whole-field search's
    displacements and peak values (funIntegerSearch.m:121-146)."""
    from staqdic import workloads
    w = workloads.uniform256(seed=3, size=128)
    f, g = w["f"], w["g"]
    ws, st, S = 16, 16, 6
    x, y, u, v, cc, _ = oracle.funIntegerSearch(f, g, S, (1, 128), (1, 128), ws, st)
    for (j, i) in [(0, 0), (1, 2), (2, 1)]:
        ii = int(round(x[j, i] - ws / 2))
        jj = int(round(y[j, i] - ws / 2))
        T = f[ii - 1:ii + ws, jj - 1:jj + ws]
        A = g[ii - 1 - S:ii + ws + S, jj - 1 - S:jj + ws + S]
        X = mg.normxcorr2_full(T, A)
        sub = X[ws - 1:X.shape[0] - ws + 1, ws - 1:X.shape[1] - ws + 1]
        pv, pu, mf = mg.findpeak(sub, True)
        zd = (math.ceil(sub.shape[0] / 2), math.ceil(sub.shape[1] / 2))
        assert abs((pu - zd[0]) - u[j, i]) < 1e-9 and abs((pv - zd[1]) - v[j, i]) < 1e-9
        assert abs(mf - cc[j, i]) < 1e-9


def test_findpeak_exact_quadratic(mg):
    r, c = np.meshgrid(np.arange(1, 10), np.arange(1, 12), indexing="ij")
    x0, y0 = 6.25, 4.75  # column, row of the apex
    F = 2.0 - 0.3 * (c - x0) ** 2 - 0.2 * (r - y0) ** 2 - 0.05 * (c - x0) * (r - y0)
    xp, yp, mf = mg.findpeak(F, True)
    assert abs(xp - x0) < 1e-3 and abs(yp - y0) < 1e-3 and abs(mf - 2.0) < 1e-4
    xp, yp, _ = mg.findpeak(F, False)
    assert (xp, yp) == (6.0, 5.0)


def test_gridfit_springs(mg):
    rng = np.random.default_rng(1)
    x = rng.uniform(0, 100, 400)
    y = rng.uniform(0, 80, 400)
    xn, yn = np.arange(0, 101, 10.0), np.arange(0, 81, 10.0)
    Z = mg.gridfit_springs(x, y, np.full(400, 3.5), xn, yn)
    assert Z.shape == (yn.size, xn.size) and np.max(np.abs(Z - 3.5)) < 1e-9
    # with a light regulariser the fit interpolates dense samples of a plane
    # (the springs pull towards a flat surface, so at smoothness 1 it is biased)
    zs = 0.02 * x - 0.01 * y + 1.0
    Z = mg.gridfit_springs(x, y, zs, xn, yn, smoothness=1e-4)
    X, Y = np.meshgrid(xn, yn)
    # (a corner node whose triangles hold no sample follows its springs only)
    assert np.mean(np.abs(Z - (0.02 * X - 0.01 * Y + 1.0)) < 1e-3) >= 0.95
    Z1 = mg.gridfit_springs(x, y, zs, xn, yn)
    assert np.max(np.abs(Z1 - (0.02 * X - 0.01 * Y + 1.0))) < 0.5 and np.std(Z1) < np.std(Z)
    # NaN data points are dropped
    z2 = zs.copy()
    z2[::7] = np.nan
    assert not np.any(np.isnan(mg.gridfit_springs(x, y, z2, xn, yn)))


def test_multigrid_search_recovers_large_translation(mg):
    from staqdic import synth
    W = H = 256
    rng = np.random.default_rng(7)
    sp = synth.Speckles(W, H, 6000, rng)
    shift = (13.0, -9.0)
    ufun = lambda X, Y: (np.full_like(X, shift[0]), np.full_like(Y, shift[1]))
    f, g, _, _ = synth.render_pair(W, H, sp, ufun, noise=0.01, rng=rng)
    f, g = synth.normalize(f), synth.normalize(g)
    xG, yG, uG, vG, pG = mg.funIntegerSearchMg(f, g, (1, W), (1, H), 32, 16)
    assert uG.shape == xG.shape and uG.size > 20
    assert np.max(np.abs(uG - shift[0])) < 0.5 and np.max(np.abs(vG - shift[1])) < 0.5
    assert np.min(pG) > 0.5


def test_qfactors_restatement_matches_full_map_definition(oracle):
    """cc.qfactors of the oracle (direct sums in C++) against the definition
    written out on the FFT-based full normxcorr2 map of this module: PCE =
    peak^2 / mean(cc_min^2) and PPE = 1 / entropy of the 30-bin histogram of
    cc_min over [0, peak] (numpy's histogram has the same uniform bins, the
    last one closed), then each column shifted and scaled to [0, 1]."""
    from oracle import mg
    from staqdic import workloads
    w = workloads.uniform256(seed=0, size=128)
    f, g = w["g"], w["f"]
    S, ws, st = 6, 32, 16
    raw, qf = oracle.integer_search_qfactors(f, g, S, (1, 128), (1, 128), ws, st)
    gx, gy, nx, ny = oracle.intsearch_grid(128, 128, (S, S), (1, 128), (1, 128), (ws, ws), (st, st))
    assert raw.shape == (nx * ny, 2) and nx * ny > 0
    for t in range(nx * ny):
        ix, iy = t % nx, t // nx
        ii, jj = int(gx[0]) + ix * st, int(gy[0]) + iy * st
        C = f[ii - 1:ii + ws, jj - 1:jj + ws]
        D = g[ii - 1 - S:ii + ws + S, jj - 1 - S:jj + ws + S]
        X = mg.normxcorr2_full(C, D)
        cm = X - X.min()
        peak = cm.max()
        pce = peak ** 2 / np.mean(cm ** 2)
        h, _ = np.histogram(cm, bins=30, range=(0.0, peak))
        p = h[h > 0] / cm.size
        ppe = 1.0 / np.sum(p * np.log(1.0 / p))
        assert abs(raw[t, 0] - pce) <= 1e-8 * pce
        assert abs(raw[t, 1] - ppe) <= 1e-8 * ppe
    for k in range(2):
        q = raw[:, k] - np.nanmin(raw[:, k])
        assert np.allclose(qf[:, k], q / np.nanmax(q), rtol=0, atol=1e-12)


def test_qfactors_constant_template_gives_inf_then_nan(oracle):
    """A point where normxcorr2 throws holds [Inf Inf] before the
    normalisation; Inf - min is Inf and Inf / Inf is NaN, so that point is
    NaN and every other point 0 (funIntegerSearch.m:156,175-176)."""
    from staqdic import workloads
    w = workloads.uniform256(seed=0, size=128)
    f = np.array(w["g"], copy=True, order="F")
    f[:60, :60] = 0.5  # the first grid point's template is constant
    raw, qf = oracle.integer_search_qfactors(f, w["f"], 6, (1, 128), (1, 128), 32, 16)
    assert np.isinf(raw[0]).all()
    assert np.isnan(qf[0]).all()
    fin = ~np.isinf(raw[:, 0])
    assert np.all(qf[fin] == 0)
