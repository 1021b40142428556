"""The ADMM loop around Subpb1 and Subpb2: nodal strain, NaN fill and the
graph-captured iteration (stdic_nodal_strain, stdic_fill_nans, stdic_admm)
against the oracle's restatement of the same steps.

Tolerances:
  * nodal strain: 1e-12 of the largest strain against the oracle (FP64, only
    the contraction of products into FMAs differs); a linear displacement
    field gives its constant gradient at every node to 1e-12.
  * NaN fill: identical to the oracle (same sums in the same order).
  * ADMM, FP64 local step: two iterations equal the oracle-driven iterations
    (oracle Subpb1, bad-point filter, fill, direct Subpb2 solve, strain) with
    identical bad-point counts, U within 1e-5 px and F within 1e-6; the graph
    replay equals direct launches to 1e-9 (only the atomic assembly order of
    Subpb2 differs).
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def sd():
    import staqdic
    return staqdic


@pytest.fixture(scope="module")
def mesh():
    from staqdic import workloads
    return workloads.hole1024(seed=1, size=256)


def test_nodal_strain_matches_oracle(sd, ctx, oracle, mesh):
    c, el = mesh["coordinatesFEM"], mesh["elementsFEM"]
    N = c.shape[0]
    rng = np.random.default_rng(2)
    U = mesh["Utrue"] + rng.normal(0, 0.05, 2 * N)
    Fo = oracle.nodal_strain(c, el, U)
    F = sd.nodal_strain(c, el, U, ctx=ctx)
    assert np.array_equal(np.isnan(F), np.isnan(Fo))
    ok = ~np.isnan(Fo)
    assert np.max(np.abs(F[ok] - Fo[ok])) <= 1e-12 * np.max(np.abs(Fo[ok]))
    A = np.array([[0.01, 0.003], [-0.002, -0.004]])
    Ul = np.stack([A[0, 0] * c[:, 0] + A[0, 1] * c[:, 1] + 1.5, A[1, 0] * c[:, 0] + A[1, 1] * c[:, 1] - 0.7], 1).ravel()
    Fl = sd.nodal_strain(c, el, Ul, ctx=ctx).reshape(-1, 4)
    okn = ~np.isnan(Fl[:, 0])
    assert okn.sum() > 0.7 * N
    assert np.max(np.abs(Fl[okn] - [A[0, 0], A[1, 0], A[0, 1], A[1, 1]])) < 1e-12


def test_fill_nans_matches_oracle(sd, ctx, oracle, mesh):
    c, el = mesh["coordinatesFEM"], mesh["elementsFEM"]
    N = c.shape[0]
    rng = np.random.default_rng(3)
    U = mesh["Utrue"] + rng.normal(0, 0.05, 2 * N)
    bad = rng.choice(N, N // 10, replace=False)
    U[2 * bad] = np.nan
    U[2 * bad + 1] = np.nan
    Uo = oracle.fill_nans(c, el, U)
    Ug = sd.fill_nans(c, el, U, ctx=ctx)
    assert np.array_equal(np.isnan(Ug), np.isnan(Uo))
    ok = ~np.isnan(Uo)
    assert np.array_equal(Ug[ok], Uo[ok])
    assert np.isnan(U).sum() > np.isnan(Ug).sum()


def _oracle_admm(oracle, d, Dref, f, g, U2, F2, vdual, wl, mu, beta, steps):
    c, el, dirichlet = d["coordinatesFEM"], d["elementsFEM"], d["dirichlet"]
    bads = []
    for _ in range(steps):
        U1, conv = oracle.icgn2(U2, F2, vdual, c, Dref, f, g, wl, mu, 1e-2)
        bad, badnum = oracle.bad_points_subpb1(conv)
        U1 = U1.copy()
        U1[2 * bad] = np.nan
        U1[2 * bad + 1] = np.nan
        U1 = oracle.fill_nans(c, el, U1)
        F1 = F2.copy()
        U2 = oracle.Subpb2Quadtree(c, el, dirichlet, None, 2, beta, mu, U1, F1, 0.0, 16)
        F2 = oracle.nodal_strain(c, el, U2)
        vdual = U2 - U1
        bads.append(badnum)
    return U1, U2, F2, vdual, bads


def test_admm_plain_matches_oracle_and_graph_matches_direct(sd, ctx, oracle):
    d = np.load(os.path.join(GOLD, "circular_hole_pair.npz"))

    def norm(I):
        I = I.astype(np.float64)
        return (I - I.mean()) / I.std(ddof=1)

    f = np.asfortranarray(norm(d["f"]) * d["maskf"])
    g = np.asfortranarray(norm(d["g"]) * d["maskg"])
    Dref = oracle.funImgGradient(f, d["maskf"])
    c, el = d["coordinatesFEM"], d["elementsFEM"]
    N = c.shape[0]
    U2 = d["U"].copy()
    F2 = oracle.nodal_strain(c, el, U2)
    F2 = np.where(np.isnan(F2), 0.0, F2)
    vdual = np.zeros(2 * N)
    udual = np.zeros(4 * N)
    wl = np.full((N, 2), 32, dtype=np.int32, order="F")
    mu, beta = 1e-3, 1e-3 * 16 ** 2 * 1e-3
    mesh = {"coordinatesFEM": c, "elementsFEM": el, "dirichlet": d["dirichlet"]}
    out_g = sd.admm(mesh, Dref, f, g, wl, U2, F2, udual, vdual, mu, beta, steps=2, precision="plain",
                    use_graph=True, ctx=ctx)
    out_d = sd.admm(mesh, Dref, f, g, wl, U2, F2, udual, vdual, mu, beta, steps=2, precision="plain",
                    use_graph=False, ctx=ctx)
    assert out_g["graph_used"] and not out_d["graph_used"]
    assert np.array_equal(out_g["badnum"], out_d["badnum"])
    for k in ("U1", "U2", "F2", "vdual"):
        a, b = out_g[k], out_d[k]
        assert np.array_equal(np.isnan(a), np.isnan(b))
        ok = ~np.isnan(a)
        assert np.max(np.abs(a[ok] - b[ok])) < 1e-9, k
    U1o, U2o, F2o, vdo, bads = _oracle_admm(oracle, d, Dref, f, g, U2, F2, vdual, wl, mu, beta, 2)
    assert list(out_g["badnum"]) == bads
    ok = ~np.isnan(U2o)
    assert np.max(np.abs(out_g["U2"][ok] - U2o[ok])) < 1e-5
    okf = ~np.isnan(F2o)
    assert np.max(np.abs(out_g["F2"][okf] - F2o[okf])) < 1e-6
    assert np.all(out_g["pcg_iters"] > 0)
