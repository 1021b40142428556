"""stdic_icgn_adjoint (gradient of the subset ZNSSD cost; no reference
counterpart) against the oracle's FP64 restatement and finite differences.

Tolerances:
  * FP64 form vs the FP64 oracle: cost_n to 1e-10 relative, dU, dF and dg to
    1e-9 of their largest magnitude (only summation order differs).
  * store and recompute modes give the same cost_n, dU, dF bit for bit (same
    arithmetic) and dg to 1e-12 (atomic accumulation order).
  * FP32 form vs the FP64 oracle: cost_n to 1e-3 relative; dU, dF within 1e-3
    of each subset's gradient norm (norm-wise), dg within 1e-3 norm-wise.
  * FP64 gradients vs central finite differences of the cost (h = 1e-3 px for
    U and F, 1e-3 for g): 1e-3 relative, norm-wise over all subsets.
  * a torch.autograd.Function around the C ABI passes torch.autograd.gradcheck
    in FP64 (the wrapper lives only in this test).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sd():
    import staqdic
    return staqdic


@pytest.fixture(scope="module")
def bumps():
    from staqdic import workloads
    w = workloads.bumps4096(seed=3, size=256)
    rng = np.random.default_rng(11)
    N = w["coordinatesFEM"].shape[0]
    U = w["Utrue"] + rng.normal(0, 0.3, 2 * N)
    F = rng.normal(0, 0.01, 4 * N)
    f = w["f"].astype(np.float64)
    g = w["g"].astype(np.float64)
    return w, f, g, U, F


@pytest.fixture(scope="module")
def hole_case():
    from staqdic import workloads
    w = workloads.hole1024(seed=1, size=256)
    rng = np.random.default_rng(12)
    N = w["coordinatesFEM"].shape[0]
    U = w["Utrue"] + rng.normal(0, 0.2, 2 * N)
    F = rng.normal(0, 0.005, 4 * N)
    return w, w["f"].astype(np.float64), w["g"].astype(np.float64), U, F


def _rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def test_adjoint_f64_matches_oracle_both_modes(sd, ctx, oracle, bumps):
    w, f, g, U, F = bumps
    c = w["coordinatesFEM"]
    co, dUo, dFo, dgo = oracle.icgn_adjoint(f, g, None, c, 32, U, F)
    outs = []
    for mode in ("recompute", "store"):
        cost, cn, dU, dF, dg = sd.icgn_adjoint(U, F, c, f, g, 32, precision="plain", mode=mode, ctx=ctx)
        ok = np.isfinite(co)
        assert np.array_equal(np.isfinite(cn), ok)
        assert np.max(np.abs(cn[ok] - co[ok]) / np.abs(co[ok])) < 1e-10
        assert abs(cost - co[ok].sum()) < 1e-10 * co[ok].sum()
        assert _rel(dU, dUo) < 1e-9 and _rel(dF, dFo) < 1e-9
        assert _rel(dg, dgo) < 1e-9
        outs.append((cn, dU, dF, dg))
    # same arithmetic per subset; dg is accumulated with atomics, so only its
    # summation order differs
    for a, b in zip(outs[0][:3], outs[1][:3]):
        assert np.array_equal(a, b)
    assert _rel(outs[0][3], outs[1][3]) < 1e-12


def test_adjoint_masked_quadtree_f64(sd, ctx, oracle, hole_case):
    w, f, g, U, F = hole_case
    c = w["coordinatesFEM"]
    wl = np.asarray(w["winsize_list"], np.int32)
    co, dUo, dFo, dgo = oracle.icgn_adjoint(f, g, w["maskf"], c, wl, U, F)
    cost, cn, dU, dF, dg = sd.icgn_adjoint(U, F, c, f, g, int(wl.max()), ImgRefMask=w["maskf"],
                                           ws_list=wl, precision="plain", mode="store", ctx=ctx)
    ok = np.isfinite(co)
    assert (~ok).any() and ok.sum() > 100  # some windows fall inside the hole
    assert np.array_equal(np.isfinite(cn), ok)
    assert np.max(np.abs(cn[ok] - co[ok]) / np.abs(co[ok])) < 1e-10
    assert _rel(dU, dUo) < 1e-9 and _rel(dF, dFo) < 1e-9 and _rel(dg, dgo) < 1e-9


def test_adjoint_f32_matches_oracle(sd, ctx, oracle, bumps):
    w, f, g, U, F = bumps
    c = w["coordinatesFEM"]
    f32, g32 = f.astype(np.float32), g.astype(np.float32)
    co, dUo, dFo, dgo = oracle.icgn_adjoint(f32.astype(np.float64), g32.astype(np.float64), None, c, 32, U, F)
    for mode in ("recompute", "store"):
        cost, cn, dU, dF, dg = sd.icgn_adjoint(U, F, c, f32, g32, 32, precision="batched", mode=mode, ctx=ctx)
        ok = np.isfinite(co)
        assert np.max(np.abs(cn[ok] - co[ok]) / np.abs(co[ok])) < 1e-3
        Go = np.concatenate([dFo.reshape(-1, 4), dUo.reshape(-1, 2)], 1)
        Gg = np.concatenate([dF.reshape(-1, 4), dU.reshape(-1, 2)], 1)
        rel = np.linalg.norm(Gg - Go, axis=1) / np.linalg.norm(Go, axis=1)
        assert np.max(rel[ok]) < 1e-3
        assert np.linalg.norm(dg - dgo) / np.linalg.norm(dgo) < 1e-3


def test_adjoint_finite_differences(sd, ctx, bumps):
    w, f, g, U, F = bumps
    c = w["coordinatesFEM"]
    h = 1e-3
    cost, cn, dU, dF, dg = sd.icgn_adjoint(U, F, c, f, g, 32, precision="plain", ctx=ctx)
    N = c.shape[0]
    G = np.zeros((N, 6))
    for k in range(6):
        if k < 4:
            Fp, Fm = F.copy(), F.copy()
            Fp[k::4] += h
            Fm[k::4] -= h
            cp = sd.icgn_adjoint(U, Fp, c, f, g, 32, precision="plain", want_dg=False, ctx=ctx)[1]
            cm = sd.icgn_adjoint(U, Fm, c, f, g, 32, precision="plain", want_dg=False, ctx=ctx)[1]
        else:
            Up, Um = U.copy(), U.copy()
            Up[k - 4::2] += h
            Um[k - 4::2] -= h
            cp = sd.icgn_adjoint(Up, F, c, f, g, 32, precision="plain", want_dg=False, ctx=ctx)[1]
            cm = sd.icgn_adjoint(Um, F, c, f, g, 32, precision="plain", want_dg=False, ctx=ctx)[1]
        G[:, k] = (cp - cm) / (2 * h)
    A = np.concatenate([dF.reshape(-1, 4), dU.reshape(-1, 2)], 1)
    ok = np.isfinite(cn)
    assert np.linalg.norm(G[ok] - A[ok]) / np.linalg.norm(A[ok]) < 1e-3
    # dg at a few pixels: the cost is quadratic-like in g, central differences are exact to O(h^2)
    rng = np.random.default_rng(5)
    for x, y in rng.integers(40, 216, (5, 2)):
        gp, gm = g.copy(), g.copy()
        gp[x, y] += h
        gm[x, y] -= h
        Cp = sd.icgn_adjoint(U, F, c, f, gp, 32, precision="plain", want_dg=False, ctx=ctx)[0]
        Cm = sd.icgn_adjoint(U, F, c, f, gm, 32, precision="plain", want_dg=False, ctx=ctx)[0]
        fd = (Cp - Cm) / (2 * h)
        assert abs(fd - dg[x, y]) <= 1e-3 * max(abs(fd), 1e-6)


def test_adjoint_torch_autograd_gradcheck(sd, ctx):
    torch = pytest.importorskip("torch")
    from staqdic import workloads
    w = workloads.bumps4096(seed=7, size=48)
    f = torch.tensor(np.asarray(w["f"], np.float64).ravel(order="F"), device="cuda")
    W, H = w["f"].shape
    c = np.array([[20.0, 20.0], [28.0, 26.0]])
    ct = torch.tensor(c.ravel(order="F"), device="cuda", dtype=torch.float64)

    class ZNSSD(torch.autograd.Function):
        @staticmethod
        def forward(ctx_, U, F, g):
            # the library runs on its own stream: order it after torch's work and before torch reads
            torch.cuda.synchronize()
            cost, cn, dU, dF, dg = sd.icgn_adjoint(U.detach().contiguous(), F.detach().contiguous(), ct, f,
                                                   g.detach().contiguous(), 16, precision="plain",
                                                   size=(W, H), ctx=ctx)
            torch.cuda.synchronize()
            ctx_.save_for_backward(dU, dF, dg)
            return cost.reshape(())

        @staticmethod
        def backward(ctx_, go):
            dU, dF, dg = ctx_.saved_tensors
            return go * dU, go * dF, go * dg

    rng = np.random.default_rng(3)
    U = torch.tensor(rng.normal(0, 0.4, 4), device="cuda", requires_grad=True)
    F = torch.tensor(rng.normal(0, 0.02, 8), device="cuda", requires_grad=True)
    g = torch.tensor(np.asarray(w["g"], np.float64).ravel(order="F"), device="cuda", requires_grad=True)
    assert torch.autograd.gradcheck(ZNSSD.apply, (U, F, g), eps=1e-6, atol=1e-6, rtol=1e-3)
