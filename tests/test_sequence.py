"""Sequence initialisation (funPOR_GPR.m): the oracle's restatement pinned by
properties of its two halves, and stdic_por_gpr against the oracle.

  * POD: the modes are orthonormal under the reference's trapezoid inner
    product, and with every nonzero mode the snapshots are rebuilt exactly
    (mean + coefficients x modes).
  * Regression: coefficients that are exactly linear in time are predicted on
    their line (the linear basis carries them; the kernel part goes to 0).
  * The library against the oracle on a 20,000-node field evolving over five
    frames: u_pred to 1e-6 of the field's scale, alpha to 1e-12, beta_GPR to
    1e-4 relative (the regression's optimum is reached to the simplex
    tolerance; the POD parts only differ in summation order).
"""
import numpy as np
import pytest


def _snapshots(nT=5, npt=20000, seed=5):
    rng = np.random.default_rng(seed)
    x = np.linspace(0, 1, npt)
    modes = np.stack([np.sin(2 * np.pi * (k + 1) * x + rng.uniform(0, 1)) for k in range(4)])
    t = np.arange(1, nT + 1, dtype=np.float64)
    coef = np.stack([0.5 * t, 0.1 * t ** 2, np.sin(t), 0.02 * t ** 3], 1)
    return t, coef @ modes + 0.3 + 1e-4 * rng.normal(size=(nT, npt))


def test_pod_modes_orthonormal_and_rebuild_snapshots():
    from oracle import sequence as sq
    t, T = _snapshots()
    nT = T.shape[0]
    ave = T.mean(0)
    fp = T - ave
    c = np.array([[sq.inner_product(fp[k], fp[j]) for j in range(nT)] for k in range(nT)])
    lam, w = np.linalg.eigh(c)
    lam, w = lam[::-1], w[:, ::-1]
    nB = nT - 1  # every nonzero mode (the mean-free snapshots have rank nT - 1)
    fi = (fp.T @ w[:, :nB]).T / np.sqrt(lam[:nB])[:, None]
    G = np.array([[sq.inner_product(fi[j], fi[k]) for k in range(nB)] for j in range(nB)])
    assert np.allclose(G, np.eye(nB), atol=1e-9)
    a = np.array([[sq.inner_product(fp[j], fi[k]) for k in range(nB)] for j in range(nT)])
    assert np.allclose(a @ fi + ave, T, atol=1e-9)


def test_regression_predicts_linear_coefficients_on_their_line():
    from oracle import sequence as sq
    t = np.arange(1.0, 6.0)
    y = 0.7 - 1.3 * t
    m, s = sq.gpr_fit_predict(t, y, np.array([6.0, 7.0]))
    assert np.allclose(m, 0.7 - 1.3 * np.array([6.0, 7.0]), atol=1e-6)
    assert np.all(s >= sq.SIGMA_LOWER * 0.999)


def test_funpor_gpr_shapes_and_invariance_to_mode_signs():
    """u_pred does not depend on the sign of the eigenvectors: flipping every
    snapshot's fluctuation flips each coefficient with its mode."""
    from oracle import sequence as sq
    t, T = _snapshots()
    u1, a1, bp1, bg1 = sq.funPOR_GPR(T, t, np.array([6.0]), 3)
    assert u1.shape == (1, T.shape[1]) and 0 < a1 <= 1 and bg1.shape == (1,)
    ave = T.mean(0)
    u2, a2, _, _ = sq.funPOR_GPR(2 * ave - T, t, np.array([6.0]), 3)
    assert np.allclose(u2, 2 * ave - u1, atol=1e-8)
    assert abs(a1 - a2) < 1e-12


@pytest.mark.gpu
def test_por_gpr_matches_oracle(ctx):
    import staqdic
    from oracle import sequence as sq
    t, T = _snapshots()
    tp = np.array([6.0, 6.5])
    uo, ao, bpo, bgo = sq.funPOR_GPR(T, t, tp, 3)
    u, a, bp, bg = staqdic.funPOR_GPR(T, t, tp, 3, ctx=ctx)
    scale = np.abs(T).max()
    assert u.shape == uo.shape
    assert np.max(np.abs(u - uo)) <= 1e-6 * scale
    assert abs(a - ao) <= 1e-12
    assert np.allclose(bg, bgo, rtol=1e-4)
    # device-resident snapshots keep the prediction on the device
    import torch
    Td = torch.as_tensor(T).cuda()
    ud, _, _, _ = staqdic.funPOR_GPR(Td, t, tp, 3, ctx=ctx)
    torch.cuda.synchronize()
    assert np.array_equal(ud.cpu().numpy(), u)
