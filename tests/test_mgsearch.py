"""stdic_integer_search_mg (funIntegerSearchMg.m) against the oracle's
restatement (oracle/mg.py) on the same images.

Bar: the last level's blocks (the reference's tempx, tempy, tempu, tempv)
bit-exact and their cc.max within 1e-9; the node grid (xGrid, yGrid)
identical; uGrid, vGrid within 1e-6 px and cc.max within 1e-6.  What remains
after the bit-exact blocks is the difference between the device's
conjugate-gradient solve of gridfit's normal equations (relative residual
1e-12) and the oracle's direct solve, and rounding of the correlation sums.
Cases: a 13 x -9 px translation at 256^2 (beyond the +-6 px whole-field
search), the 256^2 affine speckle pair, the 1024^2 and the full 2048^2 plate
with a hole (Kirsch field up to ~20 px).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sd():
    import staqdic
    return staqdic


@pytest.fixture(scope="module")
def mg():
    from oracle import mg as m
    return m


def _compare(sd, mg, ctx, f, g, ws=32, st=16):
    W, H = f.shape
    xo, yo, uo, vo, po, bo = mg.funIntegerSearchMg(f, g, (1, W), (1, H), ws, st, return_blocks=True)
    x, y, u, v, cc = sd.funIntegerSearchMg(f, g, (1, W), (1, H), ws, st, ctx=ctx, blocks=True)
    # the last level's blocks: centres and displacements bit-exact (integer
    # peaks plus findpeak offsets rounded to 1/1000), cc.max to 1e-9
    b = cc["blocks"]
    assert b.shape == bo.shape
    assert np.array_equal(b[:, :2], bo[:, :2])
    assert np.array_equal(b[:, 2:4], bo[:, 2:4], equal_nan=True), np.nonzero(np.any(b[:, 2:4] != bo[:, 2:4], 1))
    assert np.max(np.abs(b[:, 4] - bo[:, 4])) < 1e-9
    assert x.shape == xo.shape and np.array_equal(x, xo) and np.array_equal(y, yo)
    assert np.array_equal(np.isnan(u), np.isnan(uo))
    ok = ~np.isnan(uo)
    assert np.max(np.abs(u[ok] - uo[ok])) < 1e-6
    assert np.max(np.abs(v[ok] - vo[ok])) < 1e-6
    assert np.max(np.abs(cc["max"] - po)) < 1e-6
    return x, y, u, v, cc


def test_mg_translation_beyond_whole_field_range(sd, mg, ctx):
    from staqdic import synth
    W = H = 256
    rng = np.random.default_rng(7)
    sp = synth.Speckles(W, H, 6000, rng)
    ufun = lambda X, Y: (np.full_like(X, 13.0), np.full_like(Y, -9.0))
    f, g, _, _ = synth.render_pair(W, H, sp, ufun, noise=0.01, rng=rng)
    f, g = synth.normalize(f), synth.normalize(g)
    _, _, u, v, cc = _compare(sd, mg, ctx, f, g)
    assert np.max(np.abs(u - 13.0)) < 0.5 and np.max(np.abs(v + 9.0)) < 0.5


@pytest.mark.parametrize("name", ["uniform256", "hole1024", "hole2048"])
def test_mg_matches_oracle(sd, mg, ctx, name):
    from staqdic import workloads
    w = getattr(workloads, name)()
    f, g = w["f"].astype(np.float64), w["g"].astype(np.float64)
    x, y, u, v, cc = _compare(sd, mg, ctx, f, g)
    assert u.size > 100


def test_mg_two_calls_in_a_row_agree(sd, ctx):
    from staqdic import workloads
    w = workloads.uniform256()
    f, g = w["f"].astype(np.float64), w["g"].astype(np.float64)
    a = sd.funIntegerSearchMg(f, g, (1, 256), (1, 256), 32, 16, ctx=ctx)
    b = sd.funIntegerSearchMg(f, g, (1, 256), (1, 256), 32, 16, ctx=ctx)
    for p, q in zip(a[:4], b[:4]):
        assert np.allclose(p, q, rtol=0, atol=1e-9)


def test_mg_constant_region_raises(sd, ctx):
    f = np.full((128, 128), 0.25)
    g = np.random.default_rng(0).normal(size=(128, 128))
    with pytest.raises(sd.StdicError) as e:
        sd.funIntegerSearchMg(f, g, (1, 128), (1, 128), 16, 16, ctx=ctx)
    assert e.value.code == -1
