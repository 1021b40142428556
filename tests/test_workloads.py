"""The synthetic workloads have the sizes of the configurations they stand
for: C2 about 20k quadtree nodes on a 1024^2 plate with a hole, C3 about 80k
on 2048^2, C4 about 60k subsets of 32 px on 4096^2, C5 about 25k nodes per
1024^2 frame and 400k per 16-frame launch; quadtree subsets span 8..64 px.
The Dirichlet set follows the markCoordHoleEdge rule (border and refined
elements, grown twice)."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def wl():
    from staqdic import workloads
    return workloads


def _check_quadtree(w, lo, hi):
    c, el = w["coordinatesFEM"], w["elementsFEM"]
    N = c.shape[0]
    assert lo <= N <= hi
    assert el.shape[1] == 8 and el[:, :4].min() >= 1 and el.max() <= N
    ws = np.asarray(w["winsize_list"])
    assert ws.min() >= 8 and ws.max() <= 64 and set(np.unique(ws)) >= {8, 16, 32}
    return N


def test_hole1024_is_c2_sized(wl):
    w = wl.hole1024()
    assert w["f"].shape == (1024, 1024)
    _check_quadtree(w, 18000, 22000)


def test_hole2048_is_c3_sized(wl):
    from staqdic import synth
    w = wl.hole2048()
    assert w["f"].shape == (2048, 2048)
    _check_quadtree(w, 75000, 85000)
    d = synth.dirichlet_nodes(w["coordinatesFEM"], w["elementsFEM"], w["winstepsize"])
    assert np.array_equal(d, w["dirichlet"])
    border = synth.dirichlet_nodes(w["coordinatesFEM"], w["elementsFEM"], w["winstepsize"], refined=False)
    assert np.isin(border, d).all() and border.size < d.size


def test_series_is_c5_sized(wl):
    # the mesh does not depend on the number of frames; the bench stacks 16
    w = wl.series1024(pairs=2)
    N = _check_quadtree(w, 23000, 27000)
    assert len(w["g_list"]) == 2 and 16 * N > 380000


def test_bumps4096_is_c4_sized():
    # the C4 grid (subsets of 32 px every 16 px) without rendering the images
    from staqdic import synth
    xn, yn = synth.uniform_nodes(4096, 4096, 32, 16)
    N = len(xn) * len(yn)
    assert 55000 <= N <= 70000
