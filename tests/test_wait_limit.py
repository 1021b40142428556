"""Bounded device waits that run out, and a context that still works after.

The cooperative Subpb2 PCG synchronises its blocks with grid barriers whose
waits are bounded (2^24 polls by default).  With the context's wait limit set
to one poll, a block that reaches a barrier before the others gives up at once:
the call must return STDIC_E_TIMEOUT (no trap, no hang, no fault), and the
same context, with the default limit restored, must then solve the system to
the direct sparse solve's answer (1e-6 px).  The limit only shortens how long a
block waits; every wait stays bounded either way.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mesh():
    from staqdic import synth, workloads
    w = workloads.hole1024(seed=1, size=512)
    coords, elems = w["coordinatesFEM"], w["elementsFEM"]
    # the border band alone is held: the refined region is left to the PCG
    dirichlet = synth.dirichlet_nodes(coords, elems, w["winstepsize"], False)
    N = coords.shape[0]
    rng = np.random.default_rng(17)
    U = w["Utrue"] + rng.normal(0, 0.05, 2 * N)
    F = rng.normal(0, 0.01, 4 * N)
    return dict(coordinatesFEM=coords, elementsFEM=elems, dirichlet=dirichlet, neumann=None), U, F


def test_pcg_barrier_wait_runs_out_then_context_recovers(ctx, oracle, mesh):
    import staqdic
    from staqdic import _lib
    m, U, F = mesh
    N = m["coordinatesFEM"].shape[0]
    assert N > 4 * 256  # several PCG blocks, so some block waits at the first barrier
    beta, mu = 2.56e-3, 1e-3
    ctx.set_wait_limit(1)
    try:
        with pytest.raises(staqdic.StdicError) as ei:
            staqdic.Subpb2Quadtree(m, 2, beta, mu, U, F, None, None, 0.0, 32, ctx=ctx)
        assert ei.value.code == _lib.STDIC_E_TIMEOUT
        assert "grid barrier" in str(ei.value)
    finally:
        ctx.set_wait_limit(0)
    Uo = oracle.Subpb2Quadtree(m["coordinatesFEM"], m["elementsFEM"], m["dirichlet"], None, 2, beta, mu,
                               U, F, 0.0, 32)
    Uh, it = staqdic.Subpb2Quadtree(m, 2, beta, mu, U, F, None, None, 0.0, 32, ctx=ctx, return_iters=True)
    assert it > 0
    assert np.max(np.abs(Uh - Uo)) < 1e-6


def test_wait_limit_rejects_negative(ctx):
    import staqdic
    with pytest.raises(staqdic.StdicError):
        ctx.set_wait_limit(-1)
