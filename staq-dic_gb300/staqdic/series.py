"""The accumulative frame loop of main_ALDIC_Quadtree_v2.m over a sequence of
deformed frames, on the library's entry points.

Every frame is solved against the one reference frame on one mesh.  The
initial guess of frame k (the reference's ImgSeqNum = k + 2) is
(main_ALDIC_Quadtree_v2.m:179-197):
  * frame 0: the caller's U0 (the integer search's result in the reference);
  * frames 1-4 (ImgSeqNum < 7): the previous frame's result;
  * later frames: funPOR_GPR's prediction at t = k + 1 from the last nTime = 5
    results at t = k - 4 .. k, with nB = 3 modes, separately for u and v.
Each frame runs LocalICGNQuadtree (bad subsets set to NaN), the local NaN
fill, and optionally `admm_steps` ADMM iterations (stdic_admm); its result is
the filled local field, or the last Subpb2 field with ADMM.  Nodes that stay
NaN (in no element) enter the prediction as 0, the value Subpb2 gives them.

The reference keeps this loop in MATLAB and calls the same routines through
the shims; this is its mirror on the C ABI.
"""
import numpy as np

from . import api

NTIME, NB, PRE_POD = 5, 3, 5


def initial_guess(k, results, U0_first, predict):
    """The initial guess of frame k from the results of frames 0..k-1;
    predict(T, t_train, t_pre, nB) is funPOR_GPR."""
    if k == 0:
        return np.asarray(U0_first, dtype=np.float64)
    if k < PRE_POD:
        return np.asarray(results[k - 1], dtype=np.float64)
    snaps = np.stack([np.nan_to_num(np.asarray(results[j], dtype=np.float64)) for j in range(k - NTIME, k)])
    t_train = np.arange(k - NTIME + 1, k + 1, dtype=np.float64)
    t_pre = np.array([k + 1.0])
    u = predict(snaps[:, 0::2], t_train, t_pre, NB)[0]
    v = predict(snaps[:, 1::2], t_train, t_pre, NB)[0]
    U0 = np.empty(snaps.shape[1])
    U0[0::2] = np.asarray(u).ravel()
    U0[1::2] = np.asarray(v).ravel()
    return U0


def run_series(mesh, Df, ImgRef, g_list, U0_first, winsize_list, tol=1e-2, precision="batched", admm_steps=0,
               mu=1e-3, beta=None, winstepsize=16, ctx=None):
    """Solve every frame of g_list against ImgRef on DICmesh `mesh`
    (coordinatesFEM, elementsFEM, optional dirichlet).  Returns a dict of
    per-frame lists: U (2N), U0 (the initial guesses), conv (codes), badnum."""
    c = mesh["coordinatesFEM"]
    el = mesh["elementsFEM"]
    wl = np.asarray(winsize_list, dtype=np.int32)
    N = c.shape[0]
    DP = {"winsize": int(wl.max()), "winsize_per_node": wl}
    predict = lambda T, tt, tp, nb: api.funPOR_GPR(T, tt, tp, nb, ctx=ctx)[0]
    out = {"U": [], "U0": [], "conv": [], "badnum": []}
    for k, g in enumerate(g_list):
        U0 = initial_guess(k, out["U"], U0_first, predict)
        r = api.LocalICGNQuadtree(U0, c, Df, ImgRef, g, DP, "GaussNewton", tol, precision=precision, ctx=ctx)
        U, F, conv, bad = r[0], r[1], r[4], int(r[5])
        U = api.fill_nans(c, el, U, ctx=ctx)
        if admm_steps > 0:
            F2 = np.nan_to_num(api.nodal_strain(c, el, U, ctx=ctx))
            wl2 = np.asfortranarray(np.stack([wl, wl], 1))
            b = beta if beta is not None else 1e-3 * float(winstepsize) ** 2 * mu
            st = api.admm(mesh, Df, ImgRef, g, wl2, U, F2, np.zeros(4 * N), np.zeros(2 * N), mu, b,
                          steps=admm_steps, precision=precision, ctx=ctx)
            U = st["U2"]
        out["U"].append(U)
        out["U0"].append(U0)
        out["conv"].append(conv)
        out["badnum"].append(bad)
    return out
