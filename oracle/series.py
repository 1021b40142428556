"""ORACLE — test infrastructure only.

The accumulative frame loop of main_ALDIC_Quadtree_v2.m (the initial guess
of each frame from the previous results, main_ALDIC_Quadtree_v2.m:179-197)
driven by the oracle's restatements: LocalICGNQuadtree in FP64, the local NaN
fill and funPOR_GPR (oracle/sequence.py).  It is the checker of the
library's series driver (staqdic/series.py); the initial-guess rule itself is
shared with it, so that the two differ only in the routines they call.
"""
import numpy as np


def run_series(mesh, ImgRef, ImgRefMask, g_list, U0_first, winsize_list, tol=1e-2):
    from staqdic.series import initial_guess
    from . import oracle as orc
    from . import sequence as sq
    c, el = mesh["coordinatesFEM"], mesh["elementsFEM"]
    f = np.asarray(ImgRef, dtype=np.float64)
    Df = orc.funImgGradient(f, ImgRefMask)
    wl = np.asarray(winsize_list, dtype=np.int32)
    predict = lambda T, tt, tp, nb: sq.funPOR_GPR(T, tt, tp, nb)[0]
    out = {"U": [], "U0": [], "conv": [], "badnum": []}
    for k, g in enumerate(g_list):
        U0 = initial_guess(k, out["U"], U0_first, predict)
        U, F, Hp, conv, badnum, mark = orc.LocalICGNQuadtree(U0, c, Df, f, np.asarray(g, dtype=np.float64), wl, tol)
        U = orc.fill_nans(c, el, U)
        out["U"].append(U)
        out["U0"].append(U0)
        out["conv"].append(conv)
        out["badnum"].append(int(badnum))
    return out
