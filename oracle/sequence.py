"""ORACLE — test infrastructure only.

NumPy restatement of the sequence initialisation of the reference: the
prediction of a frame's displacement field from the fields of earlier frames
(func/funPOR_GPR.m:1-99, called from main_ALDIC_Quadtree_v2.m:179-197 for
frames after the sixth): a proper orthogonal decomposition of the snapshots
(mean removed; the correlation matrix of the snapshots under the
reference's trapezoid inner product; its eigenvectors give nB modes), then a
Gaussian-process regression of each mode coefficient over time, evaluated at
the time to predict.

The regression stands in for MATLAB's fitrgp(t, a, 'Basis', 'linear',
'FitMethod', 'exact', 'PredictMethod', 'exact', 'SigmaLowerBound', 2e-5), a
closed toolbox function: this restatement follows its documented model (a
squared-exponential kernel, a linear basis whose coefficients are profiled
out, the noise standard deviation at least SigmaLowerBound, hyperparameters
by maximising the exact log marginal likelihood from the documented starting
point [mean(std(t)); std(a)/sqrt(2)], sigma = std(a)/sqrt(2)).  The optimiser
is Nelder-Mead on log-parameters, written out here so that the library and
this checker walk the same path; MATLAB's own optimiser is not restated, so
this boundary is unpinned.
"""
import math

import numpy as np

SIGMA_LOWER = 2e-5


def inner_product(f1, f2):
    """innerproduct of funPOR_GPR.m:88-99: the trapezoid rule on [0, 1] with
    N = len - 1 intervals, times 0.1."""
    y = np.asarray(f1, dtype=np.float64) * np.asarray(f2, dtype=np.float64)
    N = y.size - 1
    s = y[0] / 2 + np.sum(y[1:N]) + y[N] / 2
    return 0.1 / N * s


def _nll(logp, t, y):
    """Negative exact log marginal likelihood of y = H b + f + e with the
    linear basis H = [1 t] profiled out; logp = log(sigma_l, sigma_f, sigma -
    SIGMA_LOWER)."""
    sl, sf = math.exp(logp[0]), math.exp(logp[1])
    sn = SIGMA_LOWER + math.exp(logp[2])
    n = t.size
    d = t[:, None] - t[None, :]
    K = sf * sf * np.exp(-0.5 * d * d / (sl * sl)) + sn * sn * np.eye(n)
    try:
        L = np.linalg.cholesky(K)
    except np.linalg.LinAlgError:
        return 1e300
    H = np.stack([np.ones(n), t], 1)
    Ki = lambda v: np.linalg.solve(L.T, np.linalg.solve(L, v))
    KiH = Ki(H)
    b = np.linalg.solve(H.T @ KiH, H.T @ Ki(y))
    r = y - H @ b
    return 0.5 * float(r @ Ki(r)) + float(np.sum(np.log(np.diag(L)))) + 0.5 * n * math.log(2 * math.pi)


def nelder_mead(f, x0, step=0.5, iters=2000, tol=1e-12):
    """Nelder-Mead (reflection 1, expansion 2, contraction 1/2, shrink 1/2)
    from the simplex x0, x0 + step e_k; stops when the spread of the simplex
    values falls below tol or after iters steps."""
    n = len(x0)
    pts = [np.array(x0, dtype=np.float64)]
    for k in range(n):
        p = np.array(x0, dtype=np.float64)
        p[k] += step
        pts.append(p)
    vals = [f(p) for p in pts]
    for _ in range(iters):
        order = sorted(range(n + 1), key=lambda i: (vals[i], i))
        pts = [pts[i] for i in order]
        vals = [vals[i] for i in order]
        if abs(vals[-1] - vals[0]) <= tol * (abs(vals[0]) + tol):
            break
        c = sum(pts[:-1]) / n
        xr = c + (c - pts[-1])
        fr = f(xr)
        if fr < vals[0]:
            xe = c + 2 * (c - pts[-1])
            fe = f(xe)
            if fe < fr:
                pts[-1], vals[-1] = xe, fe
            else:
                pts[-1], vals[-1] = xr, fr
        elif fr < vals[-2]:
            pts[-1], vals[-1] = xr, fr
        else:
            xc = c + 0.5 * (pts[-1] - c) if fr >= vals[-1] else c + 0.5 * (xr - c)
            fc = f(xc)
            if fc < min(fr, vals[-1]):
                pts[-1], vals[-1] = xc, fc
            else:
                for i in range(1, n + 1):
                    pts[i] = pts[0] + 0.5 * (pts[i] - pts[0])
                    vals[i] = f(pts[i])
    i = min(range(n + 1), key=lambda k: (vals[k], k))
    return pts[i]


def gpr_fit_predict(t, y, t_pre):
    """The regression of one mode: returns (prediction, standard deviation of
    a new observation) at t_pre."""
    t = np.asarray(t, dtype=np.float64).ravel()
    y = np.asarray(y, dtype=np.float64).ravel()
    tp = np.asarray(t_pre, dtype=np.float64).ravel()
    n = t.size
    sd_t = float(np.std(t, ddof=1)) if n > 1 else 1.0
    sd_y = float(np.std(y, ddof=1)) if n > 1 else 1.0
    sl0 = sd_t if sd_t > 0 else 1.0
    sf0 = sd_y / math.sqrt(2) if sd_y > 0 else 1.0
    sn0 = max(sd_y / math.sqrt(2) - SIGMA_LOWER, 1e-12) if sd_y > 0 else 1.0
    p = nelder_mead(lambda q: _nll(q, t, y), [math.log(sl0), math.log(sf0), math.log(sn0)])
    sl, sf = math.exp(p[0]), math.exp(p[1])
    sn = SIGMA_LOWER + math.exp(p[2])
    d = t[:, None] - t[None, :]
    K = sf * sf * np.exp(-0.5 * d * d / (sl * sl)) + sn * sn * np.eye(n)
    H = np.stack([np.ones(n), t], 1)
    Ki = np.linalg.inv(K)
    b = np.linalg.solve(H.T @ Ki @ H, H.T @ Ki @ y)
    alpha = Ki @ (y - H @ b)
    ks = sf * sf * np.exp(-0.5 * (tp[:, None] - t[None, :]) ** 2 / (sl * sl))
    mean = np.stack([np.ones(tp.size), tp], 1) @ b + ks @ alpha
    var = sf * sf - np.einsum("ij,jk,ik->i", ks, Ki, ks) + sn * sn
    return mean, np.sqrt(np.maximum(var, 0.0))


def funPOR_GPR(T_snap, t_train, t_pre, nB):
    """[u_pred, alpha, beta_POD, beta_GPR] = funPOR_GPR(T_snap, t_train, t_pre, nB)
    (func/funPOR_GPR.m:1-99); T_snap is nT x np, u_pred nT1 x np."""
    T = np.asarray(T_snap, dtype=np.float64)
    nT, npt = T.shape
    ave = T.mean(0)
    fp = T - ave
    c = np.empty((nT, nT))
    for k in range(nT):
        for j in range(nT):
            c[k, j] = inner_product(fp[k], fp[j])
    lam, w = np.linalg.eigh(c)
    lam, w = lam[::-1], w[:, ::-1]
    with np.errstate(divide="ignore", invalid="ignore"):
        beta_pod = float((np.log(lam[1]) - np.log(lam[nB + 1])) / nB)
    alpha = float(np.sum(lam[:nB]) / np.sum(lam))
    lamB = lam[:nB]
    fi = (fp.T @ w[:, :nB]).T / np.sqrt(lamB)[:, None]
    a = np.empty((nT, nB))
    for j in range(nT):
        for k in range(nB):
            a[j, k] = inner_product(fp[j], fi[k])
    tp = np.asarray(t_pre, dtype=np.float64).ravel()
    ypred = np.empty((tp.size, nB))
    ysd = np.empty((tp.size, nB))
    for k in range(nB):
        ypred[:, k], ysd[:, k] = gpr_fit_predict(t_train, a[:, k], tp)
    u_pred = ypred @ fi + ave
    sd = ysd @ lamB
    beta_gpr = sd / (np.abs(ypred) @ lamB)
    return u_pred, alpha, beta_pod, beta_gpr
