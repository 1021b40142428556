"""ORACLE — test infrastructure only.

NumPy/SciPy restatement of the multigrid integer search
(func/funIntegerSearchMg.m) and of the pieces it calls: normxcorr2 over the
full lag range (restated from its published definition, like the whole-field
search's restatement in ``staqdic_oracle.cpp``), findpeak (func/findpeak.m) and
gridfit with the 'springs' regularizer and 'triangle' interpolation
(func/gridfit.m).  Only the tests use it, as the checker for a device
implementation of this search; the product never imports it.

Arrays use MATLAB's index order: an image is a (W, H) array indexed
``[x-1, y-1]``; the returned grids are ny x nx (row = y), like the reference.
The quality factors (cc.qfactors) are not restated.
"""
import math

import numpy as np


def _eps(x):
    """MATLAB eps(x) for a positive double: the spacing at x."""
    return np.spacing(abs(float(x))) if x != 0 else np.finfo(float).tiny


def normxcorr2_full(T, A):
    """normxcorr2(T, A): the (M+m-1) x (N+n-1) map of the normalised cross
    correlation of template T (m x n) over A (M x N) zero-padded, entry
    (r, c) (1-based) for the template's top-left at A(r-m+1, c-n+1).
    Lags whose window variance is below sqrt(eps(max |denominator|)) give 0,
    and so do |values| above 1 + sqrt(eps(1)).  Raises ValueError for a
    constant template, as the reference does."""
    T = np.asarray(T, dtype=np.float64)
    A = np.asarray(A, dtype=np.float64)
    m, n = T.shape
    M, N = A.shape
    if not (np.all(np.isfinite(T)) and np.all(np.isfinite(A))):
        raise ValueError("non-finite input")
    if m > M or n > N:
        raise ValueError("template larger than the image")
    mn = m * n
    Tz = T - T.mean()
    stdT = math.sqrt(float((Tz * Tz).sum()) / (mn - 1))
    if not stdT != 0:
        raise ValueError("template cannot have all the same values")
    denT = math.sqrt(mn - 1) * stdT
    R, C = M + m - 1, N + n - 1
    # correlation of the zero-mean template with A at every lag, by FFT
    fr, fc = 1 << (R - 1).bit_length(), 1 << (C - 1).bit_length()
    FA = np.fft.rfft2(A, (fr, fc))
    FT = np.fft.rfft2(Tz[::-1, ::-1], (fr, fc))
    num = np.fft.irfft2(FA * FT, (fr, fc))[:R, :C]
    # window sums of A and A^2 over the m x n window ending at (r, c)
    def wsum(X):
        P = np.zeros((M + 2 * m, N + 2 * n))
        P[m:m + M, n:n + N] = X
        S = np.cumsum(np.cumsum(P, 0), 1)
        S = np.pad(S, ((1, 0), (1, 0)))
        r = np.arange(R) + m + 1
        c = np.arange(C) + n + 1
        return (S[np.ix_(r, c)] - S[np.ix_(r - m, c)] - S[np.ix_(r, c - n)] + S[np.ix_(r - m, c - n)])
    sA, sA2 = wsum(A), wsum(A * A)
    dl = sA2 - sA * sA / mn
    den = denT * np.sqrt(np.maximum(dl, 0.0))
    tol = math.sqrt(_eps(np.max(np.abs(den))))
    out = np.zeros((R, C))
    ok = den > tol
    out[ok] = num[ok] / den[ok]
    out[np.abs(out) - 1 > math.sqrt(_eps(1.0))] = 0.0
    return out


PEAK_TIE = 1e-10


def findpeak(f, subpixel=True):
    """[xpeak, ypeak, max_f] = findpeak(f, subpixel) (func/findpeak.m:27-68):
    the first column-major maximum (x = column, y = row, 1-based), refined by a
    quadratic fit over its 3 x 3 neighbourhood unless it lies on the edge or
    the fit moves it by more than one sample.  Values within PEAK_TIE of the
    maximum count as equal (the first of them is taken): a degenerate map has
    several lags equal in exact arithmetic, which rounding alone would order."""
    f = np.asarray(f, dtype=np.float64)
    flat = f.ravel(order="F")
    imax = int(np.nonzero(flat >= np.max(flat) - PEAK_TIE)[0][0])
    max_f = flat[imax]
    ypeak, xpeak = imax % f.shape[0] + 1, imax // f.shape[0] + 1
    if not subpixel or xpeak == 1 or xpeak == f.shape[1] or ypeak == 1 or ypeak == f.shape[0]:
        return float(xpeak), float(ypeak), float(max_f)
    u = f[ypeak - 2:ypeak + 1, xpeak - 2:xpeak + 1].ravel(order="F")
    x = np.array([-1, -1, -1, 0, 0, 0, 1, 1, 1], dtype=np.float64)
    y = np.array([-1, 0, 1, -1, 0, 1, -1, 0, 1], dtype=np.float64)
    X = np.stack([np.ones(9), x, y, x * y, x * x, y * y], 1)
    Acoef = np.linalg.lstsq(X, u, rcond=None)[0]
    d = Acoef[3] ** 2 - 4 * Acoef[4] * Acoef[5]
    x_off = (-Acoef[2] * Acoef[3] + 2 * Acoef[5] * Acoef[1]) / d
    y_off = -1 / d * (Acoef[3] * Acoef[1] - 2 * Acoef[4] * Acoef[2])
    if abs(x_off) > 1 or abs(y_off) > 1:
        return float(xpeak), float(ypeak), float(max_f)
    x_off = round(1000 * x_off) / 1000
    y_off = round(1000 * y_off) / 1000
    mf = float(np.array([1, x_off, y_off, x_off * y_off, x_off ** 2, y_off ** 2]) @ Acoef)
    return xpeak + x_off, ypeak + y_off, mf


def gridfit_springs(x, y, z, xnodes, ynodes, smoothness=1.0):
    """gridfit(x, y, z, xnodes, ynodes, 'regularizer', 'springs') with its
    defaults (func/gridfit.m): triangle interpolation, autoscale, nodes
    extended to the data, least squares of the stacked system (the
    interpolation rows and the spring rows scaled by smoothness ||A||_1 /
    ||Areg||_1).  Returns the ny x nx grid (row = y)."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    x, y, z = (np.asarray(v, dtype=np.float64).ravel() for v in (x, y, z))
    keep = ~(np.isnan(x) | np.isnan(y) | np.isnan(z))
    x, y, z = x[keep], y[keep], z[keep]
    xnodes = np.array(xnodes, dtype=np.float64).ravel()
    ynodes = np.array(ynodes, dtype=np.float64).ravel()
    if x.size < 3:
        raise ValueError("insufficient data for surface estimation")
    xnodes[0] = min(xnodes[0], x.min())
    xnodes[-1] = max(xnodes[-1], x.max())
    ynodes[0] = min(ynodes[0], y.min())
    ynodes[-1] = max(ynodes[-1], y.max())
    dx, dy = np.diff(xnodes), np.diff(ynodes)
    nx, ny = xnodes.size, ynodes.size
    ngrid = nx * ny
    xscale, yscale = dx.mean(), dy.mean()
    # histc cell indices (1-based), the last node folded into the last cell
    indx = np.searchsorted(xnodes, x, side="right")
    indy = np.searchsorted(ynodes, y, side="right")
    indx[indx == nx] = nx - 1
    indy[indy == ny] = ny - 1
    ind = indy + ny * (indx - 1)  # 1-based column-major grid index
    tx = np.clip((x - xnodes[indx - 1]) / dx[indx - 1], 0, 1)
    ty = np.clip((y - ynodes[indy - 1]) / dy[indy - 1], 0, 1)
    n = x.size
    L = np.where(tx > ty, ny, 1)
    t1, t2 = np.minimum(tx, ty), np.maximum(tx, ty)
    rows = np.repeat(np.arange(n), 3)
    cols = np.stack([ind, ind + ny + 1, ind + L], 1).ravel() - 1
    vals = np.stack([1 - t2, t1, t2 - t1], 1).ravel()
    A = sp.csr_matrix((vals, (rows, cols)), shape=(n, ngrid))
    regs = []
    # springs along y
    i, j = np.meshgrid(np.arange(1, nx + 1), np.arange(1, ny))
    i, j = i.ravel(order="F"), j.ravel(order="F")
    g = j + ny * (i - 1)
    st = 1.0 / (dy[j - 1] / yscale)
    m = g.size
    regs.append(sp.csr_matrix((np.stack([-st, st], 1).ravel(),
                               (np.repeat(np.arange(m), 2), np.stack([g, g + 1], 1).ravel() - 1)), shape=(m, ngrid)))
    # springs along x
    i, j = np.meshgrid(np.arange(1, nx), np.arange(1, ny + 1))
    i, j = i.ravel(order="F"), j.ravel(order="F")
    g = j + ny * (i - 1)
    st = 1.0 / (dx[i - 1] / xscale)
    m = g.size
    regs.append(sp.csr_matrix((np.stack([-st, st], 1).ravel(),
                               (np.repeat(np.arange(m), 2), np.stack([g, g + ny], 1).ravel() - 1)), shape=(m, ngrid)))
    # diagonal springs
    i, j = np.meshgrid(np.arange(1, nx), np.arange(1, ny))
    i, j = i.ravel(order="F"), j.ravel(order="F")
    g = j + ny * (i - 1)
    st = 1.0 / np.sqrt((dx[i - 1] / xscale) ** 2 + (dy[j - 1] / yscale) ** 2)
    m = g.size
    for a, b in ((g, g + ny + 1), (g + 1, g + ny)):
        regs.append(sp.csr_matrix((np.stack([-st, st], 1).ravel(),
                                   (np.repeat(np.arange(m), 2), np.stack([a, b], 1).ravel() - 1)),
                                  shape=(m, ngrid)))
    Areg = sp.vstack(regs).tocsr()
    NA = abs(A).sum(axis=0).max()
    NR = abs(Areg).sum(axis=0).max()
    K = sp.vstack([A, Areg * (smoothness * NA / NR)]).tocsc()
    rhs = np.concatenate([z, np.zeros(Areg.shape[0])])
    sol = spla.spsolve((K.T @ K).tocsc(), K.T @ rhs)
    return sol.reshape((ny, nx), order="F")


def funIntegerSearchMg(f, g, gridx, gridy, winsize, winstepsize, return_blocks=False):
    """[xGrid, yGrid, uGrid, vGrid, ccmax] = funIntegerSearchMg(f, g, gridx,
    gridy, winsize, winstepsize) (func/funIntegerSearchMg.m:3-343): a
    correlation of the whole ROI, then blocks split in halves level by level
    (along the longer side while its aspect exceeds 2), each searched within
    +-5 px of its parent's shift, down to blocks narrower than winsize; the
    block-centre displacements are then fitted to the node grid by gridfit."""
    f = np.asarray(f, dtype=np.float64)
    g = np.asarray(g, dtype=np.float64)
    W, H = f.shape
    gridx = [float(gridx[0]), float(gridx[-1])]
    gridy = [float(gridy[0]), float(gridy[-1])]
    bgx = 1 + round(0.75 * winsize)
    bgy = bgx
    if gridx[0] < bgx: gridx[0] = bgx
    if gridy[0] < bgy: gridy[0] = bgy
    if gridx[1] > W - bgx: gridx[1] = W - bgx
    if gridy[1] > H - bgy: gridy[1] = H - bgy

    def crop(img, x0, x1, y0, y1):
        # img(x0:x1, y0:y1) with MATLAB's errors for fractional or outside indices
        for v in (x0, x1, y0, y1):
            if not np.isfinite(v) or v != int(v):
                raise IndexError("non-integer index")
        x0, x1, y0, y1 = int(x0), int(x1), int(y0), int(y1)
        if x0 < 1 or y0 < 1 or x1 > img.shape[0] or y1 > img.shape[1] or x1 < x0 or y1 < y0:
            raise IndexError("index out of bounds")
        return img[x0 - 1:x1, y0 - 1:y1]

    # level 1 (:16-28)
    Cm = crop(f, gridx[0], gridx[1], gridy[0], gridy[1])
    Dm = crop(g, gridx[0], gridx[1], gridy[0], gridy[1])
    XC = normxcorr2_full(Cm, Dm)
    v1, u1, _ = findpeak(XC, True)
    zd = (math.ceil((XC.shape[0] + 1) / 2), math.ceil((XC.shape[1] + 1) / 2))
    ut, vt = u1 - zd[0], v1 - zd[1]

    def clamp(xf, xg, yf, yg):
        # border gaps and even widths (:31-42, :258-296)
        if xg[0] < bgx: xf[0] += bgx - xg[0]; xg[0] = bgx
        if yg[0] < bgy: yf[0] += bgy - yg[0]; yg[0] = bgy
        if xg[1] > W - bgx: xf[1] += (W - bgx) - xg[1]; xg[1] = W - bgx
        if yg[1] > H - bgy: yf[1] += (H - bgy) - yg[1]; yg[1] = H - bgy
        if (xf[1] - xf[0]) % 2 == 1: xf[1] -= 1; xg[1] -= 1
        if (yf[1] - yf[0]) % 2 == 1: yf[1] -= 1; yg[1] -= 1

    xf, yf = list(gridx), list(gridy)
    xg = [gridx[0] + math.ceil(ut), gridx[1] + math.ceil(ut)]
    yg = [gridy[0] + math.ceil(vt), gridy[1] + math.ceil(vt)]
    clamp(xf, xg, yf, yg)
    wx, wy = xf[1] - xf[0], yf[1] - yf[0]
    blocks = [(list(xf), list(xg), list(yf), list(yg), math.ceil(ut), math.ceil(vt))]
    ratio = wx / wy
    while ratio > 0:
        new = []
        def half(r):
            mid = 0.5 * (r[0] + r[1])
            return [r[0], mid], [mid, r[1]]
        if ratio > 2:
            wxn, wyn = wx / 2, wy
            for (bxf, bxg, byf, byg, bu, bv) in blocks:
                if bxf[1] - bxf[0] > winsize:
                    (a1, a2), (b1, b2) = half(bxf), half(bxg)
                    new += [(a1, b1, list(byf), list(byg), bu, bv), (a2, b2, list(byf), list(byg), bu, bv)]
                else:
                    new += [(list(bxf), list(bxg), list(byf), list(byg), bu, bv)] * 2
        elif ratio < 0.5:
            wxn, wyn = wx, wy / 2
            for (bxf, bxg, byf, byg, bu, bv) in blocks:
                if byf[1] - byf[0] > winsize:
                    (a1, a2), (b1, b2) = half(byf), half(byg)
                    new += [(list(bxf), list(bxg), a1, b1, bu, bv), (list(bxf), list(bxg), a2, b2, bu, bv)]
                else:
                    new += [(list(bxf), list(bxg), list(byf), list(byg), bu, bv)] * 2
        else:
            wxn, wyn = wx / 2, wy / 2
            for (bxf, bxg, byf, byg, bu, bv) in blocks:
                if bxf[1] - bxf[0] > winsize and byf[1] - byf[0] > winsize:
                    (xa, xb), (xga, xgb) = half(bxf), half(bxg)
                    (ya, yb), (yga, ygb) = half(byf), half(byg)
                    new += [(xa, xga, ya, yga, bu, bv), (xb, xgb, ya, yga, bu, bv),
                            (xa, xga, yb, ygb, bu, bv), (xb, xgb, yb, ygb, bu, bv)]
                else:
                    new += [(list(bxf), list(bxg), list(byf), list(byg), bu, bv)] * 4
        us, vs, phis = [], [], []
        for (bxf, bxg, byf, byg, bu, bv) in new:
            try:
                Cb = crop(f, bxf[0], bxf[1], byf[0], byf[1])
                Db = crop(g, bxg[0] - 5, bxg[1] + 5, byg[0] - 5, byg[1] + 5)
                w1, w2 = Cb.shape[0] - 1, Cb.shape[1] - 1
                X = normxcorr2_full(Cb, Db)
                # the column range ends one lag later than the one zero_disp
                # is taken from (funIntegerSearchMg.m:182-183)
                sub = X[w1 - 1:X.shape[0] - w1 + 1, w2 - 1:X.shape[1] - w2 + 2]
                zsub = X[w1 - 1:X.shape[0] - w1 + 1, w2 - 1:X.shape[1] - w2 + 1].shape
                pv, pu, mf = findpeak(sub, True)
                us.append(bu + (pu - math.ceil(zsub[0] / 2)))
                vs.append(bv + (pv - math.ceil(zsub[1] / 2)))
                phis.append(mf)
            except (IndexError, ValueError):
                us.append(np.nan); vs.append(np.nan); phis.append(0.0)
        if wxn < winsize and wyn < winsize:
            break
        blocks = []
        for (bxf, bxg, byf, byg, _, _), u_, v_ in zip(new, us, vs):
            cu = math.ceil(u_) if np.isfinite(u_) else np.nan
            cv = math.ceil(v_) if np.isfinite(v_) else np.nan
            nxf, nyf = list(bxf), list(byf)
            nxg = [bxf[0] + cu, bxf[1] + cu]
            nyg = [byf[0] + cv, byf[1] + cv]
            # the reference runs the clamp for every block: NaN comparisons
            # are false, and the odd-width fix still trims the f range
            clamp(nxf, nxg, nyf, nyg)
            blocks.append((nxf, nxg, nyf, nyg, cu, cv))
        wx, wy = wxn, wyn
        ratio = wx / wy
    # block centres -> the node grid (:300-343)
    tx = np.array([0.5 * (b[0][0] + b[0][1]) for b in new])
    ty = np.array([0.5 * (b[2][0] + b[2][1]) for b in new])
    tu, tv, tp = np.array(us), np.array(vs), np.array(phis)
    ix1, ix2 = int(np.argmin(tx)), int(np.argmax(tx))
    iy1, iy2 = int(np.argmin(ty)), int(np.argmax(ty))
    # np.ceil keeps a NaN shift NaN (MATLAB's ceil), and NaN comparisons are false
    gx1 = np.ceil(1 + 1.25 * winsize + tu[ix1]); gx2 = np.ceil(1 + 1.25 * winsize + tu[ix2])
    gy1 = np.ceil(1 + 1.25 * winsize + tv[iy1]); gy2 = np.ceil(1 + 1.25 * winsize + tv[iy2])
    if gridx[0] < gx1: gridx[0] = gx1
    if gridy[0] < gy1: gridy[0] = gy1
    if gridx[1] > W - gx2 + 1: gridx[1] = W - gx2 + 1
    if gridy[1] > H - gy2 + 1: gridy[1] = H - gy2 + 1
    xList = np.arange(gridx[0], gridx[1] + 1e-9, winstepsize)
    yList = np.arange(gridy[0], gridy[1] + 1e-9, winstepsize)
    sel = (tx > xList.min()) & (tx < xList.max()) & (ty > yList.min()) & (ty < yList.max())
    uG = gridfit_springs(tx[sel], ty[sel], tu[sel], xList, yList)
    vG = gridfit_springs(tx[sel], ty[sel], tv[sel], xList, yList)
    pG = gridfit_springs(tx[sel], ty[sel], tp[sel], xList, yList)
    xG, yG = np.meshgrid(xList, yList)
    if return_blocks:
        # the last level's blocks before the fit: tempx, tempy, tempu, tempv, tempPhi
        return xG, yG, uG, vG, pG, np.stack([tx, ty, tu, tv, tp], 1)
    return xG, yG, uG, vG, pG
