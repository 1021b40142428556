"""ORACLE — test infrastructure only.

NumPy front end of the CPU FP64 restatement in ``staqdic_oracle.cpp``.  Only the
tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` use
it, as the checker (or the timed CPU baseline).  The product never imports it.

Arrays use MATLAB's index order: an image is a (W, H) array indexed ``[x-1,
y-1]`` and stored Fortran-contiguous, exactly the bytes MATLAB holds for
``ImgRef``; ``coordinatesFEM`` is (N, 2); ``elementsFEM`` is (E, 8), 1-based.

Host-side pieces that the reference does in MATLAB after the per-node loops are
restated here in NumPy:
  * bad-subset filters of LocalICGNQuadtree.m:153-177 and Subpb1Quadtree.m:173-191;
  * the free-DOF selection, Dirichlet lift and direct solve of
    Subpb2Quadtree.m:284-346 (``A(Free,Free) \\ b(Free)`` -> SuperLU).
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None
_ref = None

_d = ctypes.POINTER(ctypes.c_double)
_f = ctypes.POINTER(ctypes.c_float)
_u8 = ctypes.POINTER(ctypes.c_uint8)
_i32 = ctypes.POINTER(ctypes.c_int32)
_L = ctypes.c_long


def lib():
    global _lib
    if _lib is None:
        path = _build.oracle_lib_path()
        if not os.path.exists(path):
            _build.build_oracle()
        _lib = ctypes.CDLL(path)
    return _lib


def ref_lib():
    """The reference's compiled ba_interp2.cpp, or None when not built."""
    global _ref
    if _ref is None:
        path = _build.ref_lib_path()
        if not os.path.exists(path):
            return None
        _ref = ctypes.CDLL(path)
    return _ref


def _p(a, t):
    return a.ctypes.data_as(t)


def _F(a, dtype=np.float64):
    return np.asfortranarray(a, dtype=dtype)


def set_threads(n):
    lib().orc_set_num_threads(int(n))


def num_threads():
    return int(lib().orc_num_threads())


# --------------------------------------------------------------------------
# ba_interp2
# --------------------------------------------------------------------------
def ba_interp2(F, X, Y):
    """Z = ba_interp2(F, X, Y, 'cubic') — restatement (ba_interp2.cpp:184-234)."""
    single = F.dtype == np.float32
    dt = np.float32 if single else np.float64
    Fa = _F(F, dt)
    Xa = _F(X, dt)
    Ya = _F(Y, dt)
    out = np.empty(Xa.shape, dtype=dt, order="F")
    M, N = Fa.shape
    if single:
        lib().orc_interp_bicubic_f32(_p(Fa, _f), _L(M), _L(N), _p(Xa, _f), _p(Ya, _f), _L(Xa.size), _p(out, _f))
    else:
        lib().orc_interp_bicubic_f64(_p(Fa, _d), _L(M), _L(N), _p(Xa, _d), _p(Ya, _d), _L(Xa.size), _p(out, _d))
    return out


def ref_ba_interp2(F, X, Y):
    """The reference's own compiled ba_interp2 (None if not built here)."""
    r = ref_lib()
    if r is None:
        return None
    single = F.dtype == np.float32
    dt = np.float32 if single else np.float64
    Fa, Xa, Ya = _F(F, dt), _F(X, dt), _F(Y, dt)
    out = np.empty(Xa.shape, dtype=dt, order="F")
    M, N = Fa.shape
    fn = r.ref_ba_interp2_f32 if single else r.ref_ba_interp2_f64
    t = _f if single else _d
    rc = fn(_p(Fa, t), _L(M), _L(N), _p(Xa, t), _p(Ya, t), _L(Xa.size), _p(out, t))
    if rc != 0:
        raise RuntimeError("reference ba_interp2 raised an error")
    return out


# --------------------------------------------------------------------------
# funImgGradient
# --------------------------------------------------------------------------
def funImgGradient(ImgRef, ImgRefMask=None):
    W, H = ImgRef.shape
    if ImgRefMask is None:
        ImgRefMask = np.ones((W, H), dtype=np.uint8)
    img = _F(ImgRef)
    msk = _F(ImgRefMask, np.uint8)
    dfdx = np.empty((W - 6, H - 6), order="F")
    dfdy = np.empty((W - 6, H - 6), order="F")
    lib().orc_img_gradient(_p(img, _d), _p(msk, _u8), _L(W), _L(H), _p(dfdx, _d), _p(dfdy, _d))
    return {"DfDx": dfdx, "DfDy": dfdy, "DfCropWidth": 3, "imgSize": (W, H),
            "DfAxis": (4, W - 3, 4, H - 3), "ImgRefMask": msk}


# --------------------------------------------------------------------------
# funIntegerSearch (whole field)
# --------------------------------------------------------------------------
def intsearch_grid(W, H, S, gridx, gridy, winsize, winstepsize):
    S, ws, st = _pair(S), _pair(winsize), _pair(winstepsize)
    gx_in = (ctypes.c_double * 2)(*map(float, gridx))
    gy_in = (ctypes.c_double * 2)(*map(float, gridy))
    gx, gy = (ctypes.c_double * 2)(), (ctypes.c_double * 2)()
    nx, ny = _L(), _L()
    lib().orc_intsearch_grid(_L(W), _L(H), int(S[0]), int(S[1]), gx_in, gy_in, int(ws[0]), int(ws[1]),
                             int(st[0]), int(st[1]), gx, gy, ctypes.byref(nx), ctypes.byref(ny))
    return (gx[0], gx[1]), (gy[0], gy[1]), nx.value, ny.value


def _pair(v):
    v = np.atleast_1d(np.asarray(v)).ravel()
    return (v[0], v[0]) if v.size == 1 else (v[0], v[1])


def funIntegerSearch(f, g, S, gridx, gridy, winsize, winstepsize):
    """[x,y,u,v,cc] = funIntegerSearch(f,g,S,gridx,gridy,ws,step,0,step).

    Returns x, y, u, v, ccmax as ny x nx arrays plus the integer argmax
    (row, col) of the cropped correlation map as an (ny, nx, 2) int array.
    """
    W, H = f.shape
    S, ws, st = _pair(S), _pair(winsize), _pair(winstepsize)
    _, _, nx, ny = intsearch_grid(W, H, S, gridx, gridy, ws, st)
    fa, ga = _F(f), _F(g)
    shp = (ny, nx)
    x, y, u, v, cc = (np.empty(shp, order="F") for _ in range(5))
    peak = np.zeros((ny, nx, 2), dtype=np.int32, order="F")
    gx_in = (ctypes.c_double * 2)(*map(float, gridx))
    gy_in = (ctypes.c_double * 2)(*map(float, gridy))
    lib().orc_integer_search(_p(fa, _d), _p(ga, _d), _L(W), _L(H), int(S[0]), int(S[1]), gx_in, gy_in,
                             int(ws[0]), int(ws[1]), int(st[0]), int(st[1]), _p(x, _d), _p(y, _d),
                             _p(u, _d), _p(v, _d), _p(cc, _d), _p(peak, _i32))
    return x, y, u, v, cc, peak


def integer_search_qfactors(f, g, S, gridx, gridy, winsize, winstepsize):
    """cc.qfactors of funIntegerSearch (funIntegerSearch.m:129-131,156,175-176,
    211-264): (raw, normalised), each (ny*nx) x 2 with rows in the reference's
    point order (x fastest); raw holds each point's PCE and PPE (Inf where
    normxcorr2 throws)."""
    W, H = f.shape
    S, ws, st = _pair(S), _pair(winsize), _pair(winstepsize)
    _, _, nx, ny = intsearch_grid(W, H, S, gridx, gridy, ws, st)
    fa, ga = _F(f), _F(g)
    raw = np.empty((nx * ny, 2), order="F")
    qf = np.empty((nx * ny, 2), order="F")
    gx_in = (ctypes.c_double * 2)(*map(float, gridx))
    gy_in = (ctypes.c_double * 2)(*map(float, gridy))
    lib().orc_integer_search_qfactors(_p(fa, _d), _p(ga, _d), _L(W), _L(H), int(S[0]), int(S[1]), gx_in, gy_in,
                                      int(ws[0]), int(ws[1]), int(st[0]), int(st[1]), _p(raw, _d), _p(qf, _d))
    return raw, qf


# --------------------------------------------------------------------------
# LocalICGNQuadtree / funICGNQuadtree
# --------------------------------------------------------------------------
def icgn6(U0, coords, Df, ImgRef, ImgDef, winsize, tol, variant=0):
    """Per-node loop of LocalICGNQuadtree (codes, U, F, HtempPar, hole marks).

    variant=1 selects the masked-g branch as it was before Feb 2024 (used only
    to pin the restatement against the reference's shipped result file)."""
    W, H = ImgRef.shape
    coords = _F(coords)
    N = coords.shape[0]
    U0 = np.ascontiguousarray(U0, dtype=np.float64).ravel()
    U = np.empty(2 * N)
    F = np.empty(4 * N)
    Hp = np.empty((N, 21), order="F")
    conv = np.empty(N, dtype=np.int32)
    mark = np.empty(N, dtype=np.uint8)
    f, g = _F(ImgRef), _F(ImgDef)
    msk = _F(Df["ImgRefMask"], np.uint8)
    wsa = np.atleast_1d(np.asarray(winsize))
    if wsa.size == 1:
        wl, ws0 = None, int(wsa[0])
    else:
        wl, ws0 = np.ascontiguousarray(wsa, dtype=np.int32), 0
    lib().orc_icgn6(_p(f, _d), _p(g, _d), _p(msk, _u8), _p(_F(Df["DfDx"]), _d), _p(_F(Df["DfDy"]), _d),
                    _L(W), _L(H), _p(U0, _d), _p(coords, _d), _L(N), int(ws0),
                    (_p(wl, _i32) if wl is not None else None), ctypes.c_double(tol),
                    _p(U, _d), _p(F, _d), _p(Hp, _d), _p(conv, _i32), _p(mark, _u8), int(variant))
    return U, F, Hp, conv, mark


def icgn2(UOld, FOld, vdual, coords, Df, ImgRef, ImgDef, winsize_list, mu, tol):
    """Per-node loop of Subpb1Quadtree (codes, U)."""
    W, H = ImgRef.shape
    coords = _F(coords)
    N = coords.shape[0]
    wl = _F(winsize_list, np.int32)
    U = np.empty(2 * N)
    conv = np.empty(N, dtype=np.int32)
    f, g = _F(ImgRef), _F(ImgDef)
    msk = _F(Df["ImgRefMask"], np.uint8)
    c = lambda a: np.ascontiguousarray(a, dtype=np.float64).ravel()
    UOld, FOld, vdual = c(UOld), c(FOld), c(vdual)
    lib().orc_icgn2(_p(f, _d), _p(g, _d), _p(msk, _u8), _p(_F(Df["DfDx"]), _d), _p(_F(Df["DfDy"]), _d),
                    _L(W), _L(H), _p(UOld, _d), _p(FOld, _d), _p(vdual, _d), _p(coords, _d), _L(N),
                    _p(wl, _i32), ctypes.c_double(mu), ctypes.c_double(tol), _p(U, _d), _p(conv, _i32))
    return U, conv


def icgn_adjoint(ImgRef, ImgDef, mask, coords, winsize, U, F, want_dg=True):
    """Subset ZNSSD costs and their gradients (FP64; no reference counterpart).

    Returns cost (N), dU (2N), dF (4N) and dg (W x H, None unless want_dg)."""
    W, H = ImgRef.shape
    coords = _F(coords)
    N = coords.shape[0]
    f, g = _F(ImgRef), _F(ImgDef)
    msk = None if mask is None else _F(mask, np.uint8)
    wsa = np.atleast_1d(np.asarray(winsize))
    if wsa.size == 1:
        wl, ws0 = None, int(wsa[0])
    else:
        wl, ws0 = np.ascontiguousarray(wsa, dtype=np.int32), 0
    c = lambda a: np.ascontiguousarray(a, dtype=np.float64).ravel()
    U, F = c(U), c(F)
    cost = np.empty(N)
    dU = np.empty(2 * N)
    dF = np.empty(4 * N)
    dg = np.zeros((W, H), order="F") if want_dg else None
    lib().orc_adjoint(_p(f, _d), _p(g, _d), _p(msk, _u8) if msk is not None else None, _L(W), _L(H),
                      _p(coords, _d), _L(N), int(ws0), (_p(wl, _i32) if wl is not None else None),
                      _p(U, _d), _p(F, _d), _p(cost, _d), _p(dU, _d), _p(dF, _d),
                      _p(dg, _d) if want_dg else None)
    return cost, dU, dF, dg


def nodal_strain(coords, elems, U, gauss_order=2):
    """Nodal F = [du/dx dv/dx du/dy dv/dy] per node (4N) from the element
    Gauss-point strains (see orc_nodal_strain)."""
    coords = _F(coords)
    el = _F(elems, np.int32)
    N, E = coords.shape[0], el.shape[0]
    U = np.ascontiguousarray(U, dtype=np.float64).ravel()
    F = np.empty(4 * N)
    lib().orc_nodal_strain(_p(coords, _d), _L(N), _p(el, _i32), _L(E), _p(U, _d), int(gauss_order),
                           _p(F, _d))
    return F


def fill_nans(coords, elems, U):
    """U (2N) with NaN nodes filled from their mesh neighbours (see orc_fill_nans)."""
    coords = _F(coords)
    el = _F(elems, np.int32)
    N, E = coords.shape[0], el.shape[0]
    out = np.array(U, dtype=np.float64).ravel().copy()
    lib().orc_fill_nans(_p(coords, _d), _L(N), _p(el, _i32), _L(E), _p(out, _d))
    return out


def bad_points_local(conv, maxIterNum=100):
    """LocalICGNQuadtree.m:153-169 -> (bad index array, LocalICGNBadPtNum)."""
    conv = np.asarray(conv)
    n = conv.size
    row1 = np.nonzero(conv < 0)[0]
    row2 = np.nonzero(conv > maxIterNum - 1)[0]
    row3 = np.nonzero(conv == maxIterNum + 2)[0]
    bad = np.union1d(row1, row2)
    badnum = bad.size - row3.size
    good = np.setdiff1d(np.arange(n), bad)
    vals = conv[good].astype(np.float64)
    mu = vals.mean() if vals.size else np.nan
    sig = vals.std(ddof=1) if vals.size > 1 else (0.0 if vals.size == 1 else np.nan)
    thr = np.nanmax([mu + 1 * sig, 6])
    row4 = np.nonzero(conv > thr)[0]
    return np.union1d(bad, row4), int(badnum)


def bad_points_subpb1(conv, maxIterNum=100):
    """Subpb1Quadtree.m:173-186."""
    conv = np.asarray(conv)
    n = conv.size
    row1 = np.nonzero(conv < 0)[0]
    row2 = np.nonzero(conv > maxIterNum - 1)[0]
    row3 = np.nonzero(conv == maxIterNum + 2)[0]
    bad = np.union1d(row1, row2)
    badnum = bad.size - row3.size
    good = np.setdiff1d(np.arange(n), bad)
    vals = conv[good].astype(np.float64)
    mu = vals.mean() if vals.size else np.nan
    sig = vals.std(ddof=1) if vals.size > 1 else (0.0 if vals.size == 1 else np.nan)
    thr = np.nanmax([mu + 0.25 * sig, 10])
    row4 = np.nonzero(conv > thr)[0]
    return np.union1d(bad, row4), int(badnum)


def LocalICGNQuadtree(U0, coords, Df, ImgRef, ImgDef, winsize, tol):
    """LocalICGNQuadtree without its NaN-fill tail: U/F carry NaN at bad nodes."""
    U, F, Hp, conv, mark = icgn6(U0, coords, Df, ImgRef, ImgDef, winsize, tol)
    bad, badnum = bad_points_local(conv)
    U = U.copy(); F = F.copy()
    U[2 * bad] = np.nan; U[2 * bad + 1] = np.nan
    for k in range(4):
        F[4 * bad + k] = np.nan
    return U, F, Hp, conv, badnum, np.nonzero(mark)[0] + 1


# --------------------------------------------------------------------------
# Subpb2Quadtree
# --------------------------------------------------------------------------
def subpb2_system(coords, elems, gauss_order, beta, mu, U, F, alpha=0.0):
    """Element loop + sparse() assembly: returns (A csc, b) over 2N+8 DOFs."""
    import scipy.sparse as sp
    coords = _F(coords)
    elems = _F(elems, np.int32)
    N = coords.shape[0]
    E = elems.shape[0]
    I = np.empty(E * 256, dtype=np.int32)
    J = np.empty(E * 256, dtype=np.int32)
    V = np.empty(E * 256)
    b = np.empty(2 * N + 8)
    Uc = np.ascontiguousarray(U, dtype=np.float64).ravel()
    Fc = np.ascontiguousarray(F, dtype=np.float64).ravel()
    rc = lib().orc_subpb2_assemble(_p(coords, _d), _L(N), _p(elems, _i32), _L(E), int(gauss_order),
                                   ctypes.c_double(beta), ctypes.c_double(mu), ctypes.c_double(alpha),
                                   _p(Uc, _d), _p(Fc, _d), _p(I, _i32), _p(J, _i32), _p(V, _d), _p(b, _d))
    if rc != 0:
        raise ValueError("unsupported Gauss order")
    n = 2 * N + 8
    A = sp.csc_matrix((V, (I - 1, J - 1)), shape=(n, n))
    return A, b


def Subpb2Quadtree(coords, elems, dirichlet, neumann, gauss_order, beta, mu, U, F, alpha,
                   winstepsize):
    """Uhat = Subpb2Quadtree(DICmesh, GaussPtOrder, beta, mu, U, F, udual, vdual,
    alpha, winstepsize, ~) with the duals multiplied by zero as the reference does
    (Subpb2Quadtree.m:42-44)."""
    import scipy.sparse.linalg as spla
    N = np.asarray(coords).shape[0]
    A, b = subpb2_system(coords, elems, gauss_order, beta, mu, U, F, alpha)
    n = 2 * N + 8
    Uc = np.ascontiguousarray(U, dtype=np.float64).ravel()
    Fp = np.concatenate([np.ascontiguousarray(F, dtype=np.float64).ravel(), np.zeros(16)])
    # coordsIndexInvolved = unique(elementsFEM(:,1:8)), first entry dropped
    inv = np.unique(np.asarray(elems)[:, :8])
    inv = inv[1:]
    uinv = np.empty(2 * inv.size, dtype=np.int64)
    uinv[0::2] = 2 * inv - 1
    uinv[1::2] = 2 * inv
    dirichlet = np.asarray(dirichlet, dtype=np.int64).ravel()
    dtemp = np.concatenate([2 * dirichlet, 2 * dirichlet - 1]) if dirichlet.size else np.zeros(0, np.int64)
    free = np.setdiff1d(uinv, np.unique(dtemp))
    coords_a = np.asarray(coords, dtype=np.float64)
    BCForce = -1.0 / winstepsize * Fp
    b = b.copy()
    if neumann is not None:
        for row in np.asarray(neumann).reshape(-1, 4):
            n1, n2, nx_, ny_ = int(row[0]), int(row[1]), row[2], row[3]
            ln = 0.5 * np.linalg.norm(coords_a[n1 - 1] - coords_a[n2 - 1])
            for nd in (n1, n2):
                b[2 * nd - 2] += ln * (BCForce[4 * nd - 4] * nx_ + BCForce[4 * nd - 2] * ny_)
                b[2 * nd - 1] += ln * (BCForce[4 * nd - 3] * nx_ + BCForce[4 * nd - 1] * ny_)
    Uhat = np.zeros(n)
    ud = np.unique(dirichlet)
    if ud.size:
        Uhat[2 * ud - 1] = Uc[2 * ud - 1]
        Uhat[2 * ud - 2] = Uc[2 * ud - 2]
    b = b - A @ Uhat
    fz = free - 1
    if fz.size:
        Uhat[fz] = spla.spsolve(A[fz][:, fz].tocsc(), b[fz])
    return Uhat[:2 * N].copy()
