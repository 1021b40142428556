"""Host mirror of the reference's MATLAB interface on the hot path.

Same names, argument meaning and outputs as the reference routines, computed
on the GPU through the C ABI (include/staqdic.h):

  ba_interp2            ba_interp2.cpp:318-335
  funImgGradient        func/funImgGradient.m:1-88
  funIntegerSearch      func/funIntegerSearch.m:3-80 (whole-field mode)
  funICGNQuadtree       func_quadtree/funICGNQuadtree.m:1-451 (one node)
  LocalICGNQuadtree     func_quadtree/LocalICGNQuadtree.m:1-177
  Subpb1Quadtree        func_quadtree/Subpb1Quadtree.m:1-191
  Subpb2Quadtree        func_quadtree/Subpb2Quadtree.m:1-413
  GenerateQuadtreeMesh  func_quadtree/GenerateQuadtreeMesh.m:18-133 (with MeshSetUp.m)
  funPOR_GPR            func/funPOR_GPR.m:1-99

Array conventions are MATLAB's: NumPy arrays indexed like the MATLAB array
(0-based), laid out column-major (Fortran order) exactly as MATLAB stores them;
an image is (W, H) with ``Img[x-1, y-1]``.  Torch CUDA tensors are accepted as
raw column-major buffers and keep results on the device.

The NaN-fill tails of LocalICGNQuadtree / Subpb1Quadtree (RBF and
scatteredInterpolant over the bad subsets) are not part of this path: the
returned U / F keep NaN at the bad subsets.  Only 'GaussNewton' exists (the
reference's 'LevenbergMarquardt' branch calls ImgDef.eval on a spline object
and cannot run on image arrays).
"""
import time

import numpy as np

from . import _lib
from ._lib import Frame, default_context

try:  # torch is optional plumbing for device-resident buffers
    import torch
except Exception:  # pragma: no cover
    torch = None

PRECISIONS = {"plain": _lib.STDIC_PLAIN_F64, "batched": _lib.STDIC_BATCHED_F32,
              _lib.STDIC_PLAIN_F64: _lib.STDIC_PLAIN_F64,
              _lib.STDIC_BATCHED_F32: _lib.STDIC_BATCHED_F32}


def _is_torch(a):
    return torch is not None and isinstance(a, torch.Tensor)


class _Bufs:
    """Keeps the buffers of one call alive and hands out raw pointers.

    A torch CUDA buffer binds the context to torch's current stream first, so
    torch's producers of the inputs and consumers of the outputs are ordered
    with the call without a synchronisation (the library synchronises only
    when it stages host buffers).  torch's default stream is the legacy
    default stream, which the context's own (blocking) stream is already
    ordered with: that case keeps the context's own stream."""

    def __init__(self, ctx):
        self.keep = []
        self.ctx = ctx

    def _bind(self, t):
        if t.is_cuda:
            s = torch.cuda.current_stream(t.device).cuda_stream or None
            if getattr(self.ctx, "_torch_stream", None) != s:
                self.ctx.set_stream(s)

    def ptr(self, a, dtype):
        if a is None:
            return None
        if _is_torch(a):
            self._bind(a)
            tdt = {np.float64: torch.float64, np.float32: torch.float32, np.int32: torch.int32,
                   np.uint8: torch.uint8}[np.dtype(dtype).type]
            if a.dtype != tdt or not a.is_contiguous():
                a = a.to(tdt).contiguous()
            self.keep.append(a)
            return a.data_ptr()
        arr = np.asfortranarray(a, dtype=dtype)
        self.keep.append(arr)
        return arr.ctypes.data

    def out(self, like, shape, dtype):
        """Output buffer on the device when `like` is a CUDA tensor, else NumPy."""
        if _is_torch(like) and like.is_cuda:
            self._bind(like)
            tdt = {np.float64: torch.float64, np.float32: torch.float32, np.int32: torch.int32,
                   np.uint8: torch.uint8}[np.dtype(dtype).type]
            t = torch.empty(int(np.prod(shape)), dtype=tdt, device=like.device)
            self.keep.append(t)
            return t, t.data_ptr()
        arr = np.empty(shape, dtype=dtype, order="F")
        self.keep.append(arr)
        return arr, arr.ctypes.data


def _ctx(ctx):
    return ctx if ctx is not None else default_context()


def _nodes(coords):
    """N of an N x 2 coordinate array (torch buffers may be flat, 2N long)."""
    if _is_torch(coords):
        return int(coords.numel()) // 2
    return int(np.asarray(coords).shape[0])


def _shape2(a):
    if _is_torch(a):
        raise ValueError("pass (W, H) explicitly for torch buffers")
    return a.shape


# ---------------------------------------------------------------------------
def ba_interp2(F, X, Y, method="cubic", ctx=None):
    """Z = ba_interp2(F, X, Y, 'cubic'): F is M x N (x P), X/Y any shape."""
    if str(method).lower() != "cubic":
        raise ValueError("ba_interp2 only implements 'cubic' (the reference keeps only bicubic)")
    c = _ctx(ctx)
    single = (F.dtype == np.float32) if not _is_torch(F) else F.dtype == torch.float32
    dt = np.float32 if single else np.float64
    shp = tuple(F.shape)
    M, N = shp[0], shp[1]
    P = int(np.prod(shp[2:])) if len(shp) > 2 else 1
    xs = tuple(X.shape)
    n = int(np.prod(xs))
    b = _Bufs(c)
    pF, pX, pY = b.ptr(F, dt), b.ptr(X, dt), b.ptr(Y, dt)
    out_shape = xs + tuple(shp[2:])
    Z, pZ = b.out(X, out_shape, dt)
    c.check(c.L.stdic_interp_bicubic(c.h, pF, M, N, P, pX, pY, n, pZ,
                                     _lib.STDIC_F32 if single else _lib.STDIC_F64), "ba_interp2")
    return Z


def funImgGradient(ImgRef, ImgDef=None, ImgRefMask=None, ctx=None, dtype=None):
    """Df = funImgGradient(ImgRef, ImgDef, ImgRefMask) (finite-difference mode)."""
    c = _ctx(ctx)
    W, H = _shape2(ImgRef)
    if ImgRefMask is None:
        ImgRefMask = np.ones((W, H), dtype=np.uint8, order="F")
    if dtype is None:
        dtype = np.float32 if ImgRef.dtype == np.float32 else np.float64
    b = _Bufs(c)
    pi = b.ptr(ImgRef, dtype)
    pm = b.ptr((np.asarray(ImgRefMask) != 0).astype(np.uint8), np.uint8)
    dx, pdx = b.out(None, (W - 6, H - 6), dtype)
    dy, pdy = b.out(None, (W - 6, H - 6), dtype)
    c.check(c.L.stdic_img_gradient(c.h, pi, pm, W, H, pdx, pdy,
                                   _lib.STDIC_F32 if dtype == np.float32 else _lib.STDIC_F64),
            "funImgGradient")
    return {"DfDx": dx, "DfDy": dy, "DfCropWidth": 3, "imgSize": (W, H),
            "DfAxis": (4, W - 3, 4, H - 3),
            "ImgRefMask": np.asfortranarray((np.asarray(ImgRefMask) != 0).astype(np.uint8))}


def _pair(v):
    v = np.atleast_1d(np.asarray(v)).ravel()
    return (v[0], v[0]) if v.size == 1 else (v[0], v[1])


def funIntegerSearch(f, g, tempSizeOfSearchRegion, gridx, gridy, winsize, winstepsize,
                     tempNoOfInitPt=0, *varargin, ctx=None, qfactors=True):
    """[x,y,u,v,cc] = funIntegerSearch(f,g,S,gridx,gridy,winsize,winstepsize,0,..).

    cc is a dict with 'max' (cc.max), 'qfactors' (cc.qfactors: (ny*nx) x 2, the
    normalised PCE and PPE of each point's full correlation map, rows in the
    reference's point order, x fastest; omitted with qfactors=False) and 'peak'
    (the 1-based integer argmax (row, col) of each cropped correlation map,
    ny x nx x 2)."""
    if tempNoOfInitPt != 0:
        raise NotImplementedError("only the whole-field mode (tempNoOfInitPt = 0) is on this path")
    c = _ctx(ctx)
    W, H = _shape2(f)
    S = np.asarray(_pair(tempSizeOfSearchRegion), dtype=np.int32)
    ws = np.asarray(_pair(winsize), dtype=np.int32)
    st = np.asarray(_pair(winstepsize), dtype=np.int32)
    gx = np.asarray([gridx[0], gridx[-1]], dtype=np.float64)
    gy = np.asarray([gridy[0], gridy[-1]], dtype=np.float64)
    I = lambda a: a.ctypes.data_as(_lib._i32)
    D = lambda a: a.ctypes.data_as(_lib._d)
    nx, ny = _lib._c.c_int(), _lib._c.c_int()
    c.check(c.L.stdic_integer_search_grid(W, H, I(S), D(gx), D(gy), I(ws), I(st),
                                          _lib._c.byref(nx), _lib._c.byref(ny)), "grid")
    nx, ny = nx.value, ny.value
    b = _Bufs(c)
    pf, pg = b.ptr(f, np.float64), b.ptr(g, np.float64)
    outs = [b.out(None, (ny, nx), np.float64) for _ in range(5)]
    peak, pp = b.out(None, (ny, nx, 2), np.int32)
    qf, pq = b.out(None, (nx * ny, 2), np.float64) if qfactors else (None, None)
    c.check(c.L.stdic_integer_search(c.h, pf, pg, W, H, I(S), D(gx), D(gy), I(ws), I(st),
                                     *[o[1] for o in outs], pp, pq), "funIntegerSearch")
    x, y, u, v, cm = (o[0] for o in outs)
    cc = {"max": cm, "peak": peak}
    if qfactors:
        cc["qfactors"] = qf
    return x, y, u, v, cc


def funIntegerSearchMg(f, g, gridx, gridy, winsize, winstepsize, *varargin, ctx=None, blocks=False):
    """[xGrid,yGrid,uGrid,vGrid,cc] = funIntegerSearchMg(f,g,gridx,gridy,winsize,winstepsize)
    (stdic_integer_search_mg): the multigrid search for large displacements.
    Outputs are ny x nx (row = y); cc is a dict with 'max' (cc.max) and, with
    blocks=True, 'blocks': the last level's blocks before gridfit (nblocks x 5:
    centre x, centre y, u, v, cc.max).  The reference's cc.qfactors are not
    produced (its caller on this path, IntegerSearch.m, does not read them)."""
    c = _ctx(ctx)
    W, H = _shape2(f)
    st = np.asarray(_pair(winstepsize), dtype=np.float64)
    gx = np.asarray([gridx[0], gridx[-1]], dtype=np.float64)
    gy = np.asarray([gridy[0], gridy[-1]], dtype=np.float64)
    cap = (int((gx[1] - gx[0]) // st[0]) + 1) * (int((gy[1] - gy[0]) // st[1]) + 1)
    cap = max(cap, 4)
    b = _Bufs(c)
    pf, pg = b.ptr(f, np.float64), b.ptr(g, np.float64)
    outs = [np.empty(cap) for _ in range(5)]
    counts = np.zeros(2, dtype=np.int32)
    nbl = np.zeros(1, dtype=np.int64)
    # the library refuses searches of more than 65535 last-level blocks
    bcap = 65535 if blocks else 0
    bl = np.empty(5 * bcap) if blocks else None
    D = lambda a: a.ctypes.data_as(_lib._d)
    c.check(c.L.stdic_integer_search_mg(c.h, pf, pg, W, H, D(gx), D(gy), int(_pair(winsize)[0]), D(st),
                                        *[o.ctypes.data for o in outs], cap, counts.ctypes.data,
                                        bl.ctypes.data if blocks else None, bcap, nbl.ctypes.data),
            "funIntegerSearchMg")
    nx, ny = int(counts[0]), int(counts[1])
    x, y, u, v, cm = (o[:nx * ny].reshape((ny, nx), order="F") for o in outs)
    cc = {"max": cm}
    if blocks:
        nb = int(nbl[0])
        cc["blocks"] = np.stack([bl[k * nb:(k + 1) * nb] for k in range(5)], 1)
    return x, y, u, v, cc


# ---------------------------------------------------------------------------
def _frame(b, Df, ImgRef, ImgDef, dtype, frames=1):
    W, H = Df["imgSize"]
    fr = Frame()
    fr.f = b.ptr(ImgRef, dtype)
    fr.g = b.ptr(ImgDef, dtype)
    fr.mask = b.ptr(Df["ImgRefMask"], np.uint8)
    fr.dfdx = b.ptr(Df["DfDx"], dtype)
    fr.dfdy = b.ptr(Df["DfDy"], dtype)
    fr.W, fr.H = int(W), int(H)
    fr.dtype = _lib.STDIC_F32 if dtype == np.float32 else _lib.STDIC_F64
    return fr


def _data_dtype(precision, ImgRef):
    if precision == _lib.STDIC_PLAIN_F64:
        return np.float64
    isf32 = (ImgRef.dtype == np.float32) if not _is_torch(ImgRef) else ImgRef.dtype == torch.float32
    return np.float32 if isf32 else np.float64


def LocalICGNQuadtree(U0, coordinatesFEM, Df, ImgRef, ImgDef, DICpara, ICGNmethod="GaussNewton",
                      tol=1e-2, precision="plain", ctx=None):
    """[U,F,HtempPar,LocalTime,ConvItPerEle,LocalICGNBadPtNum,markCoordHoleStrain] =
    LocalICGNQuadtree(U0,coordinatesFEM,Df,ImgRef,ImgDef,DICpara,'GaussNewton',tol).

    DICpara['winsize'] is the subset size; an optional DICpara['winsize_per_node']
    (N) gives one size per node (its maximum must not exceed winsize).
    markCoordHoleStrain is 1-based, like MATLAB's find()."""
    if ICGNmethod != "GaussNewton":
        raise NotImplementedError("only 'GaussNewton' exists on this path")
    c = _ctx(ctx)
    prec = PRECISIONS[precision]
    dtype = _data_dtype(prec, ImgRef)
    N = _nodes(coordinatesFEM)
    b = _Bufs(c)
    fr = _frame(b, Df, ImgRef, ImgDef, dtype)
    wl = DICpara.get("winsize_per_node")
    ws = int(DICpara["winsize"]) if wl is None else int(max(int(DICpara["winsize"]), int(np.max(wl))))
    like = U0 if _is_torch(U0) else None
    U, pU = b.out(like, (2 * N,), np.float64)
    F, pF = b.out(like, (4 * N,), np.float64)
    Hp, pH = b.out(like, (N, 21), np.float64)
    conv, pc = b.out(like, (N,), np.int32)
    mark, pm = b.out(like, (N,), np.uint8)
    badnum = _lib._c.c_int(0)
    t0 = time.perf_counter()
    c.check(c.L.stdic_icgn_local(c.h, _lib._c.byref(fr), b.ptr(U0, np.float64),
                                 b.ptr(coordinatesFEM, np.float64), N, ws,
                                 b.ptr(wl, np.int32) if wl is not None else None, float(tol),
                                 pU, pF, pH, pc, pm, _lib._c.byref(badnum), prec),
            "LocalICGNQuadtree")
    LocalTime = time.perf_counter() - t0
    if _is_torch(mark):
        markCoord = torch.nonzero(mark).flatten() + 1
    else:
        markCoord = np.nonzero(mark)[0] + 1
    return U, F, Hp, LocalTime, conv, int(badnum.value), markCoord


def funICGNQuadtree(U0, x0, y0, Df, ImgRef, ImgDef, winsize, tol, ICGNmethod="GaussNewton",
                    ctx=None):
    """[U,F,stepwithinwhile,HGlobal] = funICGNQuadtree(U0,x0,y0,Df,ImgRef,ImgDef,winsize,tol,method)
    for one node on the plain FP64 path.  A MATLAB run-time error of the
    reference routine is raised here as RuntimeError, as MATLAB would."""
    if ICGNmethod != "GaussNewton":
        raise NotImplementedError("only 'GaussNewton' exists on this path")
    U, F, Hp, conv = icgn_subsets(np.asarray(U0, dtype=np.float64).ravel()[:2],
                                  np.asarray([[float(x0), float(y0)]]), Df, ImgRef, ImgDef,
                                  winsize, tol, "plain", ctx=ctx)
    if int(conv[0]) == -1:
        raise RuntimeError("funICGNQuadtree raised a MATLAB run-time error for this subset")
    return U, F, int(conv[0]), np.asarray(Hp).ravel()


def icgn_subsets(U0, coordinatesFEM, Df, ImgRef, ImgDef, winsize, tol, precision="plain",
                 ws_list=None, ctx=None):
    """funICGNQuadtree over N nodes at once (no bad-subset filter):
    returns U (2N), F (4N), HGlobal (N x 21), ConvItPerEle (N)."""
    c = _ctx(ctx)
    prec = PRECISIONS[precision]
    dtype = _data_dtype(prec, ImgRef)
    N = _nodes(coordinatesFEM)
    b = _Bufs(c)
    fr = _frame(b, Df, ImgRef, ImgDef, dtype)
    ws = int(winsize) if ws_list is None else int(max(int(winsize), int(np.max(ws_list))))
    like = U0 if _is_torch(U0) else None
    U, pU = b.out(like, (2 * N,), np.float64)
    F, pF = b.out(like, (4 * N,), np.float64)
    Hp, pH = b.out(like, (N, 21), np.float64)
    conv, pc = b.out(like, (N,), np.int32)
    c.check(c.L.stdic_icgn_subsets(c.h, _lib._c.byref(fr), b.ptr(U0, np.float64),
                                   b.ptr(coordinatesFEM, np.float64), N, ws,
                                   b.ptr(ws_list, np.int32) if ws_list is not None else None,
                                   float(tol), pU, pF, pH, pc, prec), "funICGNQuadtree")
    return U, F, Hp, conv


def subpb1_subsets(UOld, FOld, vdual, coordinatesFEM, Df, ImgRef, ImgDef, winsize_List, mu, tol,
                   precision="plain", ctx=None):
    """funICGN_Subpb1 over N nodes at once (no bad-subset filter): U (2N), codes (N)."""
    c = _ctx(ctx)
    prec = PRECISIONS[precision]
    dtype = _data_dtype(prec, ImgRef)
    N = _nodes(coordinatesFEM)
    b = _Bufs(c)
    fr = _frame(b, Df, ImgRef, ImgDef, dtype)
    like = UOld if _is_torch(UOld) else None
    U, pU = b.out(like, (2 * N,), np.float64)
    conv, pc = b.out(like, (N,), np.int32)
    c.check(c.L.stdic_subpb1_subsets(c.h, _lib._c.byref(fr), b.ptr(UOld, np.float64),
                                     b.ptr(FOld, np.float64), b.ptr(vdual, np.float64),
                                     b.ptr(coordinatesFEM, np.float64), N,
                                     b.ptr(winsize_List, np.int32), float(mu), float(tol), pU, pc,
                                     prec), "funICGN_Subpb1")
    return U, conv


def Subpb1Quadtree(UOld, FOld, udual, vdual, coordinatesFEM, Df, ImgRef, ImgDef, mu, beta, HPar,
                   ALSolveStep, DICpara, ICGNmethod="GaussNewton", tol=1e-2, precision="plain",
                   ctx=None):
    """[U,HPar,ALSub1Time,ConvItPerEle,LocalICGNBadPtNum] = Subpb1Quadtree(...) for
    ALSolveStep > 1 (the driver's only use).  HPar is returned unchanged."""
    if ICGNmethod != "GaussNewton":
        raise NotImplementedError("only 'GaussNewton' exists on this path")
    if ALSolveStep <= 1:
        raise NotImplementedError("Subpb1Quadtree is called with ALSolveStep > 1 by the reference driver")
    c = _ctx(ctx)
    prec = PRECISIONS[precision]
    dtype = _data_dtype(prec, ImgRef)
    N = _nodes(coordinatesFEM)
    b = _Bufs(c)
    fr = _frame(b, Df, ImgRef, ImgDef, dtype)
    wl = DICpara["winsize_List"]
    like = UOld if _is_torch(UOld) else None
    U, pU = b.out(like, (2 * N,), np.float64)
    conv, pc = b.out(like, (N,), np.int32)
    badnum = _lib._c.c_int(0)
    t0 = time.perf_counter()
    c.check(c.L.stdic_subpb1(c.h, _lib._c.byref(fr), b.ptr(UOld, np.float64), b.ptr(FOld, np.float64),
                             b.ptr(udual, np.float64) if udual is not None else None,
                             b.ptr(vdual, np.float64), b.ptr(coordinatesFEM, np.float64), N,
                             b.ptr(wl, np.int32), float(mu), float(beta), float(tol), pU, pc,
                             _lib._c.byref(badnum), prec), "Subpb1Quadtree")
    return U, HPar, time.perf_counter() - t0, conv, int(badnum.value)


def Subpb2Quadtree(DICmesh, GaussPtOrder, beta, mu, U, F, udual, vdual, alpha, winstepsize,
                   waitBarDisplayOrNot=0, tol=1e-10, maxit=0, ctx=None, return_iters=False):
    """Uhat = Subpb2Quadtree(DICmesh,GaussPtOrder,beta,mu,U,F,udual,vdual,alpha,winstepsize,~).

    The duals enter the reference multiplied by zero (Subpb2Quadtree.m:42-44)."""
    c = _ctx(ctx)
    coords = DICmesh["coordinatesFEM"]
    elems = DICmesh["elementsFEM"]
    dirichlet = DICmesh.get("dirichlet")
    neumann = DICmesh.get("neumann")
    N = _nodes(coords)
    E = int(elems.shape[0])
    nd = 0 if dirichlet is None else int(np.asarray(dirichlet).size) if not _is_torch(dirichlet) else dirichlet.numel()
    nn = 0 if neumann is None or np.asarray(neumann).size == 0 else int(np.asarray(neumann).reshape(-1, 4).shape[0])
    b = _Bufs(c)
    like = U if _is_torch(U) else None
    Uhat, pu = b.out(like, (2 * N,), np.float64)
    iters = _lib._c.c_int(0)
    rc = c.L.stdic_subpb2(c.h, b.ptr(coords, np.float64), N, b.ptr(elems, np.int32), E,
                          b.ptr(dirichlet, np.int32) if nd else None, nd,
                          b.ptr(np.asarray(neumann).reshape(-1, 4), np.float64) if nn else None, nn,
                          int(GaussPtOrder), float(beta), float(mu), b.ptr(U, np.float64),
                          b.ptr(F, np.float64), float(alpha), float(winstepsize), float(tol),
                          int(maxit), pu, _lib._c.byref(iters))
    c.check(rc, "Subpb2Quadtree")
    if return_iters:
        return Uhat, int(iters.value)
    return Uhat


def GenerateQuadtreeMesh(x0, y0, ImgRefMask, winstepsize, elementMinSize=2, ctx=None):
    """DICmesh of GenerateQuadtreeMesh.m (stdic_quadtree_mesh): the uniform
    mesh MeshSetUp.m builds on the search grids x0, y0 (N x M, row = y, as
    MeshSetUp receives them), refined at the edges of ImgRefMask.  Returns a
    dict with coordinatesFEM (N x 2), elementsFEM (E x 8 int32), irregular
    (nI x 3), dirichlet and markCoordHoleEdge (the same set) and
    elementMinSize, numbered as the reference numbers them."""
    c = _ctx(ctx)
    x0 = np.asfortranarray(x0, dtype=np.float64)
    y0 = np.asfortranarray(y0, dtype=np.float64)
    ny, nx = x0.shape
    m = np.asfortranarray((np.asarray(ImgRefMask) != 0).astype(np.uint8))
    W, H = m.shape
    step = float(np.max(np.atleast_1d(winstepsize)))
    counts = np.zeros(4, dtype=np.int64)
    P = lambda a: a.ctypes.data if a is not None else None
    c.check(c.L.stdic_quadtree_mesh(c.h, P(m), W, H, P(x0), P(y0), ny, nx, step, float(elementMinSize), None,
                                    None, None, None, None, P(counts)), "GenerateQuadtreeMesh")
    N, E, nI, nd = (int(v) for v in counts)
    coords = np.empty((N, 2), order="F")
    elems = np.empty((E, 8), dtype=np.int32, order="F")
    irr = np.empty((nI, 3), dtype=np.int32, order="F")
    dirichlet = np.empty(nd, dtype=np.int32)
    cap = counts.copy()
    c.check(c.L.stdic_quadtree_mesh(c.h, P(m), W, H, P(x0), P(y0), ny, nx, step, float(elementMinSize),
                                    P(coords), P(elems), P(irr), P(dirichlet), P(cap), P(counts)),
            "GenerateQuadtreeMesh")
    return {"coordinatesFEM": coords, "elementsFEM": elems, "irregular": irr, "dirichlet": dirichlet,
            "markCoordHoleEdge": dirichlet.copy(), "elementMinSize": elementMinSize}


def funPOR_GPR(T_snap, t_train, t_pre, nB, ctx=None):
    """[u_pred, alpha, beta_POD, beta_GPR] = funPOR_GPR(T_snap, t_train, t_pre, nB)
    (stdic_por_gpr): T_snap is nT x np, u_pred nT1 x np.  A torch CUDA
    T_snap keeps u_pred on the device."""
    c = _ctx(ctx)
    b = _Bufs(c)
    if _is_torch(T_snap):
        nT, npt = int(T_snap.shape[0]), int(T_snap.shape[1])
        Tp = b.ptr(T_snap.t().contiguous().view(-1), np.float64)  # column-major
    else:
        T = np.asfortranarray(T_snap, dtype=np.float64)
        nT, npt = T.shape
        Tp = b.ptr(T, np.float64)
    tt = np.ascontiguousarray(np.asarray(t_train, dtype=np.float64).ravel())
    tp = np.ascontiguousarray(np.asarray(t_pre, dtype=np.float64).ravel())
    nT1 = tp.size
    like = T_snap if _is_torch(T_snap) else None
    U, pU = b.out(like, (nT1, npt), np.float64)
    alpha, bpod = _lib._c.c_double(0), _lib._c.c_double(0)
    bgpr = np.empty(nT1)
    c.check(c.L.stdic_por_gpr(c.h, Tp, nT, npt, tt.ctypes.data, tp.ctypes.data, nT1, int(nB), pU,
                              _lib._c.byref(alpha), _lib._c.byref(bpod), bgpr.ctypes.data), "funPOR_GPR")
    if _is_torch(U):
        U = U.view(npt, nT1).t()
    return U, alpha.value, bpod.value, bgpr


ADJ_MODES = {"recompute": _lib.STDIC_ADJ_RECOMPUTE, "store": _lib.STDIC_ADJ_STORE}


def icgn_adjoint(U, F, coordinatesFEM, ImgRef, ImgDef, winsize, ImgRefMask=None, ws_list=None,
                 precision="plain", mode="recompute", want_dg=True, size=None, ctx=None):
    """ZNSSD subset costs and their gradients (stdic_icgn_adjoint; no reference
    counterpart): returns (cost, cost_n, dU, dF, dg).  cost is the sum of the
    finite subset costs, dg the gradient of cost with respect to ImgDef (None
    unless want_dg).  size = (W, H) is needed for torch image buffers."""
    c = _ctx(ctx)
    prec = PRECISIONS[precision]
    dtype = _data_dtype(prec, ImgRef)
    N = _nodes(coordinatesFEM)
    W, H = size if size is not None else _shape2(ImgRef)
    b = _Bufs(c)
    fr = Frame()
    fr.f = b.ptr(ImgRef, dtype)
    fr.g = b.ptr(ImgDef, dtype)
    fr.mask = b.ptr(ImgRefMask, np.uint8)
    fr.dfdx = None
    fr.dfdy = None
    fr.W, fr.H = int(W), int(H)
    fr.dtype = _lib.STDIC_F32 if dtype == np.float32 else _lib.STDIC_F64
    like = U if _is_torch(U) else None
    cost, pcost = b.out(like, (1,), np.float64)
    cost_n, pcn = b.out(like, (N,), np.float64)
    dU, pdU = b.out(like, (2 * N,), np.float64)
    dF, pdF = b.out(like, (4 * N,), np.float64)
    dg, pdg = (None, None)
    if want_dg:
        gdt = np.float64 if prec == _lib.STDIC_PLAIN_F64 else np.float32
        dg, pdg = b.out(like, (int(W), int(H)), gdt)
    ws0 = int(winsize) if ws_list is None else int(max(int(winsize), int(np.max(ws_list))))
    c.check(c.L.stdic_icgn_adjoint(c.h, _lib._c.byref(fr), b.ptr(coordinatesFEM, np.float64), N, ws0,
                                   b.ptr(ws_list, np.int32) if ws_list is not None else None,
                                   b.ptr(U, np.float64), b.ptr(F, np.float64), pcost, pcn, pdU, pdF, pdg,
                                   ADJ_MODES[mode] if isinstance(mode, str) else int(mode), prec),
            "icgn_adjoint")
    return (cost[0] if not _is_torch(cost) else cost), cost_n, dU, dF, dg


def icgn_subsets_frames(U0_list, coordinatesFEM, Df, ImgRef, ImgDef_list, winsize, tol, ws_list=None,
                        ctx=None):
    """funICGNQuadtree for several deformed frames sharing ImgRef and one mesh,
    in one batched launch (stdic_icgn_subsets_frames; no reference
    counterpart).  Returns lists of U (2N), F (4N) and ConvItPerEle (N)."""
    c = _ctx(ctx)
    P = len(ImgDef_list)
    N = _nodes(coordinatesFEM)
    dtype = np.float32
    b = _Bufs(c)
    g = np.concatenate([np.asarray(x, dtype=dtype).ravel(order="F") for x in ImgDef_list])
    fr = _frame(b, Df, ImgRef, g, dtype)
    U0 = np.concatenate([np.asarray(u, dtype=np.float64).ravel() for u in U0_list])
    U = np.empty(2 * N * P)
    F = np.empty(4 * N * P)
    conv = np.empty(N * P, dtype=np.int32)
    ws = int(winsize) if ws_list is None else int(max(int(winsize), int(np.max(ws_list))))
    c.check(c.L.stdic_icgn_subsets_frames(c.h, _lib._c.byref(fr), P, b.ptr(U0, np.float64),
                                          b.ptr(coordinatesFEM, np.float64), N, ws,
                                          b.ptr(ws_list, np.int32) if ws_list is not None else None,
                                          float(tol), U.ctypes.data, F.ctypes.data, None, conv.ctypes.data,
                                          _lib.STDIC_BATCHED_F32), "funICGNQuadtree (frames)")
    return ([U[2 * N * k:2 * N * (k + 1)] for k in range(P)], [F[4 * N * k:4 * N * (k + 1)] for k in range(P)],
            [conv[N * k:N * (k + 1)] for k in range(P)])


def nodal_strain(coordinatesFEM, elementsFEM, U, GaussPtOrder=2, ctx=None):
    """F (4N) = [du/dx dv/dx du/dy dv/dy] per node from the element Gauss-point
    strains (stdic_nodal_strain)."""
    c = _ctx(ctx)
    b = _Bufs(c)
    N = _nodes(coordinatesFEM)
    E = int(np.asarray(elementsFEM).shape[0])
    like = U if _is_torch(U) else None
    F, pF = b.out(like, (4 * N,), np.float64)
    c.check(c.L.stdic_nodal_strain(c.h, b.ptr(coordinatesFEM, np.float64), N, b.ptr(elementsFEM, np.int32), E,
                                   b.ptr(U, np.float64), int(GaussPtOrder), pF), "nodal strain")
    return F


def fill_nans(coordinatesFEM, elementsFEM, U, ctx=None):
    """U (2N) with its NaN nodes filled from their mesh neighbours (stdic_fill_nans)."""
    c = _ctx(ctx)
    b = _Bufs(c)
    N = _nodes(coordinatesFEM)
    E = int(np.asarray(elementsFEM).shape[0])
    out = np.array(U, dtype=np.float64).ravel().copy()
    c.check(c.L.stdic_fill_nans(c.h, b.ptr(coordinatesFEM, np.float64), N, b.ptr(elementsFEM, np.int32), E,
                                out.ctypes.data), "NaN fill")
    return out


def admm(DICmesh, Df, ImgRef, ImgDef, winsize_List, U2, F2, udual, vdual, mu, beta, tol=1e-2, steps=2,
         mark_hole=None, precision="batched", use_graph=True, ctx=None):
    """ADMM iterations of the AL-DIC loop (stdic_admm).  Returns a dict with
    U1, U2, F2, udual, vdual, badnum, pcg_iters and graph_used."""
    c = _ctx(ctx)
    prec = PRECISIONS[precision]
    dtype = _data_dtype(prec, ImgRef)
    b = _Bufs(c)
    fr = _frame(b, Df, ImgRef, ImgDef, dtype)
    coords = DICmesh["coordinatesFEM"]
    elems = DICmesh["elementsFEM"]
    dirichlet = DICmesh.get("dirichlet")
    N = _nodes(coords)
    E = int(np.asarray(elems).shape[0])
    nd = 0 if dirichlet is None else int(np.asarray(dirichlet).size)
    st = {k: np.array(v, dtype=np.float64).ravel().copy()
          for k, v in (("U2", U2), ("F2", F2), ("udual", udual), ("vdual", vdual))}
    U1 = np.empty(2 * N)
    bad = np.zeros(steps, dtype=np.int32)
    its = np.zeros(steps, dtype=np.int32)
    used = _lib._c.c_int(0)
    c.check(c.L.stdic_admm(c.h, _lib._c.byref(fr), b.ptr(coords, np.float64), N, b.ptr(elems, np.int32), E,
                           b.ptr(dirichlet, np.int32) if nd else None, nd, b.ptr(winsize_List, np.int32),
                           b.ptr(mark_hole, np.uint8) if mark_hole is not None else None, float(mu),
                           float(beta), float(tol), int(steps), prec, 1 if use_graph else 0,
                           st["U2"].ctypes.data, st["F2"].ctypes.data, st["udual"].ctypes.data,
                           st["vdual"].ctypes.data, U1.ctypes.data, bad.ctypes.data, its.ctypes.data,
                           _lib._c.byref(used)), "ADMM")
    st.update(U1=U1, badnum=bad, pcg_iters=its, graph_used=bool(used.value))
    return st
