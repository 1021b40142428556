"""The MEX gateway (staq-dic_gb300/mex/staqdic_mex.cpp) driven as MATLAB would.

The gateway is compiled against the test stand-in for mex.h (oracle/mexshim)
and linked to libstaqdic.so; mexFunction is called with mxArrays built here,
and every operation is compared with the same call through the Python mirror
of the C ABI:
  * 'ba_interp2' (double and single): bit-identical to the reference's
    compiled ba_interp2.cpp (the golden vectors), output shape of X;
  * 'gradient', 'integer_search' (x, y, u, v, cc.max, cc.qfactors),
    'integer_search_mg' (xGrid, yGrid, uGrid, vGrid, cc.max),
    'icgn_local' (U, F, HtempPar, codes, markCoordHoleStrain as 1-based
    indices, the bad count), 'subpb1', 'subpb2': equal to the direct calls
    (the same kernels on the same inputs; Subpb2's atomics leave 1e-9);
  * argument errors and library errors come back as MATLAB errors with the
    'staqdic:args' / 'staqdic:call' identifiers, as ba_interp2.cpp:318-335
    reports its own.
The build needs g++ (CPU test); the calls need the GPU.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLD = os.path.join(HERE, "golden")
mxLOGICAL, mxDOUBLE, mxSINGLE, mxUINT8, mxINT32 = 3, 6, 7, 9, 12
NP = {mxDOUBLE: np.float64, mxSINGLE: np.float32, mxUINT8: np.uint8, mxLOGICAL: np.uint8, mxINT32: np.int32}


def _build(out_dir):
    from staqdic import build
    lib = build.build()
    libdir = os.path.dirname(lib)
    so = os.path.join(str(out_dir), "libstaqdic_mex_test.so")
    cmd = ["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "oracle", "mexshim"), os.path.join(ROOT, "staq-dic_gb300", "mex", "staqdic_mex.cpp"),
           os.path.join(ROOT, "oracle", "mexshim", "mexshim.cpp"), "-L", libdir, "-lstaqdic",
           "-Wl,-rpath," + libdir, "-o", so]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return so


def test_gateway_compiles_and_links(tmp_path):
    so = _build(tmp_path)
    L = ctypes.CDLL(so)
    for name in ("mexFunction", "shim_call", "shim_array", "shim_run_atexit"):
        assert hasattr(L, name)


class Mex:
    """mexFunction of the gateway, called with NumPy arrays as mxArrays."""

    def __init__(self, so):
        L = ctypes.CDLL(so)
        vp = ctypes.c_void_p
        L.shim_array.restype = vp
        L.shim_array.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_size_t), vp]
        L.shim_string.restype = vp
        L.shim_string.argtypes = [ctypes.c_char_p]
        L.shim_data.restype = vp
        L.shim_data.argtypes = [vp]
        L.shim_class.argtypes = [vp]
        L.shim_ndim.argtypes = [vp]
        L.shim_dim.restype = ctypes.c_size_t
        L.shim_dim.argtypes = [vp, ctypes.c_int]
        L.shim_free.argtypes = [vp]
        L.shim_call.argtypes = [ctypes.c_int, ctypes.POINTER(vp), ctypes.c_int, ctypes.POINTER(vp), ctypes.c_char_p,
                                ctypes.c_int]
        self.L = L

    def arr(self, a, cls=None):
        a = np.asarray(a)
        if cls is None:
            cls = {np.dtype(np.float64): mxDOUBLE, np.dtype(np.float32): mxSINGLE, np.dtype(np.uint8): mxUINT8,
                   np.dtype(np.int32): mxINT32, np.dtype(bool): mxLOGICAL}[a.dtype]
        a = np.asfortranarray(a, dtype=NP[cls])
        if a.ndim == 0:
            a = a.reshape(1, 1)
        if a.ndim == 1:
            a = a.reshape(-1, 1, order="F")
        dims = (ctypes.c_size_t * a.ndim)(*a.shape)
        return self.L.shim_array(cls, a.ndim, dims, a.ctypes.data if a.size else None)

    def get(self, p):
        cls = self.L.shim_class(p)
        shape = tuple(self.L.shim_dim(p, i) for i in range(self.L.shim_ndim(p)))
        n = int(np.prod(shape))
        dt = NP[cls]
        buf = (ctypes.c_char * (n * np.dtype(dt).itemsize)).from_address(self.L.shim_data(p)) if n else b""
        return np.frombuffer(bytes(buf), dtype=dt).reshape(shape, order="F").copy()

    def __call__(self, op, *args, nout=1):
        ins = [self.L.shim_string(op.encode())] + [a if isinstance(a, int) else self.arr(a) for a in args]
        prhs = (ctypes.c_void_p * len(ins))(*ins)
        plhs = (ctypes.c_void_p * max(nout, 1))()
        err = ctypes.create_string_buffer(1024)
        rc = self.L.shim_call(nout, plhs, len(ins), prhs, err, len(err))
        outs = [self.get(plhs[k]) for k in range(nout) if rc == 0 and plhs[k]]
        for p in ins:
            self.L.shim_free(p)
        for k in range(nout):
            if plhs[k]:
                self.L.shim_free(plhs[k])
        if rc != 0:
            raise RuntimeError(err.value.decode())
        return outs if nout > 1 else outs[0]


@pytest.fixture(scope="module")
def mex(tmp_path_factory):
    m = Mex(_build(tmp_path_factory.mktemp("mexgw")))
    yield m
    m.L.shim_run_atexit()  # what MATLAB does when the MEX file is cleared


@pytest.mark.gpu
def test_ba_interp2_op_bit_exact(mex):
    d = np.load(os.path.join(GOLD, "ba_interp2_golden.npz"))
    Z = mex("ba_interp2", d["F"], d["X"], d["Y"])
    assert Z.shape == (d["X"].size, 1)
    assert np.array_equal(Z.ravel(), d["Z64"])
    Z32 = mex("ba_interp2", d["F"].astype(np.float32), d["X"].astype(np.float32), d["Y"].astype(np.float32))
    assert np.array_equal(Z32.ravel(), d["Z32"])
    with pytest.raises(RuntimeError, match="staqdic:args.*same class"):
        mex("ba_interp2", d["F"], d["X"].astype(np.float32), d["Y"])


@pytest.mark.gpu
def test_gradient_and_integer_search_ops(mex, ctx):
    import staqdic
    from staqdic import workloads
    w = workloads.uniform256(seed=0)
    f, g = w["f"], w["g"]
    mask = np.ones(f.shape, dtype=bool)
    mask[100:120, 30:40] = False
    DfDx, DfDy = mex("gradient", f, mask, nout=2)
    Df = staqdic.funImgGradient(f, f, mask.astype(np.uint8), ctx=ctx)
    assert np.array_equal(DfDx, Df["DfDx"]) and np.array_equal(DfDy, Df["DfDy"])
    x, y, u, v, ccm, qf = mex("integer_search", g, f, np.array([6.0]), np.array([1.0, 256.0]),
                              np.array([1.0, 256.0]), np.array([32.0]), np.array([16.0]), nout=6)
    xo, yo, uo, vo, cc = staqdic.funIntegerSearch(g, f, 6, (1, 256), (1, 256), 32, 16, ctx=ctx)
    for a, b in ((x, xo), (y, yo), (u, uo), (v, vo), (ccm, cc["max"]), (qf, cc["qfactors"])):
        assert a.shape == b.shape
        assert np.array_equal(a, b, equal_nan=True)


@pytest.mark.gpu
def test_integer_search_mg_op(mex, ctx):
    """'integer_search_mg' against the direct call (gridfit's data assembly
    adds with atomics, so the fitted fields agree to rounding)."""
    import staqdic
    from staqdic import workloads
    w = workloads.uniform256(seed=0)
    f, g = w["f"].astype(np.float64), w["g"].astype(np.float64)
    outs = mex("integer_search_mg", f, g, np.array([1.0, 256.0]), np.array([1.0, 256.0]), np.array([32.0]),
               np.array([16.0]), nout=5)
    ref = staqdic.funIntegerSearchMg(f, g, (1, 256), (1, 256), 32, 16, ctx=ctx)
    for a, b in zip(outs, list(ref[:4]) + [ref[4]["max"]]):
        assert a.shape == b.shape
        assert np.allclose(a, b, rtol=0, atol=1e-9, equal_nan=True)


@pytest.mark.gpu
def test_icgn_local_subpb1_subpb2_ops(mex, ctx):
    import staqdic
    from staqdic import workloads
    w = workloads.hole1024(seed=1, size=256)
    c, el = w["coordinatesFEM"], w["elementsFEM"]
    N = c.shape[0]
    wl = np.asarray(w["winsize_list"], np.int32)
    f, g = w["f"].astype(np.float64), w["g"].astype(np.float64)
    Df = staqdic.funImgGradient(f, f, w["maskf"], ctx=ctx)
    mask = w["maskf"].astype(bool)
    for prec in (0, 1):
        U, F, H, conv, mark, bad = mex("icgn_local", w["U0"], c, Df["DfDx"], Df["DfDy"], mask, f, g,
                                       np.array([float(wl.max())]), wl.astype(np.float64), np.array([1e-2]),
                                       np.array([float(prec)]), nout=6)
        out = staqdic.LocalICGNQuadtree(w["U0"], c, Df, f, g, {"winsize": int(wl.max()), "winsize_per_node": wl},
                                        "GaussNewton", 1e-2, precision="plain" if prec == 0 else "batched", ctx=ctx)
        assert np.array_equal(conv.ravel(), out[4].astype(np.float64))
        assert np.array_equal(U.ravel(), out[0], equal_nan=True)
        assert np.array_equal(F.ravel(), out[1], equal_nan=True)
        assert np.array_equal(H, out[2])
        assert np.array_equal(mark.ravel(), out[6].astype(np.float64))
        assert int(bad.ravel()[0]) == out[5]
    # Subpb1 on the filled local result
    U2 = staqdic.fill_nans(c, el, out[0], ctx=ctx)
    F2 = np.nan_to_num(staqdic.nodal_strain(c, el, U2, ctx=ctx))
    vd = np.zeros(2 * N)
    wl2 = np.asfortranarray(np.stack([wl, wl], 1))
    Us, convs, bads = mex("subpb1", U2, F2, np.zeros(4 * N), vd, c, Df["DfDx"], Df["DfDy"], mask, f, g,
                          np.array([1e-3]), np.array([1e-3]), wl2.astype(np.float64), np.array([1e-2]),
                          np.array([0.0]), nout=3)
    Uo, _, _, co, bo = staqdic.Subpb1Quadtree(U2, F2, np.zeros(4 * N), vd, c, Df, f, g, 1e-3, 1e-3, None, 2,
                                              {"winsize_List": wl2}, "GaussNewton", 1e-2, precision="plain", ctx=ctx)
    assert np.array_equal(convs.ravel(), co.astype(np.float64))
    assert np.array_equal(Us.ravel(), Uo, equal_nan=True)
    assert int(bads.ravel()[0]) == bo
    # Subpb2: elementsFEM and the Dirichlet list as MATLAB holds them (double)
    Uh, it = mex("subpb2", c, el.astype(np.float64), np.asarray(w["dirichlet"][::5], np.float64), np.zeros((0, 4)),
                 np.array([2.0]), np.array([2.56e-3]), np.array([1e-3]), U2, F2, np.array([0.0]), np.array([32.0]),
                 nout=2)
    mesh = {"coordinatesFEM": c, "elementsFEM": el, "dirichlet": w["dirichlet"][::5], "neumann": None}
    Uhd = staqdic.Subpb2Quadtree(mesh, 2, 2.56e-3, 1e-3, U2, F2, None, None, 0.0, 32, ctx=ctx)
    assert it.ravel()[0] > 0
    assert np.max(np.abs(Uh.ravel() - Uhd)) < 1e-9


@pytest.mark.gpu
def test_errors_map_to_matlab_errors(mex):
    from staqdic import workloads
    w = workloads.uniform256(seed=0)
    f = w["f"]
    with pytest.raises(RuntimeError, match="staqdic:op"):
        mex("no_such_op", f)
    with pytest.raises(RuntimeError, match="staqdic:args"):
        mex("gradient", f[:5, :5], np.ones((5, 5)), nout=2)
    # an odd subset size is the library's argument error, reported through stdic_last_error
    Dx, Dy = mex("gradient", f, np.ones(f.shape), nout=2)
    c = w["coordinatesFEM"]
    with pytest.raises(RuntimeError, match="staqdic:call.*winsize"):
        mex("icgn_local", w["U0"], c, Dx, Dy, np.ones(f.shape), f, w["g"], np.array([31.0]), np.zeros((0, 0)),
            np.array([1e-2]), np.array([0.0]), nout=6)
