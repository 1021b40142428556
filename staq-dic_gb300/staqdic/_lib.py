"""ctypes binding of libstaqdic.so (the C ABI in include/staqdic.h).

The library is built in-tree by ``staqdic.build``; there is no CPU fallback:
loading fails loudly when the library or a CUDA device is missing.
"""
import ctypes
import os

from . import build as _build

_c = ctypes
_d = _c.POINTER(_c.c_double)
_i32 = _c.POINTER(_c.c_int32)
_u8 = _c.POINTER(_c.c_uint8)
_vp = _c.c_void_p

STDIC_OK = 0
STDIC_E_ARG = -1
STDIC_E_CUDA = -2
STDIC_E_NOMEM = -3
STDIC_E_UNSUPPORTED = -4
STDIC_E_TIMEOUT = -5
STDIC_E_NOTCONV = -6
STDIC_F64 = 0
STDIC_F32 = 1
STDIC_ADJ_RECOMPUTE = 0
STDIC_ADJ_STORE = 1
STDIC_PLAIN_F64 = 0
STDIC_BATCHED_F32 = 1

EXPORTS = [
    "stdic_ctx_create", "stdic_ctx_destroy", "stdic_ctx_set_stream", "stdic_last_error",
    "stdic_kernel_launches", "stdic_last_solver_ms", "stdic_interp_bicubic", "stdic_img_gradient",
    "stdic_integer_search_grid", "stdic_integer_search", "stdic_icgn_subsets", "stdic_icgn_local",
    "stdic_subpb1_subsets", "stdic_subpb1", "stdic_subpb2", "stdic_subpb2_noalloc",
    "stdic_icgn_adjoint", "stdic_icgn_subsets_frames", "stdic_nodal_strain", "stdic_fill_nans",
    "stdic_admm", "stdic_ctx_set_wait_limit", "stdic_quadtree_mesh", "stdic_por_gpr", "stdic_integer_search_mg",
]


class StdicError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (code %d)" % (msg, code))
        self.code = code


class Frame(_c.Structure):
    _fields_ = [("f", _vp), ("g", _vp), ("mask", _vp), ("dfdx", _vp), ("dfdy", _vp),
                ("W", _c.c_int), ("H", _c.c_int), ("dtype", _c.c_int)]


_lib = None


def lib_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load libstaqdic.so (building it first if asked and absent)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise OSError("libstaqdic.so is not built (run staqdic.build.build())")
        _build.build()
    L = _c.CDLL(path)
    L.stdic_ctx_create.argtypes = [_c.POINTER(_vp), _c.c_int]
    L.stdic_ctx_destroy.argtypes = [_vp]
    L.stdic_ctx_set_stream.argtypes = [_vp, _vp]
    L.stdic_last_error.argtypes = [_vp]
    L.stdic_last_error.restype = _c.c_char_p
    L.stdic_kernel_launches.argtypes = [_vp]
    L.stdic_kernel_launches.restype = _c.c_longlong
    L.stdic_last_solver_ms.argtypes = [_vp]
    L.stdic_last_solver_ms.restype = _c.c_double
    L.stdic_ctx_set_wait_limit.argtypes = [_vp, _c.c_longlong]
    L.stdic_por_gpr.argtypes = [_vp, _vp, _c.c_int, _c.c_int64, _vp, _vp, _c.c_int, _c.c_int, _vp, _vp, _vp, _vp]
    L.stdic_integer_search_mg.argtypes = [_vp, _vp, _vp, _c.c_int, _c.c_int, _vp, _vp, _c.c_int, _vp, _vp, _vp,
                                          _vp, _vp, _vp, _c.c_int64, _vp, _vp, _c.c_int64, _vp]
    L.stdic_quadtree_mesh.argtypes = [_vp, _vp, _c.c_int, _c.c_int, _vp, _vp, _c.c_int, _c.c_int, _c.c_double,
                                      _c.c_double, _vp, _vp, _vp, _vp, _vp, _vp]
    L.stdic_interp_bicubic.argtypes = [_vp, _vp, _c.c_int64, _c.c_int64, _c.c_int64, _vp, _vp,
                                       _c.c_int64, _vp, _c.c_int]
    L.stdic_img_gradient.argtypes = [_vp, _vp, _vp, _c.c_int, _c.c_int, _vp, _vp, _c.c_int]
    L.stdic_integer_search_grid.argtypes = [_c.c_int, _c.c_int, _i32, _d, _d, _i32, _i32,
                                            _c.POINTER(_c.c_int), _c.POINTER(_c.c_int)]
    L.stdic_integer_search.argtypes = [_vp, _vp, _vp, _c.c_int, _c.c_int, _i32, _d, _d, _i32, _i32,
                                       _vp, _vp, _vp, _vp, _vp, _vp, _vp]
    L.stdic_icgn_local.argtypes = [_vp, _c.POINTER(Frame), _vp, _vp, _c.c_int, _c.c_int, _vp,
                                   _c.c_double, _vp, _vp, _vp, _vp, _vp, _vp, _c.c_int]
    L.stdic_icgn_subsets.argtypes = [_vp, _c.POINTER(Frame), _vp, _vp, _c.c_int, _c.c_int, _vp,
                                     _c.c_double, _vp, _vp, _vp, _vp, _c.c_int]
    L.stdic_subpb1_subsets.argtypes = [_vp, _c.POINTER(Frame), _vp, _vp, _vp, _vp, _c.c_int, _vp,
                                       _c.c_double, _c.c_double, _vp, _vp, _c.c_int]
    L.stdic_subpb1.argtypes = [_vp, _c.POINTER(Frame), _vp, _vp, _vp, _vp, _vp, _c.c_int, _vp,
                               _c.c_double, _c.c_double, _c.c_double, _vp, _vp, _vp, _c.c_int]
    L.stdic_subpb2.argtypes = [_vp, _vp, _c.c_int, _vp, _c.c_int, _vp, _c.c_int, _vp, _c.c_int,
                               _c.c_int, _c.c_double, _c.c_double, _vp, _vp, _c.c_double,
                               _c.c_double, _c.c_double, _c.c_int, _vp, _vp]
    L.stdic_nodal_strain.argtypes = [_vp, _vp, _c.c_int, _vp, _c.c_int, _vp, _c.c_int, _vp]
    L.stdic_fill_nans.argtypes = [_vp, _vp, _c.c_int, _vp, _c.c_int, _vp]
    L.stdic_admm.argtypes = [_vp, _c.POINTER(Frame), _vp, _c.c_int, _vp, _c.c_int, _vp, _c.c_int, _vp, _vp,
                             _c.c_double, _c.c_double, _c.c_double, _c.c_int, _c.c_int, _c.c_int, _vp, _vp,
                             _vp, _vp, _vp, _vp, _vp, _vp]
    L.stdic_icgn_subsets_frames.argtypes = [_vp, _c.POINTER(Frame), _c.c_int, _vp, _vp, _c.c_int, _c.c_int,
                                            _vp, _c.c_double, _vp, _vp, _vp, _vp, _c.c_int]
    L.stdic_icgn_adjoint.argtypes = [_vp, _c.POINTER(Frame), _vp, _c.c_int, _c.c_int, _vp, _vp, _vp,
                                     _vp, _vp, _vp, _vp, _vp, _c.c_int, _c.c_int]
    L.stdic_subpb2_noalloc.argtypes = [_vp, _c.c_int, _vp, _c.c_int, _vp, _c.c_int, _vp, _c.c_int,
                                       _c.c_int, _c.c_double, _c.c_double, _vp, _vp, _c.c_double,
                                       _c.c_double, _c.c_double, _c.c_int, _vp, _vp, _vp, _c.c_char_p,
                                       _c.c_int]
    for name in EXPORTS:
        if name not in ("stdic_last_error", "stdic_kernel_launches", "stdic_last_solver_ms"):
            getattr(L, name).restype = _c.c_int
    _lib = L
    return L


class Context:
    """One CUDA device, one stream and one workspace (stdic_ctx)."""

    def __init__(self, device=0):
        self.L = load()
        h = _vp()
        rc = self.L.stdic_ctx_create(_c.byref(h), int(device))
        if rc != STDIC_OK:
            raise StdicError(rc, "stdic_ctx_create failed (no CUDA device %d?)" % device)
        self.h = h
        self.device = device
        self._torch_stream = None

    def check(self, rc, what):
        if rc != STDIC_OK:
            msg = self.L.stdic_last_error(self.h).decode(errors="replace")
            raise StdicError(rc, "%s: %s" % (what, msg))

    def set_stream(self, stream_ptr):
        """Run the library's work on the cudaStream_t stream_ptr (None or 0:
        the context's own stream, which is ordered with the legacy default
        stream)."""
        self.check(self.L.stdic_ctx_set_stream(self.h, _vp(stream_ptr or 0)), "set_stream")
        self._torch_stream = stream_ptr or None

    def set_wait_limit(self, polls):
        """Bound (polls) of the Subpb2 PCG grid-barrier waits; 0 = default 2^24."""
        self.check(self.L.stdic_ctx_set_wait_limit(self.h, int(polls)), "set_wait_limit")

    def last_solver_ms(self):
        """Device time (ms) of the last IC-GN solver kernel (CUDA events)."""
        return float(self.L.stdic_last_solver_ms(self.h))

    @property
    def launches(self):
        return int(self.L.stdic_kernel_launches(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.L.stdic_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default = None


def default_context():
    global _default
    if _default is None:
        _default = Context(int(os.environ.get("STAQDIC_DEVICE", "0")))
    return _default
