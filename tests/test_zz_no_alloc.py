"""stdic_subpb2_noalloc (static device scratch, no context) against stdic_subpb2.

The two entry points run the same assembly and Jacobi-PCG; the assembly adds
element matrices with double atomics, so the order of those additions (and
hence the last bits) can differ between any two runs: the solutions agree to
1e-7 px and the PCG counts to 2 iterations.  Several calls in a row on meshes of
different sizes show that nothing of one call's scratch leaks into the next.
This file is named to be collected last, and also passes alone.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="module")
def meshes():
    from staqdic import workloads
    hole = workloads.hole1024(seed=1, size=256)
    plate = workloads.uniform256(seed=0)
    rng = np.random.default_rng(21)
    out = []
    N = hole["coordinatesFEM"].shape[0]
    out.append(dict(coords=hole["coordinatesFEM"], elems=hole["elementsFEM"],
                    dirichlet=np.asarray(hole["dirichlet"][::7], np.int32), neumann=None,
                    gauss=2, beta=2.56e-3, mu=1e-3, alpha=0.0, step=32.0,
                    U=hole["Utrue"] + rng.normal(0, 0.05, 2 * N), F=rng.normal(0, 0.01, 4 * N)))
    N = plate["coordinatesFEM"].shape[0]
    out.append(dict(coords=plate["coordinatesFEM"], elems=plate["elementsFEM"],
                    dirichlet=np.array([100, 101], np.int32),
                    neumann=np.array([[1, 2, 0.0, -1.0], [2, 3, 0.0, -1.0], [15, 29, -1.0, 0.0]]),
                    gauss=3, beta=1e-2, mu=1e-3, alpha=1e-3, step=16.0,
                    U=rng.normal(0, 0.5, 2 * N), F=rng.normal(0, 0.01, 4 * N)))
    return out


def _dev(torch, a, dtype):
    a = np.asarray(a, dtype=dtype)
    return torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).cuda()


def _noalloc(torch, L, m, stream):
    N = m["coords"].shape[0]
    E = m["elems"].shape[0]
    d = {k: _dev(torch, m[k], np.float64) for k in ("coords", "U", "F")}
    el = _dev(torch, m["elems"], np.int32)
    di = _dev(torch, m["dirichlet"], np.int32)
    nn = 0 if m["neumann"] is None else m["neumann"].shape[0]
    ne = _dev(torch, m["neumann"], np.float64) if nn else None
    Uhat = torch.full((2 * N,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    iters = ctypes.c_int(-1)
    err = ctypes.create_string_buffer(256)
    rc = L.stdic_subpb2_noalloc(d["coords"].data_ptr(), N, el.data_ptr(), E, di.data_ptr(),
                                di.numel(), ne.data_ptr() if nn else None, nn, m["gauss"],
                                m["beta"], m["mu"], d["U"].data_ptr(), d["F"].data_ptr(),
                                m["alpha"], m["step"], 1e-10, 0, Uhat.data_ptr(),
                                ctypes.byref(iters), stream.cuda_stream, err, len(err))
    assert rc == 0, err.value.decode(errors="replace")
    return Uhat.cpu().numpy(), iters.value


def _with_ctx(sd, ctx, m):
    mesh = {"coordinatesFEM": m["coords"], "elementsFEM": m["elems"], "dirichlet": m["dirichlet"],
            "neumann": None if m["neumann"] is None else np.asfortranarray(m["neumann"])}
    return sd.Subpb2Quadtree(mesh, m["gauss"], m["beta"], m["mu"], m["U"], m["F"], None, None,
                             m["alpha"], m["step"], ctx=ctx, return_iters=True)


def test_noalloc_matches_context_entry(torch_cuda, ctx, meshes):
    import staqdic
    from staqdic import _lib
    torch = torch_cuda
    L = _lib.load()
    stream = torch.cuda.Stream()
    # large mesh, small mesh, large mesh again: consecutive calls share the array
    for m in (meshes[0], meshes[1], meshes[0]):
        Un, itn = _noalloc(torch, L, m, stream)
        Uc, itc = _with_ctx(staqdic, ctx, m)
        assert np.all(np.isfinite(Un))
        assert np.max(np.abs(Un - Uc)) < 1e-7
        assert itn > 0 and abs(itn - itc) <= 2


def test_noalloc_rejects_oversize_and_host_memory(torch_cuda, meshes):
    from staqdic import _lib
    torch = torch_cuda
    L = _lib.load()
    small = torch.zeros(64, dtype=torch.float64, device="cuda")
    small_i = torch.zeros(64, dtype=torch.int32, device="cuda")
    p, pi = small.data_ptr(), small_i.data_ptr()
    err = ctypes.create_string_buffer(256)
    # a 200,000-element mesh does not fit the 16 MiB array; rejected before any device access
    rc = L.stdic_subpb2_noalloc(p, 200000, pi, 200000, None, 0, None, 0, 2, 1e-3, 1e-3, p, p,
                                0.0, 16.0, 1e-10, 0, p, None, None, err, len(err))
    assert rc == _lib.STDIC_E_NOMEM
    assert b"static array" in err.value
    # host arrays are refused (this entry never stages through device memory of its own)
    m = meshes[1]
    coords = np.asfortranarray(m["coords"], np.float64)
    rc = L.stdic_subpb2_noalloc(coords.ctypes.data, coords.shape[0], pi, 1, None, 0, None, 0, 2,
                                1e-3, 1e-3, p, p, 0.0, 16.0, 1e-10, 0, p, None, None, err, len(err))
    assert rc == _lib.STDIC_E_ARG
    assert b"device memory" in err.value


def test_noalloc_reports_invalid_node_index(torch_cuda, meshes):
    """An element that names a node outside 1..N is reported as STDIC_E_ARG by
    the solve itself (the set-up kernels skip the index; the PCG stops before
    its first grid barrier)."""
    from staqdic import _lib
    torch = torch_cuda
    L = _lib.load()
    m = dict(meshes[1])
    el = np.array(m["elems"], dtype=np.int32, copy=True)
    el[3, 2] = m["coords"].shape[0] + 5
    m["elems"] = el
    N = m["coords"].shape[0]
    d = {k: _dev(torch, m[k], np.float64) for k in ("coords", "U", "F")}
    eld = _dev(torch, el, np.int32)
    di = _dev(torch, m["dirichlet"], np.int32)
    Uhat = torch.zeros(2 * N, dtype=torch.float64, device="cuda")
    err = ctypes.create_string_buffer(256)
    stream = torch.cuda.Stream()
    rc = L.stdic_subpb2_noalloc(d["coords"].data_ptr(), N, eld.data_ptr(), el.shape[0], di.data_ptr(),
                                di.numel(), None, 0, 2, 1e-2, 1e-3, d["U"].data_ptr(), d["F"].data_ptr(),
                                0.0, 16.0, 1e-10, 0, Uhat.data_ptr(), None, stream.cuda_stream, err, len(err))
    assert rc == _lib.STDIC_E_ARG
    assert b"invalid node index" in err.value
    # the array is usable again right after
    Un, itn = _noalloc(torch, L, meshes[1], stream)
    assert np.all(np.isfinite(Un)) and itn > 0


def test_noalloc_matches_direct_sparse_solve(torch_cuda, oracle, meshes):
    """The oracle's direct solve (SuperLU on A(Free,Free)) against the
    no-allocation entry, to the PCG tolerance (1e-6 px)."""
    from staqdic import _lib
    torch = torch_cuda
    L = _lib.load()
    m = meshes[0]
    Un, _ = _noalloc(torch, L, m, torch.cuda.Stream())
    Uo = oracle.Subpb2Quadtree(m["coords"], m["elems"], m["dirichlet"], None, m["gauss"], m["beta"],
                               m["mu"], m["U"], m["F"], m["alpha"], m["step"])
    assert np.max(np.abs(Un - Uo)) < 1e-6


_RESET_SCRIPT = r'''
import ctypes, sys
import numpy as np
sys.path[:0] = sys.argv[1:3]
from staqdic import _lib, workloads
L = _lib.load()
rt = ctypes.CDLL("libcudart.so.13")
w = workloads.uniform256(seed=0)
coords = np.asfortranarray(w["coordinatesFEM"], np.float64)
elems = np.asfortranarray(w["elementsFEM"], np.int32)
N, E = coords.shape[0], elems.shape[0]
rng = np.random.default_rng(3)
U = rng.normal(0, 0.5, 2 * N)
F = rng.normal(0, 0.01, 4 * N)
dirichlet = np.array([1, 2, 3, 100], np.int32)

def dev(a):
    p = ctypes.c_void_p()
    assert rt.cudaMalloc(ctypes.byref(p), ctypes.c_size_t(a.nbytes)) == 0
    assert rt.cudaMemcpy(p, a.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(a.nbytes), 1) == 0
    return p

def solve():
    assert rt.cudaSetDevice(0) == 0
    ptrs = [dev(np.ascontiguousarray(a.ravel(order="F"))) for a in (coords, elems, dirichlet, U, F)]
    out = np.zeros(2 * N)
    po = dev(out)
    err = ctypes.create_string_buffer(256)
    it = ctypes.c_int(0)
    rc = L.stdic_subpb2_noalloc(ptrs[0], N, ptrs[1], E, ptrs[2], dirichlet.size, None, 0, 2, 1e-2, 1e-3,
                                ptrs[3], ptrs[4], 0.0, 16.0, 1e-10, 0, po, ctypes.byref(it), None, err, 256)
    assert rc == 0, err.value
    assert rt.cudaMemcpy(out.ctypes.data_as(ctypes.c_void_p), po, ctypes.c_size_t(out.nbytes), 2) == 0
    for p in ptrs + [po]:
        rt.cudaFree(p)
    return out, it.value

a, ia = solve()
assert rt.cudaDeviceReset() == 0
b, ib = solve()
assert np.all(np.isfinite(a)) and ia > 0
assert np.max(np.abs(a - b)) < 1e-7 and abs(ia - ib) <= 2
print("reset ok")
'''


def test_noalloc_after_context_reset(torch_cuda):
    """A context torn down (cudaDeviceReset ends only this process's own
    context) and created again reloads the module; the next call looks the
    array up again and solves as before.  Run in a child process so that the
    reset does not touch the test session's context."""
    import os
    import subprocess
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    r = subprocess.run([sys.executable, "-c", _RESET_SCRIPT, os.path.join(root, "staq-dic_gb300"), root],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "reset ok" in r.stdout
