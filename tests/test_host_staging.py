"""Host buffers through the C ABI: pinned, pageable and device buffers give
identical results.

With pinned host buffers, stdic_icgn_local uploads the deformed frame on a
side stream while the queue, set-up and factorisation kernels run, and
downloads HtempPar during the iteration stage (the host then zeroes the rows
of subsets that the iterations ended with code -1, which the iteration stage
zeroes on the device).  It also uploads the reference frame, its gradients
and the mask in row bands (STDIC_UPLOAD_BANDS, default 4) and runs the set-up
stage one band at a time; each band count is checked in a child process,
since the library reads the variable once.  Pageable buffers take the in-order copies, device
buffers no copies at all.  The same kernels run in all three, so every output
must agree bit for bit: U, F, HtempPar, the codes, the hole marks and the
bad-point count, on the 1024^2 plate with a hole (19,924 quadtree nodes, subsets
8-64 px, masked subsets near the hole) and on a two-frame batch.
"""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-2


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _frame_and_inputs(torch, ctx, w, frames=1):
    from staqdic import _lib
    W, H = w["f"].shape
    L = ctx.L

    def dev(a, dt):
        return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=dt).ravel(order="F"))).cuda()

    f = dev(w["f"], np.float32)
    g1 = dev(w["g"], np.float32)
    g = torch.cat([g1] * frames) if frames > 1 else g1
    mask = dev(w["maskf"], np.uint8)
    gx = torch.empty((W - 6) * (H - 6), dtype=torch.float32, device="cuda")
    gy = torch.empty_like(gx)
    ctx.check(L.stdic_img_gradient(ctx.h, f.data_ptr(), mask.data_ptr(), W, H, gx.data_ptr(), gy.data_ptr(),
                                   _lib.STDIC_F32), "gradient")
    U0 = np.asarray(w["U0"], np.float64)
    if frames > 1:
        U0 = np.concatenate([U0] * frames)
    ins = dict(f=f, g=g, mask=mask, gx=gx, gy=gy, U0=dev(U0, np.float64),
               coords=dev(w["coordinatesFEM"], np.float64), ws=dev(w["winsize_list"], np.int32))
    torch.cuda.synchronize()
    return W, H, ins


def _call(torch, ctx, W, H, N, ins, where, frames=1, local=True):
    """One call with every buffer on the device, in pinned host memory or in
    pageable host memory (NumPy); returns the outputs as NumPy arrays."""
    from staqdic import _lib
    L = ctx.L
    NT = N * frames
    if where == "device":
        b = dict(ins)
        outs = dict(U=torch.empty(2 * NT, dtype=torch.float64, device="cuda"),
                    F=torch.empty(4 * NT, dtype=torch.float64, device="cuda"),
                    H=torch.empty(21 * NT, dtype=torch.float64, device="cuda"),
                    conv=torch.empty(NT, dtype=torch.int32, device="cuda"),
                    mark=torch.empty(NT, dtype=torch.uint8, device="cuda"))
        ptr = {k: v.data_ptr() for k, v in list(b.items()) + list(outs.items())}
    elif where == "pinned":
        b = {k: v.cpu().pin_memory() for k, v in ins.items()}
        outs = dict(U=torch.empty(2 * NT, dtype=torch.float64).pin_memory(),
                    F=torch.empty(4 * NT, dtype=torch.float64).pin_memory(),
                    H=torch.empty(21 * NT, dtype=torch.float64).pin_memory(),
                    conv=torch.empty(NT, dtype=torch.int32).pin_memory(),
                    mark=torch.empty(NT, dtype=torch.uint8).pin_memory())
        ptr = {k: v.data_ptr() for k, v in list(b.items()) + list(outs.items())}
    else:
        b = {k: np.ascontiguousarray(v.cpu().numpy()) for k, v in ins.items()}
        outs = dict(U=np.empty(2 * NT), F=np.empty(4 * NT), H=np.empty(21 * NT),
                    conv=np.empty(NT, np.int32), mark=np.empty(NT, np.uint8))
        ptr = {k: v.ctypes.data for k, v in list(b.items()) + list(outs.items())}
    fr = _lib.Frame()
    fr.f, fr.g, fr.mask, fr.dfdx, fr.dfdy = ptr["f"], ptr["g"], ptr["mask"], ptr["gx"], ptr["gy"]
    fr.W, fr.H, fr.dtype = W, H, _lib.STDIC_F32
    ws_max = 64
    badnum = ctypes.c_int(-7)
    if local:
        rc = L.stdic_icgn_local(ctx.h, ctypes.byref(fr), ptr["U0"], ptr["coords"], N, ws_max, ptr["ws"], TOL,
                                ptr["U"], ptr["F"], ptr["H"], ptr["conv"], ptr["mark"], ctypes.byref(badnum),
                                _lib.STDIC_BATCHED_F32)
    else:
        rc = L.stdic_icgn_subsets_frames(ctx.h, ctypes.byref(fr), frames, ptr["U0"], ptr["coords"], N, ws_max,
                                         ptr["ws"], TOL, ptr["U"], ptr["F"], ptr["H"], ptr["conv"],
                                         _lib.STDIC_BATCHED_F32)
    ctx.check(rc, where)
    torch.cuda.synchronize()
    res = {}
    for k, v in outs.items():
        if not local and k == "mark":
            continue
        res[k] = v.cpu().numpy().copy() if hasattr(v, "cpu") else v.copy()
    res["badnum"] = badnum.value if local else None
    return res


def _same(a, b):
    for k in a:
        if k == "badnum":
            assert a[k] == b[k], (k, a[k], b[k])
        else:
            assert np.array_equal(a[k], b[k], equal_nan=True), k


def test_local_pinned_pageable_device_identical(torch_cuda, ctx):
    from staqdic import workloads
    torch = torch_cuda
    w = workloads.hole1024()
    N = w["coordinatesFEM"].shape[0]
    W, H, ins = _frame_and_inputs(torch, ctx, w)
    ref = _call(torch, ctx, W, H, N, ins, "device")
    conv = ref["conv"]
    Hm = ref["H"].reshape(21, N)
    # rows of subsets ended with a run-time error are zero, the others hold
    # the set-up stage's Hessian sums
    err = conv == -1
    assert np.all(Hm[:, err] == 0.0)
    run = (conv >= 1) & (conv <= 101)
    assert np.all(np.any(Hm[:, run] != 0.0, axis=0))
    assert 0 <= ref["badnum"] < N
    for where in ("pinned", "pageable", "pinned"):
        _same(ref, _call(torch, ctx, W, H, N, ins, where))


def test_local_banded_uneven_rows(torch_cuda, ctx):
    """A 1000^2 plate: four bands of 250 rows, so band edges fall at rows that
    no subset grid lines up with; pinned (banded) and device buffers agree."""
    from staqdic import workloads
    torch = torch_cuda
    w = workloads.hole1024(size=1000)
    N = w["coordinatesFEM"].shape[0]
    W, H, ins = _frame_and_inputs(torch, ctx, w)
    ref = _call(torch, ctx, W, H, N, ins, "device")
    assert np.count_nonzero((ref["conv"] >= 1) & (ref["conv"] <= 100)) > N // 2
    _same(ref, _call(torch, ctx, W, H, N, ins, "pinned"))


def test_frames_pinned_matches_device(torch_cuda, ctx):
    from staqdic import workloads
    torch = torch_cuda
    w = workloads.hole1024(size=512)
    N = w["coordinatesFEM"].shape[0]
    W, H, ins = _frame_and_inputs(torch, ctx, w, frames=2)
    ref = _call(torch, ctx, W, H, N, ins, "device", frames=2, local=False)
    got = _call(torch, ctx, W, H, N, ins, "pinned", frames=2, local=False)
    _same(ref, got)
    # both frames are the same pair: the same results per frame
    c = ref["conv"].reshape(2, N)
    assert np.array_equal(c[0], c[1])


@pytest.mark.parametrize("bands", [0, 1, 2, 8])
def test_local_band_counts_identical(torch_cuda, bands):
    """The local pass with 0 (whole frame), 1, 2 and 8 upload bands: pinned,
    pageable and device buffers agree bit for bit in a child process."""
    if os.environ.get("STDIC_UPLOAD_BANDS") is not None:
        pytest.skip("already in a child process with a fixed band count")
    env = dict(os.environ, STDIC_UPLOAD_BANDS=str(bands))
    here = os.path.dirname(os.path.abspath(__file__))
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-x", "-p", "no:cacheprovider",
                        os.path.join(here, "test_host_staging.py") + "::test_local_pinned_pageable_device_identical"],
                       env=env, cwd=os.path.dirname(here), capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert "1 passed" in r.stdout, r.stdout[-2000:]
