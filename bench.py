"""Benchmark of the STAQ-DIC hot path on GB300.

Metric: converged IC-GN subsets per second, counting a subset only when its
code is 1..100 (and the LocalICGNQuadtree bad-subset filter kept it) and its
displacement is within 0.01 px of the plain FP64 drop-in on the same inputs.

Step (default workload hole1024): one LocalICGNQuadtree pass — the batched
FP32 persistent kernel behind stdic_icgn_local — over all nodes of a seeded
1024^2 plate-with-hole pair (Kirsch field, 1 % strain, quadtree 4..32 px,
uneven subsets 8..64 px).  Inputs are resident in HBM (`value`); the same call
with pinned host buffers, copies inside the timed region, gives `e2e`.  The L2
is flushed (256 MiB write) between timed steps.

Beside the headline the line carries, on one GPU, the 2048^2 quadtree pass
(config C3, ``c3``: batched vs plain FP64 vs the host CPU), the timing of
the adjoint on the 4096^2 bumps pair (config C4, ``adjoint_c4``) and 16 frames
in one multi-frame launch against the frames one by one (config C5, ``c5``);
--no-extras skips them.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N > 1 runs one replica per GPU (the path has no data-path collective);
`value` is all ranks' converged subsets over the slowest rank's time.
--impl reference times the CPU implementation of the path on the host cores
(the reference is MATLAB, so the oracle's C++ restatement stands in).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for p in (os.path.join(ROOT, "staq-dic_gb300"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

METRIC = "converged IC-GN subsets/s at <=0.01 px vs FP64; batched vs plain on GB300"
UNIT = "subsets/s"
TOLPX = 0.01
WS_MAX = 64
TOL = 1e-2


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ----------------------------------------------------------------------------
def make_workload(name, **kw):
    from staqdic import workloads
    t = time.time()
    w = workloads.WORKLOADS[name](**kw)
    log("workload %s: %d nodes, generated in %.1fs" % (name, w["coordinatesFEM"].shape[0], time.time() - t))
    return w


def flops_per_subset(conv, ws_list):
    """Algorithmic FLOPs of one IC-GN solve: 70 n_px set-up + 106 n_px per
    iteration (warp 8, bicubic weights 38, 16-tap sum 35, residual 4, g stats
    3, b-vector 18), n_px = (ws+1)^2."""
    npx = (ws_list.astype(np.float64) + 1) ** 2
    it = np.where((conv >= 1) & (conv <= 101), conv, np.where(conv == 102, 0, 1)).astype(np.float64)
    return 70.0 * npx + 106.0 * it * npx


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.lines = []
        self.proc = None

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
            # the timed region starts once the sampler reports (at most 3 s)
            t0 = time.perf_counter()
            while not self.lines and time.perf_counter() - t0 < 3.0 and self.proc.poll() is None:
                time.sleep(0.01)
            self.lines.clear()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def fp32_peak_tflops(torch):
    """FP32 CUDA-core throughput: cuBLAS SGEMM with TF32 disabled, 8192^3."""
    old = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        n = 8192
        a = torch.randn(n, n, device="cuda", dtype=torch.float32)
        b = torch.randn(n, n, device="cuda", dtype=torch.float32)
        for _ in range(2):
            torch.matmul(a, b)
        torch.cuda.synchronize()
        best = 1e30
        for _ in range(5):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b)
            e1.record()
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        del a, b
        return 2.0 * n ** 3 / (best * 1e-3) / 1e12
    finally:
        torch.backends.cuda.matmul.allow_tf32 = old


def traffic_from_profiles():
    """DRAM bytes per launch of the batched kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "icgn_batched_hole1024.md")
    if not os.path.exists(p):
        return None
    for ln in open(p):
        if ln.strip().startswith("dram_bytes_per_launch:"):
            try:
                return float(ln.split(":", 1)[1].strip().split()[0])
            except ValueError:
                return None
    return None


# ----------------------------------------------------------------------------
def workload_config(name, w):
    """The config object both arms print for a LocalICGNQuadtree workload."""
    W, H = w["f"].shape
    ws = np.asarray(w["winsize_list"])
    return {"workload": "%s: %dx%d plate with hole, Kirsch 1%% strain, quadtree, %d nodes, subsets 8..64 px, "
                        "one LocalICGNQuadtree pass per step" % (name, W, H, w["coordinatesFEM"].shape[0]),
            "nodes": int(w["coordinatesFEM"].shape[0]),
            "subset_sizes": {str(k): int(v) for k, v in zip(*np.unique(ws, return_counts=True))}}


def run_reference(args, world, rank):
    """CPU implementation of the path on the host cores (oracle port)."""
    if rank != 0:
        return 0
    from oracle import build as ob
    ob.build_oracle()
    from oracle import oracle as orc
    w = make_workload(args.workload)
    f = w["f"].astype(np.float64)
    g = w["g"].astype(np.float64)
    Df = orc.funImgGradient(f, w["maskf"])
    coords = w["coordinatesFEM"]
    N = coords.shape[0]
    cores = os.cpu_count() or 1
    orc.set_threads(cores)
    # bounded sample: every k-th node, about 4000 subsets per step
    k = max(1, N // 4000)
    idx = np.arange(0, N, k)
    U0 = w["U0"].reshape(-1, 2)[idx].ravel()
    cs = coords[idx]
    wl = w["winsize_list"][idx]
    for _ in range(args.warmup):
        orc.icgn6(U0, cs, Df, f, g, wl, TOL)
    t0 = time.perf_counter()
    conv_total = 0
    for _ in range(args.steps):
        U, F, Hp, conv, mark = orc.icgn6(U0, cs, Df, f, g, wl, TOL)
        conv_total += int(((conv >= 1) & (conv <= 100)).sum())
    dt = time.perf_counter() - t0
    val = conv_total / dt
    sample = "%d of %d nodes of %s (every %d-th), FP64 IC-GN, %d OpenMP threads" % (
        idx.size, N, args.workload, k, cores)
    out = {"metric": METRIC, "value": val, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "impl": "reference", "parallelism": "host threads", "precision": "FP64 (the oracle port)",
           "config": workload_config(args.workload, w),
           "cpu_baseline": {"value": val, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
           "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)
    return 0


# ----------------------------------------------------------------------------
def reduce_over_ranks(dist, ms, n, device):
    """Replica aggregation: the slowest rank's time per step and the converged
    subsets of all ranks (the path has no data-path collective; this is the
    only exchange, outside the timed region)."""
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    k = torch.tensor([float(n)], dtype=torch.float64, device=device)
    dist.all_reduce(k)
    return float(t.item()), float(k.item())


class LocalRun:
    """Device-resident frame, gradients and outputs of one LocalICGNQuadtree
    workload, and the call through the C ABI."""

    def __init__(self, ctx, w):
        import ctypes
        import torch
        from staqdic import _lib
        self.ctx, self.w = ctx, w
        L = ctx.L
        W, H = w["f"].shape
        N = int(w["coordinatesFEM"].shape[0])
        self.W, self.H, self.N = W, H, N
        self.ws_list = np.ascontiguousarray(w["winsize_list"], dtype=np.int32)

        def dev(a, dt):
            return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=dt).ravel(order="F"))).cuda()

        f32, g32 = dev(w["f"], np.float32), dev(w["g"], np.float32)
        mask = dev(w["maskf"], np.uint8)
        self.coords = dev(w["coordinatesFEM"], np.float64)
        self.U0 = dev(w["U0"], np.float64)
        self.wsl = dev(self.ws_list, np.int32)
        gx32 = torch.empty((W - 6) * (H - 6), dtype=torch.float32, device="cuda")
        gy32 = torch.empty_like(gx32)
        ctx.check(L.stdic_img_gradient(ctx.h, f32.data_ptr(), mask.data_ptr(), W, H, gx32.data_ptr(),
                                       gy32.data_ptr(), _lib.STDIC_F32), "gradient")
        f64, g64 = f32.double(), g32.double()
        gx64 = torch.empty((W - 6) * (H - 6), dtype=torch.float64, device="cuda")
        gy64 = torch.empty_like(gx64)
        ctx.check(L.stdic_img_gradient(ctx.h, f64.data_ptr(), mask.data_ptr(), W, H, gx64.data_ptr(),
                                       gy64.data_ptr(), _lib.STDIC_F64), "gradient64")
        self.keep = (f32, g32, mask, f64, g64, gx64, gy64)
        self.gx32, self.gy32 = gx32, gy32

        def frame(f, g, gx, gy, dtype):
            fr = _lib.Frame()
            fr.f, fr.g, fr.mask, fr.dfdx, fr.dfdy = f.data_ptr(), g.data_ptr(), mask.data_ptr(), gx.data_ptr(), gy.data_ptr()
            fr.W, fr.H, fr.dtype = W, H, dtype
            return fr

        self.fr32 = frame(f32, g32, gx32, gy32, _lib.STDIC_F32)
        self.fr64 = frame(f64, g64, gx64, gy64, _lib.STDIC_F64)
        self.U = torch.empty(2 * N, dtype=torch.float64, device="cuda")
        self.F = torch.empty(4 * N, dtype=torch.float64, device="cuda")
        self.Hp = torch.empty(21 * N, dtype=torch.float64, device="cuda")
        self.conv = torch.empty(N, dtype=torch.int32, device="cuda")
        self.mark = torch.empty(N, dtype=torch.uint8, device="cuda")
        self.badnum = torch.zeros(1, dtype=torch.int32, device="cuda")
        ws_max = int(self.ws_list.max())

        def solve(fr, prec):
            ctx.check(L.stdic_icgn_local(ctx.h, ctypes.byref(fr), self.U0.data_ptr(), self.coords.data_ptr(), N,
                                         ws_max, self.wsl.data_ptr(), TOL, self.U.data_ptr(), self.F.data_ptr(),
                                         self.Hp.data_ptr(), self.conv.data_ptr(), self.mark.data_ptr(),
                                         self.badnum.data_ptr(), prec), "icgn_local")

        self.solve = solve


def converged_within(Ub, cb, Up):
    """Converged subsets of a batched result within TOLPX of the plain FP64 one."""
    dU = np.abs(Ub - Up).reshape(-1, 2).max(axis=1)
    return (cb >= 1) & (cb <= 100) & ~np.isnan(Ub[0::2]) & ~np.isnan(Up[0::2]) & (dU <= TOLPX)


def measure_c3(ctx, torch, flush, steps=5):
    """The 2048^2 quadtree with hole (config C3): one LocalICGNQuadtree pass,
    batched FP32 against the plain FP64 drop-in and the host CPU."""
    from staqdic import _lib
    w = make_workload("hole2048")
    run = LocalRun(ctx, w)

    def timed(fr, prec, k):
        ms = []
        for i in range(k):
            flush.fill_(float(i))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            run.solve(fr, prec)
            e1.record()
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        return float(np.mean(ms))

    run.solve(run.fr64, _lib.STDIC_PLAIN_F64)
    torch.cuda.synchronize()
    Up, cp = run.U.cpu().numpy(), run.conv.cpu().numpy()
    plain_ms = timed(run.fr64, _lib.STDIC_PLAIN_F64, 2)
    plain_conv = int(((cp >= 1) & (cp <= 100) & ~np.isnan(Up[0::2])).sum())
    for _ in range(3):
        run.solve(run.fr32, _lib.STDIC_BATCHED_F32)
    bat_ms = timed(run.fr32, _lib.STDIC_BATCHED_F32, steps)
    Ub, cb = run.U.cpu().numpy(), run.conv.cpu().numpy()
    n_conv = int(converged_within(Ub, cb, Up).sum())
    out = {"workload": "hole2048: 2048x2048 plate with hole, Kirsch 2%% strain, quadtree, %d nodes" % run.N,
           "value": n_conv / (bat_ms * 1e-3), "ms_per_step": bat_ms, "unit": UNIT,
           "plain_fp64": {"value": plain_conv / (plain_ms * 1e-3), "ms_per_step": plain_ms},
           "codes_equal_frac": float(np.mean(cb == cp))}
    out["batched_over_plain"] = out["value"] / out["plain_fp64"]["value"]
    cpu = cpu_baseline(w, "hole2048")
    if cpu and cpu.get("value"):
        out["cpu_baseline"] = cpu
        out["batched_over_cpu"] = out["value"] / cpu["value"]
    out["admm"] = measure_admm(ctx, torch, run)
    return out


def measure_admm(ctx, torch, run):
    """ADMM iterations (Subpb1 batched FP32, fill, Subpb2 FP64 PCG, strain, dual
    update) on the C3 mesh after its local pass, through stdic_admm with
    device-resident state: the first iteration runs directly, the others
    replay one captured CUDA graph.  mu = 1e-3, beta = 1e-3 * step^2 * mu.

    Two Dirichlet sets: the reference's markCoordHoleEdge rule (border and
    every refined element, grown twice), which on this mesh leaves no free
    node, so Subpb2 reduces to its assembly; and the border band alone, which
    leaves the refined region free and makes the Jacobi-PCG solve it."""
    from staqdic import synth
    w = run.w
    el = w["elementsFEM"]
    inv = np.unique(el[:, :8])
    inv = inv[inv > 0]
    out = {}
    for name, dset in (("reference_dirichlet", w["dirichlet"]),
                       ("border_dirichlet", synth.dirichlet_nodes(w["coordinatesFEM"], el, w["winstepsize"], False))):
        r = guarded(admm_timing, ctx, torch, run, dset)
        r["free_nodes"] = int(np.setdiff1d(inv, dset).size)
        out[name] = r
    return out


def admm_timing(ctx, torch, run, dirichlet_nodes):
    import ctypes
    from staqdic import _lib
    L = ctx.L
    w = run.w
    N = run.N
    dev = lambda a, dt: torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=dt).ravel(order="F"))).cuda()
    elems = dev(w["elementsFEM"], np.int32)
    E = int(w["elementsFEM"].shape[0])
    dirichlet = dev(dirichlet_nodes, np.int32)
    nd = int(np.asarray(dirichlet_nodes).size)
    wl2 = dev(np.stack([run.ws_list, run.ws_list], 1), np.int32)
    mu = 1e-3
    beta = 1e-3 * float(w["winstepsize"]) ** 2 * mu
    # initial state: the batched local pass, filled, and its strain
    run.solve(run.fr32, _lib.STDIC_BATCHED_F32)
    U2 = run.U.clone()
    ctx.check(L.stdic_fill_nans(ctx.h, run.coords.data_ptr(), N, elems.data_ptr(), E, U2.data_ptr()), "fill")
    F2 = torch.empty(4 * N, dtype=torch.float64, device="cuda")
    ctx.check(L.stdic_nodal_strain(ctx.h, run.coords.data_ptr(), N, elems.data_ptr(), E, U2.data_ptr(), 2,
                                   F2.data_ptr()), "strain")
    F2 = torch.nan_to_num(F2)
    state0 = (U2, F2, torch.zeros(4 * N, dtype=torch.float64, device="cuda"),
              torch.zeros(2 * N, dtype=torch.float64, device="cuda"))
    U1 = torch.empty(2 * N, dtype=torch.float64, device="cuda")
    used = ctypes.c_int(0)

    def go(steps, graph):
        U2_, F2_, ud_, vd_ = (t.clone() for t in state0)
        bad = torch.zeros(steps, dtype=torch.int32, device="cuda")
        its = torch.zeros(steps, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        ctx.check(L.stdic_admm(ctx.h, ctypes.byref(run.fr32), run.coords.data_ptr(), N, elems.data_ptr(), E,
                               dirichlet.data_ptr(), nd, wl2.data_ptr(), run.mark.data_ptr(), mu, beta, TOL,
                               steps, _lib.STDIC_BATCHED_F32, 1 if graph else 0, U2_.data_ptr(), F2_.data_ptr(),
                               ud_.data_ptr(), vd_.data_ptr(), U1.data_ptr(), bad.data_ptr(), its.data_ptr(),
                               ctypes.byref(used)), "admm")
        e1.record()
        e1.synchronize()
        return e0.elapsed_time(e1), bad.cpu().tolist(), its.cpu().tolist()

    go(1, False)
    t1, _, _ = go(1, False)
    t3, bad, its = go(3, True)
    graph_used = bool(used.value)
    t4, _, _ = go(4, True)
    return {"iterations": 3, "ms_3_iterations": t3, "ms_per_graph_iteration": (t4 - t1) / 3,
            "ms_first_iteration": t1, "graph_used": graph_used, "badnum": bad, "pcg_iters": its,
            "mu": mu, "beta": beta, "dirichlet_nodes": nd}


def measure_c5(ctx, torch, flush, steps=3):
    """16 deformed frames (rotation 2k degrees plus a crack opening) of one
    1024^2 reference frame and quadtree mesh (config C5): one multi-frame
    batched launch against the 16 frames one by one, device-resident inputs."""
    import ctypes
    from staqdic import _lib
    w = make_workload("series1024")
    L = ctx.L
    W, H = w["f"].shape
    N = int(w["coordinatesFEM"].shape[0])
    P = len(w["g_list"])
    dev = lambda a, dt: torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=dt).ravel(order="F"))).cuda()
    f32 = dev(w["f"], np.float32)
    g32 = torch.cat([dev(g, np.float32) for g in w["g_list"]])
    mask = dev(w["maskf"], np.uint8)
    wl = np.ascontiguousarray(w["winsize_list"], dtype=np.int32)
    wsl, coords = dev(wl, np.int32), dev(w["coordinatesFEM"], np.float64)
    U0 = torch.cat([dev(u, np.float64) for u in w["U0_list"]])
    gx = torch.empty((W - 6) * (H - 6), dtype=torch.float32, device="cuda")
    gy = torch.empty_like(gx)
    ctx.check(L.stdic_img_gradient(ctx.h, f32.data_ptr(), mask.data_ptr(), W, H, gx.data_ptr(), gy.data_ptr(),
                                   _lib.STDIC_F32), "gradient")
    U = torch.empty(2 * N * P, dtype=torch.float64, device="cuda")
    F = torch.empty(4 * N * P, dtype=torch.float64, device="cuda")
    conv = torch.empty(N * P, dtype=torch.int32, device="cuda")
    ws_max = int(wl.max())

    def frame(gptr):
        fr = _lib.Frame()
        fr.f, fr.g, fr.mask, fr.dfdx, fr.dfdy = f32.data_ptr(), gptr, mask.data_ptr(), gx.data_ptr(), gy.data_ptr()
        fr.W, fr.H, fr.dtype = W, H, _lib.STDIC_F32
        return fr

    fr_all = frame(g32.data_ptr())

    def multi():
        ctx.check(L.stdic_icgn_subsets_frames(ctx.h, ctypes.byref(fr_all), P, U0.data_ptr(), coords.data_ptr(), N,
                                              ws_max, wsl.data_ptr(), TOL, U.data_ptr(), F.data_ptr(), None,
                                              conv.data_ptr(), _lib.STDIC_BATCHED_F32), "frames")

    frs = [frame(g32.data_ptr() + 4 * W * H * k) for k in range(P)]

    def singles():
        for k in range(P):
            ctx.check(L.stdic_icgn_subsets(ctx.h, ctypes.byref(frs[k]), U0.data_ptr() + 16 * N * k,
                                           coords.data_ptr(), N, ws_max, wsl.data_ptr(), TOL,
                                           U.data_ptr() + 16 * N * k, F.data_ptr() + 32 * N * k, None,
                                           conv.data_ptr() + 4 * N * k, _lib.STDIC_BATCHED_F32), "single")

    def timed(fn):
        for _ in range(2):
            fn()
        ms = []
        for i in range(steps):
            flush.fill_(float(i))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        return float(np.mean(ms))

    ms_single = timed(singles)
    c_single, U_single = conv.cpu().numpy(), U.cpu().numpy()
    ms_multi = timed(multi)
    c_multi, U_multi = conv.cpu().numpy(), U.cpu().numpy()
    nconv = int(((c_multi >= 1) & (c_multi <= 100) & ~np.isnan(U_multi[0::2])).sum())
    same = (c_multi == c_single) & (c_multi >= 1) & (c_multi <= 100)
    dU = np.abs(U_multi - U_single).reshape(-1, 2).max(axis=1)
    return {"workload": "series1024: %d frames of %dx%d, rotation 2k deg + crack, quadtree %d nodes" % (P, W, H, N),
            "subsets_per_launch": N * P, "value": nconv / (ms_multi * 1e-3), "unit": UNIT,
            "ms_per_launch": ms_multi, "frames_one_by_one": {"value": nconv / (ms_single * 1e-3),
                                                             "ms": ms_single},
            "codes_equal_frac": float(np.mean(c_multi == c_single)),
            "max_abs_du_px_equal_codes": float(dU[same].max()) if same.any() else None}


def measure_adjoint(ctx, torch, size=4096):
    """Adjoint of the subset ZNSSD cost on the bumps field (config C4: 4096^2,
    ws 32, step 16), FP32, both modes, with dg."""
    import staqdic
    w = make_workload("bumps4096", size=size)
    c = w["coordinatesFEM"]
    N = c.shape[0]
    rng = np.random.default_rng(0)
    dev = lambda a, dt: torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=dt).ravel(order="F"))).cuda()
    U = dev(w["Utrue"] + rng.normal(0, 0.2, 2 * N), np.float64)
    F = dev(rng.normal(0, 0.005, 4 * N), np.float64)
    f, g, ct = dev(w["f"], np.float32), dev(w["g"], np.float32), dev(c, np.float64)
    W, H = w["f"].shape
    out = {"workload": "bumps4096: %dx%d speckle, 8 Gaussian displacement bumps, %d subsets of 32 px" % (W, H, N)}
    for mode in ("recompute", "store"):
        for _ in range(2):
            staqdic.icgn_adjoint(U, F, ct, f, g, 32, precision="batched", mode=mode, size=(W, H), ctx=ctx)
        torch.cuda.synchronize()
        ms = []
        for _ in range(5):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            staqdic.icgn_adjoint(U, F, ct, f, g, 32, precision="batched", mode=mode, size=(W, H), ctx=ctx)
            e1.record()
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        out[mode] = {"ms": float(np.mean(ms)), "subsets_per_s": N / (np.mean(ms) * 1e-3)}
    return out


# ----------------------------------------------------------------------------
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="hole1024")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the 2048^2 (C3) pass and the 4096^2 adjoint (C4) timing")
    ap.add_argument("--only", choices=["c3", "admm", "adjoint", "c5"],
                    help="run one secondary measurement alone and print it (for profiling)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, world, rank)

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    import staqdic
    from staqdic import _lib

    ctx = staqdic.Context(local)
    # one non-default stream for torch and the library, so the CUDA events of
    # the timed region bracket the library's kernels
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    L = ctx.L
    if args.only:
        flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
        if args.only == "admm":
            res = measure_admm(ctx, torch, LocalRun(ctx, make_workload("hole2048")))
        elif args.only == "c3":
            res = measure_c3(ctx, torch, flush)
        elif args.only == "adjoint":
            res = measure_adjoint(ctx, torch)
        else:
            res = measure_c5(ctx, torch, flush)
        print(json.dumps({"only": args.only, "result": res}), flush=True)
        ctx.close()
        return 0
    w = make_workload(args.workload)
    run = LocalRun(ctx, w)
    W, H, N, ws_list = run.W, run.H, run.N, run.ws_list
    fr32, fr64, solve = run.fr32, run.fr64, run.solve
    U, F, conv = run.U, run.F, run.conv
    gx32, gy32 = run.gx32, run.gy32
    import ctypes

    # ---- plain FP64 drop-in: accuracy reference and the 'plain' throughput
    solve(fr64, _lib.STDIC_PLAIN_F64)
    torch.cuda.synchronize()
    U_plain = U.clone()
    F_plain = F.clone()
    conv_plain = conv.clone()
    plain_ms = []
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    for _ in range(2):
        flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        solve(fr64, _lib.STDIC_PLAIN_F64)
        e1.record()
        e1.synchronize()
        plain_ms.append(e0.elapsed_time(e1))
    plain_conv = int((((conv_plain >= 1) & (conv_plain <= 100)) & ~torch.isnan(U_plain[0::2])).sum())
    plain_value = plain_conv / (np.mean(plain_ms) * 1e-3)

    # ---- batched FP32: warm-up (the first call autotunes), then K timed steps
    for _ in range(args.warmup):
        solve(fr32, _lib.STDIC_BATCHED_F32)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = ctx.launches
    sampler = ClockSampler(local)
    sampler.start()
    step_ms, solver_ms = [], []
    t_wall0 = time.perf_counter()
    for _ in range(args.steps):
        flush.fill_(float(len(step_ms)))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        solve(fr32, _lib.STDIC_BATCHED_F32)
        e1.record()
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        solver_ms.append(ctx.last_solver_ms())
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall0
    clocks = sampler.stop()
    launches = ctx.launches - launches0
    if dist:
        dist.barrier()

    # accuracy and the converged count of the last step
    Uc, cc = U.cpu().numpy(), conv.cpu().numpy()
    Fc = F.cpu().numpy()
    Up, cp = U_plain.cpu().numpy(), conv_plain.cpu().numpy()
    dU = np.abs(Uc - Up).reshape(-1, 2).max(axis=1)
    ok = (cc >= 1) & (cc <= 100) & ~np.isnan(Uc[0::2]) & ~np.isnan(Up[0::2]) & (dU <= TOLPX)
    n_conv = int(ok.sum())
    total_ms = float(np.sum(step_ms))
    mean_ms = total_ms / len(step_ms)
    if dist:
        mean_ms, n_conv_all = reduce_over_ranks(dist, mean_ms, n_conv, "cuda")
    else:
        n_conv_all = float(n_conv)
    value = n_conv_all / (mean_ms * 1e-3)

    # ---- end to end through the C ABI with pinned host buffers
    def pinned(a, dt):
        t = torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=dt).ravel(order="F"))).pin_memory()
        return t

    hf, hg, hm = pinned(w["f"], np.float32), pinned(w["g"], np.float32), pinned(w["maskf"], np.uint8)
    hgx, hgy = gx32.cpu().pin_memory(), gy32.cpu().pin_memory()
    hU0, hc, hw = pinned(w["U0"], np.float64), pinned(w["coordinatesFEM"], np.float64), pinned(ws_list, np.int32)
    oU = torch.empty(2 * N, dtype=torch.float64).pin_memory()
    oF = torch.empty(4 * N, dtype=torch.float64).pin_memory()
    oH = torch.empty(21 * N, dtype=torch.float64).pin_memory()
    oc = torch.empty(N, dtype=torch.int32).pin_memory()
    om = torch.empty(N, dtype=torch.uint8).pin_memory()
    hb = ctypes.c_int(0)
    hfr = _lib.Frame()
    hfr.f, hfr.g, hfr.mask, hfr.dfdx, hfr.dfdy = hf.data_ptr(), hg.data_ptr(), hm.data_ptr(), hgx.data_ptr(), hgy.data_ptr()
    hfr.W, hfr.H, hfr.dtype = W, H, _lib.STDIC_F32
    h2d = sum(t.numel() * t.element_size() for t in (hf, hg, hm, hgx, hgy, hU0, hc, hw))
    d2h = sum(t.numel() * t.element_size() for t in (oU, oF, oH, oc, om)) + 4

    def solve_host():
        ctx.check(L.stdic_icgn_local(ctx.h, ctypes.byref(hfr), hU0.data_ptr(), hc.data_ptr(), N, WS_MAX,
                                     hw.data_ptr(), TOL, oU.data_ptr(), oF.data_ptr(), oH.data_ptr(),
                                     oc.data_ptr(), om.data_ptr(), ctypes.byref(hb), _lib.STDIC_BATCHED_F32),
                  "icgn_local host")

    for _ in range(2):
        solve_host()
    if dist:
        dist.barrier()
    e2e_ms = []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        solve_host()  # H2D copies, kernels, D2H copies, stream sync
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
    oUn, ocn = oU.numpy(), oc.numpy()
    dUe = np.abs(oUn - Up).reshape(-1, 2).max(axis=1)
    n_conv_e2e = int(((ocn >= 1) & (ocn <= 100) & ~np.isnan(oUn[0::2]) & ~np.isnan(Up[0::2]) & (dUe <= TOLPX)).sum())
    e2e_mean = float(np.mean(e2e_ms))
    if dist:
        e2e_mean, n_conv_e2e = reduce_over_ranks(dist, e2e_mean, n_conv_e2e, "cuda")
    e2e_value = n_conv_e2e / (e2e_mean * 1e-3)

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0

    # ---- roofline of the dominant kernel (the batched persistent IC-GN)
    peaks, src = measured_peaks()
    fp32_peak = fp32_peak_tflops(torch)
    flops = float(flops_per_subset(cc, ws_list).sum())
    sv = [s for s in solver_ms if s > 0]
    kern_ms = float(np.mean(sv)) if sv else mean_ms
    achieved = flops / (kern_ms * 1e-3) / 1e12
    alg_bytes = (2 * 4 * W * H + W * H + 2 * 4 * (W - 6) * (H - 6) + N * (16 + 16 + 4 + 16 + 32 + 168 + 4 + 1))
    traffic = traffic_from_profiles()
    roofline = {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                "frac": achieved / fp32_peak,
                "traffic": traffic,
                "peak_source": "cuBLAS SGEMM 8192^3 with TF32 off, measured in this run "
                               "(MEASURED_PEAKS.json has no FP32 CUDA-core figure)",
                "flops_per_launch": flops, "kernel_ms": kern_ms}
    roofline_hbm = {"bound": "hbm", "achieved": alg_bytes / (kern_ms * 1e-3) / 1e9,
                    "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                    "frac": alg_bytes / (kern_ms * 1e-3) / 1e9 / peaks.get("hbm_gbs"),
                    "traffic": traffic, "algorithmic_bytes_per_launch": alg_bytes,
                    "peak_source": src}

    both_conv = (cc >= 1) & (cc <= 100) & (cp >= 1) & (cp <= 100)
    dF = np.abs(Fc - F_plain.cpu().numpy()).reshape(-1, 4).max(axis=1)
    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(w, args.workload)

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": mean_ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": workload_config(args.workload, w),
           "precision": "batched FP32 (FMA sums, FP64 Hessian inverses)",
           "l2": "flushed between timed steps (256 MiB write)",
           "parallelism": "replicas" if world > 1 else "single GPU",
           "clocks": clocks,
           "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                   "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_mean},
           "gpu_launches": int(launches),
           "roofline": roofline,
           "roofline_hbm": roofline_hbm,
           "plain_fp64": {"value": plain_value, "ms_per_step": float(np.mean(plain_ms)),
                          "converged": plain_conv},
           "batched_over_plain": value / plain_value if plain_value > 0 else None,
           "accuracy": {"converged": n_conv, "nodes": N,
                        "max_abs_du_px_converged": float(np.nanmax(dU[both_conv])) if both_conv.any() else None,
                        "max_abs_dF_converged": float(np.nanmax(dF[both_conv])) if both_conv.any() else None,
                        "codes_equal_frac": float(np.mean(cc == cp))},
           "wall_s_timed": t_wall}
    if cpu:
        out["cpu_baseline"] = cpu
        out["batched_over_cpu"] = value / cpu["value"] if cpu.get("value") else None
    if world == 1 and not args.no_extras:
        out["c3"] = guarded(measure_c3, ctx, torch, flush)
        out["adjoint_c4"] = guarded(measure_adjoint, ctx, torch)
        out["c5"] = guarded(measure_c5, ctx, torch, flush)
    print(json.dumps(out), flush=True)
    if dist:
        dist.destroy_process_group()
    ctx.close()
    return 0


def guarded(fn, *args):
    """One secondary measurement: its failure is reported in its own object and
    leaves the headline line intact."""
    try:
        return fn(*args)
    except Exception as e:  # pragma: no cover
        return {"error": "%s: %s" % (type(e).__name__, e)}


def cpu_baseline(w, name):
    """The oracle (FP64 C++ restatement, OpenMP on all host cores) on a bounded
    sample of the same workload, about 10-20 s of CPU work."""
    try:
        from oracle import build as ob
        ob.build_oracle()
        from oracle import oracle as orc
    except Exception as e:  # pragma: no cover
        return {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                "sample": "oracle unavailable: %s" % e}
    f = w["f"].astype(np.float64)
    g = w["g"].astype(np.float64)
    Df = orc.funImgGradient(f, w["maskf"])
    coords = w["coordinatesFEM"]
    N = coords.shape[0]
    cores = os.cpu_count() or 1
    orc.set_threads(cores)
    k = max(1, N // 4000)
    idx = np.arange(0, N, k)
    U0 = w["U0"].reshape(-1, 2)[idx].ravel()
    cs = coords[idx]
    wl = w["winsize_list"][idx]
    orc.icgn6(U0, cs, Df, f, g, wl, TOL)
    t0 = time.perf_counter()
    nconv, reps = 0, 0
    while reps < 20 and (time.perf_counter() - t0) < 10.0:
        U, F, Hp, conv, mark = orc.icgn6(U0, cs, Df, f, g, wl, TOL)
        nconv += int(((conv >= 1) & (conv <= 100)).sum())
        reps += 1
    dt = time.perf_counter() - t0
    return {"value": nconv / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "%d of %d nodes of %s (every %d-th) x %d repeats, FP64, OpenMP %d threads" % (
                idx.size, N, name, k, reps, cores)}


if __name__ == "__main__":
    sys.exit(main())
