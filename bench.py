"""Benchmark of the STAQ-DIC hot path on GB300.

Metric: converged IC-GN subsets per second, counting a subset only when its
code is 1..100, the LocalICGNQuadtree bad-subset filter (LocalICGNQuadtree.m:
153-169) kept it (its U is not NaN) and its displacement is within 0.01 px of
the FP64 solution on the same inputs.  Both arms count by that one rule: the
GPU arm against the plain FP64 drop-in (equal to the FP64 oracle to 1e-6 px),
the CPU arm is FP64 itself.

Step (default workload hole2048, the 2048^2 quadtree config): one
LocalICGNQuadtree pass -- the batched FP32 persistent kernel behind
stdic_icgn_local -- over all 80,695 nodes of a seeded 2048^2 plate-with-hole
pair (Kirsch field at 2 % strain, quadtree 4..32 px, uneven subsets 8..64 px).
Inputs are resident in HBM (`value`); the same call with pinned host buffers,
copies inside the timed region, gives `e2e`.  The L2 is flushed (256 MiB write)
between timed steps.

Beside the headline the line carries the plain FP64 drop-in on the same pass
(`plain_fp64`, with its FP64-pipe roofline), the CPU port on the whole mesh
(`cpu_baseline`, median of 5 runs), and, on one GPU, the 1024^2 quadtree pass
(``c2``), three ADMM iterations on the 2048^2 mesh (``admm``), the adjoint on
the 4096^2 bumps pair (``adjoint_c4``) and 16 frames in one multi-frame launch
(``c5``); --no-extras skips them.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N > 1 runs one replica per GPU (the path has no data-path collective);
`value` is all ranks' converged subsets over the slowest rank's time.
--impl reference times the CPU implementation of the path on the host cores
(the reference is MATLAB, so the oracle's C++ restatement stands in) on the
same workload, the whole mesh every step.
"""
import argparse
import hashlib
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
DEFAULT_WORKLOAD = "hole2048"
# sources of the batched solver kernels: a traffic figure is quoted only from
# an ncu capture of exactly these sources
KERNEL_SOURCES = ("staq-dic_gb300/csrc/icgn_batched.cuh", "staq-dic_gb300/csrc/icgn_batched.cu",
                  "staq-dic_gb300/csrc/icgn_batched_tw1.cu", "staq-dic_gb300/csrc/icgn_batched_tw2.cu",
                  "staq-dic_gb300/csrc/icgn_batched_tw4.cu", "staq-dic_gb300/csrc/icgn_batched_tw8.cu",
                  "staq-dic_gb300/csrc/icgn_batched_tw1s.cu", "staq-dic_gb300/csrc/icgn_batched_tw2s.cu",
                  "staq-dic_gb300/csrc/icgn_batched_tw4s.cu", "staq-dic_gb300/csrc/icgn_batched_tw8s.cu",
                  "staq-dic_gb300/csrc/device_common.cuh", "staq-dic_gb300/csrc/kernels.h")


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


def converged_rule(U, conv, U_fp64=None):
    """The metric's rule: code 1..100, not NaN (kept by the bad-subset filter),
    and, when an FP64 solution is given, within 0.01 px of it."""
    ok = (conv >= 1) & (conv <= 100) & ~np.isnan(U[0::2])
    if U_fp64 is not None:
        dU = np.abs(U - U_fp64).reshape(-1, 2).max(axis=1)
        ok &= ~np.isnan(U_fp64[0::2]) & (dU <= TOLPX)
    return ok


def kernel_source_hash():
    h = hashlib.sha256()
    for rel in KERNEL_SOURCES:
        with open(os.path.join(ROOT, rel), "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()[:16]


def traffic_from_profile(workload):
    """DRAM bytes per pass of the batched solver from the committed ncu summary
    of this workload, quoted only when that capture was taken of the current
    kernel sources (the summary records their hash)."""
    p = os.path.join(ROOT, "profiles", "icgn_batched_%s.md" % workload)
    if not os.path.exists(p):
        return None, "no ncu summary of this workload"
    sha, val = None, None
    for ln in open(p):
        s = ln.strip()
        if s.startswith("kernel_sources_sha256_16:"):
            sha = s.split(":", 1)[1].strip()
        elif s.startswith("dram_bytes_per_pass:"):
            try:
                val = float(s.split(":", 1)[1].strip().split()[0])
            except ValueError:
                val = None
    cur = kernel_source_hash()
    if sha != cur:
        return None, "the ncu summary was captured on other kernel sources (%s, now %s)" % (sha, cur)
    return val, "ncu capture of these kernel sources (%s), profiles/icgn_batched_%s.md" % (cur, workload)


class ClockSampler:
    """nvidia-smi clock / throttle samples around and during the timed region:
    the last sample before it starts, every sample inside it, and the first
    after it ends (so a region shorter than the 100 ms period still has two)."""

    NAMES = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self, index=0):
        self.index = index
        self.samples = []  # (host time, line)
        self.proc = None
        self.t0 = self.t1 = None

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
            t = time.perf_counter()
            while not self.samples and time.perf_counter() - t < 3.0 and self.proc.poll() is None:
                time.sleep(0.01)
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append((time.perf_counter(), line.strip()))

    def region_start(self):
        self.t0 = time.perf_counter()

    def region_end(self):
        self.t1 = time.perf_counter()
        if self.proc is not None:
            t = time.perf_counter()
            while (not any(ts > self.t1 for ts, _ in self.samples) and time.perf_counter() - t < 1.0
                   and self.proc.poll() is None):
                time.sleep(0.01)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        s = list(self.samples)
        t0 = self.t0 if self.t0 is not None else -1e30
        t1 = self.t1 if self.t1 is not None else 1e30
        before = [x for x in s if x[0] <= t0][-1:]
        inside = [x for x in s if t0 < x[0] <= t1]
        after = [x for x in s if x[0] > t1][:1]
        sm, smax, reasons = [], [], set()
        for _, ln in before + inside + after:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(self.NAMES, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "samples_inside": len(inside)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def gemm_peak_tflops(torch, dtype, n):
    """CUDA-core throughput of one precision: a cuBLAS GEMM n^3 (TF32 off),
    best of 5 (the burst figure, for kernels timed alone)."""
    old = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        a = torch.randn(n, n, device="cuda", dtype=dtype)
        b = torch.randn(n, n, device="cuda", dtype=dtype)
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


# ----------------------------------------------------------------------------
def workload_config(name, w):
    """The config object both arms print for a LocalICGNQuadtree workload."""
    W, H = w["f"].shape
    ws = np.asarray(w["winsize_list"])
    return {"workload": "%s: %dx%d plate with hole, Kirsch %g%% strain, quadtree, %d nodes, subsets 8..64 px, "
                        "one LocalICGNQuadtree pass per step" % (name, W, H, 100 * w.get("eps", 0),
                                                                  w["coordinatesFEM"].shape[0]),
            "nodes": int(w["coordinatesFEM"].shape[0]),
            "subset_sizes": {str(k): int(v) for k, v in zip(*np.unique(ws, return_counts=True))},
            "count_rule": "code 1..100 after the LocalICGNQuadtree.m:153-169 bad-subset filter, "
                          "within 0.01 px of FP64"}


class CpuPass:
    """The oracle (FP64 C++ restatement, OpenMP over subsets on all host cores)
    running LocalICGNQuadtree over the whole mesh of a workload."""

    def __init__(self, w):
        from oracle import build as ob
        ob.build_oracle()
        from oracle import oracle as orc
        self.orc = orc
        self.w = w
        self.f = w["f"].astype(np.float64)
        self.g = w["g"].astype(np.float64)
        self.Df = orc.funImgGradient(self.f, w["maskf"])
        self.cores = os.cpu_count() or 1
        orc.set_threads(self.cores)
        self.out = None

    def run(self):
        w = self.w
        t0 = time.perf_counter()
        out = self.orc.LocalICGNQuadtree(w["U0"], w["coordinatesFEM"], self.Df, self.f, self.g,
                                         w["winsize_list"], TOL)
        dt = time.perf_counter() - t0
        self.out = out
        U, F, Hp, conv, badnum, mark = out
        return dt, int(converged_rule(U, conv).sum())

    def measure(self, runs, warm=1):
        for _ in range(warm):
            self.run()
        ts, n = [], 0
        for _ in range(runs):
            dt, n = self.run()
            ts.append(dt)
        med = float(np.median(ts))
        return {"value": n / med, "unit": UNIT, "cores": self.cores, "kind": "port",
                "ms_median": 1e3 * med, "runs": runs, "converged": n,
                "sample": "whole mesh (%d nodes) of %s, LocalICGNQuadtree with its bad-subset filter, FP64, "
                          "OpenMP %d threads, median of %d runs" % (self.w["coordinatesFEM"].shape[0],
                                                                     self.w["name"], self.cores, runs)}


def run_reference(args, world, rank):
    """CPU implementation of the path on the host cores (oracle port), on the
    same workload, metric and counting rule as the GPU arm."""
    if rank != 0:
        return 0
    w = make_workload(args.workload)
    cp = CpuPass(w)
    for _ in range(args.warmup):
        cp.run()
    ts, n = [], 0
    for _ in range(args.steps):
        dt, n = cp.run()
        ts.append(dt)
    med = float(np.median(ts))
    val = n / med
    sample = "whole mesh (%d nodes) of %s every step, FP64 LocalICGNQuadtree with its bad-subset filter, " \
             "%d OpenMP threads, median step of %d" % (w["coordinatesFEM"].shape[0], args.workload, cp.cores,
                                                       args.steps)
    out = {"metric": METRIC, "value": val, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * med, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "impl": "reference", "parallelism": "host threads", "precision": "FP64 (the oracle port)",
           "ms_per_step_mean": 1e3 * float(np.mean(ts)),
           "config": workload_config(args.workload, w),
           "cpu_baseline": {"value": val, "unit": UNIT, "cores": cp.cores, "kind": "port", "sample": sample},
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

    def host(self):
        return self.U.cpu().numpy(), self.F.cpu().numpy(), self.conv.cpu().numpy()


def timed_solves(torch, run, fr, prec, k, flush):
    """k solves, each bracketed by CUDA events on the library's stream, with
    the L2 flushed before each; returns per-call ms and the solver kernels' ms."""
    ms, kern = [], []
    for i in range(k):
        flush.fill_(float(i))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        run.solve(fr, prec)
        e1.record()
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
        kern.append(run.ctx.last_solver_ms())
    return ms, kern


def accuracy(Ub, Fb, cb, Ur, Fr, cr):
    """Batched against an FP64 solution: max |du| and |dF| over the subsets
    that stop at the same iteration in both (the strict bar: 0.01 px, 1e-4),
    the same over all subsets converged in both (a subset whose stopping test
    lands on the other side of the tolerance takes one step more or less, a
    step of up to ~1e-3 in F), and the share of equal result codes."""
    both = (cb >= 1) & (cb <= 100) & (cr >= 1) & (cr <= 100) & ~np.isnan(Ub[0::2]) & ~np.isnan(Ur[0::2])
    same = both & (cb == cr)
    dU = np.abs(Ub - Ur).reshape(-1, 2).max(axis=1)
    dF = np.abs(Fb - Fr).reshape(-1, 4).max(axis=1)
    return {"max_abs_du_px_equal_codes": float(np.max(dU[same])) if same.any() else None,
            "max_abs_dF_equal_codes": float(np.max(dF[same])) if same.any() else None,
            "max_abs_du_px_converged": float(np.max(dU[both])) if both.any() else None,
            "max_abs_dF_converged": float(np.max(dF[both])) if both.any() else None,
            "codes_equal_frac": float(np.mean(cb == cr)),
            "within_0.01px_frac_of_both_converged": float(np.mean(dU[both] <= TOLPX)) if both.any() else None}


def plain_roofline(flops, ms, fp64_peak):
    a = flops / (ms * 1e-3) / 1e12
    return {"bound": "fp64", "achieved": a, "peak": fp64_peak, "unit": "TFLOP/s", "frac": a / fp64_peak,
            "peak_source": "cuBLAS DGEMM 4096^3, measured in this run (MEASURED_PEAKS.json has no FP64 figure)"}


def measure_local_extra(ctx, torch, flush, name, steps=10, with_cpu=True):
    """One LocalICGNQuadtree workload beside the headline: batched FP32 against
    the plain FP64 drop-in and the CPU port, by the same rule."""
    from staqdic import _lib
    w = make_workload(name)
    run = LocalRun(ctx, w)
    run.solve(run.fr64, _lib.STDIC_PLAIN_F64)
    torch.cuda.synchronize()
    Up, Fp, cp = run.host()
    plain_ms, _ = timed_solves(torch, run, run.fr64, _lib.STDIC_PLAIN_F64, 2, flush)
    plain_conv = int(converged_rule(Up, cp).sum())
    for _ in range(3):
        run.solve(run.fr32, _lib.STDIC_BATCHED_F32)
    bat_ms, kern = timed_solves(torch, run, run.fr32, _lib.STDIC_BATCHED_F32, steps, flush)
    Ub, Fb, cb = run.host()
    n_conv = int(converged_rule(Ub, cb, Up).sum())
    bms = float(np.mean(bat_ms))
    out = {"workload": workload_config(name, w)["workload"], "nodes": run.N,
           "value": n_conv / (bms * 1e-3), "ms_per_step": bms, "unit": UNIT, "converged": n_conv,
           "solver_kernels_ms": float(np.mean(kern)),
           "plain_fp64": {"value": plain_conv / (np.mean(plain_ms) * 1e-3), "ms_per_step": float(np.mean(plain_ms))},
           "accuracy_vs_plain_fp64": accuracy(Ub, Fb, cb, Up, Fp, cp)}
    out["batched_over_plain"] = out["value"] / out["plain_fp64"]["value"]
    if with_cpu:
        cpu = guarded(lambda: CpuPass(w).measure(5))
        out["cpu_baseline"] = cpu
        if cpu.get("value"):
            out["batched_over_cpu"] = out["value"] / cpu["value"]
    return out


def measure_admm(ctx, torch, run):
    """ADMM iterations (Subpb1 batched FP32, fill, Subpb2 FP64 PCG, strain, dual
    update) on the 2048^2 mesh after its local pass, through stdic_admm with
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
    1024^2 reference frame and quadtree mesh: one multi-frame batched launch
    against the 16 frames one by one, device-resident inputs."""
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
    """Adjoint of the subset ZNSSD cost on the bumps field (4096^2, ws 32,
    step 16), FP32, both modes, with dg."""
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
    # the FP64 oracle on all host cores over a seeded sample of subsets: its
    # throughput, and the FP32 gradients' error against it on that sample
    from oracle import build as ob
    ob.build_oracle()
    from oracle import oracle as orc
    orc.set_threads(os.cpu_count() or 1)
    idx = np.sort(rng.choice(N, min(N, 4000), replace=False))
    Uh, Fh = U.cpu().numpy().reshape(-1, 2)[idx].ravel(), F.cpu().numpy().reshape(-1, 4)[idx].ravel()
    f64, g64 = w["f"].astype(np.float64), w["g"].astype(np.float64)
    t0 = time.perf_counter()
    co, dUo, dFo, _ = orc.icgn_adjoint(f64, g64, None, c[idx], 32, Uh, Fh)
    dt = time.perf_counter() - t0
    _, cn, dU, dF, _ = staqdic.icgn_adjoint(U, F, ct, f, g, 32, precision="batched", want_dg=False, size=(W, H),
                                            ctx=ctx)
    dU = dU.cpu().numpy().reshape(-1, 2)[idx]
    dF = dF.cpu().numpy().reshape(-1, 4)[idx]
    ok = np.isfinite(co)
    gref = np.concatenate([dUo.reshape(-1, 2), dFo.reshape(-1, 4)], 1)[ok]
    gout = np.concatenate([dU, dF], 1)[ok]
    rel = np.linalg.norm(gout - gref, axis=1) / np.linalg.norm(gref, axis=1)
    out["cpu_oracle"] = {"subsets_per_s": idx.size / dt, "cores": os.cpu_count() or 1,
                         "sample": "%d seeded subsets, FP64 with dg" % idx.size}
    out["fp32_grad_rel_err_max"] = float(rel.max())
    return out


def measure_c1(ctx, torch, steps=20):
    """C1, the reference's CPU-runnable case: the 256^2 affine speckle pair, a
    uniform 14 x 14 grid of 32-px subsets (196 nodes).  The integer search
    (S = 6), the FP64 plain and FP32 batched LocalICGNQuadtree, one Subpb2
    solve, each through the public API with host arrays (copies included);
    the oracle on all host cores beside them."""
    import staqdic
    from oracle import build as ob
    ob.build_oracle()
    from oracle import oracle as orc
    orc.set_threads(os.cpu_count() or 1)
    w = make_workload("uniform256")
    c, el = w["coordinatesFEM"], w["elementsFEM"]
    N = c.shape[0]
    f64, g64 = w["f"].astype(np.float64), w["g"].astype(np.float64)
    W, H = f64.shape
    wl = np.asarray(w["winsize_list"], np.int32)

    def timed(fn, k):
        fn()
        ts = []
        for _ in range(k):
            t0 = time.perf_counter()
            r = fn()
            ts.append(time.perf_counter() - t0)
        return 1e3 * float(np.median(ts)), r

    out = {"workload": "uniform256: 256x256 affine speckle pair, %d subsets of 32 px" % N}
    ms, _ = timed(lambda: staqdic.funIntegerSearch(f64, g64, 6, (1, W), (1, H), 32, 16, ctx=ctx, qfactors=False), steps)
    cms, _ = timed(lambda: orc.funIntegerSearch(f64, g64, 6, (1, W), (1, H), 32, 16), 3)
    out["integer_search"] = {"ms_gpu": ms, "ms_cpu_oracle": cms}
    Df = staqdic.funImgGradient(f64, ImgRefMask=w["maskf"], ctx=ctx)
    Dfo = orc.funImgGradient(f64, w["maskf"])
    DP = {"winsize": int(wl.max()), "winsize_per_node": wl}
    res = {}
    for prec in ("plain", "batched"):
        ff, gg, D = (f64, g64, Df) if prec == "plain" else (w["f"], w["g"], staqdic.funImgGradient(
            w["f"], ImgRefMask=w["maskf"], ctx=ctx, dtype=np.float32))
        ms, r = timed(lambda: staqdic.LocalICGNQuadtree(w["U0"], c, D, ff, gg, DP, "GaussNewton", TOL, precision=prec,
                                                        ctx=ctx), steps)
        res[prec] = (ms, r)
    cms, ro = timed(lambda: orc.LocalICGNQuadtree(w["U0"], c, Dfo, f64, g64, wl, TOL), 3)
    Uo, convo = ro[0], ro[3]
    for prec, (ms, r) in res.items():
        U, conv = r[0], r[4]
        n = int(converged_rule(U, conv, Uo).sum())
        out[prec] = {"ms": ms, "subsets_per_s": n / (ms * 1e-3), "converged": n,
                     "max_abs_du_px_equal_codes": float(np.nanmax(np.abs(U - Uo).reshape(-1, 2).max(1)[conv == convo]))}
    out["cpu_oracle"] = {"ms": cms, "subsets_per_s": int(converged_rule(Uo, convo).sum()) / (cms * 1e-3),
                         "cores": os.cpu_count() or 1}
    mesh = {"coordinatesFEM": c, "elementsFEM": el, "dirichlet": w["dirichlet"]}
    beta, mu = 1e-3 * 16 ** 2 * 1e-3, 1e-3
    U1 = np.nan_to_num(res["plain"][1][0])
    F1 = np.zeros(4 * N)
    ms, _ = timed(lambda: staqdic.Subpb2Quadtree(mesh, 2, beta, mu, U1, F1, np.zeros(4 * N), np.zeros(2 * N), 0.0, 16,
                                                 ctx=ctx), steps)
    cms, _ = timed(lambda: orc.Subpb2Quadtree(c, el, w["dirichlet"], None, 2, beta, mu, U1, F1, 0.0, 16), 3)
    out["subpb2"] = {"ms_gpu": ms, "ms_cpu_oracle_direct_solve": cms}
    return out


def measure_mg(ctx, torch, steps=5):
    """The multigrid integer search (funIntegerSearchMg) on the 1024^2 and
    2048^2 plates with a hole (Kirsch field, up to ~20 px at 2048^2): one call
    through the public API with host images (the copies included), median of
    `steps` calls after a warm-up call; the oracle's NumPy/SciPy restatement
    timed once on the 1024^2 case (single-threaded FFTs and a direct sparse
    solve) as the CPU reference point."""
    import staqdic
    out = {}
    for name in ("hole1024", "hole2048"):
        w = make_workload(name)
        f, g = w["f"].astype(np.float64), w["g"].astype(np.float64)
        W, H = f.shape
        call = lambda: staqdic.funIntegerSearchMg(f, g, (1, W), (1, H), 32, 16, ctx=ctx, blocks=True)
        r = call()
        ts = []
        for _ in range(steps):
            torch.cuda.synchronize()
            t = time.perf_counter()
            r = call()
            ts.append(time.perf_counter() - t)
        ms = 1e3 * float(np.median(ts))
        ent = {"workload": "%s: %dx%d, winsize 32, step 16" % (name, W, H), "ms_per_call": ms,
               "grid": list(r[2].shape), "last_level_blocks": int(r[4]["blocks"].shape[0])}
        if name == "hole1024":
            from oracle import mg
            t = time.perf_counter()
            mg.funIntegerSearchMg(f, g, (1, W), (1, H), 32, 16)
            ent["cpu_oracle_ms"] = 1e3 * (time.perf_counter() - t)
            ent["cpu_oracle"] = "oracle/mg.py (NumPy FFT, SciPy sparse direct solve), one run"
        out[name] = ent
    return out


def measure_series(ctx, torch):
    """The accumulative frame loop (staqdic.series.run_series) over a loading
    sequence of ten 1024^2 frames of the plate with a hole (Kirsch field at
    0.2 % .. 2 % far-field strain, 19.9k quadtree nodes), batched FP32: the
    initial guess of each frame from the previous result (frames 1-4) or
    funPOR_GPR (frames 5-9), LocalICGNQuadtree, the NaN fill, all through the
    public API with host arrays.  The oracle's FP64 loop (oracle/series.py)
    is timed once on the same frames as the CPU reference point."""
    import staqdic
    from staqdic import series
    w = make_workload("ramp1024")
    mesh = {"coordinatesFEM": w["coordinatesFEM"], "elementsFEM": w["elementsFEM"]}
    Df = staqdic.funImgGradient(w["f"], ImgRefMask=w["maskf"], ctx=ctx, dtype=np.float32)
    call = lambda: series.run_series(mesh, Df, w["f"], w["g_list"], w["U0_first"], w["winsize_list"],
                                     precision="batched", ctx=ctx)
    call()
    torch.cuda.synchronize()
    t = time.perf_counter()
    r = call()
    ms = 1e3 * (time.perf_counter() - t)
    P, N = len(w["g_list"]), int(w["coordinatesFEM"].shape[0])
    nconv = sum(int(((c >= 1) & (c <= 100) & ~np.isnan(u[0::2])).sum()) for c, u in zip(r["conv"], r["U"]))
    err = [float(np.nanmedian(np.abs(u - ut).reshape(-1, 2).max(1))) for u, ut in zip(r["U"], w["Utrue_list"])]
    err0 = [float(np.nanmedian(np.abs(u - ut).reshape(-1, 2).max(1))) for u, ut in zip(r["U0"], w["Utrue_list"])]
    from oracle import oracle as orc
    from oracle import series as osr
    t = time.perf_counter()
    o = osr.run_series(mesh, w["f"], w["maskf"], w["g_list"], w["U0_first"], w["winsize_list"])
    cpu_ms = 1e3 * (time.perf_counter() - t)
    both = [((a >= 1) & (a <= 100) & (b >= 1) & (b <= 100) & ~np.isnan(x[0::2]) & ~np.isnan(y[0::2]))
            for a, b, x, y in zip(r["conv"], o["conv"], r["U"], o["U"])]
    dU = [np.abs(x - y).reshape(-1, 2).max(1)[m] for x, y, m in zip(r["U"], o["U"], both)]
    return {"workload": "ramp1024: %d frames of 1024x1024, Kirsch field 0.2%%..%.0f%% strain, quadtree %d nodes"
                        % (P, 0.2 * P, N),
            "ms_per_sequence": ms, "ms_per_frame": ms / P, "converged_subsets": nconv,
            "value": nconv / (ms * 1e-3), "unit": "converged subsets/s (host arrays, copies included)",
            "median_err_vs_truth_px": err, "median_guess_err_vs_truth_px": err0,
            "within_0_01px_of_oracle_frac": float(np.mean(np.concatenate(dU) <= 0.01)),
            "cpu_oracle_ms": cpu_ms, "cpu_oracle_threads": orc.num_threads(),
            "cpu_oracle": "oracle/series.py (the FP64 LocalICGNQuadtree restatement), one run"}


def guarded(fn, *args):
    """One secondary measurement: its failure is reported in its own object and
    leaves the headline line intact."""
    try:
        return fn(*args)
    except Exception as e:  # pragma: no cover
        return {"error": "%s: %s" % (type(e).__name__, e)}


# ----------------------------------------------------------------------------
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the 1024^2 pass, the ADMM iterations, the adjoint and the multi-frame launch")
    ap.add_argument("--only", choices=["c2", "admm", "adjoint", "c5", "mg", "c1", "series"],
                    help="run one secondary measurement alone and print it (for profiling)")
    ap.add_argument("--profile", choices=["batched", "plain"],
                    help="only the headline workload's passes of one form (warm-up + steps), for ncu captures")
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

    import ctypes
    import staqdic
    from staqdic import _lib

    ctx = staqdic.Context(local)
    # one non-default stream for torch and the library, so the CUDA events of
    # the timed region bracket the library's kernels
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    L = ctx.L
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    if args.only:
        if args.only == "admm":
            res = measure_admm(ctx, torch, LocalRun(ctx, make_workload(DEFAULT_WORKLOAD)))
        elif args.only == "c2":
            res = measure_local_extra(ctx, torch, flush, "hole1024", with_cpu=False)
        elif args.only == "adjoint":
            res = measure_adjoint(ctx, torch)
        elif args.only == "mg":
            res = measure_mg(ctx, torch)
        elif args.only == "c1":
            res = measure_c1(ctx, torch)
        elif args.only == "series":
            res = measure_series(ctx, torch)
        else:
            res = measure_c5(ctx, torch, flush)
        print(json.dumps({"only": args.only, "result": res}), flush=True)
        ctx.close()
        return 0
    w = make_workload(args.workload)
    run = LocalRun(ctx, w)
    W, H, N, ws_list = run.W, run.H, run.N, run.ws_list
    if args.profile:
        fr, prec = (run.fr32, _lib.STDIC_BATCHED_F32) if args.profile == "batched" else (run.fr64, _lib.STDIC_PLAIN_F64)
        ms = []
        for _ in range(args.warmup + args.steps):
            run.solve(fr, prec)
            ms.append(ctx.last_solver_ms())
        torch.cuda.synchronize()
        print(json.dumps({"profile": args.workload, "form": args.profile, "passes": args.warmup + args.steps,
                          "solver_ms": ms}), flush=True)
        ctx.close()
        return 0

    # ---- plain FP64 drop-in: accuracy reference and the 'plain' throughput
    run.solve(run.fr64, _lib.STDIC_PLAIN_F64)
    torch.cuda.synchronize()
    U_plain, F_plain, conv_plain = run.host()
    plain_ms, plain_kern = timed_solves(torch, run, run.fr64, _lib.STDIC_PLAIN_F64, 2, flush)
    plain_conv = int(converged_rule(U_plain, conv_plain).sum())
    plain_value = plain_conv / (np.mean(plain_ms) * 1e-3)

    # ---- batched FP32: warm-up (the first call autotunes), then K timed steps
    for _ in range(args.warmup):
        run.solve(run.fr32, _lib.STDIC_BATCHED_F32)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = ctx.launches
    sampler = ClockSampler(local)
    sampler.start()
    sampler.region_start()
    step_ms, solver_ms = timed_solves(torch, run, run.fr32, _lib.STDIC_BATCHED_F32, args.steps, flush)
    torch.cuda.synchronize()
    sampler.region_end()
    clocks = sampler.stop()
    launches = ctx.launches - launches0
    if dist:
        dist.barrier()

    Uc, Fc, cc = run.host()
    n_conv = int(converged_rule(Uc, cc, U_plain).sum())
    mean_ms = float(np.mean(step_ms))
    if dist:
        mean_ms, n_conv_all = reduce_over_ranks(dist, mean_ms, n_conv, "cuda")
    else:
        n_conv_all = float(n_conv)
    value = n_conv_all / (mean_ms * 1e-3)

    # ---- end to end through the C ABI with pinned host buffers
    def pinned(a, dt):
        return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=dt).ravel(order="F"))).pin_memory()

    hf, hg, hm = pinned(w["f"], np.float32), pinned(w["g"], np.float32), pinned(w["maskf"], np.uint8)
    hgx, hgy = run.gx32.cpu().pin_memory(), run.gy32.cpu().pin_memory()
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
    n_conv_e2e = int(converged_rule(oU.numpy(), oc.numpy(), U_plain).sum())
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
    fp32_peak = gemm_peak_tflops(torch, torch.float32, 8192)
    fp64_peak = gemm_peak_tflops(torch, torch.float64, 4096)
    flops = float(flops_per_subset(cc, ws_list).sum())
    sv = [s for s in solver_ms if s > 0]
    kern_ms = float(np.mean(sv)) if sv else mean_ms
    achieved = flops / (kern_ms * 1e-3) / 1e12
    alg_bytes = (2 * 4 * W * H + W * H + 2 * 4 * (W - 6) * (H - 6) + N * (16 + 16 + 4 + 16 + 32 + 168 + 4 + 1))
    traffic, traffic_src = traffic_from_profile(args.workload)
    roofline = {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                "frac": achieved / fp32_peak, "traffic": traffic, "traffic_source": traffic_src,
                "peak_source": "cuBLAS SGEMM 8192^3 with TF32 off, measured in this run "
                               "(MEASURED_PEAKS.json has no FP32 CUDA-core figure)",
                "flops_per_launch": flops, "kernel_ms": kern_ms,
                "kernel": "icgn_batched_kernel set-up + factor6_kernel + icgn_batched_kernel iterations"}
    roofline_hbm = {"bound": "hbm", "achieved": alg_bytes / (kern_ms * 1e-3) / 1e9,
                    "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                    "frac": alg_bytes / (kern_ms * 1e-3) / 1e9 / peaks.get("hbm_gbs"),
                    "traffic": traffic, "algorithmic_bytes_per_launch": alg_bytes,
                    "peak_source": src}
    # the warped footprint of g each iteration gathers: 4 (ws+4)^2 bytes per
    # subset per iteration (taps reach one pixel before and two after)
    it_b = np.where((cc >= 1) & (cc <= 101), cc, 0).astype(np.float64)
    gather_bytes = float((4.0 * (ws_list.astype(np.float64) + 4) ** 2 * it_b).sum())
    gather_l2 = {"achieved": gather_bytes / (kern_ms * 1e-3) / 1e9, "unit": "GB/s",
                 "bytes_per_launch": gather_bytes,
                 "note": "algorithmic bytes of the warped g footprints the iterations gather (through L1 "
                         "and L2) over the solver kernels' time"}
    plain_flops = float(flops_per_subset(conv_plain, ws_list).sum())
    pk = [s for s in plain_kern if s > 0]
    plain_rf = plain_roofline(plain_flops, float(np.mean(pk)) if pk else float(np.mean(plain_ms)), fp64_peak)

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": mean_ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": workload_config(args.workload, w),
           "precision": "batched FP32 (FMA sums, FP64 Hessian inverses applied in double-float)",
           "l2": "flushed between timed steps (256 MiB write)",
           "parallelism": "replicas" if world > 1 else "single GPU",
           "clocks": clocks,
           "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                   "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_mean},
           "gpu_launches": int(launches),
           "roofline": roofline,
           "roofline_hbm": roofline_hbm,
           "gather_l2": gather_l2,
           "plain_fp64": {"value": plain_value, "ms_per_step": float(np.mean(plain_ms)),
                          "converged": plain_conv, "roofline": plain_rf},
           "batched_over_plain": value / plain_value if plain_value > 0 else None,
           "accuracy": dict(converged=n_conv, nodes=N,
                            **accuracy(Uc, Fc, cc, U_plain, F_plain, conv_plain))}
    if world == 1 and not args.no_cpu_baseline:
        cp = guarded(CpuPass, w)
        if isinstance(cp, CpuPass):
            cpu = guarded(cp.measure, 5)
            out["cpu_baseline"] = cpu
            if cpu.get("value"):
                out["batched_over_cpu"] = value / cpu["value"]
                Uo, Fo, _, co, badno, _ = cp.out
                out["accuracy_vs_fp64_oracle"] = dict(
                    converged_batched_within_0_01px=int(converged_rule(Uc, cc, Uo).sum()),
                    badnum_oracle=int(badno), **accuracy(Uc, Fc, cc, Uo, Fo, co))
                dpo = np.abs(U_plain - Uo).reshape(-1, 2).max(axis=1)
                both = (co >= 1) & (co <= 100) & ~np.isnan(Uo[0::2])
                out["accuracy_vs_fp64_oracle"]["plain_max_abs_du_px"] = float(np.nanmax(dpo[both]))
                out["accuracy_vs_fp64_oracle"]["plain_codes_equal_frac"] = float(np.mean(conv_plain == co))
        else:
            out["cpu_baseline"] = cp
    if world == 1 and not args.no_extras:
        out["c2"] = guarded(measure_local_extra, ctx, torch, flush, "hole1024")
        out["admm"] = guarded(measure_admm, ctx, torch, run)
        out["adjoint_c4"] = guarded(measure_adjoint, ctx, torch)
        out["c5"] = guarded(measure_c5, ctx, torch, flush)
        out["mg_search"] = guarded(measure_mg, ctx, torch)
        out["c1"] = guarded(measure_c1, ctx, torch)
        out["series"] = guarded(measure_series, ctx, torch)
    print(json.dumps(out), flush=True)
    if dist:
        dist.destroy_process_group()
    ctx.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
