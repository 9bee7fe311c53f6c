"""EM iterations per second of the DA-GTM annealed EM step on GB300.

Workload (the headline configuration): N = 1,000,000 synthetic binary
fingerprints (D = 166, 20 prototypes, per-feature Bernoulli p ~ U[0.05,0.5],
10 % bit flips), K = 8000 latent points (20^3, L = 3), M = 64 RBF centres
(4^3) plus bias, width 2 x spacing, deterministic annealing at the start
temperature.  One step = one EM iteration (E-step, qualities, M-step, beta)
with the data resident in HBM; the data (>= 332 MB in BF16, 1.3 GB in FP64)
is larger than L2, so no flush is needed between iterations.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
  python bench.py --anneal [--form bf16x3|fp32|fp64] [--anneal-maxloop J]
  python bench.py --ctemp [--form bf16x3|fp32|fp64] [--n N] [--ctemp-calls C]

Under torchrun each rank runs an independent replica (the path is one GPU
per problem; no data-path collective); rank 0 prints one JSON line.
``--impl reference`` times the CPU restatement of the reference's algorithm
(the oracle: the reference itself needs MPI/GSL/HDF5, which are absent) on
all host cores, on a bounded sample of the same workload.

``--anneal`` is a separate measurement, not the per-iteration contract: the
wall time of a whole annealing run of the workload through the package's
temperature loop (EXP cooling, alpha 0.99, eps 1e-6, from the start
temperature down to 1, as the reference's dagtm runs by default), host loop
and per-iteration synchronisation included.  Give it a cap: a temperature
ends only when the quality changes by less than eps (or its 50-iteration
average settles), and at the start temperature the EM keeps drifting for
thousands of iterations (an uncapped run did not finish in 15 minutes).

``--ctemp`` is another separate measurement: the wall time of the AUTO
schedule's critical-temperature call (dgtm_next_ctemp) on the workload, after
one E-step at the start temperature.

``--fe`` times the differentiation configuration: the annealed free energy
and its gradient (dgtm_fe_forward + dgtm_fe_backward for dY, dT and dbeta)
at N = 65,536 points in D = 64 (16-component mixture, sd 0.2), K = 4096,
FP32 data, L2 flushed between steps.

``--large`` times the large split-precision configuration: EM iterations at
N = 4,000,000 binary vectors (50 prototypes), K = 32,768 (32^3), M = 512
(8^3) + bias, then the gradient projection of 1,000,000 held-out points onto
the fixed map (gradient steps on F through dgtm_fe_backward's dT).
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "EM iters/sec at N=1M,K=8k,D=166: FP64 plain vs BF16x3 form at stated error"
DTYPES = {
    "bf16x3": "bf16x3 (split BF16 products, fp32 accumulate; per point the shifted sums in "
              "fp32 with Kahan compensation, the nearest distance recomputed in fp32, "
              "logarithms and sums over points in fp64; fp64 M-step and beta)",
    "fp64": "f64", "fp32": "f32 (fp64 reductions and M-step)"}
WORKLOAD = dict(N=1_000_000, D=166, K=8000, L=3, M=64, s=2.0, nproto=20, seed=0)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--form", default="bf16x3", choices=["bf16x3", "fp64", "fp32"])
    ap.add_argument("--n", type=int, default=WORKLOAD["N"], help="data points (default 1M)")
    ap.add_argument("--fp64-steps", type=int, default=2,
                    help="timed EM iterations of the FP64 form beside the headline (0: skip)")
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--ref-sample", type=int, default=8192,
                    help="points per step of the reference arm's bounded sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--anneal", action="store_true",
                    help="time a whole annealing run instead of single iterations")
    ap.add_argument("--anneal-maxloop", type=int, default=2000,
                    help="iteration cap of the annealing run (0: none; see above)")
    ap.add_argument("--ctemp", action="store_true",
                    help="time the AUTO schedule's critical-temperature call instead")
    ap.add_argument("--ctemp-calls", type=int, default=1)
    ap.add_argument("--fe", action="store_true",
                    help="time the free energy's forward + backward (differentiation config)")
    ap.add_argument("--large", action="store_true",
                    help="time the large split-precision configuration and the projection")
    ap.add_argument("--proj-steps", type=int, default=20,
                    help="gradient steps of the projection in --large")
    return ap.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def max_over_ranks(x, world):
    """Max of a per-rank number over all ranks (the slowest rank times the job)."""
    if world <= 1:
        return float(x)
    import torch
    dev = "cuda" if torch.distributed.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], device=dev, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(steps, ms, world):
    """Weak scaling: every rank runs `steps` iterations of its own problem in `ms`."""
    return world * steps / (ms / 1000.0)


def make_problem(n):
    ds = importlib.import_module("da-gtm_gb300.datasets")
    st = importlib.import_module("da-gtm_gb300.gtm_setup")
    w = WORKLOAD
    T = ds.fingerprints(n, w["D"], w["nproto"], seed=w["seed"])
    X, FI, W0, beta0 = st.random_init(T, w["L"], w["K"], w["M"], w["s"], seed=1)
    Y0 = FI @ W0
    temp0 = st.start_temp(T[: min(n, 200_000)], 0.99)
    return T, X, FI, Y0, beta0, temp0


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax = float(p[2])
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, \
            "fallback"


def traffic_summary():
    """Per-launch DRAM traffic of the dominant kernel from a committed ncu summary."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def time_steps(torch, ctx, n, beta, temp, stream):
    """n EM iterations with resident data; returns (ms, beta)."""
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(n):
        ctx.estep(beta, 1, temp)
        beta, _, _ = ctx.mstep(want_W=False)
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1), beta


R_COLS = (0, 499_776, 999_744)  # three 256-point blocks of sampled responsibilities


def probe_step(ctx, beta, temp):
    """One EM iteration from the loaded centres that also keeps what the error
    report compares: qualities, R on three 256-point blocks, G, RT, beta, Y."""
    llh, nfree = ctx.estep(beta, 1, temp)
    cols = [min(c, max(0, ctx.N - 256)) for c in R_COLS]
    R = [ctx.R_block(0, ctx.K, c, min(256, ctx.N)) for c in cols]
    b, _, Y = ctx.mstep(want_W=False, want_Y=True)
    G, RT = ctx.get_stats()
    return dict(llh=llh, nfree=nfree, R=R, beta=b, Y=Y, G=G, RT=RT)


def run_form(torch, pkg, form, T, FI, Y0, beta0, temp0, steps, warmup, rank, world, stream_cls,
             clocks=False, probe=False):
    """Warm-up, then `steps` timed EM iterations.  With probe, the first warm-up
    iteration is probe_step (it starts from Y0, beta0) and its record is returned."""
    ctx = pkg.Context(T, FI, form)
    ctx.set_Y(Y0)
    stream = stream_cls(ctx.stream())
    beta = beta0
    rec = None
    for i in range(warmup):
        if probe and i == 0:
            rec = probe_step(ctx, beta, temp0)
            beta = rec["beta"]
            continue
        ctx.estep(beta, 1, temp0)
        beta, _, _ = ctx.mstep(want_W=False)
    ctx.set_timing(True)
    ctx.reset_timing()
    if world > 1:
        torch.distributed.barrier()
    sampler = ClockSampler(torch.cuda.current_device()) if clocks else None
    if sampler:
        sampler.__enter__()
    ms, beta = time_steps(torch, ctx, steps, beta, temp0, stream)
    if sampler:
        sampler.__exit__(None, None, None)
    ms = max_over_ranks(ms, world)
    phases = ctx.timing()
    ctx.set_timing(False)
    return ctx, ms, phases, (sampler.summary() if sampler else None), beta, rec


def rel_err(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b)) / max(float(np.max(np.abs(b))), 1e-300))


def form_errors(split, ref, N, D, sum_t2):
    """The split form's first EM iteration against the FP64 form's, from the
    same centres, beta and temperature."""
    def beta_from(G, RT, Y):
        return N * D / (float((G * (Y * Y).sum(axis=1)).sum()) - 2.0 * float((Y * RT).sum())
                        + sum_t2)
    b_stats = beta_from(split["G"], split["RT"], ref["Y"])
    return {
        "beta_stats_rel": abs(b_stats / ref["beta"] - 1.0),
        "F_rel": abs(split["nfree"] - ref["nfree"]) / abs(ref["nfree"]),
        "llh_rel": abs(split["llh"] - ref["llh"]) / abs(ref["llh"]),
        "beta_rel": abs(split["beta"] - ref["beta"]) / abs(ref["beta"]),
        "R_max_abs": max(float(np.max(np.abs(a - b))) for a, b in zip(split["R"], ref["R"])),
        "G_rel": rel_err(split["G"], ref["G"]),
        "RT_rel": rel_err(split["RT"], ref["RT"]),
        "Y_rel": rel_err(split["Y"], ref["Y"]),
        "what": "first EM iteration of each form from the same Y, beta, temp: F = N nfree "
                "(the annealed free energy), llh, the new beta, R on three 256-point blocks "
                f"(points 0, mid, end of {N}), G, RT and the new Y (max-abs / max).  At this "
                "width A = FI^T G FI is numerically singular, pivots are dropped and W, Y are "
                "not determined by the data (any two solvers differ); beta_stats_rel is the "
                "determined part: beta from the split form's G and RT with the FP64 form's "
                "new centres, against the FP64 form's beta",
    }


def e2e_steps(torch, pkg, ctx, steps, beta, temp, stream_cls, warmup=3):
    """Through the host-buffer API: Y in from pinned host memory, W / Y out.
    `warmup` untimed steps first, as for the device-resident loop (the first
    calls with fresh host buffers carry one-off costs)."""
    K, D, M1 = ctx.K, ctx.D, ctx.M1
    Yh_t = torch.empty((K, D), dtype=torch.float64, pin_memory=True)
    Wh_t = torch.empty((M1, D), dtype=torch.float64, pin_memory=True)
    Yh = Yh_t.numpy()
    Wh = Wh_t.numpy()
    Yh[:] = ctx.get_Y()
    import ctypes
    lib = pkg.load_library()
    dp = ctypes.POINTER(ctypes.c_double)
    stream = stream_cls(ctx.stream())
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    b = ctypes.c_double(beta)
    llh, nfree = ctypes.c_double(), ctypes.c_double()

    def step():
        pkg._check(lib.dgtm_set_Y(ctx._h, Yh.ctypes.data_as(dp), D))
        pkg._check(lib.dgtm_estep(ctx._h, b.value, 1, temp, ctypes.byref(llh), ctypes.byref(nfree)))
        pkg._check(lib.dgtm_mstep(ctx._h, Wh.ctypes.data_as(dp), D, Yh.ctypes.data_as(dp), D,
                                  ctypes.byref(b)))

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(steps):
        step()
    ev1.record(stream)
    ev1.synchronize()
    ms = ev0.elapsed_time(ev1)
    h2d = K * D * 8
    d2h = (K * D + M1 * D) * 8 + 3 * 8
    return ms, h2d, d2h


def bf16_exact(T):
    """Whether every value of T is exactly a BF16 number (the split form then
    keeps T in one piece)."""
    t32 = T.astype(np.float32)
    return bool(np.array_equal(t32.astype(np.float64), T)
                and not np.any(t32.view(np.uint32) & np.uint32(0xFFFF)))


def canonical_flops(phase, N, K, D):
    """The kernel's share of the canonical work of one EM iteration: the
    distance product 2KND for the E-step and the R T product 2KND for the
    responsibility pass (its distance recompute is not counted)."""
    return 2.0 * K * N * D if phase in ("estep", "mstep_pass") else None


def issued_flops(form, phase, nT, N, K, D):
    """Products the kernel issues on unpadded shapes: the split form's E-step
    runs Y_hi T and Y_lo T (plus Y_hi T_lo when T is split); its
    responsibility pass recomputes those and runs R_hi T, R_lo T (and R_hi T_lo)."""
    kdn = 2.0 * K * N * D
    per = (1 + nT) if form == "bf16x3" else 1
    if phase == "estep":
        return per * kdn
    if phase == "mstep_pass":
        return 2 * per * kdn
    return None


def canonical_step_flops(N, K, D, M1):
    """Canonical work of one EM iteration: distances, the cheaper route to B,
    A and Y = FI W."""
    return (2.0 * K * N * D + min(2.0 * M1 * K * N + 2.0 * M1 * N * D,
                                  2.0 * K * N * D + 2.0 * K * M1 * D)
            + 2.0 * K * M1 * M1 + 2.0 * K * M1 * D)


def _time_iters(ws, iters, temp, budget_s, **kw):
    ws.iteration(1, temp, **kw)  # warm-up
    times = []
    t_end = time.perf_counter() + budget_s
    while True:
        t0 = time.perf_counter()
        ws.iteration(1, temp, **kw)
        times.append(time.perf_counter() - t0)
        if len(times) >= iters or time.perf_counter() > t_end:
            break
    return statistics.median(times), len(times)


def cpu_variants(T, FI, Y0, beta0, temp0, N_full, samples=(256, 1024, 8192), budget_s=10.0):
    """The reference's EM iteration on the host cores, on the first points of
    the same data and from the same initial state, in three variants:
    faithful (the C restatement, one thread: the reference as built by default
    against GSL's reference cblas, one MPI rank), port_omp (the same code with
    OpenMP on every core), blas (numpy/OpenBLAS dgemm, element loops split
    over every core).  Work is linear in N, so each rate is scaled from its
    sample to N_full: these are extrapolations."""
    from oracle import oracle as O  # the checker: CPU restatement of the reference
    from oracle import oracle_blas as OB
    O.build()
    threads = os.cpu_count() or 1
    out = {}
    n_f, n_o, n_b = (min(s, T.shape[0]) for s in samples)
    O.set_threads(1)
    t, it = _time_iters(O.Workspace(T[:n_f], FI, Y0, beta0), 1, temp0, budget_s)
    out["faithful"] = {"value": (1.0 / t) * (n_f / N_full), "cores": 1, "sample_points": n_f,
                       "iters": it, "s_per_iter": t}
    O.set_threads(threads)
    t, it = _time_iters(O.Workspace(T[:n_o], FI, Y0, beta0), 2, temp0, budget_s)
    out["port_omp"] = {"value": (1.0 / t) * (n_o / N_full), "cores": threads,
                       "sample_points": n_o, "iters": it, "s_per_iter": t}
    ws = OB.Workspace(T[:n_b], FI, Y0, beta0, threads=threads)
    t, it = _time_iters(ws, 2, temp0, budget_s)
    ws.close()
    out["blas"] = {"value": (1.0 / t) * (n_b / N_full), "cores": threads, "sample_points": n_b,
                   "iters": it, "s_per_iter": t}
    return out


def cpu_baseline(T, FI, Y0, beta0, temp0, N_full):
    v = cpu_variants(T, FI, Y0, beta0, temp0, N_full)
    best = max(v, key=lambda k: v[k]["value"])
    b = v[best]
    return {"value": b["value"], "unit": "EM iters/s", "cores": b["cores"], "kind": "port",
            "extrapolated": True, "variant": best, "variants": v,
            "sample": f"first {b['sample_points']} of the {N_full} points (K, D, M and the "
                      f"initial state unchanged), {b['iters']} timed iterations of the "
                      f"reference-semantics CPU restatement ({best}), scaled linearly in N; "
                      f"median {b['s_per_iter']:.3f} s per iteration"}


def main_gb300(args):
    import torch
    rank, world, local = dist_env()
    if world > 1:
        torch.cuda.set_device(local)
        torch.distributed.init_process_group("nccl")
    pkg = importlib.import_module("da-gtm_gb300")
    pkg.load_library()
    stream_cls = torch.cuda.ExternalStream
    T, X, FI, Y0, beta0, temp0 = make_problem(args.n)
    N, D = T.shape
    K, M1 = FI.shape
    form = args.form
    want_err = rank == 0 and form != "fp64" and args.fp64_steps > 0
    ctx, ms, phases, clocks, beta, rec = run_form(
        torch, pkg, form, T, FI, Y0, beta0, temp0, args.steps, max(args.warmup, 1), rank, world,
        stream_cls, clocks=(rank == 0), probe=want_err)
    ms_step = ms / args.steps
    value = whole_job_rate(args.steps, ms, world)
    launches = sum(p["launches"] for p in phases.values())
    e2e_ms, h2d, d2h = e2e_steps(torch, pkg, ctx, max(1, args.e2e_steps), beta, temp0, stream_cls,
                                 warmup=max(3, args.warmup))
    e2e_ms = max_over_ranks(e2e_ms, world)
    e2e_value = whole_job_rate(max(1, args.e2e_steps), e2e_ms, world)
    nT = 1 if bf16_exact(T) else 2
    exact_slices = ctx.path == "exact_slices"
    ctx.close()

    peaks, peak_src = measured_peaks()
    dom = max(("estep", "mstep_pass"), key=lambda p: phases[p]["ms"])
    per_launch_ms = phases[dom]["ms"] / max(1, phases[dom]["calls"])
    canon = canonical_flops(dom, N, K, D)
    issued = issued_flops(form, dom, nT, N, K, D)
    achieved = canon / (per_launch_ms / 1000.0) / 1e12
    burst = peaks.get("bf16_tflops", 1900.0)
    sustained = peaks.get("bf16_tflops_sustained", burst)
    if form == "bf16x3":
        peak = burst / 3.0
        peak_note = (f"bf16 dense burst ({peak_src}) / 3: three BF16 products stand for one "
                     "canonical FP32-accurate product")
        tensor_util = issued / (per_launch_ms / 1000.0) / 1e12 / burst
    elif form == "fp64" and exact_slices:
        # the exact-slice form: integer distance products on the tensor cores,
        # double-float epilogues on the FP32 pipe; the FP64 pipe's nominal
        # peak is the ceiling of an FP64-pipe implementation, so frac is the
        # gain over that ceiling (and may exceed 1)
        peak = 1.25
        peak_note = ("fp64 pipe nominal (1.25 TFLOP/s): the ceiling of an FP64-pipe form; this "
                     "form runs on the tensor and FP32 pipes, frac > 1 is the gain over it")
        slices = 7 if dom == "estep" else 7 + 6  # distance slices (+ R digits in pass 2)
        tensor_util = slices * 2.0 * K * N * D / (per_launch_ms / 1000.0) / 1e12 / burst
    else:
        peak = 1.25 if form == "fp64" else 75.0
        peak_note = f"{form} nominal (no measured {form} peak)"
        tensor_util = None
    traffic = traffic_summary().get(f"{form}:{dom}")
    traffic_note = None
    if traffic is not None:
        traffic = traffic.get("bytes_per_point", 0.0) * N
        traffic_note = ("ncu dram__bytes_read.sum + dram__bytes_write.sum per point "
                        "(profiles/traffic.json), x N")
    step_flops = canonical_step_flops(N, K, D, M1)
    roofline = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak, "traffic": traffic, "kernel": dom,
                "per_launch_ms": per_launch_ms, "canonical_flop_per_launch": canon,
                "peak_source": peak_note,
                "frac_of_sustained": (achieved / (sustained / 3.0)) if form == "bf16x3" else None,
                "tensor_util": tensor_util,
                "tensor_util_what": "products the kernel issues (unpadded) / launch time / "
                                    "bf16 dense burst peak",
                "step": {"canonical_flop": step_flops,
                         "achieved": step_flops / (ms_step / 1000.0) / 1e12,
                         "frac": step_flops / (ms_step / 1000.0) / 1e12 / peak},
                "traffic_source": traffic_note}

    fp64 = None
    errors = None
    if args.fp64_steps > 0 and form != "fp64":
        c64, ms64, ph64, _, _, rec64 = run_form(torch, pkg, "fp64", T, FI, Y0, beta0, temp0,
                                                args.fp64_steps, 1, rank, world, stream_cls,
                                                probe=want_err)
        path64 = c64.path
        c64.close()
        fp64 = {"value": world * args.fp64_steps / (ms64 / 1000.0), "unit": "EM iters/s",
                "ms_per_step": ms64 / args.fp64_steps, "steps": args.fp64_steps, "path": path64}
        if want_err:
            errors = form_errors(rec, rec64, N, D, float((T * T).sum()))
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(T, FI, Y0, beta0, temp0, N)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "EM iters/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": DTYPES[form],
            "data": "synthetic (seeded binary fingerprints, stand-in for the 166-bit "
                    "chemical-fingerprint data set)",
            "config": {"workload": f"DA-GTM EM iteration, N={N}, D={D}, K={K} (20^3), "
                                   f"M=64 (4^3) + bias, {form} form",
                       "N": N, "D": D, "K": K, "M": 64, "L": 3, "form": form,
                       "path": "exact_slices" if exact_slices else ("split_bf16" if form == "bf16x3"
                                                                     else "cuda_cores"),
                       "temp": temp0, "l2": "inputs larger than L2 (no flush)",
                       "parallelism": f"replicas x{world}"},
            "e2e": {"value": e2e_value, "unit": "EM iters/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "steps": args.e2e_steps,
                    "warmup": max(3, args.warmup)},
            "gpu_launches": int(launches),
            "clocks": clocks,
            "roofline": roofline,
            "phases_ms_per_step": {p: v["ms"] / args.steps for p, v in phases.items()},
            "fp64_form": fp64,
            "errors_vs_fp64_form": errors,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main_anneal(args):
    """Wall time of a whole annealing run (rank 0 of one GPU)."""
    import torch
    pkg = importlib.import_module("da-gtm_gb300")
    T, X, FI, Y0, beta0, temp0 = make_problem(args.n)
    ctx = pkg.Context(T, FI, args.form)
    ctx.set_Y(Y0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    run = pkg.anneal(ctx, beta0, temp0, alpha=0.99, eps=1e-6, maxloop=args.anneal_maxloop)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    temps = len(set(run.temp_trace))
    w = WORKLOAD
    print(json.dumps({
        "mode": "anneal",
        "metric": "wall seconds of a whole DA-GTM annealing run (EXP, alpha 0.99, eps 1e-6)",
        "value": wall, "unit": "s", "higher_is_better": False,
        "iterations": run.nloop, "temperatures": temps, "iters_per_s": run.nloop / wall,
        "final": {"temp": run.temp, "beta": run.beta, "llh": run.llh_trace[-1],
                  "nfree": run.nfree_trace[-1]},
        "start": {"temp": temp0, "beta": beta0},
        "dtype": args.form, "data": "synthetic (seeded binary fingerprints)",
        "config": {"workload": f"DA-GTM annealing run, N={args.n}, D={w['D']}, K={w['K']} "
                               f"(20^3), M={w['M']} (4^3) + bias, {args.form} form",
                   "N": args.n, "D": w["D"], "K": w["K"], "M": w["M"], "L": w["L"],
                   "maxloop": args.anneal_maxloop}}), flush=True)
    ctx.close()


def main_ctemp(args):
    """Wall time of dgtm_next_ctemp on the workload (rank 0 of one GPU)."""
    import torch
    pkg = importlib.import_module("da-gtm_gb300")
    T, X, FI, Y0, beta0, temp0 = make_problem(args.n)
    times = []
    with pkg.Context(T, FI, args.form) as ctx:
        ctx.set_Y(Y0)
        ctx.estep(beta0, 1, temp0)
        torch.cuda.synchronize()
        for _ in range(max(1, args.ctemp_calls)):
            t0 = time.perf_counter()
            ct = ctx.next_ctemp(temp0, beta0, 1e-6)
            times.append(time.perf_counter() - t0)
    w = WORKLOAD
    print(json.dumps({
        "mode": "ctemp",
        "metric": "wall seconds of one AUTO critical-temperature call (dgtm_next_ctemp)",
        "value": times[-1], "unit": "s", "higher_is_better": False, "calls_s": times,
        "ctemp": ct, "temp": temp0, "beta": beta0,
        "dtype": args.form, "data": "synthetic (seeded binary fingerprints)",
        "config": {"workload": f"AUTO critical temperature, N={args.n}, D={w['D']}, K={w['K']} "
                               f"(20^3), {args.form} form, after one E-step at the start "
                               "temperature",
                   "N": args.n, "D": w["D"], "K": w["K"]}}), flush=True)


class L2Flush:
    """Writes a buffer larger than L2 (129 MB) between timed steps."""

    def __init__(self, torch, mb=512):
        self.buf = torch.empty(mb << 18, dtype=torch.float32, device="cuda")

    def __call__(self):
        self.buf.fill_(1.0)


def fe_buffers(torch, pkg, N, K, D):
    import ctypes
    lib = pkg.load_library()
    size = ctypes.c_size_t()
    pkg._check(lib.dgtm_fe_workspace_size(N, K, D, ctypes.byref(size)))
    ws = torch.empty(size.value + 256, dtype=torch.uint8, device="cuda")
    return lib, ws, ws.data_ptr() + ((-ws.data_ptr()) % 256), size.value


def main_fe(args):
    """Forward + backward of the annealed free energy at the differentiation
    configuration, through the C ABI on torch's stream."""
    import torch
    pkg = importlib.import_module("da-gtm_gb300")
    ds = importlib.import_module("da-gtm_gb300.datasets")
    N, D, K = 65536, 64, 4096
    beta, temp = 4.0, 2.0
    Th = ds.gaussian_mixture(N, D, 16, 0.2, seed=0).astype(np.float32)
    rng = np.random.default_rng(0)
    Yh = (Th[rng.integers(0, N, K)] + 0.05 * rng.standard_normal((K, D))).astype(np.float32)
    T = torch.tensor(Th, device="cuda")
    Y = torch.tensor(Yh, device="cuda")
    lib, ws, wp, wsz = fe_buffers(torch, pkg, N, K, D)
    F = torch.empty((), dtype=torch.float64, device="cuda")
    g = torch.ones((), dtype=torch.float64, device="cuda")
    dY = torch.empty_like(Y)
    dT = torch.empty_like(T)
    db = torch.empty((), dtype=torch.float64, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    flush = L2Flush(torch)

    def fwd():
        pkg._check(lib.dgtm_fe_forward(Y.data_ptr(), T.data_ptr(), N, K, D, beta, temp, wp, wsz,
                                       st, F.data_ptr()))

    def bwd():
        pkg._check(lib.dgtm_fe_backward(Y.data_ptr(), T.data_ptr(), N, K, D, beta, temp, wp, wsz,
                                        st, g.data_ptr(), dY.data_ptr(), dT.data_ptr(),
                                        db.data_ptr()))

    for _ in range(max(3, args.warmup)):
        fwd()
        bwd()
    torch.cuda.synchronize()
    t_f, t_b = [], []
    for _ in range(args.steps):
        flush()
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record()
        fwd()
        e1.record()
        bwd()
        e2.record()
        e2.synchronize()
        t_f.append(e0.elapsed_time(e1))
        t_b.append(e0.elapsed_time(e2) - e0.elapsed_time(e1))
    ms_f, ms_b = statistics.mean(t_f), statistics.mean(t_b)
    ms = ms_f + ms_b
    canon = 3 * 2.0 * K * N * D
    peaks, src = measured_peaks()
    peak = peaks.get("bf16_tflops", 1900.0) / 3.0
    print(json.dumps({
        "mode": "fe",
        "metric": "free-energy forward + backward (dY, dT, dbeta) per second",
        "value": 1000.0 / ms, "unit": "fwd+bwd/s", "higher_is_better": True,
        "ms_per_step": ms, "ms_forward": ms_f, "ms_backward": ms_b, "steps": args.steps,
        "F": F.item(), "finite": bool(torch.isfinite(dT).all() and torch.isfinite(dY).all()),
        "roofline": {"bound": "tensor", "canonical_flop": canon, "achieved": canon / ms / 1e9,
                     "peak": peak, "unit": "TFLOP/s", "frac": canon / ms / 1e9 / peak,
                     "peak_source": f"bf16 dense burst ({src}) / 3"},
        "dtype": "fp32 data, split-BF16 tensor-core products, fp64 reductions",
        "data": "synthetic (16-component Gaussian mixture, sd 0.2)",
        "config": {"workload": f"annealed free energy and gradient, N={N}, D={D}, K={K}, "
                               f"beta={beta}, temp={temp}", "N": N, "D": D, "K": K,
                   "l2": "flushed between steps (512 MB write)"}}), flush=True)


def main_large(args):
    """EM iterations of the large split-precision configuration, then the
    gradient projection of held-out points onto the fixed map."""
    import ctypes
    import torch
    pkg = importlib.import_module("da-gtm_gb300")
    ds = importlib.import_module("da-gtm_gb300.datasets")
    st = importlib.import_module("da-gtm_gb300.gtm_setup")
    N, D, K, M, L = 4_000_000, 166, 32768, 512, 3
    T = ds.fingerprints(N, D, 50, seed=0)
    # width 0.5: at the reference's 2 the 512 basis functions on a 32^3 grid
    # are numerically dependent (cond(FI^T FI) = 3e19) and W is undetermined
    X, FI, W0, beta0 = st.random_init(T[:200_000], L, K, M, 0.5, seed=1)
    Y0 = FI @ W0
    temp0 = st.start_temp(T[:200_000], 0.99)
    ctx = pkg.Context(T, FI, "bf16x3")
    ctx.set_Y(Y0)
    beta = beta0
    for _ in range(max(1, args.warmup)):
        ctx.estep(beta, 1, temp0)
        beta, _, _ = ctx.mstep(want_W=False)
    ctx.set_timing(True)
    ctx.reset_timing()
    steps = max(1, args.steps)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        ctx.estep(beta, 1, temp0)
        beta, _, _ = ctx.mstep(want_W=False)
    torch.cuda.synchronize()
    em_s = (time.perf_counter() - t0) / steps
    phases = {p: v["ms"] / steps for p, v in ctx.timing().items()}
    Ymap = torch.tensor(ctx.get_Y(), dtype=torch.float32, device="cuda")
    ctx.close()
    del T
    # held-out points: the same generator, another seed
    Nh = 1_000_000
    Th = torch.tensor(ds.fingerprints(Nh, D, 50, seed=7, dtype=np.float32), device="cuda")
    lib, ws, wp, wsz = fe_buffers(torch, pkg, Nh, K, D)
    F = torch.empty((), dtype=torch.float64, device="cuda")
    g = torch.ones((), dtype=torch.float64, device="cuda")
    dT = torch.empty_like(Th)
    sptr = torch.cuda.current_stream().cuda_stream
    step = 1.0 / beta
    P = Th.clone()

    def grad_step():
        pkg._check(lib.dgtm_fe_forward(Ymap.data_ptr(), P.data_ptr(), Nh, K, D, beta, 1.0, wp,
                                       wsz, sptr, F.data_ptr()))
        pkg._check(lib.dgtm_fe_backward(Ymap.data_ptr(), P.data_ptr(), Nh, K, D, beta, 1.0, wp,
                                        wsz, sptr, g.data_ptr(), None, dT.data_ptr(), None))
        P.add_(dT, alpha=step)

    grad_step()
    P.copy_(Th)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.proj_steps):
        grad_step()
    e1.record()
    e1.synchronize()
    proj_ms = e0.elapsed_time(e1)
    moved = float((P - Th).norm(dim=1).mean())
    print(json.dumps({
        "mode": "large",
        "metric": "EM iters/sec at N=4M, K=32768, M=512 (bf16x3) and projected points/sec",
        "value": 1.0 / em_s, "unit": "EM iters/s", "higher_is_better": True,
        "ms_per_step": em_s * 1000.0, "steps": steps, "phases_ms_per_step": phases,
        "projection": {"points": Nh, "gradient_steps": args.proj_steps,
                       "ms": proj_ms, "ms_per_gradient_step": proj_ms / args.proj_steps,
                       "points_per_s": Nh / (proj_ms / 1000.0),
                       "step_size": "1/beta (one step is the fixed-point update at temp 1)",
                       "mean_displacement": moved, "finite": bool(torch.isfinite(P).all())},
        "dtype": "bf16x3 (split BF16 products, fp32 accumulate, fp64 reductions)",
        "data": "synthetic (seeded binary fingerprints, 50 prototypes)",
        "config": {"workload": f"DA-GTM EM iteration, N={N}, D={D}, K={K} (32^3), M={M} (8^3) "
                               "+ bias, width 0.5, bf16x3 form; projection of 1M held-out "
                               "points", "N": N, "D": D, "K": K, "M": M, "L": L,
                   "temp": temp0}}), flush=True)


def main_reference(args):
    """The reference's CPU path (restated: the reference itself needs MPI, GSL
    and HDF5) on the host cores, from the same data and initial state as the
    GPU arm; each step is one EM iteration on the first points of the data,
    scaled linearly to N (an extrapolation, flagged as such)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle_blas as OB
    T, X, FI, Y0, beta0, temp0 = make_problem(args.n)
    N_full = T.shape[0]
    n_sample = min(args.ref_sample, N_full)
    threads = os.cpu_count() or 1
    ws = OB.Workspace(T[:n_sample], FI, Y0, beta0, threads=threads)
    for _ in range(args.warmup):
        ws.iteration(1, temp0)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ws.iteration(1, temp0)
    dt = (time.perf_counter() - t0) / args.steps
    ws.close()
    value = (1.0 / dt) * (n_sample / N_full)
    variants = cpu_variants(T, FI, Y0, beta0, temp0, N_full, budget_s=5.0)
    sample = (f"first {n_sample} of the {N_full} points per step (K, D, M and the initial "
              f"state unchanged), numpy/OpenBLAS restatement of the reference's iteration on "
              f"{threads} threads, {dt:.3f} s per step, scaled linearly in N")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "EM iters/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": dt * 1000.0 * (N_full / n_sample), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded binary fingerprints)",
            "extrapolated": True, "sample_points": n_sample,
            "config": {"workload": f"DA-GTM EM iteration, N={N_full}, D=166, K=8000 (20^3), "
                                   "M=64 (4^3) + bias, reference CPU path (restated)",
                       "N": N_full, "D": 166, "K": 8000, "M": 64, "L": 3},
            "cpu_baseline": {"value": value, "unit": "EM iters/s", "cores": threads,
                             "kind": "port", "extrapolated": True, "sample": sample,
                             "variants": variants},
            "e2e": {"value": value, "unit": "EM iters/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    a = parse()
    if a.anneal:
        if dist_env()[0] == 0:
            main_anneal(a)
    elif a.ctemp:
        if dist_env()[0] == 0:
            main_ctemp(a)
    elif a.fe:
        if dist_env()[0] == 0:
            main_fe(a)
    elif a.large:
        if dist_env()[0] == 0:
            main_large(a)
    elif a.impl == "reference":
        main_reference(a)
    else:
        main_gb300(a)
