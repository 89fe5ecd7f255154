"""Benchmark of the OPTIMET sphere path on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload c2|c1]

Metric: wavelength-solves per second of the precision form (complex64
matrix, FP32 inner GMRES inside FP64 outer FGMRES) next to the plain FP64
form, at <= 1e-6 relative extinction-efficiency error, with per-solve
latency percentiles. One "step" = one wavelength-solve of the whole cluster:
per-wavelength set-up, source vector, assembly of S, solve, internal
coefficients and the four cross sections. Successive steps scan the
wavelength (650 nm + 0.25 nm per step) so nothing is reused between steps.

Default workload (c2): N = 400 non-overlapping spheres (seeded rejection
sampling, 20 nm gap) in a 4 um cube, radii U[40, 70] nm, refractive index
2.0+0.05i in vacuum, nMax = 8 -> 64,000 unknowns; plane wave along +z,
x-polarised. Synthetic data. Inputs exceed L2 (S alone is 32.8 GB complex64 +
65.5 GB complex128), so no L2 flush is needed between steps.

The headline number is the batched/served form: om_server with two slots
(device contexts with their own streams and host threads) takes the scan's
wavelengths in order, so one wavelength's assembly overlaps the
previous wavelength's HBM-bound solve; the FP64 form is served the same way.
The single-stream numbers of both forms are reported beside it.

Multi-GPU: independent replicas (one cluster scan per rank, no collective);
value = the sum over ranks of the wavelength-solves each completed, divided
by the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "wavelength-solves/sec mixed vs FP64 on 1 GB300 at 1e-6 Qext err; p50/p99 latency"

# DRAM bytes read per launch of k_matvec_tma<true> over its algorithmic
# 4 n^2 bytes: 163.912 MB / 163.840 MB in an ncu capture at n = 6,400 (the
# reads grow with n^2; the writes are the split-K partial sums, 8 bytes per
# row and 1,024-column chunk at the c2 size)
BF16_READ_RATIO = 163.912 / 163.840
UNIT = "wavelength-solves/s"
nm = 1e-9

WORKLOADS = {
    "c2": dict(N=400, edge=4000 * nm, rmin=40 * nm, rmax=70 * nm, index=2.0 + 0.05j, host=1.0,
               nmax=8, lam=650 * nm, seed=20260402,
               desc="N=400 spheres, nMax=8 (64,000 unknowns), 4 um cube, radii U[40,70] nm, "
                    "index 2.0+0.05i in vacuum, plane wave +z x-polarised, lambda 650 nm + 0.25 nm/step"),
    "small": dict(N=40, edge=1500 * nm, rmin=40 * nm, rmax=70 * nm, index=2.0 + 0.05j, host=1.0,
                  nmax=8, lam=650 * nm, seed=20260403,
                  desc="profiling case: N=40 spheres, nMax=8 (6,400 unknowns), 1.5 um cube, "
                       "radii U[40,70] nm, index 2.0+0.05i in vacuum"),
    "mid": dict(N=120, edge=4000 * nm * (120 / 400) ** (1 / 3), rmin=40 * nm, rmax=70 * nm, index=2.0 + 0.05j,
                host=1.0, nmax=8, lam=650 * nm, seed=20260402,
                desc="profiling case: N=120 spheres at the c2 number density, nMax=8 (19,200 unknowns, "
                     "complex64 S 2.95 GB)"),
    "c1": dict(N=100, edge=2000 * nm, rmin=50 * nm, rmax=80 * nm, index=0.3 + 3.0j, host=1.33,
               nmax=8, lam=650 * nm, seed=20260401,
               desc="N=100 spheres, nMax=8 (16,000 unknowns), 2 um cube, radii U[50,80] nm, "
                    "index 0.3+3.0i in host index 1.33, plane wave +z x-polarised, lambda 650 nm"),
}


def cluster(w, rank=0):
    rng = np.random.default_rng(w["seed"] + 7919 * rank)
    xyz, rad = [], []
    while len(xyz) < w["N"]:
        r = rng.uniform(w["rmin"], w["rmax"])
        c = rng.uniform(-w["edge"] / 2 + r, w["edge"] / 2 - r, size=3)
        if xyz:
            d = np.linalg.norm(np.array(xyz) - c, axis=1) - np.array(rad) - r
            if d.min() < 20 * nm:
                continue
        xyz.append(c)
        rad.append(r)
    return np.array(xyz), np.array(rad)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for name, v in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                                "sw_power_cap"), f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(times, world, device="cpu"):
    """Replica timing: every rank's times reduced with MAX (the slowest rank
    sets the job's time; the work is the sum over ranks)."""
    if world <= 1:
        return list(times)
    import torch
    import torch.distributed as dist
    tt = torch.tensor(times, device=device, dtype=torch.float64)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return [float(v) for v in tt.cpu()]


def replica_value(units_per_rank, seconds, world, device="cpu"):
    """Whole-job throughput of independent replicas: units summed over ranks
    divided by the slowest rank's time."""
    if world <= 1:
        return units_per_rank / seconds
    import torch
    import torch.distributed as dist
    u = torch.tensor([float(units_per_rank)], device=device, dtype=torch.float64)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(u.item()) / max_over_ranks([seconds], world, device)[0]


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def gpu_arm(args, w):
    import optimet_gb300 as G
    from optimet_gb300 import build
    rank, world, local = dist_env()
    build.build()
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    ctx = G.Context(local)
    xyz, rad = cluster(w, rank)
    n_index = complex(w["index"])
    sp = G.spheres_array(xyz, rad, n_index ** 2, w["nmax"])
    bg = G.medium(complex(w["host"]) ** 2)
    pr = G.Problem(ctx, sp, bg, G.plane_wave(w["lam"]))
    n = pr.n
    # outer tolerance 1e-7, inner 1e-3: two outer steps of 4 FP32 matvecs each.
    # Q_ext then sits ~2e-9 from FP64, set by the complex64 rounding of S (the
    # same as with tol 1e-8 / inner 1e-4, which takes 10 FP32 matvecs)
    mixed_opts = G.options(G.SOLVE_FGMRES_MIXED, tol=1e-7, max_iter=30, restarts=4, inner_iter=80,
                           inner_tol=1e-3)
    fp64_opts = G.options(G.SOLVE_GMRES, tol=1e-10, max_iter=400, restarts=6)

    def step(i, mixed):
        pr.set_wavelength(w["lam"] + 0.25 * nm * i)
        launches = ctx.last_launches
        pr.source_vector(copy=False)
        launches += ctx.last_launches
        pr.assemble(G.FF, G.C64 if mixed else G.C128)
        launches += ctx.last_launches
        st = pr.solve(mixed_opts if mixed else fp64_opts)
        launches += ctx.last_launches
        xs = pr.cross_sections()
        launches += ctx.last_launches
        return xs, st, launches

    def barrier():
        ctx.synchronize()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    # ---- precision form (the metric's numerator) ----
    for i in range(args.warmup):
        step(i, True)
    barrier()
    ctx.timers(True)
    lat, xs_mixed, total_launches, inner, outer = [], [], 0, 0, 0
    with ClockSampler(local) as clk:
        ctx.mark()
        for i in range(args.steps):
            xs, st, launches = step(args.warmup + i, True)
            lat.append(ctx.mark() * 1e-3)
            xs_mixed.append(xs)
            total_launches += launches
            inner += st.inner_iterations
            outer += st.iterations
        barrier()
        t_mixed = float(np.sum(lat))
    kt = ctx.timers(False)
    kin = ctx.inner_timers()
    clocks = clk.summary()

    # ---- plain FP64 form on the same wavelengths ----
    step(0, False)
    barrier()
    lat64, xs64, it64 = [], [], 0
    ctx.timers(True)
    k64 = max(1, min(args.steps, 3))
    ctx.mark()
    for i in range(k64):
        xs, st, _ = step(args.warmup + i, False)
        lat64.append(ctx.mark() * 1e-3)
        xs64.append(xs)
        it64 += st.iterations
    barrier()
    t_fp64 = float(np.sum(lat64))
    kt64 = ctx.timers(False)

    # Q_ext = C_ext / sum(pi a^2): the relative error equals that of C_ext
    err = max(abs(xs_mixed[i][0] - xs64[i][0]) / abs(xs64[i][0]) for i in range(k64))
    err_all = max(float(np.max(np.abs(xs_mixed[i] - xs64[i]) / np.abs(xs64[i]))) for i in range(k64))


    pr.close()
    if args.single_stream:
        ctx.close()
        return {"metric": METRIC + " (single stream)", "value": args.steps / t_mixed,
                "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1e3 * t_mixed / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "c64 (FP32) inner + c128 (FP64) outer/assembly",
                "data": "synthetic (seeded random clusters)",
                "config": {"workload": args.workload + ": " + w["desc"], "unknowns": n},
                "fp64": {"value": k64 / t_fp64}, "kernels_ms": {k: v[0] / max(v[1], 1) for k, v in kt.items()},
                "inner_products": {k: {"ms_avg": v[0] / max(v[1], 1), "launches": v[1]} for k, v in kin.items()},
                "iterations": {"outer": outer / args.steps, "inner": inner / args.steps},
                "qext_rel_err_vs_fp64": err,
                "gpu_launches": total_launches, "clocks": clocks}

    # ---- batched / served form: om_server with `slots` contexts on the GPU ----
    # Successive wavelengths of the scan run on alternating slots, so one
    # wavelength's assembly overlaps the previous one's solve (both
    # HBM-bound). Same requests for both forms; a slot keeps its problem resident
    # across wavelengths (cluster_key) like the reference's scan keeps its
    # Geometry.
    def served(opts, precision, k, key, tuning=None, tune_count=6):
        srv = G.Server(local, 0, args.slots)
        lam = lambda i: G.plane_wave(w["lam"] + 0.25 * nm * i)
        # launch tuning: the server's autotuner on warm-up requests (untimed)
        if tuning is None:
            tuning = srv.autotune(sp, bg, lam(0), opts, precision, 1, tune_count)
        else:
            srv.tune(**tuning)
        # warm-up: at least two requests per slot, so that every slot's
        # problem buffers are in the memory pool before the timed requests
        nwarm = max(args.warmup, 2 * args.slots)
        for t in [srv.submit(sp, bg, lam(i), opts, precision, key) for i in range(nwarm)]:
            srv.poll(t)
        srv.launches()
        srv.mark()
        s0 = time.perf_counter()
        tickets = [srv.submit(sp, bg, lam(nwarm + i), opts, precision, key) for i in range(k)]
        res = [srv.poll(t) for t in tickets]
        wall = time.perf_counter() - s0
        dev_ms = srv.mark()
        launches = srv.launches()
        srv.close()
        bad = [r["status"] for r in res if r["status"] not in (G.OK,)]
        if bad:
            raise RuntimeError(f"served solve failed: status {bad}")
        return dev_ms * 1e-3, wall, res, launches, tuning

    barrier()
    with ClockSampler(local) as clk_srv:
        t_srv, _, res_srv, srv_launches, tuning = served(mixed_opts, G.C64, args.steps, 1)
    clocks_srv = clk_srv.summary()
    k64s = max(1, min(args.steps, 4))
    t_srv64, _, res_srv64, _, tuning64 = served(fp64_opts, G.C128, k64s, 1, tune_count=2)
    err_srv = max(abs(res_srv[i]["xsec"][0] - res_srv64[i]["xsec"][0]) / abs(res_srv64[i]["xsec"][0])
                  for i in range(k64s))
    err_srv_all = max(float(np.max(np.abs(res_srv[i]["xsec"] - res_srv64[i]["xsec"]) /
                                   np.abs(res_srv64[i]["xsec"]))) for i in range(k64s))
    svc = [r["service_ms"] for r in res_srv]
    svc64 = [r["service_ms"] for r in res_srv64]

    # ---- end to end through the C ABI with host buffers: every request
    # copies its spheres and wave from the host, sets its problem up from
    # scratch (cluster_key 0), and returns its cross sections to the host ----
    with ClockSampler(local) as clk_e2e:
        _, wall_e2e, res_e2e, _, _ = served(mixed_opts, G.C64, args.steps, 0, tuning=tuning)
    import ctypes
    h2d = ctypes.sizeof(G.Sphere) * len(sp) + ctypes.sizeof(G.Medium) + \
        ctypes.sizeof(G.PlaneWave) + ctypes.sizeof(G.SolveOptions)
    d2h = ctypes.sizeof(G.Result)

    # aggregate over ranks (max time, summed work)
    t_srv_all, t_srv64_all, e2e_all, t_mixed_all, t64_all = max_over_ranks(
        [t_srv, t_srv64, wall_e2e, t_mixed, t_fp64], world, f"cuda:{local}")
    value = world * args.steps / t_srv_all
    value64 = world * k64s / t_srv64_all
    value_ss = world * args.steps / t_mixed_all
    value64_ss = world * k64 / t64_all

    hbm, how = peaks()
    mv_ms, mv_n = kt["matvec_c64"]
    bytes_mv = 8.0 * n * n  # complex64 matrix streamed once per product
    achieved_c64 = bytes_mv / (mv_ms / mv_n * 1e-3) / 1e9 if mv_n else None
    # the inner products on the bf16 copy (4 bytes per entry), and the one
    # complex64 product per solve that writes the copy (8 bytes read, 4 written)
    b16_ms, b16_n = kin["bf16"]
    cp_ms, cp_n = kin["copy"]
    bytes_b16 = 4.0 * n * n
    achieved = bytes_b16 / (b16_ms / b16_n * 1e-3) / 1e9 if b16_n else 0.0
    asm_ms, asm_n = kt["assemble"]
    bytes_asm = 8.0 * n * n  # complex64 matrix written
    mv64_ms, mv64_n = kt64["matvec_c128"]
    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_srv_all / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64 (FP32) matrix; inner FP32 GMRES on its bf16 copy (FP32 accumulation); "
                 "c128 (FP64) outer residuals (compensated) and assembly",
        "data": "synthetic (seeded random clusters)",
        "config": {"workload": args.workload + ": " + w["desc"], "unknowns": n,
                   "parallelism": f"replicas x{world}, {args.slots} serving slots per GPU",
                   "l2": "inputs larger than L2 (no flush)",
                   "solver": "FGMRES(FP64 outer, tol 1e-7) + GMRES(FP32 inner, 80 it, tol 1e-3; its "
                             "products on a bf16 copy of the complex64 matrix, written by the first)",
                   "timing": "CUDA events on every slot's stream (om_server_mark) around the K requests",
                   "launch_tuning": {"mixed": tuning, "fp64": tuning64,
                                     "how": "om_server_autotune on warm-up requests"}},
        "latency_ms": {"p50": float(np.percentile(svc, 50)), "p99": float(np.percentile(svc, 99)),
                       "what": "per-request service time on its slot (host clock), overlapping the other slot"},
        "fp64": {"value": value64, "unit": UNIT, "steps": k64s, "ms_per_step": 1e3 * t_srv64_all / k64s,
                 "latency_ms": {"p50": float(np.percentile(svc64, 50)),
                                "p99": float(np.percentile(svc64, 99))},
                 "solver": "GMRES(FP64, tol 1e-10)", "gmres_iterations": it64 / k64},
        "speedup_vs_fp64": value / value64,
        "qext_rel_err_vs_fp64": err_srv, "xsec_max_rel_err_vs_fp64": err_srv_all,
        "single_stream": {
            "mixed": {"value": value_ss, "ms_per_step": 1e3 * t_mixed_all / args.steps,
                      "latency_ms": {"p50": 1e3 * float(np.percentile(lat, 50)),
                                     "p99": 1e3 * float(np.percentile(lat, 99))}},
            "fp64": {"value": value64_ss, "ms_per_step": 1e3 * t64_all / k64,
                     "latency_ms": {"p50": 1e3 * float(np.percentile(lat64, 50)),
                                    "p99": 1e3 * float(np.percentile(lat64, 99))}},
            "speedup_vs_fp64": value_ss / value64_ss,
            "qext_rel_err_vs_fp64": err, "xsec_max_rel_err_vs_fp64": err_all},
        "iterations": {"outer": outer / args.steps, "inner": inner / args.steps},
        "e2e": {"value": world * args.steps / e2e_all, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "path": "om_server_submit/om_server_poll (C ABI, host buffers, problem set-up "
                        "from the host every request, host wall clock)",
                "service_ms": {"p50": float(np.percentile([r["service_ms"] for r in res_e2e], 50)),
                               "max": float(max(r["service_ms"] for r in res_e2e))},
                "queue_ms_max": float(max(r["queue_ms"] for r in res_e2e)),
                "clocks": clk_e2e.summary()},
        "roofline": {"bound": "hbm",
                     "kernel": "k_matvec_tma<true> (inner FP32 product on the bf16 copy, TMA-staged; "
                               "timed in the single-stream part, where a context uses it)",
                     "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "peak_source": how + " (MEASURED_PEAKS.json hbm_gbs)",
                     "traffic": bytes_b16 * BF16_READ_RATIO + 8.0 * n * -(-n // 1024),
                     "algorithmic_bytes_per_launch": bytes_b16},
        "kernels": {
            "assemble_mixed": {"ms_avg": asm_ms / max(asm_n, 1), "launches": asm_n,
                               "written_GBps": bytes_asm / (asm_ms / max(asm_n, 1) * 1e-3) / 1e9
                               if asm_n else None,
                               "frac_of_hbm_peak": bytes_asm / (asm_ms / max(asm_n, 1) * 1e-3) / 1e9 / hbm
                               if asm_n else None,
                               "kernel": "k_assemble_rot (rotated z-axis translations)",
                               "bound": "hbm write (8 n^2 B per assembly)"},
            "matvec_bf16_inner": {"ms_avg": b16_ms / max(b16_n, 1), "launches": b16_n,
                                  "GBps": achieved, "bound": "hbm (4 n^2 B read)"},
            "matvec_c64_writing_copy": {"ms_avg": cp_ms / max(cp_n, 1), "launches": cp_n,
                                        "GBps": 12.0 * n * n / (cp_ms / cp_n * 1e-3) / 1e9 if cp_n else None,
                                        "bound": "hbm (8 n^2 B read + 4 n^2 B written)"},
            "matvec_c64": {"ms_avg": mv_ms / max(mv_n, 1), "launches": mv_n,
                           "GBps": achieved_c64, "bound": "hbm"},
            "matvec_c64_compensated": {"ms_avg": kt["matvec_c64_df"][0] / max(kt["matvec_c64_df"][1], 1),
                                       "launches": kt["matvec_c64_df"][1],
                                       "GBps": bytes_mv / (kt["matvec_c64_df"][0] / max(kt["matvec_c64_df"][1], 1) * 1e-3) / 1e9 if kt["matvec_c64_df"][1] else None},
            "matvec_c128": {"ms_avg": mv64_ms / max(mv64_n, 1), "launches": mv64_n,
                            "bound": "fp64 ALU (4 FMA per 16 B)"},
        },
        "gpu_launches": srv_launches,
        "gpu_launches_single_stream": total_launches,
        "clocks": clocks_srv,
        "clocks_single_stream": clocks,
    }
    if rank == 0 and not args.no_cpu_baseline:
        cb = cpu_baseline(w, xyz, rad, it64 / k64, threads=None, budget_s=15.0)
        cb["model_check"] = cpu_model_check()
        cb["model_error"] = cb["model_check"]["model_error"]
        result["cpu_baseline"] = cb
    ctx.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return result if rank == 0 else None


def cpu_baseline(w, xyz, rad, gmres_iters, threads=None, budget_s=15.0):
    """The oracle (a restatement of the reference's CPU algorithm: map-cached
    Stout recurrences, dense matvec GMRES) timed on a bounded sample of the
    same wavelength-solve on this host, extrapolated to one full solve."""
    from oracle import oracle as O
    O.lib()
    threads = threads or O.max_threads()
    O.set_threads(threads)
    cl = O.Cluster(xyz=xyz, radius=rad, eps=complex(w["index"]) ** 2, nmax=w["nmax"],
                   wavelength=w["lam"], bg_eps=complex(w["host"]) ** 2)
    pr = O.Problem(cl)
    N, P = cl.n_spheres, cl.P
    n = cl.n_unknowns
    rng = np.random.default_rng(1)
    # assembly sample: ordered pairs i != j
    npairs = max(threads, 8)
    t_pair = None
    while True:
        pairs = []
        while len(pairs) < npairs:
            i, j = rng.integers(0, N, 2)
            if i != j:
                pairs.append((i, j))
        t0 = time.perf_counter()
        O.assemble_pairs(pr, pairs)
        dt = time.perf_counter() - t0
        t_pair = dt / npairs
        if dt > budget_s / 3 or npairs >= N * (N - 1):
            break
        npairs = min(N * (N - 1), 1024, int(npairs * max(2.0, (budget_s / 3) / max(dt, 1e-3))))
        if npairs >= 1024 and dt > 0.05:
            break
    t_asm = t_pair * N * (N - 1)
    # matvec sample: a block of rows of a dense complex128 matrix of the full width
    rows = max(64, min(n, int(2e8 // (16 * n))))
    A = (rng.standard_normal((rows, n)) + 1j * rng.standard_normal((rows, n))).astype(np.complex128)
    A = np.asfortranarray(A)
    x = rng.standard_normal(n) + 0j
    O.matvec(A, x)
    reps = 0
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < budget_s / 3:
        O.matvec(A, x)
        reps += 1
    t_mv = (time.perf_counter() - t0) / reps * (n / rows)
    t_solve = t_asm + t_mv * (gmres_iters + 2)
    O.set_threads(1)
    return {"value": 1.0 / t_solve, "unit": UNIT, "cores": threads, "kind": "port",
            "estimate": "extrapolated from a bounded sample (sampled pair blocks x N(N-1), "
                        "row-block matvec x GMRES iterations)",
            "sample": (f"oracle on {threads} host threads: {npairs} sampled pair blocks "
                       f"({t_pair * 1e3:.2f} ms/pair, x N(N-1)={N * (N - 1)}) + dense FP64 "
                       f"matvec on {rows} of {n} rows ({t_mv * 1e3:.1f} ms/full matvec) x "
                       f"{gmres_iters + 2:.0f} GMRES iterations; extrapolated {t_solve:.1f} s/solve"),
            "gmres_iterations": gmres_iters, "seconds_per_solve": t_solve}


def cpu_model_check(threads=None, budget_s=3.0):
    """The extrapolation model of cpu_baseline against a full oracle
    wavelength-solve where one fits in seconds (workload `small`: N = 40,
    nMax = 8, 6,400 unknowns): source vector, all N(N-1) blocks, GMRES to
    1e-10 with the dense matvec, internal coefficients, cross sections. The
    model gets the measured run's own GMRES iteration count."""
    from oracle import oracle as O
    O.lib()
    threads = threads or O.max_threads()
    w = WORKLOADS["small"]
    xyz, rad = cluster(w)
    O.set_threads(threads)
    cl = O.Cluster(xyz=xyz, radius=rad, eps=complex(w["index"]) ** 2, nmax=w["nmax"],
                   wavelength=w["lam"], bg_eps=complex(w["host"]) ** 2)
    pr = O.Problem(cl)
    t0 = time.perf_counter()
    _, _, _, it = pr.wavelength_solve("gmres", tol=1e-10, maxit=400, restarts=6)
    measured = time.perf_counter() - t0
    O.set_threads(1)
    predicted = cpu_baseline(w, xyz, rad, it, threads=threads, budget_s=budget_s)["seconds_per_solve"]
    return {"workload": "small: " + w["desc"], "cores": threads, "gmres_iterations": it,
            "measured_s": measured, "predicted_s": predicted, "model_error": predicted / measured - 1.0}


def reference_arm(args, w):
    rank, world, local = dist_env()
    if rank != 0:
        return None
    xyz, rad = cluster(w, 0)
    # FP64 GMRES iterations to 1e-10 on this workload's matrix, measured by the
    # GPU arm's plain form (bench.py c2: fp64.gmres_iterations = 11; c1: 59).
    # The reference arm runs in its own process and cannot hold the complex128
    # C2 matrix (65.5 GB) to count them itself.
    iters = {"c2": 11, "c1": 59, "small": 13, "mid": 12}[args.workload]
    check = cpu_model_check()
    lat, wall = [], []
    for i in range(args.warmup + args.steps):
        s0 = time.perf_counter()
        cb = cpu_baseline(w, xyz, rad, iters, threads=None, budget_s=6.0)
        if i >= args.warmup:
            lat.append(cb["seconds_per_solve"])
            wall.append(time.perf_counter() - s0)
    t = float(np.mean(lat))
    return {"metric": METRIC, "value": 1.0 / t, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128 (FP64)",
            "data": "synthetic (seeded random clusters)", "impl": "reference",
            "config": {"workload": args.workload + ": " + w["desc"]},
            "estimate": ("each step times a bounded sample of one wavelength-solve and extrapolates it: "
                         "ms_per_step is the extrapolated solve time, not the step's wall time "
                         f"({1e3 * float(np.mean(wall)):.0f} ms); model error from a full solve in this "
                         f"run: {check['model_error']:+.3f}"),
            "sample_wall_ms_per_step": 1e3 * float(np.mean(wall)),
            "model_check": check,
            "cpu_baseline": {"value": 1.0 / t, "unit": UNIT, "cores": cb["cores"], "kind": "port",
                             "estimate": cb["estimate"], "model_error": check["model_error"],
                             "gmres_iterations": iters, "sample": cb["sample"]},
            "e2e": {"value": 1.0 / t, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


# ---------------------------------------------------------------------------
# Batching (c3) and serving (c4) workloads: ragged requests through om_server.
# ---------------------------------------------------------------------------
def c1_volume_fraction():
    """Volume fraction of the c1 cluster (N = 100, radii U[50, 80] nm, 2 um cube)."""
    xyz, rad = cluster(WORKLOADS["c1"])
    return float(np.sum(4.0 / 3.0 * np.pi * rad ** 3) / (2000 * nm) ** 3)


def nmax_rule(radii, lam):
    """nMax = clamp(ceil(x + 4 x^(1/3) + 2), 4, 12), x = 2 pi a / lambda; the
    reference needs one nMax per cluster, so the largest over its spheres."""
    x = 2.0 * np.pi * np.asarray(radii) / lam
    return int(np.clip(np.ceil(x + 4.0 * np.cbrt(x) + 2.0), 4, 12).max())


def ragged_cluster(rng, N, rmin, rmax, frac):
    """N spheres, radii U[rmin, rmax], in the smallest cube edge that gives the
    volume fraction `frac` (seeded rejection sampling, 20 nm gap)."""
    rad = rng.uniform(rmin, rmax, N)
    edge = float(np.cbrt(np.sum(4.0 / 3.0 * np.pi * rad ** 3) / frac))
    edge = max(edge, 2.0 * rad.max() + 40 * nm)
    while True:
        xyz = np.zeros((N, 3))
        ok = True
        for k, r in enumerate(rad):
            lim = (rad[:k] + r + 20 * nm) ** 2
            for _ in range(1000):
                cand = rng.uniform(-edge / 2 + r, edge / 2 - r, size=(4, 3))
                if k == 0:
                    xyz[0] = cand[0]
                    break
                diff = cand[:, None, :] - xyz[None, :k, :]
                good = np.nonzero(((diff * diff).sum(axis=2) >= lim).all(axis=1))[0]
                if good.size:
                    xyz[k] = cand[good[0]]
                    break
            else:
                ok = False
                break
        if ok:
            return xyz, rad, edge
        edge *= 1.1


def c3_cases(n_clusters, n_lambda, seed=20260404):
    """The spectral sweep: clusters of 2-64 spheres (radii U[30, 120] nm,
    index U[1.5, 4.0] + i U[0.001, 0.1] per cluster) at wavelengths uniform in
    [400, 900] nm; every case is the fundamental solve plus the SH solve
    driven by the surface chi(2) (perp-perp-perp 1.0, par-perp-par 0.25)."""
    import optimet_gb300 as G
    rng = np.random.default_rng(seed)
    frac = c1_volume_fraction()
    lams = np.linspace(400 * nm, 900 * nm, 256)
    pick = np.linspace(0, 255, n_lambda).round().astype(int)
    cases = []
    for c in range(n_clusters):
        N = int(rng.integers(2, 65))
        xyz, rad, edge = ragged_cluster(rng, N, 30 * nm, 120 * nm, frac)
        index = complex(rng.uniform(1.5, 4.0), rng.uniform(0.001, 0.1))
        arrays = {}
        for li in pick:
            lam = float(lams[li])
            nmax = nmax_rule(rad, lam)
            if nmax not in arrays:
                arrays[nmax] = G.spheres_array(xyz, rad, index ** 2, nmax, ksippp=1.0,
                                               ksiparppar=0.25)
            cases.append(dict(sp=arrays[nmax], wave=G.plane_wave(lam, sh=True), key=c * 16 + nmax,
                              N=N, nmax=nmax))
    return cases


def run_cases(G, cases, opts, precision, slots, bg, device=0, budget=0):
    srv = G.Server(device, budget, slots)
    # warm-up: one request per size class
    seen = {}
    for cs in cases:
        seen.setdefault((cs["N"], cs["nmax"]), cs)
    for t in [srv.submit(cs["sp"], bg, cs["wave"], opts, precision, 0) for cs in list(seen.values())[:8]]:
        srv.poll(t)
    srv.launches()
    srv.mark()
    tickets = [srv.submit(cs["sp"], bg, cs["wave"], opts, precision, cs["key"]) for cs in cases]
    res = [srv.poll(t) for t in tickets]
    dev_s = srv.mark() * 1e-3
    launches = srv.launches()
    srv.close()
    return dev_s, res, launches


def run_batch(G, ctx, cases, opts, precision, bg):
    """The cases through om_batch_solve (size classes, one assembly launch and
    graph-captured lockstep GMRES per batch); returns (seconds, results,
    launches)."""
    reqs = [(cs["sp"], bg, cs["wave"], opts, precision) for cs in cases]
    ctx.synchronize()
    ctx.mark()
    res = G.batch_solve(ctx, reqs)
    dev_s = ctx.mark() * 1e-3
    return dev_s, res, ctx.last_launches


def c3_profile_case(G, mixed, bg):
    """The small c3 case the ncu captures use: 24 requests with N >= 40 of two
    wavelengths per cluster, precision form, batch arena 6 GiB."""
    cases = [c for c in c3_cases(64, 2) if c["N"] >= 40][:24]
    ctx = G.Context(0)
    t0 = time.perf_counter()
    res = G.batch_solve(ctx, [(c["sp"], bg, c["wave"], mixed, G.C64) for c in cases],
                        arena_bytes=6 << 30)
    dt = time.perf_counter() - t0
    ctx.close()
    return {"workload": "c3 profiling case: 24 requests with N >= 40, precision form, 6 GiB arena",
            "seconds": dt, "statuses": sorted({r["status"] for r in res})}


def batch_arm(args):
    """c3: the ragged spectral sweep through the batching form
    (om_batch_solve), precision form against the FP64 form on the same cases;
    the same cases through the server are reported beside it."""
    import optimet_gb300 as G
    from optimet_gb300 import build
    build.build()
    bg = G.medium(1.0)
    mixed = G.options(G.SOLVE_FGMRES_MIXED, tol=1e-8, max_iter=30, restarts=4, inner_iter=60,
                      inner_tol=args.c3_inner_tol)
    if args.c3_profile:
        return c3_profile_case(G, mixed, bg)
    cases = c3_cases(args.c3_clusters, args.c3_wavelengths)
    fp64 = G.options(G.SOLVE_GMRES, tol=1e-10, max_iter=300, restarts=6)
    ctx = G.Context(0)
    # warm-up: the whole sweep once in both forms (coefficient and SH coupling
    # tables, the auxiliary contexts, and the autotuner's choice of matvec
    # tiles for every size class, made at a class's first batch)
    for opts, prec in ((mixed, G.C64), (fp64, G.C128)):
        run_batch(G, ctx, cases, opts, prec, bg)
    with ClockSampler(0) as clk:
        t_mx, res_mx, launches = run_batch(G, ctx, cases, mixed, G.C64, bg)
    t_64, res_64, _ = run_batch(G, ctx, cases, fp64, G.C128, bg)
    tiles = G.batch_tiles(ctx)
    ctx.close()
    ok = [i for i in range(len(cases)) if res_mx[i]["status"] == G.OK and res_64[i]["status"] == G.OK]
    err = max(abs(res_mx[i]["xsec"][0] - res_64[i]["xsec"][0]) / abs(res_64[i]["xsec"][0]) for i in ok)
    err_sh = max(float(np.max(np.abs(res_mx[i]["xsec_sh"] - res_64[i]["xsec_sh"]) /
                              np.abs(res_64[i]["xsec_sh"]))) for i in ok)
    lat = [r["latency_ms"] for r in res_mx]
    served = {}
    if not args.no_server:
        ts_mx, rs_mx, _ = run_cases(G, cases, mixed, G.C64, args.batch_slots, bg)
        ts_64, rs_64, _ = run_cases(G, cases, fp64, G.C128, args.batch_slots, bg)
        served = {"slots": args.batch_slots, "mixed": len(cases) / ts_mx, "fp64": len(cases) / ts_64,
                  "unit": UNIT, "speedup_vs_fp64": ts_64 / ts_mx,
                  "failed": {"mixed": sum(r["status"] != G.OK for r in rs_mx),
                             "fp64": sum(r["status"] != G.OK for r in rs_64)}}
    Ns = [cs["N"] for cs in cases]
    nm_ = [cs["nmax"] for cs in cases]
    count = lambda res: {str(k): v for k, v in sorted(
        __import__("collections").Counter(r["status"] for r in res).items())}
    return {"metric": METRIC, "value": len(cases) / t_mx, "unit": UNIT + " (FF + SH per case)",
            "n_gpus": 1, "steps": len(cases), "warmup": len(cases), "ms_per_step": 1e3 * t_mx / len(cases),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c64 (FP32) inner + c128 (FP64) outer/assembly", "data": "synthetic (seeded)",
            "config": {"workload": f"c3: {args.c3_clusters} clusters x {args.c3_wavelengths} of the "
                                   "256 wavelengths in [400, 900] nm, N U{2..64}, radii U[30,120] nm, "
                                   "index U[1.5,4]+iU[0.001,0.1], nMax rule clamp(ceil(x+4x^(1/3)+2),4,12) "
                                   "(max over each cluster), FF + SH (ksippp 1, ksiparppar 0.25)",
                       "path": "om_batch_solve (size classes; one assembly launch and graph-captured "
                               "lockstep GMRES per batch)",
                       "N_range": [min(Ns), max(Ns)], "nmax_range": [min(nm_), max(nm_)],
                       "solver": f"precision form: GMRES-based refinement to 1e-8 (FP64 residuals on the "
                                 f"complex64 matrices), FP32 Arnoldi to {args.c3_inner_tol:g} per cycle on "
                                 f"scaled fp16 copies; FP64 form: GMRES to 1e-10"},
            "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                           "note": "call start -> the request's batch done (all requests submitted at once)"},
            "fp64": {"value": len(cases) / t_64, "unit": UNIT},
            "speedup_vs_fp64": t_64 / t_mx,
            "qext_rel_err_vs_fp64": err, "sh_xsec_rel_err_vs_fp64": err_sh,
            "statuses": {"mixed": count(res_mx), "fp64": count(res_64)},
            "served": served,
            "gpu_launches": launches, "matvec_tiles_autotuned": tiles, "clocks": clk.summary()}


def c4_requests(rate, duration, seed=20260405):
    """Poisson arrivals; N log-uniform in [1, 300]; radii, index and nMax as
    c3; wavelength U[400, 900] nm; random linear polarisation and direction;
    SH attached to 30% of the requests."""
    import optimet_gb300 as G
    rng = np.random.default_rng(seed)
    frac = c1_volume_fraction()
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            break
        N = int(np.clip(np.floor(np.exp(rng.uniform(0.0, np.log(301.0)))), 1, 300))
        xyz, rad, _ = ragged_cluster(rng, N, 30 * nm, 120 * nm, frac)
        index = complex(rng.uniform(1.5, 4.0), rng.uniform(0.001, 0.1))
        lam = rng.uniform(400 * nm, 900 * nm)
        nmax = nmax_rule(rad, lam)
        sh = bool(rng.uniform() < 0.3)
        psi = rng.uniform(0, np.pi)
        th, ph = float(np.arccos(rng.uniform(-1, 1))), float(rng.uniform(0, 2 * np.pi))
        sp = G.spheres_array(xyz, rad, index ** 2, nmax, ksippp=1.0 if sh else 0.0,
                             ksiparppar=0.25 if sh else 0.0)
        out.append(dict(t=t, sp=sp, wave=G.plane_wave(lam, th, ph, np.cos(psi), np.sin(psi), sh=sh),
                        N=N, nmax=nmax))
    return out


def serve_arm(args):
    """c4: Poisson request stream admitted against a 150 GB HBM budget."""
    import optimet_gb300 as G
    from optimet_gb300 import build
    build.build()
    reqs = c4_requests(args.c4_rate, args.c4_seconds)
    bg = G.medium(1.0)
    forms = {"mixed": (G.options(G.SOLVE_FGMRES_MIXED, tol=1e-8, max_iter=30, restarts=4,
                                 inner_iter=60, inner_tol=args.c3_inner_tol), G.C64),
             "fp64": (G.options(G.SOLVE_GMRES, tol=1e-10, max_iter=300, restarts=6), G.C128)}
    forms = {k: v for k, v in forms.items() if k in args.c4_forms.split(",")}
    out = {}
    for name, (opts, prec) in forms.items():
        srv = G.Server(0, 150 << 30, args.batch_slots)
        if args.c4_batching > 1:
            srv.batching(args.c4_batching, 0, int(args.c4_batch_limit_gb * (1 << 30)))
        for r in reqs[:4]:
            srv.poll(srv.submit(r["sp"], bg, r["wave"], opts, prec, 0))
        tickets = []
        s0 = time.perf_counter()
        with ClockSampler(0) as clk:
            for r in reqs:
                delay = s0 + r["t"] - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                tickets.append(srv.submit(r["sp"], bg, r["wave"], opts, prec, 0))
            res = [srv.poll(t) for t in tickets]
            wall = time.perf_counter() - s0
        srv.close()
        lat = np.array([r["latency_ms"] for r in res if r["status"] == G.OK])
        out[name] = {"solves_per_s": len(lat) / wall, "offered_per_s": len(reqs) / args.c4_seconds,
                     "latency_ms": {"p50": float(np.percentile(lat, 50)),
                                    "p99": float(np.percentile(lat, 99)),
                                    "p99.9": float(np.percentile(lat, 99.9))},
                     "completed": int(len(lat)),
                     "refused_budget": int(sum(r["status"] == G.ERR_BUDGET for r in res)),
                     "other_failures": int(sum(r["status"] not in (G.OK, G.ERR_BUDGET) for r in res)),
                     "failed": [{"request": i, "status": r["status"], "N": q["N"], "nmax": q["nmax"],
                                 "sh": int(q["wave"].sh)}
                                for i, (r, q) in enumerate(zip(res, reqs))
                                if r["status"] not in (G.OK, G.ERR_BUDGET)][:20],
                     "service_ms_by_N": {f"{lo}-{hi}": float(np.median([r["service_ms"] for r, q in zip(res, reqs)
                                                                        if lo <= q["N"] <= hi] or [0]))
                                         for lo, hi in ((1, 10), (11, 30), (31, 100), (101, 300))},
                     "wall_s": wall, "clocks": clk.summary(), "xsec": [r["xsec"][0] for r in res]}
    both = [i for i in range(len(reqs)) if len(out) == 2 and out["mixed"]["xsec"][i] and
            out["fp64"]["xsec"][i]]
    err = max(abs(out["mixed"]["xsec"][i] - out["fp64"]["xsec"][i]) / abs(out["fp64"]["xsec"][i])
              for i in both) if both else None
    for v in out.values():
        v.pop("xsec")
    m = out.get("mixed") or next(iter(out.values()))
    return {"metric": METRIC, "value": m["solves_per_s"], "unit": UNIT, "n_gpus": 1,
            "steps": len(reqs), "warmup": 4, "ms_per_step": 1e3 / m["solves_per_s"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c64 (FP32) inner + c128 (FP64) outer/assembly", "data": "synthetic (seeded)",
            "config": {"workload": f"c4: Poisson arrivals {args.c4_rate}/s for {args.c4_seconds} s, "
                                   "N log-uniform [1,300], radii/index/nMax as c3, lambda U[400,900] nm, "
                                   "random polarisation and direction, SH on 30%, HBM budget 150 GB",
                       "slots": args.batch_slots,
                       "batching": (f"runs of up to {args.c4_batching} queued requests with a batched "
                                    f"footprint up to {args.c4_batch_limit_gb} GiB per om_batch_solve "
                                    "call; larger ones one at a time" if args.c4_batching > 1 else "off")},
            "latency_ms": m["latency_ms"], "forms": out, "qext_rel_err_vs_fp64": err}


def fp64_gemm_tflops():
    """FP64 throughput measured with cuBLAS DGEMM (torch.matmul, 8192^3, best of 5)."""
    import torch
    a = torch.randn(8192, 8192, dtype=torch.float64, device="cuda")
    b = torch.randn_like(a)
    best = 1e30
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) * 1e-3)
    return 2.0 * 8192 ** 3 / best / 1e12


def tc_update_arm(args):
    """One tensor-core trailing update C (m x m) -= A (m x k) B (k x m), complex64
    (om_cgemm_sub_c64: host buffers in and out), m = --tc-m, k = --tc-k: the
    kernel the LU role's rank-k updates run, as a stand-alone case for ncu."""
    import optimet_gb300 as G
    from optimet_gb300 import build
    build.build()
    m, k = args.tc_m, args.tc_k
    rng = np.random.default_rng(1)
    A = (rng.standard_normal((m, k)) + 1j * rng.standard_normal((m, k))).astype(np.complex64)
    B = (rng.standard_normal((k, m)) + 1j * rng.standard_normal((k, m))).astype(np.complex64)
    Cm = (rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m))).astype(np.complex64)
    ctx = G.Context(0)
    ctx.tune(lu_tensor_cores=args.lu_update)
    t0 = time.perf_counter()
    out = G.cgemm_sub_c64(ctx, A, B, Cm)
    wall = time.perf_counter() - t0
    ctx.close()
    return {"workload": f"tensor-core rank-{k} update, {m} x {m} complex64",
            "kernel": {1: "k_cgemm_sub_tc3 (persistent)", 2: "k_cgemm_sub_tc2 (one CTA per tile)",
                       3: "k_cgemm_sub_tc3 (persistent) for k > 64, else k_cgemm_sub_tc2"}.get(
                args.lu_update, "none"),
            "wall_s_with_copies": wall, "checksum": float(np.abs(out[:4, :4]).sum())}


def lu_mixed_arm(args):
    """c2 through the precision form's LU role: FP32 LU of the complex64
    matrix (tensor-core trailing updates) as the preconditioner of FP64 outer
    FGMRES with compensated residuals (GMRES-based iterative refinement), one
    wavelength-solve per step, against the FP64 GMRES solve of the same
    cluster."""
    import optimet_gb300 as G
    from optimet_gb300 import build
    build.build()
    w = WORKLOADS[args.lu_case]
    xyz, rad = cluster(w)
    ctx = G.Context(0)
    sp = G.spheres_array(xyz, rad, complex(w["index"]) ** 2, w["nmax"])
    pr = G.Problem(ctx, sp, G.medium(complex(w["host"]) ** 2), G.plane_wave(w["lam"]))
    pr.source_vector(copy=False)
    pr.assemble(G.FF, G.C128)
    pr.solve(G.options(G.SOLVE_GMRES, tol=1e-10, max_iter=400, restarts=6))
    ref = pr.cross_sections()
    pr.close()
    pr = G.Problem(ctx, sp, G.medium(complex(w["host"]) ** 2), G.plane_wave(w["lam"]))
    ctx.tune(lu_tensor_cores=args.lu_update, lu_persistent=args.lu_persistent)
    opts = G.options(G.SOLVE_LU_MIXED, tol=1e-9, max_iter=30, restarts=4)
    times, st = [], None
    # one untimed solve first: the LU kernels' first launches (module loading,
    # shared-memory attributes, the memory pool growing to the LU's workspace)
    ctx.synchronize()
    ctx.mark()
    t_first = time.perf_counter()
    pr.source_vector(copy=False)
    pr.assemble(G.FF, G.C64)
    pr.solve(opts)
    ctx.synchronize()
    first_ms = {"device": ctx.mark(), "host": 1e3 * (time.perf_counter() - t_first)}
    with ClockSampler(0) as clk:
        for _ in range(max(1, args.steps)):
            ctx.synchronize()
            ctx.mark()
            pr.source_vector(copy=False)
            pr.assemble(G.FF, G.C64)
            st = pr.solve(opts)
            xs = pr.cross_sections()
            times.append(ctx.mark() * 1e-3)
    # one more solve, untimed, with the phase timers on (an event pair per
    # panel, trailing update and triangular solve)
    ctx.timers(True)
    ctx.lu_timers()
    pr.solve(opts)
    ph = ctx.lu_timers()
    ctx.timers(False)
    t = float(np.median(times))
    err = float(abs(xs[0] - ref[0]) / abs(ref[0]))
    n = pr.n
    pr.close()
    ctx.close()
    blk = 256 if args.lu_update else 32  # rank of the trailing updates
    upd_bytes = 16.0 * sum((n - K) ** 2 for K in range(blk, n, blk))  # C read + written, complex64
    phases = {"factor_ms": ph["factor"][0], "panel_ms": ph["panel"][0], "panels": ph["panel"][1],
              "update_ms": ph["update"][0], "updates": ph["update"][1],
              "update_hbm_frac_of_measured": upd_bytes / (ph["update"][0] * 1e-3) / 1e9 / peaks()[0]
              if ph["update"][0] > 0 else None,
              "tri_solve_ms": ph["tri_solve"][0], "tri_solves": ph["tri_solve"][1]}
    return {"metric": METRIC, "value": 1.0 / t, "unit": UNIT, "n_gpus": 1, "steps": len(times),
            "warmup": 1, "ms_per_step": 1e3 * t, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c64 (FP32) LU + c128 (FP64) refinement",
            "data": "synthetic (seeded)",
            "config": {"workload": args.lu_case + " LU role: " + w["desc"],
                       "solver": "GMRES-based iterative refinement: FP64 residuals, GMRES on the system left-preconditioned by the FP32 LU (tensor-core trailing updates), tol 1e-9",
                       "trailing_update": {1: "persistent", 2: "one CTA per tile",
                                           3: "persistent for the trailing updates, one CTA per tile "
                                              "for the rank-32 in-block and U12 updates",
                                           0: "FP32 CUDA cores, rank 32"}[args.lu_update],
                       "panels_and_sweeps": {1: "one launch per panel / sweep",
                                             2: "per-column panel launches, per-block sweep launches"}[args.lu_persistent]},
            "refinement_iterations": st.iterations, "qext_rel_err_vs_fp64": err, "phases": phases,
            "first_solve_ms": first_ms,
            "clocks": clk.summary()}


def near_field_arm(args):
    """c1 near field: |E|^2 on a 256 x 256 grid in the z = 0 plane (two z
    layers at +-0.1 nm, as the reference's grid needs two steps: 131,072
    points) around the c1 cluster after its FP64 GMRES solve."""
    import optimet_gb300 as G
    from optimet_gb300 import build
    from optimet_gb300.optimet import grid_points
    build.build()
    w = WORKLOADS["c1"]
    xyz, rad = cluster(w)
    ctx = G.Context(0)
    sp = G.spheres_array(xyz, rad, complex(w["index"]) ** 2, w["nmax"])
    pr = G.Problem(ctx, sp, G.medium(complex(w["host"]) ** 2), G.plane_wave(w["lam"]))
    pr.source_vector(copy=False)
    pr.assemble(G.FF, G.C128)
    st = pr.solve(G.options(G.SOLVE_GMRES, tol=1e-10, max_iter=400, restarts=6))
    params = [-1000 * nm, 1000 * nm, 256, -1000 * nm, 1000 * nm, 256, -0.1 * nm, 0.1 * nm, 2]
    pts = grid_points(params)
    for _ in range(args.warmup):
        pr.near_field(pts[:8192])
    times = []
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            ctx.mark()
            E, H = pr.near_field(pts)
            times.append(ctx.mark() * 1e-3)
    t = float(np.median(times))
    inside = 0
    for c, r in zip(xyz, rad):
        inside += int(np.sum(np.linalg.norm(pts - c, axis=1) <= r))
    N, P = w["N"], w["nmax"] * (w["nmax"] + 2)
    flops = 8.0 * 6 * N * P * (len(pts) - inside)  # 6 complex MAC per (point, sphere, harmonic)
    peak = fp64_gemm_tflops()
    res = {"metric": "near-field points/s (|E|^2, c1 grid)", "value": len(pts) / t, "unit": "points/s",
           "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128 (FP64)",
           "data": "synthetic (seeded)",
           "config": {"workload": "c1 near field: " + w["desc"] + "; grid 256 x 256 x 2 over "
                                  "[-1, 1] um^2 at z = +-0.1 nm", "points": len(pts),
                      "points_inside_spheres": inside, "gmres_iterations": st.iterations},
           "max_abs_E2": float(np.max(np.sum(np.abs(E) ** 2, axis=1))),
           "roofline": {"bound": "fp64", "achieved": flops / t / 1e12, "peak": peak, "unit": "TFLOP/s",
                        "frac": flops / t / 1e12 / peak,
                        "peak_source": "measured here: cuBLAS DGEMM 8192^3 (torch.matmul float64)",
                        "algorithmic_flops": flops},
           "clocks": clk.summary()}
    if not args.no_cpu_baseline:
        from oracle import oracle as O
        O.lib()
        O.set_threads(O.max_threads())
        cl = O.Cluster(xyz=xyz, radius=rad, eps=complex(w["index"]) ** 2, nmax=w["nmax"],
                       wavelength=w["lam"], bg_eps=complex(w["host"]) ** 2)
        po = O.Problem(cl)
        xs, xi = pr.coefficients()
        sample = pts[:: max(1, len(pts) // 2048)]
        s0 = time.perf_counter()
        po.near_field(xs, xi, sample)
        dt = time.perf_counter() - s0
        res["cpu_baseline"] = {"value": len(sample) / dt, "unit": "points/s", "cores": O.max_threads(),
                               "kind": "port", "sample": f"oracle eh_fields on {len(sample)} of the grid points"}
        O.set_threads(1)
    pr.close()
    ctx.close()
    return res


def aca_arm(args):
    """ACA-compressed FP64 form (the reference's ACA + Gmres_Zcomp role:
    eps 1e-3, GMRES tol 1e-6, 240 iterations, 2 restarts) on the c2 cluster
    and on a 1,000-sphere cluster whose dense matrix would not fit comfortably."""
    import optimet_gb300 as G
    from optimet_gb300 import build
    build.build()
    ctx = G.Context(0)
    opts = G.options(G.SOLVE_GMRES, tol=1e-6, max_iter=240, restarts=2)
    out = {}
    cases = [("c2", WORKLOADS["c2"]),
             ("n1000", dict(WORKLOADS["c2"], N=1000, edge=6000 * nm, nmax=6, seed=20260406,
                            desc="N=1000 spheres, nMax=6 (96,000 unknowns), 6 um cube, radii U[40,70] nm"))]
    for name, w in cases:
        xyz, rad = cluster(w)
        sp = G.spheres_array(xyz, rad, complex(w["index"]) ** 2, w["nmax"])
        pr = G.Problem(ctx, sp, G.medium(complex(w["host"]) ** 2), G.plane_wave(w["lam"]))
        times = []
        for i in range(args.warmup + args.steps):
            pr.set_wavelength(w["lam"] + 0.25 * nm * i)
            ctx.mark()
            pr.source_vector(copy=False)
            pr.assemble(G.FF, G.ACA)
            t_asm = ctx.mark()
            st = pr.solve(opts)
            xs = pr.cross_sections()
            t_sol = ctx.mark()
            if i >= args.warmup:
                times.append((t_asm, t_sol))
        info = pr.aca_info()
        n = pr.n
        res = {"unknowns": n, "ms_assemble_compress": float(np.mean([t[0] for t in times])),
               "ms_solve": float(np.mean([t[1] for t in times])), "gmres_iterations": st.iterations,
               "store_GB": info["store_bytes"] / 1e9, "dense_c128_GB": 16.0 * n * n / 1e9,
               "compressed_blocks": info["compressed"], "dense_blocks": info["dense"],
               "mean_rank": info["mean_rank"], "max_rank": info["max_rank"], "xsec": list(xs)}
        if name == "c2":
            pr.assemble(G.FF, G.C128)
            pr.solve(G.options(G.SOLVE_GMRES, tol=1e-10, max_iter=400, restarts=6))
            ref = pr.cross_sections()
            res["qext_rel_err_vs_dense_fp64"] = abs(xs[0] - ref[0]) / abs(ref[0])
        res["wavelength_solves_per_s"] = 1e3 / (res["ms_assemble_compress"] + res["ms_solve"])
        out[name] = res
        pr.close()
    ctx.close()
    return {"metric": "ACA-compressed wavelength-solves/s (FP64)", "value": out["c2"]["wavelength_solves_per_s"],
            "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 / out["c2"]["wavelength_solves_per_s"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128 (FP64), ACA eps 1e-3",
            "data": "synthetic (seeded)", "config": {"workload": "aca: c2 and a 1,000-sphere cluster"},
            "cases": out}


C0 = dict(xyz=np.array([[0.0, 0.0, -125 * nm], [0.0, 0.0, 125 * nm]]), radius=100 * nm, index=3.5 + 0.01j,
          host=1.0, nmax=6, lam=600 * nm,
          desc="two spheres a = 100 nm, n = 3.5+0.01i, centres 250 nm apart on z, vacuum, x-polarised "
               "plane wave along +z at 600 nm, nMax = 6 (192 unknowns), direct LU")


def pct(v, q):
    return float(np.percentile(np.asarray(v) * 1e3, q))


def c0_cpu(repeats):
    """C0 in full on the host, `repeats` times each: the serial reference
    algorithm on one thread (map-cached recurrences, column-pivoted QR, as
    PreconditionedMatrixSolver.h:45-79) and the LU on all host threads."""
    from oracle import oracle as O
    O.lib()
    cl = O.Cluster(xyz=C0["xyz"], radius=C0["radius"], eps=C0["index"] ** 2, nmax=C0["nmax"],
                   wavelength=C0["lam"])
    out = {}
    for name, method, threads in (("serial_qr_1core", "qr", 1), ("lu_all_cores", "lu", O.max_threads())):
        O.set_threads(threads)
        pr = O.Problem(cl)
        pr.wavelength_solve(method)
        lat = []
        for _ in range(repeats):
            t0 = time.perf_counter()
            xs = pr.wavelength_solve(method)[0]
            lat.append(time.perf_counter() - t0)
        out[name] = {"cores": threads, "repeats": repeats, "solves_per_s": repeats / float(np.sum(lat)),
                     "p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99), "xsec": list(xs)}
    O.set_threads(1)
    return out


def c0_arm(args):
    """C0 (the reference's CPU-runnable case) end to end: om_wavelength_solve
    from host buffers (set-up, source, assembly, LU, cross sections) repeated
    1,000 times on the GPU, p50 / p99 latency, beside the host's serial
    reference algorithm and all-core LU over as many repeats."""
    import optimet_gb300 as G
    from optimet_gb300 import build
    build.build()
    repeats = 1000
    ctx = G.Context(0)
    sp = G.spheres_array(C0["xyz"], C0["radius"], C0["index"] ** 2, C0["nmax"])
    bg, wave = G.medium(1.0), G.plane_wave(C0["lam"])
    opts = G.options(G.SOLVE_LU)
    for _ in range(args.warmup):
        G.wavelength_solve(ctx, sp, bg, wave, opts)
    lat = []
    for _ in range(repeats):
        t0 = time.perf_counter()
        xs = G.wavelength_solve(ctx, sp, bg, wave, opts)[0]
        lat.append(time.perf_counter() - t0)
    ctx.close()
    cpu = c0_cpu(repeats)
    err = float(np.max(np.abs(xs - cpu["lu_all_cores"]["xsec"]) / np.abs(cpu["lu_all_cores"]["xsec"])))
    t = float(np.sum(lat))
    return {"metric": "C0 wavelength-solves/s (FP64, LU, host buffers) and p50/p99 latency",
            "value": repeats / t, "unit": UNIT, "n_gpus": 1, "steps": repeats, "warmup": args.warmup,
            "ms_per_step": 1e3 * t / repeats, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128 (FP64)", "data": "synthetic (the C0 geometry)",
            "config": {"workload": "c0: " + C0["desc"]},
            "latency_ms": {"p50": pct(lat, 50), "p99": pct(lat, 99)},
            "xsec_max_rel_err_vs_cpu_lu": err, "cpu": cpu}


def c1_cpu_full():
    """C1 in full on all host threads: source vector, all N(N-1) blocks, GMRES
    to 1e-10 with the dense matvec, internal coefficients and cross sections;
    beside the extrapolation model's prediction for the same solve."""
    from oracle import oracle as O
    O.lib()
    w = WORKLOADS["c1"]
    xyz, rad = cluster(w)
    threads = O.max_threads()
    O.set_threads(threads)
    cl = O.Cluster(xyz=xyz, radius=rad, eps=complex(w["index"]) ** 2, nmax=w["nmax"],
                   wavelength=w["lam"], bg_eps=complex(w["host"]) ** 2)
    pr = O.Problem(cl)
    t0 = time.perf_counter()
    xs, _, _, it = pr.wavelength_solve("gmres", tol=1e-10, maxit=400, restarts=6)
    measured = time.perf_counter() - t0
    O.set_threads(1)
    pred = cpu_baseline(w, xyz, rad, it, threads=threads, budget_s=6.0)["seconds_per_solve"]
    return {"metric": "C1 wavelength-solve on the host (oracle port, FP64 GMRES to 1e-10)",
            "value": 1.0 / measured, "unit": UNIT, "seconds": measured, "cores": threads,
            "gmres_iterations": it, "xsec": list(xs), "model_predicted_s": pred,
            "model_error": pred / measured - 1.0, "config": {"workload": "c1: " + w["desc"]},
            "impl": "reference", "kind": "port"}


def assemble_arm(args, w):
    """Precision-form assemblies only (profiling): warm-up then `steps` timed
    om_assemble(FF, C64) calls of the workload's cluster, CUDA-event timers."""
    import optimet_gb300 as G
    from optimet_gb300 import build
    build.build()
    ctx = G.Context(0)
    xyz, rad = cluster(w)
    sp = G.spheres_array(xyz, rad, complex(w["index"]) ** 2, w["nmax"])
    pr = G.Problem(ctx, sp, G.medium(complex(w["host"]) ** 2), G.plane_wave(w["lam"]))
    for _ in range(args.warmup):
        pr.assemble(G.FF, G.C64)
    ctx.timers(True)
    for _ in range(args.steps):
        pr.assemble(G.FF, G.C64)
    ms, launches = ctx.timers(False)["assemble"]
    n = pr.n
    pr.close()
    ctx.close()
    per = ms / max(launches, 1)
    return {"workload": w["desc"], "unknowns": n, "ms_per_assembly": per, "launches": launches,
            "written_GB": 8.0 * n * n / 1e9, "written_GBps": 8.0 * n * n / 1e6 / per}


def spawn_ranks(n):
    """`bench.py --gpus N` without a launcher: start N copies of this command,
    one per GPU, with RANK / LOCAL_RANK / WORLD_SIZE and a local rendezvous
    (what `torch.distributed.run --nproc-per-node N` sets); rank 0 prints the
    line. Returns the largest exit code."""
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    procs = []
    for r in range(n):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(n), LOCAL_WORLD_SIZE=str(n),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, os.path.abspath(__file__)] + sys.argv[1:], env=env))
    return max(p.wait() for p in procs)


def dry_arm(args):
    """The multi-rank plumbing without GPU work (gloo): rank r reports r + 1
    units in 0.5 (r + 1) seconds; the line aggregates them as the real arms do
    (summed units over the slowest rank's time)."""
    import torch.distributed as dist
    rank, world, _ = dist_env()
    if world > 1:
        dist.init_process_group("gloo")
    units, seconds = rank + 1, 0.5 * (rank + 1)
    t = max_over_ranks([seconds], world)[0]
    value = replica_value(units, seconds, world)
    if world > 1:
        dist.destroy_process_group()
    if rank != 0:
        return None
    return {"metric": "dry run (no GPU work)", "value": value, "unit": "units/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "none", "data": "none",
            "config": {"workload": "dry"}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--slots", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c2",
                    choices=sorted(WORKLOADS) + ["c0", "c1f", "c1full", "c2lu", "c3", "c4", "aca", "tcupd"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--assemble-only", action="store_true",
                    help="only timed precision-form assemblies of the workload (profiling runs)")
    ap.add_argument("--single-stream", action="store_true",
                    help="only the single-stream measurement of both forms (profiling runs)")
    ap.add_argument("--c3-clusters", type=int, default=64)
    ap.add_argument("--c3-wavelengths", type=int, default=16)
    ap.add_argument("--c3-inner-tol", type=float, default=1e-3,
                    help="c3: relative tolerance of each refinement cycle's FP32 Arnoldi (precision form)")
    ap.add_argument("--c4-rate", type=float, default=200.0)
    ap.add_argument("--c4-seconds", type=float, default=60.0)
    ap.add_argument("--batch-slots", type=int, default=6, help="server slots for c3 / c4")
    ap.add_argument("--c4-forms", default="mixed,fp64", help="c4: forms to run (comma-separated)")
    ap.add_argument("--lu-update", type=int, default=3, choices=[0, 1, 2, 3],
                    help="c2lu: trailing-update kernel (1 persistent, 2 one CTA per tile, 3 persistent for "
                         "rank 256 and one CTA per tile for rank 32, 0 FP32 CUDA cores)")
    ap.add_argument("--lu-case", default="c2", choices=sorted(WORKLOADS),
                    help="c2lu: the cluster of the LU role's solve (c2 by default)")
    ap.add_argument("--tc-m", type=int, default=8192, help="tcupd: rows and columns of C")
    ap.add_argument("--tc-k", type=int, default=128, help="tcupd: rank of the update")
    ap.add_argument("--lu-persistent", type=int, default=1, choices=[1, 2],
                    help="c2lu: panels and triangular sweeps (1 one launch each, 2 per column / per block)")
    ap.add_argument("--c4-batch-limit-gb", type=float, default=1.0,
                    help="c4: largest batched footprint of a request that is batched")
    ap.add_argument("--c4-batching", type=int, default=64,
                    help="c4: requests per batched run of a slot (<= 1: one request at a time)")
    ap.add_argument("--no-server", action="store_true", help="c3: skip the server comparison")
    ap.add_argument("--c3-profile", action="store_true",
                    help="c3: only the small batched case that the ncu captures use")
    ap.add_argument("--dry", action="store_true", help="multi-rank plumbing only (gloo, no GPU work)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(spawn_ranks(args.gpus))
    if args.dry:
        out = dry_arm(args)
        if out is not None:
            print(json.dumps(out))
        return
    if args.workload == "c0":
        out = c0_arm(args) if args.impl != "reference" else {"impl": "reference", **c0_cpu(1000)}
    elif args.workload == "c1full":
        out = c1_cpu_full()
    elif args.workload == "aca":
        out = aca_arm(args) if args.impl != "reference" else None
    elif args.workload == "c1f":
        out = near_field_arm(args) if args.impl != "reference" else None
    elif args.workload == "tcupd":
        out = tc_update_arm(args) if args.impl != "reference" else None
    elif args.workload == "c2lu":
        out = lu_mixed_arm(args) if args.impl != "reference" else None
    elif args.workload == "c3":
        out = batch_arm(args) if args.impl != "reference" else None
    elif args.workload == "c4":
        out = serve_arm(args) if args.impl != "reference" else None
    elif args.assemble_only:
        out = assemble_arm(args, WORKLOADS[args.workload]) if args.impl != "reference" else None
    else:
        w = WORKLOADS[args.workload]
        out = reference_arm(args, w) if args.impl == "reference" else gpu_arm(args, w)
    if out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
