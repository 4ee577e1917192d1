"""Benchmark: IMEX-DG DoF-steps/s of the flow-over-hill dynamical core on GB300.

A "step" is one full 3-stage IMEX step (Picard loops, Schur GMRES solves,
stage combination, sponge) of one member, run by the library's time loop.
Default workload: 320x160 cells, Q4 (25 nodes/cell, 5.12 M DoFs), FP64,
acoustic CFL 5, solver eps 1e-8 (the reference parameter file).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                  [--nx 320 --nz 160 --degree 4]

One JSON line on stdout (rank 0).  ``--impl reference`` times the CPU FP64
restatement of the reference algorithm (the oracle; the deal.II reference
cannot be built here) on the host cores for the same workload and metric.
Under torchrun (N > 1) every rank runs its own independent member
(replicas; no collective on the data path) and the timing is the max over
ranks.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "IMEX-DG DoF-steps/s"
UNIT = "DoF-steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--nx", type=int, default=320)
    ap.add_argument("--nz", type=int, default=160)
    ap.add_argument("--degree", type=int, default=4)
    ap.add_argument("--cfl", type=float, default=5.0)
    ap.add_argument("--eps", type=float, default=1e-8)
    ap.add_argument("--precision", default="fp64", choices=["fp64"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--fma-probe", action="store_true",
                    help="print the measured FP64/FP32 FMA peaks and exit")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def workload(args):
    return {"workload": f"flow-over-hill {args.nx}x{args.nz} Q{args.degree} "
                        f"{'FP64' if args.precision == 'fp64' else args.precision}, "
                        f"acoustic CFL {args.cfl:g}, eps {args.eps:g}",
            "nx": args.nx, "nz": args.nz, "degree": args.degree,
            "dofs": 4 * args.nx * args.nz * (args.degree + 1) ** 2,
            "l2_policy": "working set (state, stage vectors, geometry, cell inverses) "
                         "is larger than the 129 MB L2; no flush between steps",
            "parallelism": "one member per GPU (replicas)"}


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_bench_{os.getpid()}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


# FP64 FMA throughput of this machine's GB300 (1255 GFLOP/s measured with an
# independent-chain DFMA probe; profiles/fp64_fp32_fma_peak.md)
FP64_PEAK_TFLOPS = 1.255


def cpu_baseline(case, eps):
    """FP64 CPU restatement (oracle) on all host cores: one IMEX step."""
    from oracle.oracle import OracleSolver, num_threads

    s = OracleSolver(case, eps=eps, inner_tol=1e-12)
    t0 = time.perf_counter()
    s.run(1)
    dt = time.perf_counter() - t0
    return {"value": case.n_dofs / dt, "unit": UNIT, "cores": num_threads(), "kind": "port",
            "sample": f"1 IMEX step of the same {case.params.nx}x{case.params.nz} "
                      f"Q{case.degree} member ({dt:.2f} s), CPU FP64 restatement of the "
                      f"reference algorithm (nested CG A^-1 in the Schur apply)"}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from atmospheric_flows_gb300.hill import HillParams, build_case
    from oracle.oracle import OracleSolver, num_threads

    case = build_case(HillParams(nx=args.nx, nz=args.nz, degree=args.degree, cfl=args.cfl))
    s = OracleSolver(case, eps=args.eps, inner_tol=1e-12)
    for _ in range(args.warmup):
        s.run(1)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        s.run(1)
    el = time.perf_counter() - t0
    v = case.n_dofs * args.steps / el
    cores = num_threads()
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload(args),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{args.steps} IMEX steps of the workload after "
                                       f"{args.warmup} warm-up steps, CPU FP64 restatement "
                                       "of the reference (deal.II is not installable here)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_gb300(args):
    import torch

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    from atmospheric_flows_gb300 import _lib
    from atmospheric_flows_gb300.euler_solver import EulerSolver
    from atmospheric_flows_gb300.hill import HillParams, build_case

    L = _lib.load()
    case = build_case(HillParams(nx=args.nx, nz=args.nz, degree=args.degree, cfl=args.cfl))
    solver = EulerSolver(case, eps=args.eps, precision=0)
    h = solver.op.handle

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
            torch.cuda.synchronize()

    for _ in range(args.warmup):
        solver.run(1)
    barrier()
    # ------------------------------------------------ device-resident timing
    nfam = len(_lib.KERNEL_FAMILIES)
    _lib.check(L.atm_timing_read(h, None, None, None, None, 0), "timing reset")
    _lib.call("atm_timing_enable", h, 1)
    launches0 = L.atm_kernel_launches()
    with ClockSampler(local) as clk:
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        barrier()
        ev0.record()
        solver.run(args.steps)
        ev1.record()
        barrier()
    launches = L.atm_kernel_launches() - launches0
    ms = (ctypes.c_double * nfam)()
    cnt = (ctypes.c_long * nfam)()
    byt = (ctypes.c_double * nfam)()
    flp = (ctypes.c_double * nfam)()
    _lib.call("atm_timing_read", h, ms, cnt, byt, flp, nfam)
    _lib.call("atm_timing_enable", h, 0)
    el_ms = ev0.elapsed_time(ev1)
    if ws > 1:
        t = torch.tensor([el_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        el_ms = float(t.item())
    value = ws * case.n_dofs * args.steps / (el_ms * 1e-3)
    stats = solver.stats()
    # -------------------------------------------- end-to-end through the ABI
    ns = solver.n_scalar
    host = {k: torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
            for k, n in (("rho", ns), ("u", 2 * ns), ("p", ns))}
    r0, u0, p0 = solver.get_state()
    host["rho"][:] = r0
    host["u"][:] = u0
    host["p"][:] = p0
    dp = ctypes.POINTER(ctypes.c_double)
    ptrs = [host[k].ctypes.data_as(dp) for k in ("rho", "u", "p")]
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        _lib.call("atm_solver_set_state", h, *ptrs)
        _lib.call("atm_solver_run", h, 1)
        _lib.call("atm_solver_get_state", h, *ptrs)
    barrier()
    e2e_s = time.perf_counter() - t0
    if ws > 1:
        t = torch.tensor([e2e_s], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e = {"value": ws * case.n_dofs * args.steps / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": int(8 * 4 * ns), "d2h_bytes_per_step": int(8 * 4 * ns)}
    if rank != 0:
        if ws > 1:
            torch.distributed.destroy_process_group()
        return 0
    # ----------------------------------------------------------- roofline
    fams = _lib.KERNEL_FAMILIES
    dom = max(range(nfam), key=lambda i: ms[i])
    avg_ms = ms[dom] / max(cnt[dom], 1)
    gbs = byt[dom] / max(cnt[dom], 1) / (avg_ms * 1e-3) / 1e9
    tflops = flp[dom] / max(cnt[dom], 1) / (avg_ms * 1e-3) / 1e12
    peak, peak_kind = measured_peaks()
    traffic = os.environ.get("ATM_NCU_TRAFFIC_BYTES")
    roofline = {"bound": "hbm", "kernel": f"{fams[dom]}", "achieved": gbs, "peak": peak,
                "unit": "GB/s", "frac": gbs / peak, "peak_source": peak_kind,
                "traffic": float(traffic) if traffic else None,
                "algorithmic_bytes_per_launch": byt[dom] / max(cnt[dom], 1),
                "avg_launch_ms": avg_ms, "launches": int(cnt[dom]),
                "fp64": {"achieved_tflops": tflops, "peak_tflops": FP64_PEAK_TFLOPS,
                         "frac": tflops / FP64_PEAK_TFLOPS,
                         "note": "FP64 FMA pipe is the binding limit on GB300"},
                "families": {fams[i]: {"ms": ms[i], "launches": int(cnt[i]),
                                       "share": ms[i] / max(sum(ms), 1e-30)}
                             for i in range(nfam) if cnt[i]}}
    cpu = None
    if not args.no_cpu_baseline:
        try:
            cpu = cpu_baseline(case, args.eps)
        except Exception as exc:  # the baseline must not kill the GPU line
            cpu = {"value": None, "unit": UNIT, "cores": None, "kind": "port",
                   "sample": f"failed: {exc}"}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": el_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload(args), "e2e": e2e, "gpu_launches": int(launches),
            "roofline": roofline, "cpu_baseline": cpu, "clocks": clk.summary(),
            "solver": {"picard_per_step": stats["picard_total"] / max(stats["steps"], 1),
                       "krylov_per_step": stats["krylov_total"] / max(stats["steps"], 1),
                       "solve_fail": stats["solve_fail"]}}
    print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def fma_probe():
    import torch

    from atmospheric_flows_gb300 import _lib

    torch.cuda.set_device(0)
    f64, f32 = ctypes.c_double(), ctypes.c_double()
    _lib.call("atm_probe_fma_peak", ctypes.byref(f64), ctypes.byref(f32))
    print(json.dumps({"fp64_fma_gflops": f64.value, "fp32_fma_gflops": f32.value,
                      "ratio": f32.value / f64.value}), flush=True)
    return 0


def main():
    args = parse()
    if args.fma_probe:
        return fma_probe()
    if args.impl == "reference":
        return run_reference(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
