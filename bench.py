#!/usr/bin/env python
"""Benchmark: 10M-cell steady-state solve time to IMS closure on one GB300.

Workload (1000x1000x10 DIS, 7-point, 10,000,000 cells, 67,960,000 nonzeros):
per-layer lognormal Kh (ln K ~ N(0, 1.5^2), 20-cell correlation), Kv = 0.1 Kh,
CHD 20 m / 0 m on the west / east faces, 5,000 wells U(-500, -50) m3/d,
seeded synthetic data.  PCG + ILU0, INNER_DVCLOSE 1e-4 m, INNER_RCLOSE 1e-5
m3/d, OUTER_DVCLOSE 1e-4 m.

A step is one steady-state time step from the initial heads to closure: the
NumericalSolution outer loop (fill, sln_ls fix-ups, IMS solve, dxmax) until
OUTER_DVCLOSE holds.  `value` is the device-resident plain FP64 drop-in
(inputs in HBM); `mixed_s` the FP32-matrix/FP64-refinement form; `e2e` the
same FP64 step driven through the C ABI with host buffers (gbims_apply:
amat, rhs and x copied host->device, x copied back, every outer iteration).

--impl reference times the CPU restatement of the reference's IMS (the
oracle; MODFLOW 6 itself is Fortran and no Fortran compiler exists on either
machine) on a bounded sample of the same workload, on the host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "10M-cell solve time to IMS closure: FP64 vs mixed vs warm-start; SpMV HBM GB/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb", choices=["gb", "reference"])
    ap.add_argument("--scale", type=float, default=1.0, help="grid scale (1.0 = 1000x1000x10)")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-ensemble", action="store_true")
    ap.add_argument("--no-warmstart", action="store_true")
    ap.add_argument("--no-c3", action="store_true", help="skip the C1 and C3 forms")
    ap.add_argument("--no-grids", action="store_true", help="skip the DISV, DISU and XT3D form")
    ap.add_argument("--grids", action="store_true",
                    help="only the DISV, DISU and XT3D steady steps (one JSON line)")
    ap.add_argument("--grid-cases", default="disv,disu,xt3d",
                    help="which of the general-grid workloads to run")
    ap.add_argument("--no-tune", action="store_true",
                    help="keep the library's default sweep tiling and reduction grid")
    ap.add_argument("--kernels", action="store_true",
                    help="per-kernel device times on direct launches (no solve)")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    lrank = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, lrank


def max_over_ranks(v: float, ws: int) -> float:
    """The slowest rank's time: every rank times its own replica of the step;
    the job's time is the maximum (NCCL on GPUs, gloo on CPU)."""
    if ws <= 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], device=dev, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload_config(a, m):
    from modflow6_gb300.workloads import C2_IMS, C2_OUTER
    return {"workload": f"DIS {m.nlay}x{m.nrow}x{m.ncol} confined steady state (10M-cell case)"
            if a.scale == 1.0 else f"DIS {m.nlay}x{m.nrow}x{m.ncol} (scaled {a.scale})",
            "cells": m.nodes, "nonzeros": int(m.nodes + 2 * (m.nlay * m.nrow * (m.ncol - 1)
                                                            + m.nlay * (m.nrow - 1) * m.ncol
                                                            + (m.nlay - 1) * m.nrow * m.ncol)),
            "accelerator": "PCG", "preconditioner": "ILU0", "inner_dvclose": C2_IMS["dvclose"],
            "inner_rclose": C2_IMS["rclose"], "outer_dvclose": C2_OUTER["dvclose"],
            "wells": int(m.wel_node.size), "seed": a.seed,
            "l2_flush": "inputs larger than L2 (amat alone 544 MB vs 129 MB L2)"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.p = None
        self.lines = []

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.p = None
        return self

    def _read(self):
        for line in self.p.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic():
    p = ROOT / "profiles" / "traffic.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except Exception:
            return {}
    return {}


# ---------------------------------------------------------------------------
# CPU restatement (oracle): bounded sample, scaled to a solve to closure
# ---------------------------------------------------------------------------
def cpu_sample(m, inner_total: int, outer: int, budget_s: float = 25.0) -> dict:
    """Times the oracle's IMS (PCG + ILU0, 1 core) on the same system: setup
    (ILU0 factor + initial residual) and a few inner iterations, then scales
    to outer * setup + inner_total * per-iteration."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    from modflow6_gb300.workloads import C2_IMS

    t0 = time.perf_counter()
    g = oracle.Gwf(m, oracle.settings(**C2_IMS))
    x0 = g.x.copy()
    x0[m.chd_node] = m.chd_head
    amat, rhs = g.assemble(x0)
    t_fill = time.perf_counter() - t0
    amat, rhs = g.fixups(amat, rhs, x0, isymmetric=True)

    def run(iters):
        s = dict(C2_IMS)
        s["iter1"] = iters
        s["dvclose"] = 0.0
        s["rclose"] = 1e-300
        ims = oracle.Ims(oracle.settings(**s), g.con["ia"], g.con["ja"])
        x = x0.copy()
        t = time.perf_counter()
        ims.apply(amat.copy(), rhs.copy(), x)
        return time.perf_counter() - t

    k1 = 2
    t1 = run(k1)
    per_guess = max(t1 / (k1 + 2), 1e-6)
    k2 = k1 + max(3, min(40, int((budget_s - t1) / per_guess / 2)))
    t2 = run(k2)
    t_iter = max((t2 - t1) / (k2 - k1), 1e-9)
    t_setup = max(t1 - k1 * t_iter, 0.0)
    est = outer * (t_fill + t_setup) + inner_total * t_iter
    return {"value": est, "unit": "s", "cores": 1, "kind": "port",
            "sample": (f"oracle C restatement of IMS (gcc -O2, 1 thread) on the same system: "
                       f"fill {t_fill:.2f}s, ILU0 factor + residual {t_setup:.2f}s, "
                       f"{t_iter:.3f}s per PCG iteration from {k1}- and {k2}-iteration runs; "
                       f"scaled to {outer} outer x (fill + setup) + {inner_total} inner iterations"),
            "t_iter_s": t_iter, "t_setup_s": t_setup, "t_fill_s": t_fill}


def reference_arm(a):
    """The oracle (the C restatement of the reference's IMS, one core) on the
    same steady-state step: one full time step from the initial heads to
    closure -- fill, sln_ls fix-ups, PCG + ILU0 to the inner closure, outer
    loop to OUTER_DVCLOSE -- measured once, wall clock.  That single measured
    solve is the line's value.  The warm-up and the further steps repeat only
    the bounded per-iteration sample (setup and a few PCG iterations), whose
    linear model is reported beside it as a cross-check."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    from modflow6_gb300.dis import make_config
    from modflow6_gb300.workloads import C2_IMS, C2_OUTER
    ws, rank, _ = dist_env()
    if ws > 1 and rank != 0:
        return
    m = make_config("c2", seed=a.seed, scale=a.scale)
    t0 = time.perf_counter()
    g = oracle.Gwf(m, oracle.settings(**C2_IMS))
    t_setup = time.perf_counter() - t0
    t0 = time.perf_counter()
    st = g.timestep(kper=1, kstp=1, delt=1.0, transient=False, **C2_OUTER)
    t_full = time.perf_counter() - t0
    samples = []
    for _ in range(max(1, a.warmup + a.steps - 1)):
        samples.append(cpu_sample(m, st["inner_total"], st["outer"],
                                  budget_s=max(3.0, 30.0 / max(1, a.warmup + a.steps))))
    cb = {"value": t_full, "unit": "s", "cores": 1, "kind": "port",
          "sample": (f"measured: one full steady step of the oracle (C restatement of IMS, "
                     f"gcc -O2, 1 thread): {st['outer']} outer / {st['inner_total']} inner "
                     f"iterations in {t_full:.1f} s (model setup {t_setup:.1f} s not counted)"),
          "measured_steps": 1, "converged": int(st["converged"]),
          "outer_iterations": int(st["outer"]), "inner_iterations": int(st["inner_total"]),
          "sampled_model_s": float(np.median([c["value"] for c in samples])),
          "sampled_s_per_iteration": float(np.median([c["t_iter_s"] for c in samples]))}
    line = {"metric": METRIC, "value": t_full, "unit": "s", "impl": "reference",
            "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup, "ms_per_step": t_full * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "cpu_baseline": cb,
            "e2e": {"value": t_full, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "config": workload_config(a, m)}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GB300 arm
# ---------------------------------------------------------------------------
def gb_arm(a):
    import torch

    ws, rank, lrank = dist_env()
    torch.cuda.set_device(lrank)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from modflow6_gb300 import _lib, build
    build.build()
    from modflow6_gb300.dis import make_config
    from modflow6_gb300.ims import ImsLinear, ImsLinearSettings
    from modflow6_gb300.solution import GwfSolution, Nonlinear, sln_ls_fixups
    from modflow6_gb300.workloads import C2_IMS, C2_OUTER
    import ctypes as C

    lib = _lib.load()
    m = make_config("c2", seed=a.seed, scale=a.scale)
    shape = (m.nlay, m.nrow, m.ncol)
    nl = Nonlinear(dvclose=C2_OUTER["dvclose"], mxiter=C2_OUTER["mxiter"])

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()

    def maxr(v):
        return max_over_ranks(v, ws)

    def run_form(precision, clocks=False):
        sol = GwfSolution(m, ImsLinearSettings(precision=precision, structure=shape, **C2_IMS), nl)
        stats = []
        tuning = None
        for i in range(a.warmup):
            sol.restart()
            st = sol.timestep(1, 1, 1.0)
            assert st["converged"] == 1, st
            if i == 0 and not a.no_tune:
                # the autotuner picks the sweep tiling and reduction grid on
                # the factored system; the later warm-up steps re-capture
                # the inner-loop graph with them
                tuning = autotune(lib, sol.ims_handle())
        ims_h = sol.ims_handle()
        l0 = lib.gbims_kernel_launches(ims_h)
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        sampler = ClockSampler(lrank) if clocks else None
        if sampler:
            sampler.__enter__()
        e0.record()
        for _ in range(a.steps):
            sol.restart()
            stats.append(sol.timestep(1, 1, 1.0))
        e1.record()
        barrier()
        if sampler:
            sampler.__exit__(None, None, None)
        ms = e0.elapsed_time(e1) / max(1, a.steps)
        launches = lib.gbims_kernel_launches(ims_h) - l0
        # per-step kernels outside the IMS handle: memsets excluded; npf_cf, fill,
        # fix-ups, dxmax per outer iteration, CHD reset per step
        launches += sum(4 * s["outer"] + 1 for s in stats)
        heads = sol.heads
        return sol, ms, stats, launches, sampler.summary() if sampler else None, heads, tuning

    sol64, ms64, st64, launches64, clocks, h64, tune64 = run_form(_lib.GBIMS_FP64, clocks=True)
    ms64 = maxr(ms64)
    # per-kernel device times (CUDA events on the library stream) for the roofline
    kt = _lib.GbimsKernelTimes()
    rc = lib.gbims_time_kernels(sol64.ims_handle(), 20, C.byref(kt))
    assert rc == 0, rc
    peak, peak_kind = measured_peaks()
    spmv_gbs = kt.spmv_bytes / (kt.spmv_ms * 1e-3) / 1e9
    pre_gbs = kt.precond_bytes / (kt.precond_ms * 1e-3) / 1e9
    traffic = ncu_traffic()
    pre_name = ("k_dia7_sweep<double> forward + backward (structured wavefront ILU0; "
                "the forward sweep reads r and the backward sweep writes z in natural order)")
    mixed = None
    if not a.no_mixed:
        solm, msm, stm, lm, _, hm, tunem = run_form(_lib.GBIMS_MIXED)
        msm = maxr(msm)
        ktm = _lib.GbimsKernelTimes()
        lib.gbims_time_kernels(solm.ims_handle(), 20, C.byref(ktm))
        mixed = {"value": msm / 1e3, "unit": "s", "inner_iterations": stm[-1]["inner_total"],
                 "outer_iterations": stm[-1]["outer"],
                 "max_head_diff_vs_fp64": float(np.max(np.abs(hm - h64))),
                 "heads_within_0.1_inner_dvclose": bool(np.max(np.abs(hm - h64))
                                                        <= 0.1 * C2_IMS["dvclose"]),
                 "spmv_fp32_gbs": ktm.spmv_bytes / (ktm.spmv_ms * 1e-3) / 1e9,
                 "precond_fp32_ms": ktm.precond_ms, "spmv_fp32_ms": ktm.spmv_ms,
                 "tuning": tunem}
        solm.close()
    # e2e: the same FP64 step driven by a host through the C ABI with host
    # buffers, as MODFLOW 6 drives imslinear_apply: every outer iteration the
    # heads go to the device, the conductance fill runs there and AMAT/RHS
    # come back to pinned host arrays (gbsln_formulate), the host applies the
    # sln_ls loose ends, and gbims_apply copies AMAT, RHS and X in and X out
    e2e = None
    if not a.no_e2e:
        from modflow6_gb300.solution import LsFixups
        con = m.connections()
        ia, ja = con["ia"], con["ja"]
        fx = LsFixups(ia, ja, m.ibound, isymmetric=True)
        pin = lambda arr: torch.from_numpy(arr).pin_memory()
        t_amat, t_rhs = pin(np.zeros(ja.size)), pin(np.zeros(m.nodes))
        t_x = pin(m.strt.copy())
        amat_h, rhs_h, xv = t_amat.numpy(), t_rhs.numpy(), t_x.numpy()
        ims = ImsLinear(ImsLinearSettings(structure=shape, **C2_IMS)).imslinear_allocate(m.nodes, ia, ja)
        active = m.ibound > 0
        amat_p = C.cast(t_amat.data_ptr(), C.POINTER(C.c_double))
        rhs_p = C.cast(t_rhs.data_ptr(), C.POINTER(C.c_double))
        x_p = C.cast(t_x.data_ptr(), C.POINTER(C.c_double))
        x0 = m.strt.copy()
        x0[m.chd_node] = m.chd_head

        def e2e_step():
            xv[:] = x0
            outer = 0
            for kiter in range(1, nl.mxiter + 1):
                xtemp = xv.copy()
                rc = lib.gbsln_set_heads(sol64._h, x_p)
                assert rc >= 0, rc
                rc = lib.gbsln_formulate(sol64._h, 0.0, None, amat_p, rhs_p)
                assert rc >= 0, rc
                fx.apply(amat_h, rhs_h, xv)
                ic, it = C.c_int(), C.c_int()
                rc = lib.gbims_apply(ims._h, amat_p, rhs_p, x_p, 1, kiter, C.byref(ic), C.byref(it), None)
                assert rc >= 0, lib.gbims_last_error(ims._h)
                outer = kiter
                if np.max(np.abs((xv - xtemp)[active])) <= nl.dvclose:
                    break
            return outer

        for _ in range(min(a.warmup, 1)):
            e2e_step()
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        outers = [e2e_step() for _ in range(a.steps)]
        e1.record()
        barrier()
        ms_e2e = maxr(e0.elapsed_time(e1) / max(1, a.steps))
        no = float(np.mean(outers))
        nb = amat_h.nbytes + 2 * rhs_h.nbytes
        e2e = {"value": ms_e2e / 1e3, "unit": "s",
               "h2d_bytes_per_step": int(no * (nb + xv.nbytes)),
               "d2h_bytes_per_step": int(no * nb),
               "path": "per outer iteration: heads to the device, GPU fill, AMAT/RHS to host, "
                       "host sln_ls, gbims_apply (pinned host AMAT/RHS/X)"}
        ims.imslinear_da()
    ens = None if a.no_ensemble else ensemble_form(a, lib, barrier, maxr)
    c3 = None if a.no_c3 else c3_form(a, barrier)
    c1 = None if a.no_c3 else c1_form(a, barrier)
    grids = None if a.no_grids else grids_form(a, barrier)
    ws_res = None if a.no_warmstart else warmstart_form(a)
    last = st64[-1]
    cpu = None
    if rank == 0 and not a.no_cpu:
        c = cpu_sample(m, last["inner_total"], last["outer"])
        cpu = {k: c[k] for k in ("value", "unit", "cores", "kind")}
        cpu["sample"] = (f"oracle, 1 thread: setup + a few PCG iterations timed, "
                         f"{c['t_iter_s']:.3f} s/iteration, scaled to {last['outer']} outer / "
                         f"{last['inner_total']} inner iterations")
    roof = {"bound": "hbm", "achieved": pre_gbs, "peak": peak, "unit": "GB/s",
            "frac": pre_gbs / peak, "traffic": traffic.get("precond_fp64_bytes_per_launch"),
            "kernel": "k_dia7_sweep fwd+bwd (FP64 wavefront ILU0)",
            "algorithmic_bytes_per_launch": kt.precond_bytes, "launch_ms": kt.precond_ms,
            "peak_kind": f"{peak_kind} copy bandwidth"}
    # the details (tuning candidates, per-form breakdowns) go to stderr as one
    # line; stdout carries the contract line, with the forms' summary last
    detail = {"tuning_fp64": tune64, "mixed": mixed, "ensemble": ens, "warm_start": ws_res,
              "c3": c3, "c1": c1, "grids": grids,
              "roofline_spmv": {"kernel": "k_dia7_spmv<double>", "achieved": spmv_gbs,
                                "frac": spmv_gbs / peak, "launch_ms": kt.spmv_ms,
                                "traffic": traffic.get("spmv_fp64_bytes_per_launch")},
              "device_ms_per_step": float(np.mean([s["total_ms"] for s in st64])),
              "fill_ms_per_step": float(np.mean([s["fill_ms"] for s in st64]))}
    if rank == 0:
        print("detail: " + json.dumps(detail), file=sys.stderr, flush=True)
    forms = {"fp64_s": ms64 / 1e3, "fp64_inner": last["inner_total"], "fp64_outer": last["outer"]}
    if mixed:
        forms.update(mixed_s=mixed["value"], mixed_vs_fp64=mixed["value"] / (ms64 / 1e3),
                     mixed_inner=mixed["inner_iterations"],
                     mixed_max_head_diff_m=mixed["max_head_diff_vs_fp64"])
    if ens:
        forms.update(ensemble_s=ens["value"], ensemble_members_per_s=ens["members_per_s"])
        if ens.get("mixed"):
            forms.update(ensemble_mixed_s=ens["mixed"]["value"],
                         ensemble_mixed_vs_fp64=ens["mixed"]["vs_fp64"])
    if c1:
        forms.update(c1_fp64_s=c1["fp64"]["value"], c1_inner=c1["fp64"]["inner"])
        if "oracle" in c1:
            forms.update(c1_oracle_s=c1["oracle"]["value"])
    if c3:
        forms.update(c3_fp64_s=c3["fp64"]["value"], c3_outer=c3["fp64"]["outer"])
        if "mixed" in c3:
            forms.update(c3_mixed_s=c3["mixed"]["value"], c3_mixed_vs_fp64=c3["mixed_vs_fp64"],
                         c3_mixed_max_head_diff_m=c3["mixed_max_head_diff_m"])
    if grids:
        for gname, gr in grids.items():
            forms[f"{gname}_s"] = gr["value"]
            if "oracle" in gr:
                forms[f"{gname}_oracle_s"] = gr["oracle"]["value"]
    if ws_res:
        h = ws_res["heldout"]
        forms.update(warmstart_time_ratio=h.get("time_ratio"),
                     warmstart_iteration_ratio=h.get("iteration_ratio"),
                     warmstart_extrap_only_iteration_ratio=h.get("iteration_ratio_extrap"),
                     warmstart_train_models=ws_res["train_models"],
                     warmstart_heldout_models=h.get("models"))
    line = {
        "metric": METRIC, "value": ms64 / 1e3, "unit": "s", "n_gpus": ws, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": ms64, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded lognormal K, CHD, WEL)",
        "config": workload_config(a, m), "gpu_launches": int(launches64), "clocks": clocks,
        "e2e": e2e, "roofline": roof, "spmv_gbs": spmv_gbs,
        "kernels": {"precond_ms": kt.precond_ms, "spmv_ms": kt.spmv_ms, "dot_ms": kt.dot_ms,
                    "update_ms": kt.update_ms},
        "cpu_baseline": cpu, "forms": forms,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def autotune(lib, h, reps=5):
    """gbims_autotune on a factored handle: the chosen wavefront tiling and
    reduction grid, with the time of every tiling tried."""
    import ctypes as C
    from modflow6_gb300 import _lib
    t = _lib.GbimsTuning()
    rc = lib.gbims_autotune(h, reps, C.byref(t))
    assert rc == 0, lib.gbims_last_error(h)
    out = {"reduction_blocks": t.reduction_blocks}
    if t.level_mode >= 0:
        out.update(level_mode=("sync-free" if t.level_mode == 1 else "per-level launches"),
                   level_ms=[round(t.level_ms[0], 4), round(t.level_ms[1], 4)],
                   sync_free_ms_by_threads_per_row=dict(zip(
                       ("1", "2", "4", "8", "16"),
                       (round(t.candidate_ms[i], 4) for i in range(t.ncandidates)))))
    if t.sweep_config >= 0:
        out.update(sweep_config=t.sweep_config, sweep_config_backward=t.sweep_config_backward,
                   sweep_chunk=t.sweep_chunk, sweep_ring=t.sweep_ring,
                   sweep_prefetch=t.sweep_prefetch, sweep_occupancy=t.sweep_occupancy,
                   precond_ms=t.precond_ms,
                   candidates_ms=[round(t.candidate_ms[i], 4) for i in range(t.ncandidates)])
    return out


def ensemble_form(a, lib, barrier, maxr) -> dict:
    """The 256-member batched ensemble (C4): every member assembled on the
    GPU (gbnpf_fill + sln_ls fix-ups), concatenated, and solved to its own
    closure by one batched PCG + ILU0 (gbims_batch_apply_device, the
    wavefront preconditioner over all members).  Inputs stay in HBM; each
    timed step restores x and solves all members.  The same members are then
    solved in the mixed form (FP32 inner loop per member, FP64 refinement)
    unless --no-mixed."""
    import torch
    from modflow6_gb300 import _lib
    from modflow6_gb300.ensemble import (EnsembleLinear, assemble_member, concat_systems,
                                         make_ensemble)
    from modflow6_gb300.ims import ImsLinearSettings
    from modflow6_gb300.workloads import C4_IMS

    count = 256 if a.scale == 1.0 else 16
    members = make_ensemble(count, seed=a.seed, scale=a.scale)
    systems = [assemble_member(m) for m in members]
    mrow, ia, ja, amat, rhs, x0 = concat_systems([s[0] for s in systems], [s[1] for s in systems],
                                                 [s[2] for s in systems], [s[3] for s in systems])
    del systems
    shapes = [(m.nlay, m.nrow, m.ncol) for m in members]
    dev = torch.device("cuda")
    d_amat, d_rhs = torch.from_numpy(amat).to(dev), torch.from_numpy(rhs).to(dev)
    d_x0 = torch.from_numpy(x0).to(dev)
    d_x = d_x0.clone()

    def run(precision):
        ens = EnsembleLinear(ImsLinearSettings(precision=precision, **C4_IMS)).allocate(
            mrow, ia, ja, shapes)
        res = None
        tuning = None
        for i in range(min(a.warmup, 2)):
            d_x.copy_(d_x0)
            res = ens.apply_device(d_amat.data_ptr(), d_rhs.data_ptr(), d_x.data_ptr())
            if i == 0 and not a.no_tune:
                tuning = autotune(lib, ens._h, reps=3)
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        nsteps = max(1, min(a.steps, 3))
        e0.record()
        for _ in range(nsteps):
            d_x.copy_(d_x0)
            res = ens.apply_device(d_amat.data_ptr(), d_rhs.data_ptr(), d_x.data_ptr())
        e1.record()
        barrier()
        ms = maxr(e0.elapsed_time(e1) / nsteps)
        its = np.array([r.in_iter for r in res])
        ens.close()
        return {"value": ms / 1e3, "unit": "s", "members_per_s": count / (ms / 1e3),
                "converged": int(sum(r.icnvg for r in res)),
                "inner_iterations": {"min": int(its.min()), "mean": float(its.mean()),
                                     "max": int(its.max())},
                "refinements_max": int(max(r.summary["refinements"] for r in res)),
                "tuning": tuning}

    out = {"workload": f"{count} DIS members, nrow/ncol U{{50..450}} x scale {a.scale}, "
                       f"nlay U{{1..5}}",
           "members": count, "cells": int(mrow[-1]), "nonzeros": int(ia[-1]),
           "form": "FP64 batched PCG + wavefront ILU0, one CUDA graph for all members"}
    out.update(run(_lib.GBIMS_FP64))
    if not a.no_mixed:
        mixed = run(_lib.GBIMS_MIXED)
        mixed["form"] = ("FP32 matrix, factors and inner loop per member inside FP64 "
                         "refinement, same closure")
        mixed["vs_fp64"] = mixed["value"] / out["value"]
        out["mixed"] = mixed
    return out


def c1_form(a, barrier) -> dict:
    """The 100x100x1 steady confined case (C1, the reference's CPU-runnable
    case): one steady step to closure (INNER_DVCLOSE 1e-8, INNER_RCLOSE 1e-6,
    PCG + ILU0) on the device, FP64 and mixed, CUDA events over 20 solves from
    the initial heads; beside it the oracle's full solve of the same step on
    one core (wall clock, median of 5)."""
    import torch
    from modflow6_gb300 import _lib
    from modflow6_gb300.dis import make_config
    from modflow6_gb300.ims import ImsLinearSettings
    from modflow6_gb300.solution import GwfSolution, Nonlinear
    from modflow6_gb300.workloads import C1_IMS, C1_OUTER

    m = make_config("c1", seed=a.seed)
    nl = Nonlinear(dvclose=C1_OUTER["dvclose"], mxiter=C1_OUTER["mxiter"])
    out = {"workload": f"DIS {m.nlay}x{m.nrow}x{m.ncol} confined steady state", "cells": m.nodes}
    heads = {}
    reps = 20
    for name, prec in (("fp64", _lib.GBIMS_FP64), ("mixed", _lib.GBIMS_MIXED)):
        if name == "mixed" and a.no_mixed:
            continue
        sol = GwfSolution(m, ImsLinearSettings(precision=prec, structure=(m.nlay, m.nrow, m.ncol),
                                               **C1_IMS), nl)
        sol.timestep(1, 1, 1.0)  # warm-up: builds the graphs
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        tot, sts = 0.0, []
        for _ in range(reps):
            sol.restart()
            e0.record()
            sts.append(sol.timestep(1, 1, 1.0))
            e1.record()
            torch.cuda.synchronize()
            tot += e0.elapsed_time(e1)
        heads[name] = sol.heads
        sol.close()
        out[name] = {"value": tot / reps / 1e3, "unit": "s", "outer": int(sts[-1]["outer"]),
                     "inner": int(sts[-1]["inner_total"]),
                     "converged": int(all(st["converged"] == 1 for st in sts))}
    if "mixed" in heads:
        out["mixed_max_head_diff_m"] = float(np.max(np.abs(heads["mixed"] - heads["fp64"])))
    if not a.no_cpu:
        sys.path.insert(0, str(ROOT / "oracle"))
        import oracle
        ts = []
        for _ in range(5):
            g = oracle.Gwf(m, oracle.settings(**C1_IMS))
            t0 = time.perf_counter()
            so = g.timestep(kper=1, kstp=1, delt=1.0, transient=False, **C1_OUTER)
            ts.append(time.perf_counter() - t0)
        out["oracle"] = {"value": float(np.median(ts)), "unit": "s", "cores": 1,
                         "outer": int(so["outer"]), "inner": int(so["inner_total"]),
                         "max_head_diff_vs_gpu_fp64_m": float(np.max(np.abs(g.x - heads["fp64"])))}
    return out


def c3_form(a, barrier) -> dict:
    """The 500x500x5 convertible NEWTON transient workload (C3): its first
    stress period (10 steps, TSMULT 1.2 over 10 d, BiCGSTAB + ILU0, DBD) on
    the device-resident solution, in FP64 and in the mixed form, timed with
    CUDA events from the initial heads to the end of the period; the heads of
    the two forms are compared at the end."""
    import torch
    from modflow6_gb300 import _lib
    from modflow6_gb300.dis import make_config
    from modflow6_gb300.ims import ImsLinearSettings
    from modflow6_gb300.solution import GwfSolution, Nonlinear
    from modflow6_gb300.workloads import C3_IMS, C3_OUTER, C3_PERIOD, step_lengths

    m = make_config("c3", seed=a.seed, scale=a.scale)
    o = dict(C3_OUTER)
    nl = Nonlinear(dvclose=o["dvclose"], mxiter=o["mxiter"], nonmeth=o["nonmeth"],
                   theta=o["theta"], akappa=o["akappa"], gamma=o["gamma"], amomentum=o["amomentum"])
    delts = step_lengths(C3_PERIOD["perlen"], C3_PERIOD["nstp"], C3_PERIOD["tsmult"])
    out = {"workload": f"DIS {m.nlay}x{m.nrow}x{m.ncol} convertible NEWTON, stress period 1 "
                       f"({len(delts)} steps)", "cells": m.nodes}
    heads = {}
    for name, prec in (("fp64", _lib.GBIMS_FP64), ("mixed", _lib.GBIMS_MIXED)):
        if name == "mixed" and a.no_mixed:
            continue
        sol = GwfSolution(m, ImsLinearSettings(precision=prec, structure=(m.nlay, m.nrow, m.ncol),
                                               **C3_IMS), nl)
        sol.timestep(1, 1, delts[0])  # warm-up: builds the graphs
        sol.restart()
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        sts = [sol.timestep(1, k, d) for k, d in enumerate(delts, start=1)]
        e1.record()
        barrier()
        heads[name] = sol.heads
        sol.close()
        out[name] = {"value": e0.elapsed_time(e1) / 1e3, "unit": "s",
                     "outer": int(sum(s["outer"] for s in sts)),
                     "inner": int(sum(s["inner_total"] for s in sts)),
                     "converged": int(all(s["converged"] == 1 for s in sts))}
    if "mixed" in heads:
        out["mixed_vs_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
        out["mixed_max_head_diff_m"] = float(np.max(np.abs(heads["mixed"] - heads["fp64"])))
    rec = ROOT / "tests" / "golden" / "c3_oracle_period1.json"
    if rec.exists() and a.scale == 1.0:
        d = json.loads(rec.read_text())
        out["oracle_recorded_s"] = d["oracle_seconds"]
        out["oracle_recorded_note"] = "oracle, 1 thread, on the x86 build host, same period"
    return out


GRID_IMS = dict(dvclose=1e-8, rclose=1e-6, iter1=4000)
GRID_OUTER = dict(dvclose=1e-8, mxiter=20)


def grids_form(a, barrier) -> dict:
    """The general grids and the full-tensor formulation, one steady step to
    closure each (INNER_DVCLOSE 1e-8, INNER_RCLOSE 1e-6, OUTER_DVCLOSE 1e-8):
    a DISV hexagon grid and a DISU locally refined grid (SELL-32 product,
    sync-free level-scheduled ILU0 sweeps, PCG), and a DIS grid with XT3D
    (the wider pattern, BiCGSTAB).  FP64 on the device-resident solution:
    the time step's own CUDA-event times (fill, solve, total), the median of
    3 steps from the initial heads after a warm-up step and (unless
    --no-tune) gbims_autotune on the factored system (level-sweep form and
    threads per row, reduction grid).  Beside each, the
    oracle's full solve of the same step on one core (wall clock) and the
    largest head difference."""
    from modflow6_gb300 import _lib
    from modflow6_gb300.dis import make_config
    from modflow6_gb300.disu import make_disu_model
    from modflow6_gb300.disv import make_disv_model
    from modflow6_gb300.ims import ImsLinearSettings
    from modflow6_gb300.solution import GwfSolution, Nonlinear

    lib = _lib.load()
    s = a.scale
    nv, nu = max(8, int(round(250 * s))), max(6, int(round(240 * s)))
    cases = (("disv", f"DISV 4x{nv}x{nv} hexagons", lambda: make_disv_model(4, nv, nv, seed=a.seed), 1),
             ("disu", f"DISU 3 layers, {nu}x{nu} cells with the middle ninth refined 2x2",
              lambda: make_disu_model(3, nu, nu, seed=a.seed), 1),
             ("xt3d", None, lambda: make_config("xt3d", seed=a.seed, scale=s), 2))
    out = {}
    want = set(a.grid_cases.split(","))
    for name, desc, build, ilinmeth in cases:
        if name not in want:
            continue
        m = build()
        if desc is None:
            desc = f"DIS {m.nlay}x{m.nrow}x{m.ncol} XT3D, K11:K22:K33 1:0.2:0.05, angles 30/15/5"
        tol = dict(ilinmeth=ilinmeth, **GRID_IMS)
        sol = GwfSolution(m, ImsLinearSettings(**tol), Nonlinear(**GRID_OUTER))
        sol.timestep(1, 1, 1.0)  # warm-up: builds the graphs, factors the matrix
        tuning = None if a.no_tune else autotune(lib, sol.ims_handle())
        barrier()
        sts = []
        for _ in range(3):
            sol.restart()
            sts.append(sol.timestep(1, 1, 1.0))
        heads = sol.heads
        sol.close()
        med = lambda f: float(np.median([st[f] for st in sts]))
        r = {"workload": desc, "cells": int(len(m.k11)), "value": med("total_ms") / 1e3, "unit": "s",
             "fill_ms": med("fill_ms"), "solve_ms": med("solve_ms"),
             "outer": int(sts[-1]["outer"]), "inner": int(sts[-1]["inner_total"]),
             "converged": int(all(st["converged"] == 1 for st in sts)), "tuning": tuning}
        if not a.no_cpu:
            sys.path.insert(0, str(ROOT / "oracle"))
            import oracle
            g = oracle.Gwf(m, oracle.settings(**tol))
            t0 = time.perf_counter()
            so = g.timestep(kper=1, kstp=1, delt=1.0, transient=False, **GRID_OUTER)
            r["oracle"] = {"value": time.perf_counter() - t0, "unit": "s", "cores": 1,
                           "outer": int(so["outer"]), "inner": int(so["inner_total"]),
                           "max_head_diff_vs_gpu_m": float(np.max(np.abs(g.x - heads)))}
        out[name] = r
    return out


def warmstart_form(a) -> dict:
    """The learned warm start on the transient 256x256x3 workload (C5): the
    network is trained on the GPU (its own BF16 tensor-core kernels) on heads
    the plain solver produces for seeded training models, then every time step
    of held-out models is solved from the previous heads, from the energy
    projection onto the last step's change alone, and from the projection onto
    the last change and the network's guess, all to the same closure."""
    import time as _t
    from modflow6_gb300.warmstart import WarmStartNet, evaluate, generate, train

    full = a.scale == 1.0
    ntrain, nheld, steps = (48, 16, 20) if full else (4, 2, 8)
    sc = 1.0 if full else 0.1
    t0 = _t.perf_counter()
    data, dh_scale = generate(range(1000, 1000 + ntrain), steps=steps, scale=sc)
    t_gen = _t.perf_counter() - t0
    net = WarmStartNet(data[0][0], seed=a.seed)
    t0 = _t.perf_counter()
    hist = train(net, data, dh_scale, epochs=4, lr=1e-3)
    t_train = _t.perf_counter() - t0
    del data
    res = evaluate(net, range(5000, 5000 + nheld), steps=steps, scale=sc)
    net.close()
    return {"workload": f"DIS 3x{int(256 * sc)}x{int(256 * sc)} transient, {steps} steps of 0.5 d, "
                        f"50 wells; PCG + ILU0 to INNER_DVCLOSE 1e-6, INNER_RCLOSE 1e-4",
            "train_models": ntrain, "train_samples": ntrain * steps, "data_s": t_gen,
            "head_change_scale_asinh_units": dh_scale,
            "train_s": t_train, "epochs": 4, "loss_per_epoch": hist, "heldout": res,
            "network": "8-layer message passing, hidden 64, BF16 mma.sync GEMMs, FP32 Adam"}


def kernels_arm(a):
    """Per-kernel device times of one inner iteration's kernels (SpMV,
    ILU0 application, dot, update) on direct stream launches, for both
    precisions: one system assembled on the GPU, factored, then each kernel
    launched `--steps` times after one warm-up (gbims_time_kernels)."""
    import ctypes as C

    import torch
    from modflow6_gb300 import _lib, build
    build.build()
    from modflow6_gb300.dis import make_config
    from modflow6_gb300.ims import GENERAL, ImsLinear, ImsLinearSettings
    from modflow6_gb300.solution import GwfSolution, Nonlinear, sln_ls_fixups
    from modflow6_gb300.workloads import C2_IMS

    torch.cuda.set_device(0)
    lib = _lib.load()
    m = make_config("c2", seed=a.seed, scale=a.scale)
    shape = (m.nlay, m.nrow, m.ncol)
    con = m.connections()
    sol = GwfSolution(m, ImsLinearSettings(structure=shape, **C2_IMS), Nonlinear())
    x0 = m.strt.copy()
    x0[m.chd_node] = m.chd_head
    sol.heads = x0
    amat, rhs = sol.formulate(0.0)
    sol.close()
    amat, rhs = sln_ls_fixups(con["ia"], con["ja"], m.ibound, amat, rhs, x0, isymmetric=True)
    out = {"workload": workload_config(a, m)["workload"], "reps": a.steps}
    # the full-grid (index-free SpMV, wavefront sweeps) forms, then the
    # general-pattern form (SELL-32 SpMV, level-scheduled sweeps) in FP64
    for name, prec, st in (("fp64", _lib.GBIMS_FP64, shape), ("mixed", _lib.GBIMS_MIXED, shape),
                           ("fp64_general", _lib.GBIMS_FP64, GENERAL)):
        ims = ImsLinear(ImsLinearSettings(precision=prec, structure=st, **C2_IMS))
        ims.imslinear_allocate(m.nodes, con["ia"], con["ja"])
        rc = lib.gbims_factor(ims._h, _lib.dptr(amat), None)
        assert rc >= 0, lib.gbims_last_error(ims._h)
        tuning = None if a.no_tune else autotune(lib, ims._h)
        kt = _lib.GbimsKernelTimes()
        rc = lib.gbims_time_kernels(ims._h, max(1, a.steps), C.byref(kt))
        assert rc == 0, lib.gbims_last_error(ims._h)
        out[name] = {"spmv_ms": kt.spmv_ms, "precond_ms": kt.precond_ms, "dot_ms": kt.dot_ms,
                     "update_ms": kt.update_ms,
                     "spmv_gbs": kt.spmv_bytes / (kt.spmv_ms * 1e-3) / 1e9,
                     "precond_gbs": kt.precond_bytes / (kt.precond_ms * 1e-3) / 1e9,
                     "spmv_bytes": kt.spmv_bytes, "precond_bytes": kt.precond_bytes,
                     "tuning": tuning}
        ims.imslinear_da()
    print(json.dumps(out), flush=True)


def grids_arm(a):
    """The general-grid steady steps alone (for launch lists and quick
    measurements); prints the form's results as one JSON line."""
    import torch
    from modflow6_gb300 import build
    build.build()
    torch.cuda.set_device(0)
    print(json.dumps(grids_form(a, torch.cuda.synchronize)), flush=True)


def main():
    a = parse()
    if a.kernels:
        kernels_arm(a)
    elif a.grids:
        grids_arm(a)
    elif a.impl == "reference":
        reference_arm(a)
    else:
        gb_arm(a)


if __name__ == "__main__":
    main()
