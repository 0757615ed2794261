#!/usr/bin/env python
"""Benchmark: explicit Cahn-Hilliard, [0,64]^3, 64^3 cells, FE_Q degree 2, periodic, FP64.

One step = one increment of the application's solve loop: the c block (c from old c and
grad old mu) then the mu block (mu from c and grad c), each an explicit solve
u = invM (.) A_rhs followed by the constraints. Metric: DoF-updates/s = 2 N per step
(N = 129^3 lattice DoFs per field, periodic images included as deal.II keeps them).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`value` is device time with the state resident in HBM (per-step CUDA events on the
engine's stream, L2 flushed between steps). `e2e` is the same metric through the public C
ABI with the step's inputs uploaded from pinned host memory and its result downloaded every
step. `--impl reference` times the CPU restatement of the reference algorithm (the oracle;
the reference itself needs deal.II/MPI/p4est, which neither machine has) on all host cores.
Under torchrun (or with --sharded) one simulation is sharded over the ranks: z-slabs of
64^3 cells per rank stacked along z (weak scaling), halo node planes exchanged after every
block (phasefield_gb300/sharding.py); rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import csv
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "DoF-updates/s (explicit Cahn-Hilliard Q2 3-D step, FP64)"
UNIT = "DoF-updates/s"
WORKLOAD = dict(refine=6, degree=2, size=64.0, dt=1e-4)
# dram__bytes_read.sum + dram__bytes_write.sum of the cell kernel (the lane kernel, the mode the
# bench's timing picks) from one ncu capture of this workload, mean of the c-block
# (59.93 + 0.04 MB) and mu-block (42.76 + 0.00 MB) launches
TRAFFIC_PER_LAUNCH = 51.37e6


def workload_config(extra=None):
    cfg = {"workload": "cahn_hilliard_3d explicit, [0,64]^3, 64^3 cells, FE_Q(2) on GL points, periodic, "
                       "dt=1e-4, M=1, kappa=1.5, f=c^2(1-c)^2, c0=0.5+0.05U(-1,1)",
           "dofs_per_field": 129 ** 3, "fields_updated_per_step": 2, "l2": "flushed between timed steps (256 MiB write)"}
    if extra:
        cfg.update(extra)
    return cfg


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            return float(d.get("hbm_gbs") or d.get("hbm_GBs") or 6800.0), "of measured"
        except Exception:
            pass
    return 6800.0, "of fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    def __init__(self, index: int = 0):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.2)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            with open(self.path) as f:
                for r in csv.reader(f):
                    if len(r) >= 9:
                        rows.append([x.strip() for x in r])
        except Exception:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for n, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def cell_flops_per_step(degree=2, dim=3):
    """Algorithmic FP64 flops of one CH step per cell (sum factorisation + pointwise).

    per block: gradient of one field (dim*nq*n FMA) + integration of the gradient term
    (dim*nq*n FMA) + JxW scaling of value (nq) and gradient terms (dim*nq) + the callback
    (c block: 4 flops/q; mu block: 8 flops/q). FMA counts 2.
    """
    n = degree + 1
    nq = n ** dim
    sf = 2 * (2 * dim * nq * n) + nq + dim * nq
    return (sf + 4 * nq) + (sf + 8 * nq)


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import pyoracle
    from phasefield_gb300 import workloads as W
    threads = os.cpu_count() or 1
    wl = W.cahn_hilliard_3d(**WORKLOAD)
    o = pyoracle.Oracle(wl, threads=threads)
    o.run(0)
    inc = 1
    for _ in range(args.warmup):
        o.run(inc)
        inc += 1
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.run(inc)
        inc += 1
    dt = time.perf_counter() - t0
    N = 129 ** 3
    value = 2 * N * args.steps / dt
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded)", "impl": "reference",
            "config": workload_config({"parallelism": "host threads (OpenMP)"}),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{args.steps} full steps of the workload"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def cpu_baseline_sample(budget_s=12.0):
    from oracle import pyoracle
    from phasefield_gb300 import workloads as W
    threads = os.cpu_count() or 1
    wl = W.cahn_hilliard_3d(**WORKLOAD)
    o = pyoracle.Oracle(wl, threads=threads)
    o.run(0)
    o.run(1)  # warm-up
    steps, t0 = 0, time.perf_counter()
    while True:
        o.run(2 + steps)
        steps += 1
        el = time.perf_counter() - t0
        if el > budget_s or steps >= 200:
            break
    N = 129 ** 3
    return {"value": 2 * N * steps / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{steps} full steps of the workload on {threads} threads ({el:.1f} s)"}


def gmg_cg_measure(refine=6, depth=7):
    """GMG-CG time to a relative residual of 1e-10 on the 3-D elasticity workload
    ([0,64]^3, 64^3 cells, Q2 vector, 40 seeded inclusions, u = 0 on x = 0), plain FP64 V-cycle
    against the FP32 smoother/transfers V-cycle inside the FP64 CG. The system is the
    unscaled one (tolerance type AbsoluteResidual) with tolerance 1e-10 ||b||; each solve
    starts from zero and includes building the level hierarchy, the diagonal probes and the
    eigenvalue estimates (reported per phase)."""
    import torch
    from phasefield_gb300 import workloads as W
    wl = W.eshelby_3d(refine=refine, degree=2, size=64.0, n_incl=40)
    out = {"workload": f"eshelby_3d: [0,64]^3, {2 ** refine}^3 cells, FE_Q(2) vector, 40 inclusions, "
                       f"C11/C12/C44 = 250/150/100, mg_depth {depth}, Chebyshev degree 4, range 15, 10 eig-CG its",
           "criterion": "||b - A x|| <= 1e-10 ||b|| (AbsoluteResidual with tolerance 1e-10 ||b||)"}
    p0 = wl.make_problem()
    b = p0.apply(0, 0, None, scale=0)
    bnorm = float(np.linalg.norm(b))
    p0.close()
    sols = {}
    for mixed in (0, 1):
        p = wl.make_problem()
        p.set_linear_params(0, tolerance_type=0, tolerance=1e-10 * bnorm, max_iterations=500, preconditioner=2,
                            mg_depth=depth, smoother_degree=4, mixed_precision=mixed)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        its, res = p.linear_solve(0, allow_noconv=True)
        p.synchronize()
        el = time.perf_counter() - t0
        key = "mixed" if mixed else "fp64"
        out[key + "_s"] = el
        out[key + "_phases_ms"] = p.linear_stats(0)
        out[key + "_iterations"] = its
        out[key + "_rel_residual"] = res / bnorm
        out[key + "_contraction_mode"] = p.contraction_mode(0, 1)
        sols[key] = p.download(0)
        p.close()
    out["speedup_mixed_vs_fp64"] = out["fp64_s"] / out["mixed_s"]
    out["solution_rel_diff"] = float(np.linalg.norm(sols["mixed"] - sols["fp64"]) / np.linalg.norm(sols["fp64"]))
    return out


def amr_measure():
    """The reference Allen-Cahn application's adaptive configuration
    (applications/allen_cahn/explicit/parameters.prm: [0,100]^2, global refinement 8, min 3,
    max 8, remeshing period 800, refinement where 0.01 < n < 0.99; Q1) on seeded grains: the
    initial refinement passes, the explicit increments 3..799 (no remeshing), the remeshing
    increment 800, and the same number of increments on the uniform 256^2 mesh of the finest
    level."""
    import numpy as np
    import torch
    from phasefield_gb300 import workloads as W
    wl = W.allen_cahn_amr_2d(refine=8, degree=1, min_level=3, max_level=8, period=800, n_grains=12, size=100.0,
                             dt=0.01)
    p = wl.make_problem()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    p.solve(0)
    torch.cuda.synchronize()
    init_s = time.perf_counter() - t0
    dofs0 = p.n_nodes
    levels0 = np.bincount(p.cells()[:, 0], minlength=9).tolist()
    p.solve(2)
    torch.cuda.synchronize()
    # increments 3 .. 799 hold no remeshing step; increment 800 remeshes
    t0 = time.perf_counter()
    p.solve(799)
    torch.cuda.synchronize()
    ada_s = time.perf_counter() - t0
    v0 = p.mesh_version
    t0 = time.perf_counter()
    p.solve(800)
    torch.cuda.synchronize()
    remesh_s = time.perf_counter() - t0
    assert p.mesh_version == v0 + 1
    remesh_phases = p.remesh_stats()
    dofs1 = p.n_nodes
    p.close()
    steps = 797
    wu = W.allen_cahn_2d(refine=8, degree=1, n_grains=12, size=100.0, dt=0.01)
    pu = wu.make_problem()
    pu.solve(2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    pu.solve(2 + steps)
    torch.cuda.synchronize()
    uni_s = time.perf_counter() - t0
    dofs_u = pu.n_nodes
    pu.close()
    return {"workload": "Allen-Cahn [0,100]^2 Q1, 12 seeded grains, global refinement 8, min 3, max 8, "
                        "remeshing period 800, refine where 0.01 < n < 0.99, dt 0.01",
            "steps": steps, "initial_refinement_s": init_s, "dofs_after_initial_refinement": dofs0,
            "cells_per_level": levels0, "dofs_after_remesh": dofs1,
            "adaptive_ms_per_step": ada_s / steps * 1e3,
            "adaptive_dof_updates_per_s": dofs0 * steps / ada_s,
            "remeshing_increment_ms": remesh_s * 1e3, "remesh_phases_ms": remesh_phases,
            "uniform_finest_dofs": dofs_u, "uniform_finest_ms_per_step": uni_s / steps * 1e3,
            "speedup_adaptive_vs_uniform_finest": uni_s / ada_s}


def ensemble_measure(steps=30):
    """Aggregate DoF-updates/s of the 256-instance Allen-Cahn ensemble (cells per side
    32..256, Q1/Q2, per-instance m_well/kappa, grain ICs), one persistent launch per step
    under a captured graph after the autotuner's choice, against the same instances run one
    simulation per launch sequence (a handle each, ppf_run)."""
    import torch
    from phasefield_gb300 import ensemble as E
    from phasefield_gb300 import workloads as W
    meshes, mw, ka, ics = E.allen_cahn_ensemble(n_instances=256)
    dofs = sum(len(ic) for ic in ics)
    dt = 0.01
    ens = E.Ensemble(meshes, mw, ka, dt)
    for i, ic in enumerate(ics):
        ens.upload(i, ic)
    tune_ms, shape, grid = ens.autotune(steps=3)
    ens.run(3)
    ens.synchronize()
    t0 = time.perf_counter()
    ens.run(steps)
    ens.synchronize()
    batched_s = time.perf_counter() - t0
    ens.close()
    # one simulation per launch sequence
    probs = []
    for i, m in enumerate(meshes):
        wl = W.allen_cahn_2d(degree=m.degree, refine=m.global_refinement, m_well=mw[i], kappa=ka[i], dt=dt,
                             subdivisions=m.subdivisions[:2])
        wl.initial = {0: ics[i]}
        p = wl.make_problem()
        p.solve(1)
        probs.append(p)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(steps):
        for p in probs:
            p.lib.ppf_run(p.h, 2 + k, 0)
    torch.cuda.synchronize()
    single_s = time.perf_counter() - t0
    for p in probs:
        p.close()
    return {"workload": "256 Allen-Cahn instances, [0,100]^2, cells per side U{32..256}, Q1/Q2, "
                        "m_well U[0.5,2], kappa U[1,4], 12 seeded grains each, dt 0.01",
            "dofs_total": dofs, "steps": steps,
            "batched_dof_updates_per_s": dofs * steps / batched_s,
            "single_dof_updates_per_s": dofs * steps / single_s,
            "speedup_batched_vs_single": single_s / batched_s,
            "autotune": {"ms_per_step": tune_ms, "shape": shape, "grid_multiplier": grid},
            "launches_per_step_batched": 1}


def adjoint_measure(steps=500, snapshots=32):
    """Adjoint calibration workload: coupled Allen-Cahn/Cahn-Hilliard 2-D, [0,128]^2, 256^2
    cells, Q2, dt 1e-3, 500 explicit steps; loss J = sum_i m_i (c_K - c_target)^2 with the
    target produced by (1.5 Mc, 0.5 Kn); gradient w.r.t. (Mc, Kn, n_0) by the adjoint with 32
    binomial checkpoint slots, checked against central differences (Mc, Kn) in the same run."""
    from phasefield_gb300 import workloads as W

    def final_c(Mc, Kn):
        wl = W.coupled_acch_2d(Mc=Mc, Kn=Kn)
        p = wl.make_problem()
        p.solve(steps)
        c = p.download(0, age=1)
        m = 1.0 / p.invm()
        p.close()
        return c, m

    base = W.coupled_acch_2d()
    Mc, Mn, Kn = base.constants
    target, mass = final_c(1.5 * Mc, 0.5 * Kn)
    p = base.make_problem()
    N = p.n_nodes
    p.synchronize()
    t0 = time.perf_counter()
    p.adjoint_forward(0, steps, snapshots)
    cK = p.download(0)
    dJ = np.concatenate([2.0 * mass * (cK - target), np.zeros(N)])
    dparams, du0, fsteps = p.adjoint_backward(dJ)
    el = time.perf_counter() - t0
    p.close()
    fd = []
    for i, (val, key) in enumerate(((Mc, "Mc"), (Kn, "Kn"))):
        eps = 1e-5 * val
        args_p = {"Mc": Mc, "Kn": Kn}
        args_m = dict(args_p)
        args_p[key] = val + eps
        args_m[key] = val - eps
        jp = float(np.sum(mass * (final_c(**args_p)[0] - target) ** 2))
        jm = float(np.sum(mass * (final_c(**args_m)[0] - target) ** 2))
        fd.append((jp - jm) / (2 * eps))
    rel = [abs(dparams[i] - fd[i]) / abs(fd[i]) for i in range(2)]
    return {"workload": "coupled AC/CH 2-D, [0,128]^2, 256^2 cells, FE_Q(2), dt 1e-3, 500 steps, "
                        "target from (1.5 Mc, 0.5 Kn), loss sum m (c_K - c_t)^2",
            "snapshots": snapshots, "forward_plus_backward_s": el, "forward_steps_taken": int(fsteps),
            "dJ_dMc": float(dparams[0]), "dJ_dKn": float(dparams[1]), "fd_dJ_dMc": fd[0], "fd_dJ_dKn": fd[1],
            "rel_err_vs_fd": rel, "dJ_dn0_norm": float(np.linalg.norm(du0[N:]))}


def run_ours(args):
    import torch
    import torch.distributed as dist

    ws, rank, local = dist_env()
    if ws > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    from phasefield_gb300 import build as pbuild
    if rank == 0:
        pbuild.build()
    if ws > 1:
        dist.barrier()
    from phasefield_gb300 import capi
    from phasefield_gb300 import workloads as W
    lib = capi.load()

    wl = W.cahn_hilliard_3d(**WORKLOAD)
    p = wl.make_problem()
    N = p.n_nodes
    stream = torch.cuda.current_stream(dev)
    lib.ppf_set_stream(p.h, C.c_void_p(stream.cuda_stream))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    p.solve(0)  # increment 0: initial condition + mu block
    inc = 1
    for _ in range(args.warmup):
        p.solve(inc)
        inc += 1
    torch.cuda.synchronize()

    # ---- device-timed steps ----
    lib.ppf_kernel_stats_reset(p.h)
    lib.ppf_kernel_timing(p.h, 1)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            flush.zero_()
            evs[k][0].record(stream)
            p.solve(inc)
            evs[k][1].record(stream)
            inc += 1
        torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    step_ms = [a.elapsed_time(b) for a, b in evs]
    total_ms = float(sum(step_ms))
    cell_ms = C.c_double()
    cell_n, all_n = C.c_longlong(), C.c_longlong()
    lib.ppf_kernel_stats(p.h, C.byref(cell_ms), C.byref(cell_n), C.byref(all_n))
    lib.ppf_kernel_timing(p.h, 0)
    # 0 FP64 contractions, 1 fixed-point derivatives + FP64 integration, 2 both fixed point,
    # 3 FP64 derivatives + fixed-point integration, 4 the lane kernel (all in fixed point)
    modes = {"c_block": p.contraction_mode(0, 0), "mu_block": p.contraction_mode(1, 0)}
    from phasefield_gb300 import replicas
    max_ms, dof_updates = replicas.aggregate(total_ms, 2 * N * args.steps, dist if ws > 1 else None, dev)
    value = dof_updates / (max_ms * 1e-3)

    # ---- end to end through the C ABI with host buffers ----
    # every step uploads old c and old mu from pinned host memory and returns both results to
    # pinned host memory. Pipelined (the headline): the inputs are staged on the upload stream
    # (ppf_upload_state_staged), the increment is queued (ppf_run_async) and the results stream
    # out of staging copies (ppf_set_output_stream), so step k+1's uploads and step k's
    # downloads overlap the computation; ppf_wait at the end returns once every copy landed.
    # Serial (reported beside it): one blocking ppf_run per step with queued uploads.
    pin = [torch.empty(N, dtype=torch.float64, pin_memory=True) for _ in range(4)]
    for f in (0, 1):
        p.lib.ppf_download_state(p.h, f, 1, C.cast(pin[f].data_ptr(), C.POINTER(C.c_double)), 0)
    for f in (0, 1):
        p.set_output_stream(f, pin[2 + f])
    hp = [C.cast(pin[f].data_ptr(), C.POINTER(C.c_double)) for f in (0, 1)]
    e2e_steps = max(3, args.steps)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        for f in (0, 1):  # inputs of this step: old c and old mu
            assert lib.ppf_upload_state_staged(p.h, f, 1, hp[f]) == 0
        assert lib.ppf_run_async(p.h, inc, 0) == 0  # results land in pin[2], pin[3]
        inc += 1
    assert lib.ppf_wait(p.h) == 0
    e2e_s = time.perf_counter() - t0
    assert np.array_equal(pin[2].numpy(), p.download_solution(0))
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        for f in (0, 1):
            assert lib.ppf_upload_state_async(p.h, f, 1, hp[f], 0) == 0
        p.solve(inc)
        inc += 1
    torch.cuda.synchronize()
    serial_s = time.perf_counter() - t0
    for f in (0, 1):
        p.set_output_stream(f, None)
    assert np.array_equal(pin[2].numpy(), p.download_solution(0))
    e2e = {"value": 2 * N * e2e_steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 2 * 8 * N,
           "d2h_bytes_per_step": 2 * 8 * N, "steps": e2e_steps,
           "pipelined": "ppf_upload_state_staged + ppf_run_async per step, one ppf_wait at the end",
           "serial_value": 2 * N * e2e_steps / serial_s}

    if rank == 0:
        peak, peak_src = measured_peaks()
        avg_launch_s = cell_ms.value * 1e-3 / max(cell_n.value, 1)
        bytes_per_launch = 20 * N  # c block 24N (read c_old, mu_old, write c), mu block 16N: mean 20N
        achieved = bytes_per_launch / avg_launch_s / 1e9
        fp64_peak = C.c_double()
        lib.ppf_device_fp64_peak(C.byref(fp64_peak))
        ncells = 64 ** 3
        flops_per_launch = cell_flops_per_step() * ncells / 2
        fp64_achieved = flops_per_launch / avg_launch_s / 1e12
        cpu = cpu_baseline_sample()
        gmg = gmg_cg_measure() if not args.skip_extras else None
        ens = ensemble_measure() if not args.skip_extras else None
        adj = adjoint_measure() if not args.skip_extras else None
        amr = amr_measure() if not args.skip_extras else None
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": max_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
                "config": workload_config({"parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"}),
                "e2e": e2e, "gpu_launches": int(all_n.value), "clocks": clk.summary(),
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "traffic": TRAFFIC_PER_LAUNCH,
                             "traffic_unit": "bytes/launch", "peak_source": peak_src,
                             "kernel": ("cell_kernel_lanes<CahnHilliard<3,2>>" if set(modes.values()) == {4}
                                        else "cell_kernel<CahnHilliard<3,2>>"),
                             "bytes_per_launch": bytes_per_launch, "avg_launch_ms": avg_launch_s * 1e3},
                "fp64_equivalent": {"achieved": fp64_achieved, "peak": fp64_peak.value, "unit": "TFLOP/s",
                                    "frac": fp64_achieved / fp64_peak.value if fp64_peak.value else None,
                                    "flops_per_launch": flops_per_launch, "peak_source": "measured in this run",
                                    "note": "FP64 flops of the same launch with FP64 contractions; the kernel "
                                            "contracts exactly in 64-bit integers"},
                "contraction_modes": modes,
                "cpu_baseline": cpu, "gmg_cg": gmg, "ensemble": ens, "adjoint": adj, "amr": amr}
        print(json.dumps(line), flush=True)
    p.close()
    if ws > 1:
        dist.destroy_process_group()
    return 0


def run_sharded(args):
    """The same workload as one simulation sharded over the ranks (weak scaling: 64^3 cells per
    GPU, the GPUs' slabs stacked along z into [0,64]^2 x [0,64N], periodic), the halo planes
    exchanged after every block with NCCL point-to-point messages (phasefield_gb300/sharding.py).
    `value` counts the DoF updates of the whole simulation."""
    import torch
    import torch.distributed as dist

    ws, rank, local = dist_env()
    if ws > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from phasefield_gb300 import build as pbuild
    if rank == 0:
        pbuild.build()
    if ws > 1:
        dist.barrier()
    from phasefield_gb300 import capi
    from phasefield_gb300 import sharding as S
    from phasefield_gb300 import workloads as W
    lib = capi.load()

    wl = W.cahn_hilliard_3d(**WORKLOAD, subdivisions=(1, 1, ws))
    wl.mesh.size = (64.0, 64.0, 64.0 * ws)
    P = wl.mesh.nodes[0] * wl.mesh.nodes[1]
    c0 = wl.initial[0].copy()
    c0[-P:] = c0[:P]  # periodic along the split axis
    wl.initial = {0: c0}
    Ng = int(np.prod(wl.mesh.nodes))
    slab = S.partition(wl.mesh, rank, ws)
    lw = S.local_workload(wl, slab)
    p = lw.make_problem()
    drv = S.ShardedExplicit(slab, S.EngineLocal(p), wl.fields, wl.blocks, dist if ws > 1 else None)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    drv.run(0)
    for _ in range(args.warmup):
        drv.run(drv.increment)
    torch.cuda.synchronize()
    lib.ppf_kernel_stats_reset(p.h)
    lib.ppf_kernel_timing(p.h, 1)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            flush.zero_()
            evs[k][0].record(stream)
            drv.run(drv.increment)
            evs[k][1].record(stream)
        torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    total_ms = float(sum(a.elapsed_time(b) for a, b in evs))
    cell_ms = C.c_double()
    cell_n, all_n = C.c_longlong(), C.c_longlong()
    lib.ppf_kernel_stats(p.h, C.byref(cell_ms), C.byref(cell_n), C.byref(all_n))
    lib.ppf_kernel_timing(p.h, 0)
    from phasefield_gb300 import replicas
    max_ms, _ = replicas.aggregate(total_ms, 0, dist if ws > 1 else None, dev)
    value = 2 * Ng * args.steps / (max_ms * 1e-3)
    # end to end: each rank's slab through the C ABI with host buffers
    Nl = p.n_nodes
    pin = [torch.empty(Nl, dtype=torch.float64, pin_memory=True) for _ in range(4)]
    for f in (0, 1):
        p.lib.ppf_download_state(p.h, f, 1, C.cast(pin[f].data_ptr(), C.POINTER(C.c_double)), 0)
    e2e_steps = max(3, min(args.steps, 10))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for f in (0, 1):
            assert lib.ppf_upload_state(p.h, f, 1, C.cast(pin[f].data_ptr(), C.POINTER(C.c_double)), 0) == 0
        drv.run(drv.increment)
        for f in (0, 1):
            assert lib.ppf_download_state(p.h, f, 1, C.cast(pin[2 + f].data_ptr(), C.POINTER(C.c_double)), 0) == 0
    torch.cuda.synchronize()
    e2e_ms, _ = replicas.aggregate((time.perf_counter() - t0) * 1e3, 0, dist if ws > 1 else None, dev)
    if rank == 0:
        peak, peak_src = measured_peaks()
        avg_launch_s = cell_ms.value * 1e-3 / max(cell_n.value, 1)
        bytes_per_launch = 20 * Nl
        achieved = bytes_per_launch / avg_launch_s / 1e9
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": max_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
                "config": {"workload": f"cahn_hilliard_3d explicit sharded: [0,64]^2 x [0,{64 * ws}], "
                                       f"64x64x{64 * ws} cells, FE_Q(2) on GL points, periodic, dt=1e-4",
                           "dofs_per_field": Ng, "fields_updated_per_step": 2,
                           "l2": "flushed between timed steps (256 MiB write)",
                           "parallelism": f"slab sharding x{ws}, ghost cells + NCCL halo planes"},
                "e2e": {"value": 2 * Ng * e2e_steps / (e2e_ms * 1e-3), "unit": UNIT,
                        "h2d_bytes_per_step": 2 * 8 * Nl * ws, "d2h_bytes_per_step": 2 * 8 * Nl * ws},
                "gpu_launches": int(all_n.value), "clocks": clk.summary(),
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "traffic": TRAFFIC_PER_LAUNCH * Nl / 129 ** 3,
                             "traffic_unit": "bytes/launch (scaled from the 64^3 capture)",
                             "peak_source": peak_src, "kernel": "cell_kernel<CahnHilliard<3,2>>",
                             "bytes_per_launch": bytes_per_launch, "avg_launch_ms": avg_launch_s * 1e3},
                "cpu_baseline": None}
        print(json.dumps(line), flush=True)
    p.close()
    if ws > 1:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--skip-extras", action="store_true", help="omit the GMG-CG, ensemble, adjoint and adaptive-mesh measurements")
    ap.add_argument("--sharded", action="store_true",
                    help="run the sharded simulation also on one GPU (more than one GPU always shards)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    if args.impl == "reference":
        return run_reference(args)
    if args.sharded or dist_env()[0] > 1:
        return run_sharded(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
