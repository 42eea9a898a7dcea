"""Benchmark of the GB300 monodomain time step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Workload: ORd (tissue myocyte) on the 20 x 7 x 3 mm slab at h = 0.1 mm
(200 x 70 x 30 = 420,000 cells), dt = 5 us, implicit backward-Euler/BDF2
diffusion with PCG (tol 1e-8), corner box stimulus 5e4 A/m^3 for 2 ms,
Vm0 = -84 mV, starting at t = 0.  Synthetic (the reference publishes no
dataset for this path).  A step is one runTime++/evolve over all cells.

The headline `value` is the mixed-precision form's device-resident
throughput in cell-steps/s over K steps of the wavefront window (from
t = 10 ms, step 2000: the front inside the slab, about 21,600 cells
activated); the rest-state window right after the warm-up is reported
beside it, with the RHS evaluations per cell-step of each window.  The FP64
plain form is timed in the same window and both forms are compared at its
end (activation times, Vm).  `e2e` repeats the mixed run through the C ABI
with Vm copied in from and out to pinned host memory every step.  Under
torchrun every rank runs an independent replica on its own GPU (the step
has no cross-rank exchange at one GPU per replica).  `--impl reference`
times the CPU oracle (the reference's ionic code and restated OpenFOAM
numerics) on a bounded corner piece of the slab at the same window.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "monodomain cell-steps/s, mixed vs FP64 on GB300 at ≤0.05 ms activation error"
SIGMA = (0.1334, 0.0, 0.0, 0.0176, 0.0, 0.0176)
BOX = [((0.0, 0.0, 0.0), (1.5e-3, 1.5e-3, 1.5e-3), 0.0, 2e-3, 5e4)]
WORKLOAD = ("ORd myocyte monodomain slab 20x7x3 mm, h=0.1 mm (200x70x30 = 420000 cells), "
            "dt=5e-6 s, implicit (backward ddt, PIMPLE residualControl 1e-6, PCG tol 1e-8), "
            "corner stimulus 5e4 A/m^3 x 2 ms, from t=0; timed window from t=10 ms "
            "(step 2000, the wavefront inside the slab)")
DIMS = (200, 70, 30)
H = 1e-4
DT = 5e-6
# DRAM bytes (read + write) of one mixed ORd ionic launch on this workload,
# from an ncu capture of the current kernel (dram__bytes_read.sum +
# dram__bytes_write.sum); ncu cannot run inside the timed region, so the
# figure is carried here and refreshed with each capture.
IONIC_TRAFFIC_BYTES = 120.6e6
IONIC_TRAFFIC_SOURCE = "profiles/ionic_mixed_kernel_ord_420k.md"
# states read and written (31 FP32 + 10 FP32 hi/lo pairs = 204 B) + Vm in + Iion out
IONIC_STATE_BYTES = 2 * 204 + 16


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


def opcounts():
    return json.loads((ROOT / "cardiacfoam_gb300/csrc/models/opcounts.json").read_text())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self, index: int):
        self.proc = None
        self.path = Path(tempfile.gettempdir()) / f"cfg_bench_clocks_{os.getpid()}.csv"
        self.index = index

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}",
                 "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()
            self.fh.close()

    def summary(self):
        if not self.proc or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        rows = [r.split(", ") for r in self.path.read_text().strip().splitlines() if r]
        sm = [float(r[1]) for r in rows if len(r) >= 9 and r[1].strip().isdigit()]
        mx = [float(r[2]) for r in rows if len(r) >= 9 and r[2].strip().isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows if len(r) >= 9
                          for i in range(4) if r[5 + i].strip() == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(sm)}


def max_over_ranks(seconds: float, world: int) -> float:
    """The slowest rank's time (whole-job timing of replicas): an all-reduce
    MAX on a tensor of the process group's device (CUDA under NCCL, CPU
    under gloo)."""
    if world <= 1:
        return seconds
    import torch
    dist = torch.distributed
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([seconds], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_value(cells: int, steps: int, world: int, seconds: float) -> float:
    """cell-steps/s of all replicas together (each rank advances its own
    copy of the workload; scaling "weak")."""
    return cells * steps * world / seconds


def build_mesh():
    from cardiacfoam_gb300.mesh import box_mesh
    nx, ny, nz = DIMS
    return box_mesh(nx, ny, nz, nx * H, ny * H, nz * H)


GRAPH = True


def make_model(mesh, precision):
    from cardiacfoam_gb300 import api
    m = api.Monodomain(mesh, "ORd", "myocyte", SIGMA, dt=DT, precision=precision, boxes=BOX,
                       max_steps=10 ** 6)
    if not GRAPH:
        m.set_graph(False)   # every kernel launched on its own (for per-kernel profiling)
    return m


def timed_steps(md, k, flush, dt=DT):
    """Run k steps, timing each with CUDA events on the context's stream.
    Before each step L2 is flushed (a 256 MB write) on that stream, ahead of
    the start event: the host submits the step while the flush runs, so the
    events bracket the step's device work and not the host's launch
    latency (the end-to-end figure keeps that)."""
    import torch
    stream = torch.cuda.ExternalStream(md.stream())
    total = 0.0
    for _ in range(k):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            flush.zero_()
        e0.record(stream)
        md.step(dt)
        e1.record(stream)
        e1.synchronize()
        total += e0.elapsed_time(e1)
    torch.cuda.synchronize()
    return total / 1e3


def gpu_arm(args, rank, world):
    """The headline: the mixed form timed over K steps of the wavefront
    window (steps window_start .. window_start + K, t = 10 ms by default, the
    front inside the slab), after W warm-up steps and an untimed advance to
    the window.  The rest-state window right after the warm-up (t ~ 0.05 ms,
    one RKF45 substep per cell) is timed too and reported beside it.  The FP64
    form runs to the same window, is timed there, and both forms are compared
    at the window's end (activation times over every cell both activated,
    Vm L-inf)."""
    import torch
    from cardiacfoam_gb300 import build as gpu_build, lib
    if rank == 0 or not (ROOT / "cardiacfoam_gb300/libcardiac_gpu.so").exists():
        gpu_build.build()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.set_device(rank % max(torch.cuda.device_count(), 1))
    dev = torch.cuda.current_device()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")   # 256 MB > L2
    mesh = build_mesh()
    n = mesh.n_cells
    K = args.steps

    # ---------------- mixed form (headline)
    mixed = make_model(mesh, lib.PRECISION_MIXED)
    for _ in range(args.warmup):
        mixed.step(DT)
    tune_mixed = mixed.autotune() if not args.no_autotune else None
    mixed.step(DT)                 # rebuilds the step graph with the chosen shape
    # rest-state window (secondary figure)
    mixed.set_timing(True)
    e0 = mixed.rhs_evaluations()
    t_rest = timed_steps(mixed, K, flush)
    rest_ionic_ms, rest_diff_ms, _, _ = mixed.timings()
    rest_evals = mixed.rhs_evaluations() - e0
    mixed.set_timing(False)
    # untimed advance to the wavefront window
    done = args.warmup + 1 + K
    window_start = max(args.window_start, done)
    mixed.run(DT, window_start - done)
    mixed.set_timing(True)
    evals0 = mixed.rhs_evaluations()
    if world > 1:
        torch.distributed.barrier()
    with ClockSampler(dev) as clk:
        t_mixed = timed_steps(mixed, K, flush)
    t_mixed = max_over_ranks(t_mixed, world)
    ionic_ms, diff_ms, nsteps, launches = mixed.timings()
    evals = mixed.rhs_evaluations() - evals0
    mixed.set_timing(False)
    clocks = clk.summary()
    total_steps = window_start + K

    # ---------------- FP64 plain form: to the same window, timed there, then
    # on to the mixed context's step for the comparison
    k64 = max(1, min(K, args.fp64_steps))
    fp64 = make_model(mesh, lib.PRECISION_FP64)
    for _ in range(args.warmup):
        fp64.step(DT)
    tune_fp64 = fp64.autotune() if not args.no_autotune else None
    fp64.run(DT, window_start - args.warmup)
    fp64.set_timing(True)
    t_fp64 = timed_steps(fp64, k64, flush)
    ionic64_ms, diff64_ms, _, _ = fp64.timings()
    fp64.set_timing(False)
    fp64.run(DT, total_steps - window_start - k64)
    a64, amx = fp64.activation(), mixed.activation()
    both = (a64 > 0) & (amx > 0)
    act_err_ms = float(np.max(np.abs(a64[both] - amx[both])) * 1e3) if both.any() else None
    mismatch = int(np.sum((a64 > 0) != (amx > 0)))
    vm_err = float(np.max(np.abs(fp64.vm() - mixed.vm())))
    in_box = np.zeros(n, dtype=bool)
    lo, hi = BOX[0][0], BOX[0][1]
    c = mesh.centres
    in_box[:] = np.all((c >= np.array(lo)) & (c <= np.array(hi)), axis=1)
    propagated = int(np.sum(both & ~in_box))
    fp64_time = fp64.time()
    del fp64

    # ---------------- end to end through the C ABI with host copies, in the
    # wavefront window
    pin_in = torch.empty(n, dtype=torch.float64, pin_memory=True)
    pin_out = torch.empty(n, dtype=torch.float64, pin_memory=True)
    ke2e = max(1, min(K, args.e2e_steps))
    vm_host = pin_in.numpy()
    vm_host[:] = mixed.vm()
    vm_out = pin_out.numpy()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(ke2e):
        mixed.set_field(lib.FIELD_VM, vm_host)
        mixed.step(DT)
        lib.check(mixed._lib.cfg_monodomain_get_field(mixed.h, lib.FIELD_VM, lib.dptr(vm_out)))
        vm_host, vm_out = vm_out, vm_host
    t_e2e = time.perf_counter() - t0

    # ---------------- roofline of the dominant kernel (ionic, mixed form)
    pk, src = peaks()
    ops = opcounts()["ORd"]
    sm_mhz = pk.get("sm_max_mhz", 2070.0)
    fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12        # TFLOP/s, FP32 FMA pipe
    ionic_s = ionic_ms / 1e3
    # executed work: the stage loop per evaluation, the membrane-potential-only
    # part once per cell-step; and the same evaluations counted as the
    # reference's body evaluates them
    per_eval = ops["flops"] + ops["transcendental"]
    inv = ops.get("invariant_flops", 0.0) + ops.get("invariant_transcendental", 0.0)
    executed = evals * (per_eval - inv) + n * K * inv
    achieved = executed / ionic_s / 1e12
    reference_equivalent = evals * per_eval / ionic_s / 1e12
    nnz = 2 * mesh.n_faces
    return dict(n=n, t_mixed=t_mixed, t_fp64=t_fp64, k64=k64, ionic_ms=ionic_ms,
                diff_ms=diff_ms, ionic64_ms=ionic64_ms, diff64_ms=diff64_ms, evals=evals,
                executed_ops=executed, reference_equivalent=reference_equivalent,
                launches=launches, clocks=clocks, act_err_ms=act_err_ms, act_mismatch=mismatch,
                act_cells=int(both.sum()), act_cells_outside_box=propagated, vm_err=vm_err,
                window_start=window_start, compared_at_step=total_steps,
                compared_at_time=fp64_time, t_e2e=t_e2e, ke2e=ke2e, achieved=achieved,
                fp32_peak=fp32_peak, peaks=pk, peak_src=src, nnz=nnz,
                n_active_mixed=int((amx > 0).sum()),
                rest={"t": t_rest, "ionic_ms": rest_ionic_ms, "diff_ms": rest_diff_ms,
                      "evals": rest_evals, "start_step": args.warmup + 1},
                autotune={"mixed": tune_mixed, "fp64": tune_fp64})


LV_DT = 1e-5
LV_INTENSITY = 5e4       # A/m^3, for 2 ms


def bidomain_arm(args):
    """The bidomain tutorial's manufactured case (bidomainSolver,
    bidomainFDAManufactured, 3D unit cube at 40 cells per direction, dt of the
    tutorial's sweep, two PIMPLE correctors, PCG tolerance 1e-12 for Vm and
    phiE): GPU steps timed with CUDA events after warm-up, with the PCG of both
    systems in float pairs (the headline) and in FP64, the oracle (DIC, one
    thread) on a bounded sample of the same steps, and each GPU form
    compared with it after that sample."""
    import torch
    from cardiacfoam_gb300 import api, lib
    from cardiacfoam_gb300 import verification as V
    from oracle import pyoracle
    dim, n = 3, args.bidomain_cells
    dt = V.SWEEP.get(n, 0.2 / (10 * n * n / 4))
    mesh = V.geometry_mesh_for(dim, n)

    def gpu(arithmetic):
        bd = api.Bidomain(mesh, model="bidomainFDAManufactured", tissue=f"{dim}D",
                          sigma_i=V.BIDOMAIN_SIGMA_I, sigma_e=V.BIDOMAIN_SIGMA_E, chi=V.CHI,
                          cm=V.CM, dt=dt, pcg_tol=1e-12, phie_tol=1e-12, phie_max_iter=4000,
                          n_outer=2, ref_point=V.BIDOMAIN_REF_POINT,
                          grad_scheme=lib.GRAD_GAUSS_LINEAR)
        bd.set_pcg_arithmetic(arithmetic)
        vm, pe, _, u1, u2, u3 = V.bidomain_fields(mesh.centres, 0.0, dim)
        bd.set_field(lib.FIELD_VM, vm)
        bd.set_field(lib.FIELD_PHIE, pe)
        bd.set_states(np.stack([vm, u1, u2, u3]))
        return bd

    ks = args.bidomain_sample

    def timed(arithmetic):
        """ks sample steps (kept for the oracle comparison), 3 warm-up
        steps, then the timed steps"""
        bd = gpu(arithmetic)
        bd.run(dt, ks)
        sample = (bd.vm(), bd.phie())
        bd.run(dt, 3)
        s = torch.cuda.ExternalStream(bd.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        its_v, its_e = [], []
        torch.cuda.synchronize()
        e0.record(s)
        for _ in range(args.bidomain_steps):
            bd.step(dt)
            (_, _, iv), (_, _, ie) = bd.stats()
            its_v.append(int(iv.sum()))
            its_e.append(int(ie.sum()))
        e1.record(s)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / args.bidomain_steps
        bd.close()
        return ms, its_v, its_e, sample

    runs = {name: timed(a) for name, a in (("float_pairs", lib.PCG_FLOAT_PAIRS),
                                           ("fp64", lib.PCG_FP64))}
    # oracle sample: the same first steps from the same state
    d = pyoracle.tissue_desc("bidomainFDAManufactured", 10 + dim, V.BIDOMAIN_SIGMA_I, chi=V.CHI,
                             cm=V.CM, implicit=True, precond_dic=True, pcg_tol=1e-12,
                             pcg_rel_tol=0.0, pcg_max_iter=2000, n_outer=2, outer_tol=0.0,
                             grad_gauss=True)
    B = pyoracle.Bidomain(d, V.BIDOMAIN_SIGMA_E, pyoracle.Mesh.general(mesh),
                          V.BIDOMAIN_REF_POINT, 0.0, 1e-12, 0.0, 4000)
    vm, pe, _, u1, u2, u3 = V.bidomain_fields(mesh.centres, 0.0, dim)
    B.tissue.set_vm(vm)
    B.tissue.set_states(np.stack([vm, u1, u2, u3]), dt)
    B.set_phie(pe)
    t0 = time.perf_counter()
    for _ in range(ks):
        B.step(dt)
    t_cpu = time.perf_counter() - t0
    cells = mesh.n_cells

    def vs_oracle(sample):
        g_vm, g_pe = sample
        return {"vm_max_rel": float(np.max(np.abs(g_vm - B.tissue.vm())) /
                                    np.max(np.abs(B.tissue.vm()))),
                "phie_max_rel": float(np.max(np.abs(g_pe - B.phie())) / np.max(np.abs(B.phie())))}

    ms, its_v, its_e, sample = runs["float_pairs"]
    ms64, its_v64, its_e64, sample64 = runs["fp64"]
    return {"workload": (f"bidomain tutorial manufactured case, 3D unit cube {n}^3 = {cells} "
                         f"cells, dt {dt} s, Gi/Ge of the tutorial, backward ddt, 2 PIMPLE "
                         f"correctors, PCG 1e-12 (Vm, phiE), Gauss linear gradients, FP64 "
                         f"ionic update"),
            "pcg_arithmetic": "float pairs (about 48 significant bits, FP32 pipe)",
            "value": cells / (ms * 1e-3), "unit": "cell-steps/s", "ms_per_step": ms,
            "steps": args.bidomain_steps,
            "pcg_iterations_per_step": {"vm": its_v, "phie": its_e},
            "us_per_phie_iteration": ms * 1e3 / max(1, np.mean(its_e)),
            "gpu_vs_oracle_after_sample": vs_oracle(sample),
            "fp64_pcg": {"value": cells / (ms64 * 1e-3), "ms_per_step": ms64,
                         "pcg_iterations_per_step": {"vm": its_v64, "phie": its_e64},
                         "gpu_vs_oracle_after_sample": vs_oracle(sample64)},
            "cpu_oracle": {"value": cells * ks / t_cpu, "unit": "cell-steps/s", "cores": 1,
                           "kind": "port", "sample": f"the first {ks} steps, DIC preconditioner"}}


def ecg_timing(L, source, launches: int = 50):
    """Both arithmetic forms of the pseudo-ECG (float pairs, the default, and
    FP64 multiply-adds), each timed as below."""
    from cardiacfoam_gb300 import lib
    out = {"float_pairs": ecg_timing_one(L, source, launches, lib.ECG_FLOAT_PAIRS),
           "fp64": ecg_timing_one(L, source, launches, lib.ECG_FP64)}
    a, b = out["float_pairs"].pop("_values"), out["fp64"].pop("_values")
    out["pairs_vs_fp64_max_rel"] = float(np.max(np.abs(a - b)) / np.max(np.abs(b)))
    return out


def ecg_timing_one(L, source, launches: int, arithmetic):
    """The pseudo-ECG at the LV's five electrodes (PseudoECGSolver::compute,
    folded into one lead row per electrode): `launches` evaluations recorded
    back to back between CUDA events on the stream they run on (a
    Monodomain's, or torch's current stream for a CUDA tensor of Vm).  One
    evaluation reads the rows and Vm once, (electrodes + 1) x 8 bytes per
    cell: 191 MB on the 4.0 M-tet LV, more than L2 holds."""
    import torch
    from cardiacfoam_gb300 import api
    el = L.ecg_electrodes()
    t0 = time.perf_counter()
    pe = api.PseudoECG(L.mesh, el, conductivity_per_cell=L.conductivity, max_rows=launches + 3,
                       arithmetic=arithmetic)
    t_setup = time.perf_counter() - t0
    if isinstance(source, api.Monodomain):
        s = torch.cuda.ExternalStream(source.stream())
    else:
        s = torch.cuda.current_stream()
    for _ in range(3):
        pe.record(source)
    pe.reset()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(s)
    for _ in range(launches):
        pe.record(source)
    e1.record(s)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / launches
    _, values = pe.series()
    pe.close()
    n = L.mesh.n_cells
    nbytes = n * 8 * (len(el) + 1)
    pk, src = peaks()
    peak = pk["hbm_gbs"]
    gbs = nbytes / (ms * 1e-3) / 1e9
    return {"electrodes": len(el), "cells": n, "setup_seconds": t_setup, "launches": launches,
            "us_per_evaluation": ms * 1e3, "bytes_per_evaluation": nbytes,
            "achieved_gbs": gbs, "hbm_peak_gbs": peak, "peak_src": src,
            "frac_of_hbm_peak": gbs / peak,
            "values_at_t": [float(v) for v in values[-1]], "_values": values[-1]}


def ecg_arm(args):
    """The pseudo-ECG kernel alone on the LV mesh, on a seeded random Vm field
    (uniform in [-90, 40] mV; the pass reads the same bytes for any values)."""
    import torch
    from cardiacfoam_gb300 import lv
    dims = tuple(int(v) for v in args.lv_dims.split(",")) if args.lv_dims else lv.config_sizes()
    L = lv.left_ventricle(*dims)
    g = torch.Generator(device="cuda").manual_seed(7)
    vm = torch.rand(L.mesh.n_cells, dtype=torch.float64, device="cuda", generator=g) * 0.13 - 0.09
    return ecg_timing(L, vm, launches=args.ecg_launches)


def lv_arm(args, flush):
    """The left-ventricle configuration: a truncated prolate-ellipsoid shell
    of about 4.0 M tetrahedra with rule-based fibres (per-cell conductivity
    tensors) and TNNP endo/M/epi cells, apical stimulus, the Laplacian with
    its explicit non-orthogonal and tangential corrections; mixed form in
    the step graph, timed over a bounded number of steps of the 400 ms run,
    FP64 form timed on the same steps, and activation times of both forms
    compared after an accuracy window."""
    import torch
    from cardiacfoam_gb300 import api, lib, lv
    ops = opcounts()["TNNP"]
    t0 = time.perf_counter()
    dims = tuple(int(v) for v in args.lv_dims.split(",")) if args.lv_dims else lv.config_sizes()
    L = lv.left_ventricle(*dims)
    t_mesh = time.perf_counter() - t0
    lo, hi = L.apex_box(2e-3)
    boxes = [(lo, hi, 0.0, 2e-3, LV_INTENSITY)]

    def make(precision):
        m = api.Monodomain(L.mesh, "TNNP", "epicardialCells", dt=LV_DT, precision=precision,
                           boxes=boxes, tissue_per_cell=L.tissue,
                           conductivity_per_cell=L.conductivity, stencil=False,
                           max_steps=10 ** 6)
        if precision == lib.PRECISION_MIXED and args.lv_pcg != "default":
            m.set_pcg_arithmetic(lib.PCG_FLOAT_PAIRS if args.lv_pcg == "pairs" else lib.PCG_FP64)
        return m

    t0 = time.perf_counter()
    mixed = make(lib.PRECISION_MIXED)
    t_setup = time.perf_counter() - t0
    for _ in range(args.warmup):
        mixed.step(LV_DT)
    tune = mixed.autotune() if not args.no_autotune else None
    mixed.step(LV_DT)
    mixed.set_timing(True)
    evals0 = mixed.rhs_evaluations()
    t_mixed = timed_steps(mixed, args.lv_steps, flush, LV_DT)
    ionic_ms, diff_ms, nsteps, launches = mixed.timings()
    evals = mixed.rhs_evaluations() - evals0
    mixed.set_timing(False)
    ecg = ecg_timing(L, mixed)
    iters, corrs = [], []
    for _ in range(5):
        mixed.step(LV_DT)
        it = mixed.stats()[2]
        iters.append(int(it.sum()))
        corrs.append(int(it.size))
    fp64 = make(lib.PRECISION_FP64)
    for _ in range(1):
        fp64.step(LV_DT)
    fp64.set_timing(True)
    k64 = max(1, min(args.lv_steps, args.lv_fp64_steps))
    t_fp64 = timed_steps(fp64, k64, flush, LV_DT)
    ionic64_ms, diff64_ms, _, _ = fp64.timings()
    fp64.set_timing(False)
    window = max(args.lv_accuracy_steps, 1 + k64)
    fp64.run(LV_DT, window - 1 - k64)
    mixed_b = make(lib.PRECISION_MIXED)
    mixed_b.run(LV_DT, window)
    # (the window counts the warm-up and tuning steps of the mixed context
    # only through mixed_b, which starts from t = 0 like fp64)
    a64, amx = fp64.activation(), mixed_b.activation()
    both = (a64 > 0) & (amx > 0)
    n = L.mesh.n_cells
    out = {
        "workload": (f"TNNP endo/M/epi by transmural fraction (0-0.3/0.3-0.6/0.6-1) on a "
                     f"truncated prolate-ellipsoid LV shell (endo 25x25x60 mm, wall 10 mm, base "
                     f"z=0): {dims[0]} x ({dims[1]}^2 + 4x{dims[1]}x{dims[2]}) hexahedra x 6 = "
                     f"{n} tetrahedra; fibres +60 (endo) to -60 deg (epi), sigma_l 0.1334, "
                     f"sigma_t 0.0176 S/m per cell; apical 2 mm cube stimulus 5e4 A/m^3 x 2 ms; "
                     f"dt 1e-5 s; implicit backward ddt, Gauss linear corrected Laplacian "
                     f"(leastSquares gradient), PIMPLE residualControl 1e-6, PCG tol 1e-8 "
                     f"(FP64 PCG: the mixed form's default on corrected meshes)"),
        "cells": n, "faces": L.mesh.n_faces, "wall_faces": L.mesh.n_boundary_faces,
        "autotune": None if tune is None else {"block": tune[0], "cells_per_thread": tune[1],
                                               "ionic_ms": tune[2]},
        "mesh_seconds": t_mesh, "setup_seconds": t_setup,
        "mixed": {"value": n * args.lv_steps / t_mixed, "unit": "cell-steps/s",
                  "steps": args.lv_steps, "ms_per_step": t_mixed / args.lv_steps * 1e3,
                  "ionic_ms_per_step": ionic_ms / max(nsteps, 1),
                  "diffusion_ms_per_step": diff_ms / max(nsteps, 1),
                  "gpu_launches": launches,
                  "rhs_evaluations_per_cell_step": evals / (n * args.lv_steps),
                  "ionic_fp32_tflops": evals * (ops["flops"] + ops["transcendental"]) /
                                       (ionic_ms / 1e3) / 1e12 if ionic_ms > 0 else None,
                  "pcg_iterations_per_step": iters, "pimple_correctors_per_step": corrs},
        "fp64": {"value": n * k64 / t_fp64, "unit": "cell-steps/s", "steps": k64,
                 "ms_per_step": t_fp64 / k64 * 1e3,
                 "ionic_ms_per_step": ionic64_ms / k64, "diffusion_ms_per_step": diff64_ms / k64},
        "speedup_mixed_vs_fp64": (n * args.lv_steps / t_mixed) / (n * k64 / t_fp64),
        "accuracy": {"window_steps": window, "activated_cells": int(both.sum()),
                     "activation_flag_mismatches": int(np.sum((a64 > 0) != (amx > 0))),
                     "activation_error_ms": float(np.max(np.abs(a64[both] - amx[both])) * 1e3)
                     if both.any() else None,
                     "vm_linf_error_V": float(np.max(np.abs(fp64.vm() - mixed_b.vm())))},
        "pseudo_ecg": ecg,
        "l2": "flushed (256 MB write) between timed steps",
    }
    del mixed, mixed_b, fp64
    torch.cuda.synchronize()
    return out


def adjoint_arm(args):
    """The adjoint configuration: a 128 x 128 TNNP sheet (h = 0.25 mm),
    sigma_l = sigma_t = 0.1334 S/m at the evaluation point, corner stimulus,
    200 ms at dt 0.01 ms (5 fixed RKF45 substeps per step), per-cell log-scale
    fields of g_Na and g_K1 from a seeded smooth Gaussian random field
    (correlation 5 mm, std 0.2), 64 seeded probes sampled every 1 ms against a
    target run from a second seeded field, checkpoints every 200 steps.

    The mixed form's gradient is timed over the full 200 ms.  On a window of
    `--adjoint-check-steps` steps the FP64 form gives the reference gradient
    (mixed against it), and the FP64 gradient is checked against central
    differences of the FP64 forward at eps = 1e-6 and 1e-8 on seeded random
    directions."""
    from cardiacfoam_gb300 import api, lib
    from cardiacfoam_gb300.fields import gaussian_random_field
    from cardiacfoam_gb300.mesh import box_mesh
    nx = ny = 128
    h = 2.5e-4
    dt = 1e-5
    mesh = box_mesh(nx, ny, 1, nx * h, ny * h, h)
    rng = np.random.default_rng(2024)
    probes = rng.choice(mesh.n_cells, 64, replace=False)
    boxes = [((0.0, 0.0, 0.0), (1.5e-3, 1.5e-3, h), 0.0, 2e-3, 5e4)]
    sig = (0.1334, 0.1334)

    def fields(seed):
        return (gaussian_random_field((ny, nx), h, 5e-3, 0.2, seed).ravel(),
                gaussian_random_field((ny, nx), h, 5e-3, 0.2, seed + 1).ravel())

    def problem(steps, precision):
        return api.AdjointProblem(mesh, steps, dt, probes, 100, checkpoint_every=200,
                                  substeps=5, boxes=boxes, precision=precision)

    a, b = fields(1)
    n = mesh.n_cells
    out = {"workload": (f"TNNP epicardial sheet 128x128 (h 0.25 mm), dt 0.01 ms with 5 fixed "
                        f"RKF45 substeps, implicit Euler diffusion, PCG to 1e-13, GRF log-scales "
                        f"of g_Na and g_K1 (corr 5 mm, std 0.2), 64 probes every 1 ms against a "
                        f"second seeded field, checkpoints every 200 steps"),
           "cells": n}
    # full run, mixed form
    steps = args.adjoint_steps
    pm = problem(steps, lib.PRECISION_MIXED)
    _, target = pm.forward(*fields(7), *sig)
    pm.set_target(target)
    t0 = time.perf_counter()
    J, _ = pm.forward(a, b, *sig)
    t_f = time.perf_counter() - t0
    t0 = time.perf_counter()
    gm = pm.backward()
    t_b = time.perf_counter() - t0
    pm.close()
    out["mixed"] = {"steps": steps, "loss": J, "forward_seconds": t_f,
                    "gradient_seconds": t_f + t_b,
                    "forward_cell_steps_per_s": n * steps / t_f,
                    "gradient_cell_steps_per_s": n * steps / (t_f + t_b)}
    # check window: FP64 reference gradient and central differences
    ks = args.adjoint_check_steps
    res = {}
    for name, prec in (("fp64", lib.PRECISION_FP64), ("mixed", lib.PRECISION_MIXED)):
        p = problem(ks, prec)
        _, tgt = p.forward(*fields(7), *sig)
        p.set_target(tgt)
        t0 = time.perf_counter()
        Jc, _ = p.forward(a, b, *sig)
        tf = time.perf_counter() - t0
        t0 = time.perf_counter()
        g = p.backward()
        tb = time.perf_counter() - t0
        res[name] = (p, Jc, g, tf, tb)
    p64, J64, g64, tf64, tb64 = res["fp64"]
    _, Jmx, gmx, tfm, tbm = res["mixed"]
    res["mixed"][0].close()
    rel = lambda x, y: float(np.linalg.norm(x - y) / np.linalg.norm(y))
    checks = []
    r = np.random.default_rng(100)
    for d in range(args.adjoint_fd_directions):
        va, vb = r.standard_normal(a.size), r.standard_normal(b.size)
        vs = r.standard_normal(2) * np.array(sig)
        ad = float(g64[0] @ va + g64[1] @ vb + g64[2] @ vs)
        adm = float(gmx[0] @ va + gmx[1] @ vb + gmx[2] @ vs)
        row = {"adjoint_fp64": ad, "adjoint_mixed": adm}
        for eps in (1e-6, 1e-8):
            jp, _ = p64.forward(a + eps * va, b + eps * vb, sig[0] + eps * vs[0], sig[1] + eps * vs[1])
            jm, _ = p64.forward(a - eps * va, b - eps * vb, sig[0] - eps * vs[0], sig[1] - eps * vs[1])
            fd = (jp - jm) / (2 * eps)
            row[f"fd_eps_{eps:g}"] = fd
            row[f"rel_err_eps_{eps:g}"] = abs(ad - fd) / max(abs(fd), 1e-300)
        row["mixed_vs_fp64_rel"] = abs(adm - ad) / max(abs(ad), 1e-300)
        checks.append(row)
    p64.close()
    out["check_window"] = {
        "steps": ks, "fp64_loss": J64, "mixed_loss": Jmx,
        "fp64_gradient_seconds": tf64 + tb64, "mixed_gradient_seconds": tfm + tbm,
        "mixed_vs_fp64_gradient_rel_l2": {"log_gna": rel(gmx[0], g64[0]),
                                          "log_gk1": rel(gmx[1], g64[1]),
                                          "sigma": rel(gmx[2], g64[2])},
        "directions": checks,
        "note": ("TNNP's h and j gate rates are piecewise in Vm with a jump at -40 mV; a "
                 "perturbation that moves a stage evaluation across it changes J by a "
                 "step, which a central difference divides by 2 eps.  The adjoint is the "
                 "derivative of the smooth branches; the smaller eps makes such "
                 "crossings unlikely."),
    }
    return out


def cpu_baseline(nthreads=None, cells=(30, 30, 30), window_start=2000, steps=10):
    """The oracle (restated reference numerics) on a bounded sample of the
    workload: a 3 x 3 x 3 mm corner piece of the slab (30 x 30 x 30 cells,
    holding the stimulus box), advanced untimed to the timed window's start,
    then `steps` steps timed with OpenMP over the host's cores."""
    from oracle import pyoracle as po
    nthreads = nthreads or os.cpu_count() or 1
    nx, ny, nz = cells
    mesh = po.Mesh(nx, ny, nz, nx * H, ny * H, nz * H)
    d = po.tissue_desc("ORd", 4, SIGMA, implicit=True, precond_dic=True, pcg_tol=1e-8,
                       boxes=BOX, ode=po.ode_settings(max_steps=10 ** 6))
    T = po.Tissue(d, mesh)
    T.step(DT, nthreads)           # first step outside the timing (allocation)
    for _ in range(window_start - 1):
        T.step(DT, nthreads)
    t0 = time.perf_counter()
    for _ in range(steps):
        T.step(DT, nthreads)
    el = time.perf_counter() - t0
    n = nx * ny * nz
    return {"value": n * steps / el, "unit": "cell-steps/s", "cores": nthreads, "kind": "port",
            "sample": f"CPU oracle (reference ionic code + restated OpenFOAM numerics, DIC-PCG) "
                      f"on a {nx}x{ny}x{nz} = {n}-cell corner piece of the slab, advanced "
                      f"untimed to step {max(window_start, 1)}, then {steps} steps timed, "
                      f"{nthreads} threads"}


def reference_arm(args, rank, world):
    """The reference arm: the CPU oracle (reference ionic code + restated
    OpenFOAM numerics, DIC-PCG) with every host thread on a bounded sample of
    the slab: its corner piece of `--ref-cells` cells (by default 6 x 3.5 x
    3 mm, 63,000 cells, which holds the stimulus and the wavefront of the
    timed window), advanced untimed to the GPU arm's timed window (W warm-up
    steps end at its start), then exactly K steps timed.  The full slab
    would spend six minutes in the untimed advance alone."""
    if rank != 0:
        return None
    from oracle import build as ob
    ob.build()
    from oracle import pyoracle as po
    nthreads = os.cpu_count() or 1
    nx, ny, nz = (int(v) for v in args.ref_cells.split(","))
    mesh = po.Mesh(nx, ny, nz, nx * H, ny * H, nz * H)
    d = po.tissue_desc("ORd", 4, SIGMA, implicit=True, precond_dic=True, pcg_tol=1e-8,
                       boxes=BOX, ode=po.ode_settings(max_steps=10 ** 6))
    T = po.Tissue(d, mesh)
    k, w = args.steps, args.warmup
    window_start = max(args.window_start, w)
    t_ff = time.perf_counter()
    for _ in range(window_start - w):
        T.step(DT, nthreads)
    for _ in range(w):
        T.step(DT, nthreads)
    t_ff = time.perf_counter() - t_ff
    t0 = time.perf_counter()
    for _ in range(k):
        T.step(DT, nthreads)
    el = time.perf_counter() - t0
    value = mesh.n * k / el
    sample = (f"CPU oracle (reference ionic code + restated OpenFOAM numerics, DIC-PCG) on the "
              f"{nx}x{ny}x{nz} = {mesh.n}-cell corner piece of the slab: advanced untimed to "
              f"step {window_start} (t = "
              f"{window_start * DT * 1e3:g} ms, the last {w} of those steps as warm-up), then "
              f"{k} timed steps, {nthreads} threads")
    return {"metric": METRIC, "impl": "reference", "value": value, "unit": "cell-steps/s",
            "n_gpus": world, "steps": k, "warmup": w,
            "ms_per_step": el / k * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "cells": DIMS[0] * DIMS[1] * DIMS[2],
                       "sample_cells": mesh.n, "precision": "fp64",
                       "parallelism": "host threads", "window_start_step": window_start},
            "untimed_advance_seconds": t_ff,
            "cpu_baseline": {"value": value, "unit": "cell-steps/s", "cores": nthreads,
                             "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "cell-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def batch_population(n, seed=2024):
    """Batched single cells of the ToRORd_dynCl population: per-cell
    log-uniform scales in [0.5, 2] on GNa GCaL GKr GKs GK1 Gto, S1 cycle
    length U[300, 1000] ms, beat count U{5..50}, stimulus 53 uA/uF for 1 ms."""
    from cardiacfoam_gb300 import api
    rng = np.random.default_rng(seed)
    scales = np.exp(rng.uniform(np.log(0.5), np.log(2.0), (6, n)))
    cl = rng.uniform(300.0, 1000.0, n)
    beats = rng.integers(5, 51, n)
    stimuli = [api.stimulus_desc(10.0, float(cl[c]), 1.0, 53.0, int(beats[c])) for c in range(n)]
    return stimuli, scales, cl, beats


def batch_arm(args):
    """Batched single cells: throughput of the persistent work-stealing
    kernels on a bounded window of the 65,536-cell population (dt 0.01 ms),
    and the mixed form's APD90 / peak-Ca error against FP64 over one full
    beat of a subset (dt 0.1 ms: a lone FP64 thread integrates ToRORd_dynCl at
    GB300's FP64 rate, so full beats at 0.01 ms would take minutes)."""
    from cardiacfoam_gb300 import api, lib
    n, dt = args.batch_cells, 1e-5
    stimuli, scales, cl, beats = batch_population(n)
    out = {"workload": f"{n} ToRORd_dynCl endocardialCells single cells, per-cell scales, "
                       f"S1 CL U[300,1000] ms x U{{5..50}} beats, stimulus 53 uA/uF x 1 ms, "
                       f"dt 0.01 ms", "unit": "cell-steps/s"}
    for name, prec, window in (("mixed", lib.PRECISION_MIXED, args.batch_window),
                               ("fp64", lib.PRECISION_FP64, args.batch_window_fp64)):
        end = np.full(n, window * dt)
        b = api.BatchCells("ToRORd_dynCl", "endocardialCells", dt, stimuli, end,
                           precision=prec, scales=scales, ode=api.ode_desc(max_steps=10 ** 6),
                           chunk=window)
        t0 = time.perf_counter()
        b.run()
        el = time.perf_counter() - t0
        evals, steps, launches = b.stats()
        out[name] = {"value": steps / el, "steps_per_cell": window, "seconds": el,
                     "rhs_evaluations": evals, "launches": launches}
        b.close()
    out["speedup_mixed_vs_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    # accuracy over one beat of a subset
    m, dt_acc = args.batch_accuracy_cells, 1e-4
    stim1 = [api.stimulus_desc(10.0, float(cl[c]), 1.0, 53.0, 1) for c in range(m)]
    end = np.full(m, 0.01 + 0.5)        # one beat and 500 ms to repolarise
    res = []
    for prec in (lib.PRECISION_FP64, lib.PRECISION_MIXED):
        b = api.BatchCells("ToRORd_dynCl", "endocardialCells", dt_acc, stim1, end,
                           precision=prec, scales=scales[:, :m].copy(),
                           ode=api.ode_desc(max_steps=10 ** 6))
        b.run()
        res.append(b.results())
        b.close()
    (nb0, apd0, _, ca0), (nb1, apd1, _, ca1) = res
    ok = ~np.isnan(apd0) & ~np.isnan(apd1)
    out["accuracy"] = {
        "cells": m, "dt_s": dt_acc, "beats": 1, "window_s": 0.5,
        "apd90_max_abs_error_ms": float(np.max(np.abs(apd0[ok] - apd1[ok]))) if ok.any() else None,
        "apd90_cells_compared": int(ok.sum()),
        "apd90_fp64_range_ms": [float(np.nanmin(apd0)), float(np.nanmax(apd0))],
        "peak_ca_max_rel_error": float(np.max(np.abs(ca1 - ca0) / np.abs(ca0))),
        "beat_count_mismatches": int(np.sum(nb0 != nb1))}
    return out


def full_run_arm(args):
    """The headline slab's whole run: both forms from t = 0 through
    `--full-run-steps` steps (20,000 x 5 us = 100 ms, the configuration's
    length), compared at the end over every cell either form activated:
    activation times, Vm L-inf, flag mismatches; the mixed form's time per
    step over the whole run."""
    import torch
    from cardiacfoam_gb300 import build as gpu_build, lib
    gpu_build.build()
    mesh = build_mesh()
    n = mesh.n_cells
    steps = args.full_run_steps
    out = {"workload": WORKLOAD.split("; timed window")[0], "cells": n, "steps": steps,
           "simulated_ms": steps * DT * 1e3}
    runs = {}
    for name, prec in (("mixed", lib.PRECISION_MIXED), ("fp64", lib.PRECISION_FP64)):
        m = make_model(mesh, prec)
        s = torch.cuda.ExternalStream(m.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(s)
        m.run(DT, steps)
        e1.record(s)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        runs[name] = (m.activation(), m.vm())
        out[name] = {"seconds": ms / 1e3, "ms_per_step": ms / steps,
                     "cell_steps_per_s": n * steps / (ms / 1e3),
                     "rhs_evaluations_per_cell_step": m.rhs_evaluations() / (n * steps)}
        m.close()
    (a64, v64), (amx, vmx) = runs["fp64"], runs["mixed"]
    both = (a64 > 0) & (amx > 0)
    c = mesh.centres
    in_box = np.all((c >= np.array(BOX[0][0])) & (c <= np.array(BOX[0][1])), axis=1)
    out["accuracy"] = {
        "activated_fp64": int((a64 > 0).sum()), "activated_mixed": int((amx > 0).sum()),
        "activated_both": int(both.sum()),
        "activated_both_outside_stimulus_box": int((both & ~in_box).sum()),
        "activation_flag_mismatches": int(((a64 > 0) != (amx > 0)).sum()),
        "activation_error_ms_max": float(np.max(np.abs(a64[both] - amx[both])) * 1e3),
        "activation_error_ms_p99": float(np.percentile(np.abs(a64[both] - amx[both]), 99) * 1e3),
        "latest_activation_ms": float(np.max(a64) * 1e3),
        "vm_linf_error_V": float(np.max(np.abs(v64 - vmx)))}
    err = np.where(both, np.abs(a64 - amx), 0.0)
    worst = int(np.argmax(err))
    out["accuracy"].update({
        "cells_over_0.01_ms": int((err > 1e-5).sum()), "cells_over_0.05_ms": int((err > 5e-5).sum()),
        "worst_cell": {"centre_mm": [float(x) * 1e3 for x in c[worst]],
                       "activation_fp64_ms": float(a64[worst] * 1e3),
                       "activation_mixed_ms": float(amx[worst] * 1e3)}})
    if args.full_run_save:
        np.savez_compressed(args.full_run_save, activation_fp64=a64, activation_mixed=amx,
                            vm_fp64=v64, vm_mixed=vmx, centres=c)
    out["speedup_mixed_vs_fp64"] = out["fp64"]["seconds"] / out["mixed"]["seconds"]
    return out


def tissue_apd_arm(args):
    """APD90 of a tissue run in both forms: ORd myocyte on a 6 x 2 x 1 mm
    piece of the slab at its own h = 0.1 mm (60 x 20 x 10 = 12,000 cells; at
    h = 0.5 mm ORd does not propagate), dt 5 us, corner stimulus, 400 ms (one
    full beat and its repolarisation), per-cell beat detection on Vm every
    0.1 ms (cfg_monodomain_track_apd); mixed against FP64: APD90,
    activation times and Vm at the end."""
    from cardiacfoam_gb300 import build as gpu_build, lib, api
    from cardiacfoam_gb300.mesh import box_mesh
    gpu_build.build()
    nx, ny, nz, h = 60, 20, 10, H
    mesh = box_mesh(nx, ny, nz, nx * h, ny * h, nz * h)
    steps, every = args.tissue_apd_steps, 20
    res = {}
    for name, prec in (("fp64", lib.PRECISION_FP64), ("mixed", lib.PRECISION_MIXED)):
        m = api.Monodomain(mesh, "ORd", "myocyte", SIGMA, dt=DT, precision=prec, boxes=BOX,
                           max_steps=10 ** 6)
        m.track_apd(every)
        t0 = time.perf_counter()
        m.run(DT, steps)
        nb, apd, tup = m.apd_results()
        res[name] = {"seconds": time.perf_counter() - t0, "beats": nb, "apd": apd,
                     "act": m.activation(), "vm": m.vm()}
        m.close()
    f, x = res["fp64"], res["mixed"]
    ok = ~np.isnan(f["apd"]) & ~np.isnan(x["apd"])
    both = (f["act"] > 0) & (x["act"] > 0)
    return {"workload": (f"ORd myocyte slab 6x2x1 mm at h 0.1 mm ({mesh.n_cells} cells), dt 5 us, "
                         f"{steps * DT * 1e3:g} ms, corner stimulus 5e4 A/m^3 x 2 ms; per-cell "
                         f"APD90 from Vm sampled every {every * DT * 1e3:g} ms"),
            "fp64_seconds": f["seconds"], "mixed_seconds": x["seconds"],
            "apd90_cells_compared": int(ok.sum()),
            "apd90_fp64_range_ms": [float(np.nanmin(f["apd"])), float(np.nanmax(f["apd"]))],
            "apd90_max_abs_error_ms": float(np.max(np.abs(f["apd"][ok] - x["apd"][ok])))
            if ok.any() else None,
            "beat_count_mismatches": int(np.sum(f["beats"] != x["beats"])),
            "activation_error_ms": float(np.max(np.abs(f["act"][both] - x["act"][both])) * 1e3)
            if both.any() else None,
            "activated_cells": int(both.sum()),
            "vm_linf_error_V": float(np.max(np.abs(f["vm"] - x["vm"])))}


def batch_apd_arm(args):
    """Last-beat APD90 and peak Ca of the batched ToRORd_dynCl population at
    the configuration's own dt (0.01 ms) over each cell's whole protocol, in
    both forms, for the `--batch-apd-cells` cells of the 65,536 with the
    shortest protocols (beats x cycle length): a lone FP64 thread integrates
    ToRORd_dynCl at GB300's FP64 rate, so the whole population in FP64 would
    take hours."""
    from cardiacfoam_gb300 import build as gpu_build, api, lib
    gpu_build.build()
    n_all, dt = args.batch_cells, 1e-5
    stimuli, scales, cl, beats = batch_population(n_all)
    length = (10.0 + cl * beats) * 1e-3 + 0.5           # s: the protocol and 500 ms after it
    pick = np.argsort(length, kind="stable")[:args.batch_apd_cells]
    st = [stimuli[int(c)] for c in pick]
    end = length[pick].copy()
    res = {}
    for name, prec in (("fp64", lib.PRECISION_FP64), ("mixed", lib.PRECISION_MIXED)):
        b = api.BatchCells("ToRORd_dynCl", "endocardialCells", dt, st, end, precision=prec,
                           scales=scales[:, pick].copy(), ode=api.ode_desc(max_steps=10 ** 6))
        t0 = time.perf_counter()
        b.run()
        res[name] = (time.perf_counter() - t0,) + tuple(b.results())
        b.close()
    (t64, nb0, apd0, _, ca0), (tmx, nb1, apd1, _, ca1) = res["fp64"], res["mixed"]
    ok = ~np.isnan(apd0) & ~np.isnan(apd1)
    return {"workload": (f"the {pick.size} ToRORd_dynCl endocardialCells cells of the {n_all}-cell "
                         f"population with the shortest protocols (per-cell scales, S1 CL "
                         f"U[300,1000] ms x U{{5..50}} beats from 10 ms, stimulus 53 uA/uF x 1 ms, "
                         f"+500 ms), dt 0.01 ms, whole protocols"),
            "simulated_s_per_cell": [float(end.min()), float(end.max())],
            "beats_per_cell": [int(beats[pick].min()), int(beats[pick].max())],
            "fp64_seconds": t64, "mixed_seconds": tmx,
            "apd90_cells_compared": int(ok.sum()),
            "apd90_fp64_range_ms": [float(np.nanmin(apd0)), float(np.nanmax(apd0))],
            "apd90_max_abs_error_ms": float(np.max(np.abs(apd0[ok] - apd1[ok]))) if ok.any() else None,
            "peak_ca_max_rel_error": float(np.nanmax(np.abs(ca1 - ca0) / np.abs(ca0))),
            "beat_count_mismatches": int(np.sum(nb0 != nb1))}


def mms_arm():
    """Manufactured-solution convergence of the FP64 step on GPU: the 3D
    monodomainFDAManufactured case over the tutorial's sweep (10/20/40/80
    cells per direction, dt shrinking with h^2, to t = 0.2 s)."""
    from cardiacfoam_gb300 import verification as vf
    rows = []
    for n in (10, 20, 40, 80):
        t0 = time.perf_counter()
        r = vf.run(3, n)
        rows.append({"n": n, "dt": r["dt"], "steps": r["steps"],
                     "seconds": time.perf_counter() - t0,
                     "V_L1": r["V"][0], "V_L2": r["V"][1], "V_Linf": r["V"][2],
                     "u1_Linf": r["u1"][2], "u2_Linf": r["u2"][2]})
    rates = [{"n": (a["n"], b["n"]),
              "V_Linf": vf.rate(a["V_Linf"], b["V_Linf"], a["n"], b["n"]),
              "V_L2": vf.rate(a["V_L2"], b["V_L2"], a["n"], b["n"])}
             for a, b in zip(rows, rows[1:])]
    return {"case": "3D unit cube, sigma diag(0.1115, 0.1216, 0.0304), chi 3, Cm 2, "
                    "backward ddt, 2 correctors, PCG tol 1e-12, t = 0.2 s",
            "errors": rows, "rates": rates}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--fp64-steps", type=int, default=12)
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--window-start", type=int, default=2000,
                    help="step at which the timed window starts (2000 x 5 us = 10 ms: the "
                         "wavefront inside the slab); the FP64 and mixed forms are compared "
                         "at the window's end")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched single cells")
    ap.add_argument("--no-mms", action="store_true", help="skip the manufactured-solution sweep")
    ap.add_argument("--no-lv", action="store_true", help="skip the left-ventricle configuration")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint configuration")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the ionic kernels' default launch shape")
    ap.add_argument("--adjoint-only", action="store_true")
    ap.add_argument("--adjoint-steps", type=int, default=20000)
    ap.add_argument("--adjoint-fd-directions", type=int, default=2)
    ap.add_argument("--adjoint-check-steps", type=int, default=2000)
    ap.add_argument("--no-bidomain", action="store_true", help="skip the bidomain case")
    ap.add_argument("--bidomain-only", action="store_true")
    ap.add_argument("--bidomain-cells", type=int, default=40)
    ap.add_argument("--bidomain-steps", type=int, default=20)
    ap.add_argument("--bidomain-sample", type=int, default=3)
    ap.add_argument("--ecg-only", action="store_true",
                    help="time the pseudo-ECG kernel alone on the LV mesh (--lv-dims)")
    ap.add_argument("--ecg-launches", type=int, default=50)
    ap.add_argument("--lv-only", action="store_true",
                    help="run only the left-ventricle configuration (profiling)")
    ap.add_argument("--lv-dims", default="",
                    help="nt,m,nr of the LV mesh (default: the 4.0 M-tet configuration)")
    ap.add_argument("--lv-steps", type=int, default=20)
    ap.add_argument("--lv-pcg", default="default", choices=["default", "fp64", "pairs"],
                    help="PCG arithmetic of the LV's mixed form (default: the library's)")
    ap.add_argument("--lv-fp64-steps", type=int, default=3)
    ap.add_argument("--lv-accuracy-steps", type=int, default=250)
    ap.add_argument("--batch-cells", type=int, default=65536)
    ap.add_argument("--batch-window", type=int, default=2000,
                    help="solver steps per cell timed for the mixed batch")
    ap.add_argument("--batch-window-fp64", type=int, default=100)
    ap.add_argument("--batch-accuracy-cells", type=int, default=256)
    ap.add_argument("--no-graph", action="store_true",
                    help="host-driven PIMPLE/PCG loops instead of the step graph")
    ap.add_argument("--full-run", action="store_true",
                    help="only the whole 100 ms run of both forms and their comparison")
    ap.add_argument("--ref-cells", default="60,35,30",
                    help="corner piece of the slab the reference arm runs on (nx,ny,nz)")
    ap.add_argument("--full-run-steps", type=int, default=20000)
    ap.add_argument("--full-run-save", default=None,
                    help="write both forms' activation times and Vm (npz) to this path")
    ap.add_argument("--tissue-apd", action="store_true",
                    help="only the tissue APD90 comparison of both forms (reduced ORd slab)")
    ap.add_argument("--tissue-apd-steps", type=int, default=80000)
    ap.add_argument("--batch-apd", action="store_true",
                    help="only the batched cells' APD90 over whole protocols, both forms")
    ap.add_argument("--batch-apd-cells", type=int, default=304)
    args = ap.parse_args()
    global GRAPH
    GRAPH = not args.no_graph
    if args.warmup < 3 and args.impl == "gb300":
        args.warmup = 3
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch
        backend = "nccl" if args.impl == "gb300" else "gloo"
        torch.distributed.init_process_group(backend)
    if args.impl == "reference":
        out = reference_arm(args, rank, world)
        if out is not None:
            print(json.dumps(out), flush=True)
        return
    if args.full_run:
        print(json.dumps({"full_run": full_run_arm(args)}), flush=True)
        return
    if args.tissue_apd:
        print(json.dumps({"tissue_apd": tissue_apd_arm(args)}), flush=True)
        return
    if args.batch_apd:
        print(json.dumps({"batch_apd": batch_apd_arm(args)}), flush=True)
        return
    if args.adjoint_only:
        from cardiacfoam_gb300 import build as gpu_build
        gpu_build.build()
        print(json.dumps({"adjoint": adjoint_arm(args)}), flush=True)
        return
    if args.bidomain_only:
        from cardiacfoam_gb300 import build as gpu_build
        gpu_build.build()
        print(json.dumps({"bidomain": bidomain_arm(args)}), flush=True)
        return
    if args.ecg_only:
        from cardiacfoam_gb300 import build as gpu_build
        gpu_build.build()
        print(json.dumps({"pseudo_ecg": ecg_arm(args)}), flush=True)
        return
    if args.lv_only:
        import torch
        from cardiacfoam_gb300 import build as gpu_build
        gpu_build.build()
        flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
        print(json.dumps({"left_ventricle": lv_arm(args, flush)}), flush=True)
        return
    r = gpu_arm(args, rank, world)
    if rank != 0:
        return
    n = r["n"]
    value = whole_job_value(n, args.steps, world, r["t_mixed"])
    fp64_value = n * r["k64"] / r["t_fp64"]
    e2e_value = n * r["ke2e"] / r["t_e2e"]
    ionic_s = r["ionic_ms"] / 1e3
    out = {
        "metric": METRIC, "value": value, "unit": "cell-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": r["t_mixed"] / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64 (mixed)",
        "data": "synthetic (seeded geometry/stimulus of the ORd slab configuration)",
        "config": {"workload": WORKLOAD, "cells": n, "dt_s": DT, "precision": "mixed",
                   "pcg": "float pairs (FP32 pipe, about 48 significant bits); FP64 source",
                   "l2": "flushed (256 MB write) between timed steps",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "fp64": {"value": fp64_value, "unit": "cell-steps/s", "steps": r["k64"],
                 "ms_per_step": r["t_fp64"] / r["k64"] * 1e3,
                 "ionic_ms_per_step": r["ionic64_ms"] / r["k64"],
                 "diffusion_ms_per_step": r["diff64_ms"] / r["k64"]},
        "speedup_vs_fp64": value / world / fp64_value,
        "timed_window": {"start_step": r["window_start"], "start_time_s": r["window_start"] * DT,
                         "steps": args.steps,
                         "rhs_evaluations_per_cell_step": r["evals"] / (n * args.steps)},
        "rest_window": {"start_step": r["rest"]["start_step"], "steps": args.steps,
                        "value": n * args.steps / r["rest"]["t"], "unit": "cell-steps/s",
                        "ms_per_step": r["rest"]["t"] / args.steps * 1e3,
                        "phases_ms_per_step": {"ionic": r["rest"]["ionic_ms"] / args.steps,
                                               "diffusion": r["rest"]["diff_ms"] / args.steps},
                        "rhs_evaluations_per_cell_step":
                            r["rest"]["evals"] / (n * args.steps)},
        "accuracy": {"compared_at_step": r["compared_at_step"],
                     "compared_at_time_s": r["compared_at_time"],
                     "activation_error_ms": r["act_err_ms"],
                     "activated_cells_compared": r["act_cells"],
                     "activated_cells_outside_stimulus_box": r["act_cells_outside_box"],
                     "activation_flag_mismatches": r["act_mismatch"],
                     "vm_linf_error_V": r["vm_err"]},
        "phases_ms_per_step": {"ionic": r["ionic_ms"] / args.steps,
                               "diffusion": r["diff_ms"] / args.steps},
        "e2e": {"value": e2e_value, "unit": "cell-steps/s", "h2d_bytes_per_step": 8 * n,
                "d2h_bytes_per_step": 8 * n, "steps": r["ke2e"],
                "path": "cfg_monodomain_set_field(Vm) + cfg_monodomain_step + "
                        "cfg_monodomain_get_field(Vm), pinned host buffers"},
        "roofline": {"bound": "fp32", "kernel": "ionic_mixed_kernel<ORd, tissue 4>",
                     "achieved": r["achieved"], "peak": r["fp32_peak"], "unit": "TFLOP/s",
                     "frac": r["achieved"] / r["fp32_peak"],
                     "traffic": IONIC_TRAFFIC_BYTES, "traffic_unit": "bytes per launch",
                     "traffic_source": IONIC_TRAFFIC_SOURCE,
                     "algorithmic_bytes": IONIC_STATE_BYTES * n,
                     "work": f"{r['evals']} RHS evaluations: executed {r['executed_ops']:.4g} "
                             f"operations (stage loop {opcounts()['ORd']['flops'] - opcounts()['ORd']['invariant_flops']:.0f} FLOP + "
                             f"{opcounts()['ORd']['transcendental'] - opcounts()['ORd']['invariant_transcendental']:.0f} "
                             f"transcendental per evaluation, the membrane-potential-only "
                             f"{opcounts()['ORd']['invariant_flops']:.0f} + "
                             f"{opcounts()['ORd']['invariant_transcendental']:.0f} once per cell-step)",
                     "reference_equivalent_tflops": r["reference_equivalent"],
                     "reference_equivalent_work": f"{opcounts()['ORd']['flops']:.0f} FLOP + "
                             f"{opcounts()['ORd']['transcendental']:.0f} transcendental per "
                             f"evaluation, as the reference's body evaluates them",
                     "peak_source": f"152 SMs x 128 FP32 lanes x 2 x {r['peaks'].get('sm_max_mhz')} "
                                    f"MHz (MEASURED_PEAKS.json sm_max_mhz, {r['peak_src']}); "
                                    "no FP32 figure is measured"},
        "gpu_launches": r["launches"],
        "clocks": r["clocks"],
        "autotune": {k: (None if v is None else {"block": v[0], "cells_per_thread": v[1],
                                                 "ionic_ms": v[2]})
                     for k, v in r["autotune"].items()},
    }
    if not args.no_lv:
        import torch
        flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
        out["left_ventricle"] = lv_arm(args, flush)
        del flush
    if not args.no_batch:
        out["batched_single_cells"] = batch_arm(args)
    if not args.no_adjoint:
        out["adjoint"] = adjoint_arm(args)
    if not args.no_mms:
        out["manufactured_solution"] = mms_arm()
    if not args.no_bidomain:
        out["bidomain"] = bidomain_arm(args)
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(window_start=args.window_start)
        # one thread: a 10 x 70 x 30 piece timed from t = 0 (the advance to the
        # wavefront window would take minutes on one core)
        one = cpu_baseline(nthreads=1, cells=(10, 70, 30), window_start=0, steps=5)
        out["cpu_baseline"]["single_thread"] = {k: one[k] for k in ("value", "cores", "sample")}
        import platform
        cpu = platform.processor() or platform.machine()
        try:
            with open("/proc/cpuinfo") as fh:
                for line in fh:
                    if line.lower().startswith(("model name", "cpu part")):
                        cpu = line.split(":", 1)[1].strip()
                        break
        except OSError:
            pass
        out["cpu_baseline"]["cpu"] = f"{cpu}, nproc {os.cpu_count()}"
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
