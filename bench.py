"""Benchmark of the residual-and-timestep path on GB300.

Workload (the plain large configuration): steady 2D Euler flow past a cylinder
on a 512 (radial) x 1024 (circumferential) O-grid, radius 0.5 to 20 with
geometric radial stretching 1.01, freestream Mach 0.3; Roe flux, MUSCL with
the van Albada limiter, least-squares gradients, ssp34 with local timestepping
at CFL 0.5, FP64.  One step = one full RK step (4 stages) over all cells;
the metric is cell-updates/s (cells x steps / s).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Under torchrun (N > 1) every rank advances its own replica of the workload
(the path does not shard; replicas only) and value is the whole-job total.
--impl reference times the reference algorithm's CPU implementation (the
OpenMP oracle port built with the reference's flags) on the host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-updates/s (MUSCL+Roe+RK)"
UNIT = "cell-updates/s"
NR, NTH, MACH = 512, 1024, 0.3
FLUX, LIMITER, RKT, DTMODE, CFL = "roe", "vanalbada", "ssp34", "local", 0.5
NSTAGES = 4
# algorithmic bytes per cell per RK stage: read q_stage, read q0, write q_next
# (3 x 4 values) + 2 geometry values, in FP64
ALG_BYTES_PER_CELL_STAGE = (3 * 4 + 2) * 8
L2_BYTES = 129 * 2 ** 20
PROFILE_TRAFFIC = os.path.join(ROOT, "profiles", "stage_kernel_fp64_ogrid.md")


def workload_config():
    """The workload's description, identical on both arms of the benchmark."""
    ncell = NR * NTH
    ws = (3 * 4 + 3 * 5) * 8 * ncell / 2 ** 20 + 2 * 14 * 8 * ncell / 2 ** 20
    return {"workload": f"cylinder O-grid {NR}x{NTH}, r 0.5..20, stretch 1.01, M{MACH}",
            "cells": ncell, "flux": FLUX, "limiter": LIMITER, "gradients": "lsq", "rk": RKT,
            "dt": DTMODE, "cfl": CFL, "precision": "fp64", "step": "one RK step (4 stages) over all cells",
            "l2": f"no flush: per-step working set {ws:.0f} MiB > {L2_BYTES / 2 ** 20:.0f} MiB L2"}


def oracle_cylinder(nr: int, nth: int, mach: float, rc: float = 0.5, rb: float = 20.0, stretch: float = 1.01):
    """The O-grid workload built by the oracle alone (its own make_cylinder_mesh), so that
    the CPU arm loads nothing of the product: nodes, boundary types, far-field reference,
    uniform freestream state, species (rho 1, p 1/gamma, velocity (mach, 0))."""
    from oracle import oracle_py
    nodes = oracle_py.pointwise(fast=True).cylinder_nodes(nr, nth, rc, rb, stretch)
    qinf = np.array([mach, 0.0, 1.0, 1.0 / 1.4])
    q = np.broadcast_to(qinf[:, None, None], (4, nr, nth)).copy()
    ref = [None, np.broadcast_to(qinf[:, None], (4, nth)).copy(), None, None]
    return nodes, ["wall", "riemann", "periodic", "periodic"], ref, q, (1.4, 287.058, mach)


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_value(key: str):
    """A figure recorded in the committed FP64 stage-kernel summary, if any."""
    if not os.path.exists(PROFILE_TRAFFIC):
        return None
    for line in open(PROFILE_TRAFFIC):
        if line.startswith(key + ":"):
            return float(line.split(":", 1)[1].split()[0])
    return None


def profiled_traffic_per_cell():
    """dram bytes per cell per stage launch from the committed ncu summary, if any."""
    return profile_value("traffic_bytes_per_cell_stage")


def fp64_peak_tflops(n: int = 4096, reps: int = 5):
    """FP64 peak measured here: a float64 GEMM through cuBLAS (2 n^3 per call), best
    of `reps`, CUDA events."""
    import torch
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    best = None
    for _ in range(reps):
        e0, e1 = _events()
        torch.cuda.synchronize()
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        best = ms if best is None else min(best, ms)
    del a, b
    return 2.0 * n ** 3 / (best / 1e3) / 1e12


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 20 ms while the context is
    open (the bench opens it before the warm-up and closes it after the timed region)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.path = os.path.join("/tmp", f"hc_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def wait_first(self, timeout_s: float = 3.0):
        """Block until the sampler has written its first sample (nvidia-smi takes a moment
        to start), at most timeout_s, so that the samples cover what follows."""
        t0 = time.perf_counter()
        while self.proc is not None and time.perf_counter() - t0 < timeout_s:
            if os.path.exists(self.path) and os.path.getsize(self.path) > 0:
                return
            time.sleep(0.01)

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
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
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "samples": len(sm),
                "reasons": sorted(reasons), "window": "the warm-up and the timed region, 20 ms samples"}


def cpu_baseline(sample_s: float = 4.0, samples: int = 3, threads: int | None = None):
    """The reference algorithm on the host cores: OpenMP oracle port built with the
    reference's flags (-O3 -ffast-math -fopenmp), `samples` timed samples of about
    `sample_s` seconds each (at most 200 RK steps) of the same workload; the median."""
    from oracle import oracle_py
    threads = threads or os.cpu_count() or 1
    os.environ.setdefault("OMP_PROC_BIND", "close")
    lib = oracle_py.load(fast=True)
    lib.hco_set_threads(int(threads))
    nodes, bc, ref, q, species = oracle_cylinder(NR, NTH, MACH)
    o = oracle_py.OracleSolver(NR, NTH, nodes, bc, flux=FLUX, limiter=LIMITER, rk=RKT, dt=DTMODE, cfl=CFL,
                               species=species, ghost_ref=ref, fast=True)
    o.set_state(q)
    o.step(1)  # warm-up (first touch of the arrays)
    rates, steps = [], []
    for _ in range(samples):
        n, t0 = 0, time.perf_counter()
        while True:
            o.step(1)
            n += 1
            el = time.perf_counter() - t0
            if el >= sample_s or n >= 200:
                break
        rates.append(NR * NTH * n / el)
        steps.append(n)
    v = statistics.median(rates)
    return {"value": v, "unit": UNIT, "cores": int(lib.hco_get_threads()), "kind": "port",
            "samples": rates,
            "sample": f"median of {samples} samples of {min(steps)}-{max(steps)} RK steps of the {NR}x{NTH} "
                      f"O-grid workload (~{sample_s:.0f} s each), OpenMP oracle port, -O3 -ffast-math -fopenmp"}


def _events():
    import torch
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def measure_precision(stream, steps: int, prec: str):
    """The same workload at another precision ("fp32": everything FP32; "fp64_df":
    FP64 storage with double-float stage arithmetic): throughput, HBM roofline
    and the relative L-inf difference of the conserved quantities from FP64 after
    one step and after 20 steps from the same start (the two momentum components
    against the momentum scale: one step from the uniform freestream the normal
    momentum is still small)."""
    import torch
    from hyperboliconvergence_gb300 import cases
    from hyperboliconvergence_gb300.solver import Solver
    mesh, bc, ref, q, species = cases.cylinder(NR, NTH, mach=MACH)
    out = {}
    states = {}
    for p in (prec, "fp64"):
        s = Solver(mesh, bc, ref, flux=FLUX, limiter=LIMITER, rk=RKT, precision=p, dt=DTMODE, cfl=CFL,
                   species=species, stream=stream.cuda_stream)
        s.set_state(q)
        s.step(3)
        if p == prec:
            e0, e1 = _events()
            torch.cuda.synchronize()
            e0.record(stream)
            s.step_async(steps)
            e1.record(stream)
            s.sync()
            ms = e0.elapsed_time(e1) / steps
            cells = NR * NTH
            stage_ms = ms / NSTAGES
            esz = 4 if prec == "fp32" else 8
            ach = (3 * 4 + 2) * esz * cells / (stage_ms / 1e3) / 1e9
            peak, _ = measured_peaks()
            out = {"value": cells / (ms / 1e3), "unit": UNIT, "ms_per_step": ms,
                   "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                                "frac": ach / peak, "alg_bytes_per_cell_stage": 14 * esz}}
            # the step's buffers (3 states, 4 stage residuals, the face records, volumes): in
            # FP32 about the size of L2, so the back-to-back steps above reuse what L2 holds;
            # the same steps again, each after a write of twice L2's size, time them cold
            ws = (3 * 4 + 4 * 5 + 2 * 14 + 1) * esz * cells / 2 ** 20
            flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
            cold = 0.0
            for _ in range(steps):
                with torch.cuda.stream(stream):
                    flush.zero_()
                e0, e1 = _events()
                e0.record(stream)
                s.step_async(1)
                e1.record(stream)
                s.sync()
                torch.cuda.synchronize()
                cold += e0.elapsed_time(e1)
            del flush
            out["l2"] = (f"back-to-back steps, no flush: the step's buffers take {ws:.0f} MiB against "
                         f"{L2_BYTES / 2 ** 20:.0f} MiB of L2")
            out["l2_flushed"] = {"value": cells / (cold / steps / 1e3), "unit": UNIT, "ms_per_step": cold / steps,
                                 "how": "L2 flushed (a write of twice its size) before each timed step"}
        s.set_state(q)
        s.step(1)
        one = s.get_state()
        s.step(19)
        states[p] = (one, s.get_state())
        s.close()
    g = 1.4

    def cons(w):
        u, v, r, p = w
        return np.stack([r * u, r * v, r, p / (g - 1) + 0.5 * r * (u * u + v * v)])

    def rel(a, b):
        # relative L-inf per conserved quantity: mass, momentum (both components
        # against the momentum scale), energy
        ca, cb = cons(a), cons(b)
        err = np.abs(ca - cb).reshape(4, -1).max(1)
        scale = np.abs(cb).reshape(4, -1).max(1)
        scale[0:2] = scale[0:2].max()
        return float((err / scale).max())
    out["error_vs_fp64_after_1_step"] = rel(states[prec][0], states["fp64"][0])
    out["error_vs_fp64_after_20_steps"] = rel(states[prec][1], states["fp64"][1])
    # branch flips: the FP64 state after 20 steps evaluated at both precisions
    from hyperboliconvergence_gb300.solver import branch_flips
    sigs = {}
    for p in (prec, "fp64"):
        s = Solver(mesh, bc, ref, flux=FLUX, limiter=LIMITER, rk=RKT, precision=p, dt=DTMODE, cfl=CFL,
                   species=species, stream=stream.cuda_stream)
        s.set_state(states["fp64"][1])
        sigs[p] = s.face_signatures(with_args=(p == "fp64"))
        s.close()
    out["branch_flips_vs_fp64"] = branch_flips(sigs[prec], sigs["fp64"][0], args=sigs["fp64"][1],
                                               limiter=LIMITER) | {
        "state": "the FP64 state after 20 steps, evaluated at both precisions",
        "faces_above_roundoff_means": "flips whose FP64 limiter arguments are more than 1e-9 of the variable's "
                                "scale from a breakpoint (the others are round-off arguments, zero in "
                                "exact arithmetic)"}
    return out


def _time_batch(stream, insts, steps, precision="fp32"):
    import torch
    from hyperboliconvergence_gb300.batch import Batch
    b = Batch(insts, flux="slau", limiter="vanalbada", rk="ssp34", precision=precision, dt="global", cfl=0.5,
              stream=stream.cuda_stream)
    cells = b.cells
    tuned = b.autotune(steps=1)
    res = {"instances": len(insts), "cells": cells, "schedule": tuned}
    b.capture(steps)
    b.replay()
    b.sync()
    for mode in ("graph", "per_instance"):
        e0, e1 = _events()
        torch.cuda.synchronize()
        e0.record(stream)
        if mode == "graph":
            b.replay()
        else:
            b.step_async(steps, "per_instance")
        e1.record(stream)
        b.sync()
        ms = e0.elapsed_time(e1) / steps
        res[mode] = {"ms_per_step": ms, "value": cells / (ms / 1e3), "unit": UNIT}
    res["batched_over_per_instance"] = res["per_instance"]["ms_per_step"] / res["graph"]["ms_per_step"]
    b.close()
    return res


def measure_batched(stream, ninst: int = 256, steps: int = 3, seed: int = 2026):
    """The uneven batch: 256 four-quadrant Riemann instances, Ni, Nj from {64,96,...,1024},
    SLAU + van Albada, ssp34, global dt per instance, FP32.  Persistent batched launches
    replayed from a CUDA graph against plain per-instance launches.  Beside it, a
    launch-bound batch of 1024 small instances (Ni, Nj from {16,32,...,128}), where
    per-instance launches cannot fill the GPU."""
    from hyperboliconvergence_gb300.batch import uneven_riemann_batch
    insts = uneven_riemann_batch(ninst, seed)
    res = _time_batch(stream, insts, steps)
    res["small_instances"] = _time_batch(stream, uneven_riemann_batch(1024, seed, sizes=tuple(range(16, 129, 16))),
                                         steps)
    res["accuracy"] = _batch_accuracy(insts)
    return res


def _batch_accuracy(insts, steps: int = 200, nsub: int = 8):
    """The configuration's 200 steps on the first `nsub` instances of the batch in FP32 and
    in FP64 (whose parity with the CPU oracle the tests hold): the largest relative L-inf
    difference of the conserved variables, per variable against its own scale."""
    from hyperboliconvergence_gb300.batch import Batch
    g = 1.4

    def cons(w):
        u, v, r, p = w
        return np.stack([r * u, r * v, r, p / (g - 1) + 0.5 * r * (u * u + v * v)])

    def rel(a, b):
        ca, cb = cons(a), cons(b)
        return float((np.abs(ca - cb).reshape(4, -1).max(1) / np.abs(cb).reshape(4, -1).max(1)).max())

    sub = insts[:nsub]
    states = {}
    for prec in ("fp32", "fp64"):
        b = Batch(sub, flux="slau", limiter="vanalbada", precision=prec)
        b.step_async(steps)
        b.sync()
        states[prec] = [b.get_state(k) for k in range(len(sub))]
        b.close()
    def rel1(a, b):
        ca, cb = cons(a), cons(b)
        return float((np.abs(ca - cb).reshape(4, -1).sum(1) / np.abs(cb).reshape(4, -1).sum(1)).max())

    pairs = list(zip(states["fp32"], states["fp64"]))
    return {"steps": steps, "instances": len(sub), "cells": int(sum(m.ni * m.nj for m, *_ in sub)),
            "fp32_vs_fp64_max_rel_linf": max(rel(x, y) for x, y in pairs),
            "fp32_vs_fp64_max_rel_l1": max(rel1(x, y) for x, y in pairs),
            "note": "the shocks and contacts of the quadrant problems move by round-off-sized amounts "
                    "between precisions, so the pointwise (L-inf) difference at a discontinuity is O(1) "
                    "of its jump; the L1 difference measures the solution error"}


def measure_vortex(stream):
    """The isentropic-vortex configuration (periodic [0,10]^2, 128^2, Roe, MUSCL + van Leer,
    LSQ, ssp34, CFL 0.5 global dt, FP64, 100 steps): cell-updates/s, and the L1 / L-inf
    error of the conserved variables against the exact vortex translated by (t, t) at
    t = 4 sum(dt); with the reference's Roe flux and with the face-frame one, and for the
    face-frame flux the observed orders over 64^2 / 128^2 / 256^2 (50 / 100 / 200 steps).
    Parity with the CPU oracle at steps 1, 50 and 100 is held by the tests."""
    import torch
    from hyperboliconvergence_gb300 import HCError, cases
    from hyperboliconvergence_gb300.solver import Solver
    g = 1.4

    def cons(w):
        u, v, r, p = w
        return np.stack([r * u, r * v, r, p / (g - 1) + 0.5 * r * (u * u + v * v)])

    states = {}

    def run(n, steps, flux, timed=False, precision="fp64"):
        mesh, bc, ref, q, sp = cases.isentropic_vortex(n)
        s = Solver(mesh, bc, ref, flux=flux, limiter="vanleer", rk="ssp34", dt="global", cfl=0.5, species=sp,
                   stream=stream.cuda_stream, precision=precision)
        s.set_state(q)
        res = {}
        try:
            if timed:
                s.step(3)
                s.set_state(q)
                s.set_time(0.0, 0)
                e0, e1 = _events()
                torch.cuda.synchronize()
                e0.record(stream)
                s.step_async(steps)
                e1.record(stream)
                st = s.sync()
                ms = e0.elapsed_time(e1)
                res.update(value=n * n * steps / (ms / 1e3), unit=UNIT, ms_per_step=ms / steps)
            else:
                st = s.step(steps)
        except HCError as exc:
            s.close()
            return {"error": str(exc)}
        c = mesh.centres()
        states[(n, flux, precision)] = cons(s.get_state())
        e = np.abs(cons(s.get_state()) - cons(cases.vortex_state(c[0], c[1], 4.0 * st.t)))
        res.update(t_physical=4.0 * st.t, l1=[float(x) for x in e.reshape(4, -1).mean(1)],
                   linf=[float(x) for x in e.reshape(4, -1).max(1)])
        s.close()
        return res

    out = {"grid": "128x128", "steps": 100, "flux_reference": run(128, 100, "roe", timed=True),
           "flux_face_frame": run(128, 100, "roe_face", timed=True)}
    conv = {n: run(n, k, "roe_face") for n, k in ((64, 50), (128, 100), (256, 200))}
    ref256 = run(256, 200, "roe")
    if all("l1" in v for v in conv.values()):
        out["face_frame_orders"] = {
            f"{a}->{b}": {"l1": [float(np.log2(x / y)) for x, y in zip(conv[a]["l1"], conv[b]["l1"])],
                          "linf": [float(np.log2(x / y)) for x, y in zip(conv[a]["linf"], conv[b]["linf"])]}
            for a, b in ((64, 128), (128, 256))}
    out["reference_roe_256"] = ref256
    # FP32: the same 100 steps, against the FP64 run (per variable, relative to its largest magnitude)
    out["fp32_face_frame"] = run(128, 100, "roe_face", timed=True, precision="fp32")
    a, b = states.get((128, "roe_face", "fp32")), states.get((128, "roe_face", "fp64"))
    if a is not None and b is not None:
        d = np.abs(a - b).reshape(4, -1)
        scale = np.abs(b).reshape(4, -1).max(1)
        out["fp32_vs_fp64_after_100_steps"] = {"rel_linf": float((d.max(1) / scale).max()),
                                               "rel_mean": float((d.mean(1) / scale).max())}
    return out


def measure_steady(stream, steps: int = 2000, fluxes=("roe_face", "slau", "ausmpup"), machs=(0.3, 0.8)):
    """The steady O-grid configuration: from the uniform freestream, local timestepping at
    CFL 0.5 (ssp34, MUSCL + van Albada, LSQ) towards a density-residual drop of 1e-10, with
    a cap of `steps` steps, for each flux at M 0.3 and 0.8 in FP64 and FP32.  The runs take
    the corrections of the reference's defects (the face-frame Roe dissipation, the 1/0
    MachSplit_P1, the far fields' outflow test); one run of the reference's own Roe flux and
    far field, uncorrected, is reported beside them.  Per run: steps, residual drop, whether
    1e-10 was reached, ms per step, the drag coefficient C_d = F_x / (rho U^2 / 2 * 2 r_c)
    of the final state, and the FP32 state's relative L-inf / L1 difference from FP64."""
    import torch
    from hyperboliconvergence_gb300 import HCError, cases
    from hyperboliconvergence_gb300.solver import Solver
    g = 1.4

    def cons(w):
        u, v, r, p = w
        return np.stack([r * u, r * v, r, p / (g - 1) + 0.5 * r * (u * u + v * v)])

    def one(mach, flux, prec, corr):
        mesh, bc, ref, q, species = cases.cylinder(NR, NTH, mach=mach)
        s = Solver(mesh, bc, ref, flux=flux, limiter=LIMITER, rk=RKT, precision=prec, dt=DTMODE, cfl=CFL,
                   species=species, stream=stream.cuda_stream, corrections=corr)
        s.set_state(q)
        e0, e1 = _events()
        torch.cuda.synchronize()
        e0.record(stream)
        try:
            st, hist = s.steady(steps, residual_drop=1e-10, check_every=max(1, steps // 20))
            ok = True
        except HCError as exc:
            ok = False
            err = str(exc)
        e1.record(stream)
        torch.cuda.synchronize()
        if not ok:
            s.close()
            return {"error": err, "steps_before_failure": s.steps_done}, None
        res = {"steps": int(st.steps), "residual_drop": float(st.res / st.res0), "converged_1e-10": bool(st.converged),
               "ms_per_step": e0.elapsed_time(e1) / max(1, st.steps),
               "cd": s.wall_force((1.0, 0.0)) / (0.5 * mach * mach * 1.0)}
        state = cons(s.get_state())
        s.close()
        return res, state

    out = {"cap_steps": steps, "limiter": LIMITER, "cfl": CFL, "corrections": "all"}
    for mach in machs:
        for flux in fluxes:
            r64, s64 = one(mach, flux, "fp64", "all")
            r32, s32 = one(mach, flux, "fp32", "all")
            entry = {"fp64": r64, "fp32": r32}
            if s64 is not None and s32 is not None:
                d = np.abs(s32 - s64).reshape(4, -1)
                entry["fp32_vs_fp64_rel_linf"] = float((d.max(1) / np.abs(s64).reshape(4, -1).max(1)).max())
                entry["fp32_vs_fp64_rel_l1"] = float((d.mean(1) / np.abs(s64).reshape(4, -1).mean(1)).max())
            out[f"{flux}_M{mach}"] = entry
    lit, _ = one(0.3, "roe", "fp64", None)
    out["reference_roe_uncorrected_M0.3_fp64"] = lit
    return out


def measure_steady_full(stream, max_steps: int = 300000, mach: float = 0.3):
    """Configuration 2 run to convergence on its full 512 x 1024 O-grid (opt-in:
    `--steady-full`, minutes of FP64 time): face-frame Roe, unlimited reconstruction
    (NoLimit2; van Albada stalls near a 1e-4 drop), ssp34 with local timestepping at CFL 1.5,
    the corrections, M 0.3, from the uniform freestream until the density residual fell by
    1e-10 (cap `max_steps`); then FP32 with the same settings for as many steps, and its
    difference from the FP64 converged state (per variable, relative to its largest
    magnitude).  Reported: steps, drop, the residual history, C_d and C_l, times."""
    import torch
    from hyperboliconvergence_gb300 import cases
    from hyperboliconvergence_gb300.solver import Solver
    g = 1.4

    def cons(w):
        u, v, r, p = w
        return np.stack([r * u, r * v, r, p / (g - 1) + 0.5 * r * (u * u + v * v)])

    kw = dict(flux="roe_face", limiter="nolimit2", rk="ssp34", dt="local", cfl=1.5, corrections="all")
    out = {"workload": f"cylinder O-grid {NR}x{NTH}, M{mach}, " + ", ".join(f"{k} {v}" for k, v in kw.items())}
    states = {}
    nsteps = max_steps
    for prec in ("fp64", "fp32"):
        mesh, bc, ref, q, species = cases.cylinder(NR, NTH, mach=mach)
        s = Solver(mesh, bc, ref, precision=prec, species=species, stream=stream.cuda_stream, **kw)
        s.set_state(q)
        e0, e1 = _events()
        torch.cuda.synchronize()
        e0.record(stream)
        st, hist = s.steady(nsteps, residual_drop=1e-10, check_every=5000)
        e1.record(stream)
        torch.cuda.synchronize()
        qd = 0.5 * mach * mach
        out[prec] = {"steps": int(st.steps), "residual_drop": float(st.res / st.res0),
                     "converged_1e-10": bool(st.converged), "seconds": e0.elapsed_time(e1) / 1e3,
                     "history_every_5000_steps": [float(h) for h in np.asarray(hist).ravel()[:80]],
                     "cd": s.wall_force((1.0, 0.0)) / qd, "cl": s.wall_force((0.0, 1.0)) / qd}
        states[prec] = cons(s.get_state())
        s.close()
        nsteps = int(st.steps)  # FP32: as many steps as FP64 took
    d = np.abs(states["fp32"] - states["fp64"]).reshape(4, -1)
    scale = np.abs(states["fp64"]).reshape(4, -1).max(1)
    out["fp32_vs_fp64_converged"] = {"rel_linf": float((d.max(1) / scale).max()),
                                     "rel_mean": float((d.mean(1) / scale).max())}
    return out


def measure_developed(stream, steps: int = 10):
    """The headline workload (FP64) started from a state that is non-uniform
    everywhere -- the freestream times 1 + 1% of a smooth field of r and theta --
    so that no face has zero slopes.  From the uniform freestream the far field
    has zero slopes for many steps, and the limiter skips its division there."""
    import torch
    from hyperboliconvergence_gb300 import cases
    from hyperboliconvergence_gb300.solver import Solver
    mesh, bc, ref, q, species = cases.cylinder(NR, NTH, mach=MACH)
    c = mesh.centres()
    r, th = np.hypot(c[0], c[1]), np.arctan2(c[1], c[0])
    f = np.sin(3 * th + 0.5) * np.cos(0.7 * r) + 0.5 * np.cos(5 * th) * np.sin(0.3 * r + 1.0)
    qd = q * (1.0 + 0.01 * f[None])
    s = Solver(mesh, bc, ref, flux=FLUX, limiter=LIMITER, rk=RKT, precision="fp64", dt=DTMODE, cfl=CFL,
               species=species, stream=stream.cuda_stream)
    s.set_state(qd)
    s.step(3)
    e0, e1 = _events()
    torch.cuda.synchronize()
    e0.record(stream)
    s.step_async(steps)
    e1.record(stream)
    s.sync()
    ms = e0.elapsed_time(e1) / steps
    s.close()
    return {"value": NR * NTH / (ms / 1e3), "unit": UNIT, "ms_per_step": ms,
            "start": "freestream x (1 + 0.01 f(r, theta)), f smooth and non-zero almost everywhere"}


def measure_variants(stream, steps: int = 10):
    """The O-grid workload with each flux at M 0.3 and 0.8: FP64 cell-updates/s over
    `steps` RK steps after 3 warm-up steps, and the FP32 relative L-inf difference of
    the conserved variables from FP64 after 20 steps from the freestream.  SLAU runs
    the literal reference form first and the mass-flux-upwinded form if the literal
    one goes non-physical."""
    import torch
    from hyperboliconvergence_gb300 import HCError, cases
    from hyperboliconvergence_gb300.solver import Solver
    g = 1.4

    def cons(w):
        u, v, r, p = w
        return np.stack([r * u, r * v, r, p / (g - 1) + 0.5 * r * (u * u + v * v)])

    out = {}
    for mach in (0.3, 0.8):
        mesh, bc, ref, q, species = cases.cylinder(NR, NTH, mach=mach)
        for flux in ("roe", ("slau_ref", "slau"), "ausmpup"):
            tries = flux if isinstance(flux, tuple) else (flux,)
            for fl in tries:
                key = f"{fl}_M{mach}"
                try:
                    states = {}
                    res = {}
                    for prec in ("fp64", "fp32"):
                        s = Solver(mesh, bc, ref, flux=fl, limiter=LIMITER, rk=RKT, precision=prec, dt=DTMODE,
                                   cfl=CFL, species=species, stream=stream.cuda_stream)
                        s.set_state(q)
                        if prec == "fp64":
                            s.step(3)
                            e0, e1 = _events()
                            torch.cuda.synchronize()
                            e0.record(stream)
                            s.step_async(steps)
                            e1.record(stream)
                            s.sync()
                            ms = e0.elapsed_time(e1) / steps
                            res = {"value": NR * NTH / (ms / 1e3), "unit": UNIT, "ms_per_step": ms}
                            s.set_state(q)
                        s.step(20)
                        states[prec] = cons(s.get_state())
                        s.close()
                    a, b = states["fp32"], states["fp64"]
                    res["fp32_error_vs_fp64_after_20_steps"] = float(
                        (np.abs(a - b).reshape(4, -1).max(1) / np.abs(b).reshape(4, -1).max(1)).max())
                    out[key] = res
                    break
                except HCError as exc:
                    out[key] = {"error": str(exc)}
    return out


def measure_adjoint(nsteps: int = 400, snapshots: int = 20, precisions=("fp64", "fp64_df"), compare_no_tapes=True):
    """Differentiated case: 256x512 O-grid (0.5 to 20), M 0.4, Roe + van Albada, ssp34,
    nsteps from uniform freestream; drag coefficient averaged over the steps; gradient
    with respect to every cell's initial state and the far-field state (hence Mach and
    angle of attack); binomial checkpointing with `snapshots` stored states.  Run with
    FP64 stages and with double-float forward stages (the reverse sweep is FP64 in
    both).  The adjoint-step metric is reverse-sweep time (checkpoint recomputation
    included) per step over forward-sweep time per step, with the default stage tapes
    (snapshots + 1: each reversed step's stage states kept from the advance that computed
    it last) and, for FP64, without them (every reversed step replayed)."""
    import math
    from hyperboliconvergence_gb300.solver import Mesh, Solver
    nr, nth, mach, alpha = 256, 512, 0.4, 0.0
    mesh = Mesh.cylinder(nr, nth, 0.5, 20.0, 1.01)
    qinf = np.array([mach * math.cos(alpha), mach * math.sin(alpha), 1.0, 1.0 / 1.4])
    ref = [None, np.broadcast_to(qinf[:, None], (4, nth)).copy(), None, None]
    out = {"workload": f"cylinder O-grid {nr}x{nth}, M{mach}, {nsteps} ssp34 steps, {snapshots} snapshots"}
    for prec in precisions:
        s = Solver(mesh, ["wall", "fixed", "periodic", "periodic"], ref, flux="roe", limiter="vanalbada",
                   rk="ssp34", precision=prec, dt="global", cfl=0.5, species=(1.4, 287.058, mach))
        q0 = np.broadcast_to(qinf[:, None, None], (4, nr, nth)).copy()
        scale = 1.0 / (0.5 * mach * mach * 2 * 0.5)
        no_tapes = None
        if prec == "fp64" and compare_no_tapes:
            s.set_adjoint_tapes(0)
            s.set_state(q0)
            J0, g0, _, _, st0 = s.gradient(nsteps, snapshots=snapshots, kind="drag", scale=scale)
            f0 = st0.ms_forward
            no_tapes = {"adjoint_step_over_forward_step": (st0.ms_total - f0) / f0,
                        "adjoint_step_over_forward_step_excl_recompute": (st0.ms_total - f0 - st0.ms_recompute) / f0,
                        "replays": int(st0.replays), "forward_steps_total": int(st0.forward_steps)}
            s.set_adjoint_tapes(-1)
        s.set_state(q0)
        J, g, refb, rates, st = s.gradient(nsteps, snapshots=snapshots, kind="drag", scale=scale)
        s.close()
        if no_tapes is not None:
            no_tapes["gradient_bit_identical"] = bool(J0 == J and np.array_equal(g0, g))
        fwd, rev, rec = st.ms_forward, st.ms_total - st.ms_forward, st.ms_recompute
        state_mib = 4 * nr * nth * 8 / 2 ** 20
        # freestream derivatives: q0 and the far-field layer both equal qinf(M, alpha);
        # Cd = scale(M) * D with scale ~ 1/M^2
        dq_dm = np.array([math.cos(alpha), math.sin(alpha), 0.0, 0.0])
        dq_da = np.array([-mach * math.sin(alpha), mach * math.cos(alpha), 0.0, 0.0])
        gsum = g.reshape(4, -1).sum(axis=1) + refb[1].reshape(4, -1).sum(axis=1)
        out[prec] = {
            "J_time_avg_cd": J,
            "dJ_dmach": float(gsum @ dq_dm - 2.0 * J / mach), "dJ_dalpha": float(gsum @ dq_da),
            "grad_norm_q0": float(np.linalg.norm(g)),
            "forward_ms": fwd, "reverse_ms": rev, "recompute_ms": rec,
            "forward_step_ms": fwd / nsteps,
            "adjoint_step_over_forward_step": rev / fwd,
            "adjoint_step_over_forward_step_excl_recompute": (rev - rec) / fwd,
            "forward_steps_total": int(st.forward_steps), "adjoint_steps": int(st.adjoint_steps),
            "replays": int(st.replays), "stage_tapes": int(st.stage_tapes),
            "snapshot_mib": snapshots * state_mib, "stage_tape_mib": int(st.stage_tapes) * 4 * state_mib}
        if no_tapes is not None:
            out[prec]["without_stage_tapes"] = no_tapes
    if "fp64" in out and "fp64_df" in out:
        a, b = out["fp64"], out["fp64_df"]
        out["df_vs_fp64_grad_rel_diff"] = {k: abs(b[k] - a[k]) / max(abs(a[k]), 1e-300)
                                           for k in ("J_time_avg_cd", "dJ_dmach", "grad_norm_q0")}
    return out


def measure_batched_adjoint(ninst: int = 64, nsteps: int = 100, snapshots: int = 20, seed: int = 2027,
                            compare: int = 8, law: str = "euler", budget: int = 50):
    """Batched and differentiated case: `ninst` periodic instances on [0,1]^2, n x n
    cells with n drawn from {128, 192, ..., 1024}.  Euler: density = 5 plus 8 seeded
    Gaussians (widths 0.02..0.2, amplitudes -0.5..0.5) on u = 0.5, v = 0.25, p = 1;
    scalar advection (law="scalar"): the scalar = 1 plus 8 such Gaussians, advected by
    a seeded constant velocity per instance (|u|, |v| <= 1).  Rusanov with NoLimit3
    reconstruction (smooth, so FP32 and FP64 differentiate the
    same branches), ssp34, global dt, CFL 0.5.  L2 loss of each instance's state after
    `nsteps` steps against its own seeded target; gradient with respect to every
    instance's initial state in FP32 from one batched adjoint (hc_batch_adjoint_gradient:
    one persistent launch per forward stage and one launch per reverse pass over all
    instances, `snapshots` checkpoints of the whole batch; timed again with `budget`
    checkpoints).  Checks: the smallest
    instance's FP32 gradient from the batch against its FP64 single-mesh gradient, and
    the first `compare` instances timed as single-mesh adjoints against the batched
    adjoint of the same instances."""
    from hyperboliconvergence_gb300 import cases
    from hyperboliconvergence_gb300.batch import Batch
    from hyperboliconvergence_gb300.solver import Solver
    rng = np.random.default_rng(seed)
    sizes = [int(n) for n in rng.choice(np.arange(128, 1025, 64), ninst)]
    base = (0.5, 0.25, 5.0, 1.0)
    insts, targets = [], []
    sp = (1.4, 287.058, 0.3)
    for n in sizes:
        if law == "scalar":
            vel = rng.uniform(-1.0, 1.0, 2)
            mesh, bc, ref, q = cases.scalar_gaussian_sum(n, n, rng, velocity=vel)
            insts.append((mesh, bc, ref, q))
            targets.append(cases.scalar_gaussian_sum(n, n, rng, velocity=vel)[3])
        else:
            mesh, bc, ref, q, sp = cases.gaussian_sum(n, n, rng, base=base)
            insts.append((mesh, bc, ref, q))
            targets.append(cases.gaussian_sum(n, n, rng, base=base)[3])
    kw = dict(flux="rusanov", limiter="nolimit3", rk="ssp34", dt="global", cfl=0.5, species=sp, law=law)
    kmin = int(np.argmin(sizes))
    t0 = time.perf_counter()
    bt = Batch(insts, precision="fp32", **kw)
    J, grads, st = bt.gradient(nsteps, targets, snapshots=snapshots, want=[kmin])
    wall = time.perf_counter() - t0
    # the same batch through the torch.autograd.Function: per-instance J from CUDA tensors,
    # loss.backward() one batched reverse sweep from the forward's checkpoints
    import torch
    from hyperboliconvergence_gb300.autograd import batch_l2_objective
    q0s = [torch.tensor(q, dtype=torch.float64, device="cuda", requires_grad=True) for (_, _, _, q) in insts]
    tgs = [torch.tensor(t, dtype=torch.float64, device="cuda") for t in targets]
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    first_ms = None
    for rep in range(2):  # the first call carries torch's one-time costs; the second is timed
        for q in q0s:
            q.grad = None
        torch.cuda.synchronize()
        ev[0].record()
        Jt = batch_l2_objective(bt, q0s, tgs, nsteps, snapshots=snapshots)
        ev[1].record()
        Jt.sum().backward()
        ev[2].record()
        torch.cuda.synchronize()
        if rep == 0:
            first_ms = ev[0].elapsed_time(ev[2])
    fst = bt.last_stats
    fn = {"forward_ms": ev[0].elapsed_time(ev[1]), "backward_ms": ev[1].elapsed_time(ev[2]),
          "library_reverse_ms": fst.ms_total - fst.ms_forward, "library_forward_ms": fst.ms_forward,
          "library_reverse_sweep_ms": fst.ms_reverse, "one_call_reverse_sweep_ms": st.ms_reverse,
          "replays": int(fst.replays), "stage_tapes": int(fst.stage_tapes),
          "first_call_total_ms": first_ms,
          "J_equal_one_call": bool(np.array_equal(Jt.detach().cpu().numpy(), J)),
          "grad_equal_one_call": bool(np.array_equal(q0s[kmin].grad.cpu().numpy(), grads[kmin]))}
    fn["backward_over_forward"] = fn["backward_ms"] / fn["forward_ms"]
    del q0s, tgs, Jt
    # the same gradient with a larger checkpoint budget (the configuration names none; the
    # single-mesh differentiated one names 20): fewer recomputed steps for more memory
    state_gib = sum(n * n for n in sizes) * 4 * 4 / 2 ** 30
    try:
        _, _, stb = bt.gradient(nsteps, targets, snapshots=budget, want=[])
        larger = {"snapshots": budget, "snapshot_gib": budget * state_gib, "forward_ms": stb.ms_forward,
                  "reverse_ms": stb.ms_total - stb.ms_forward, "recompute_ms": stb.ms_recompute,
                  "stage_tapes": int(stb.stage_tapes),
                  "adjoint_step_over_forward_step": (stb.ms_total - stb.ms_forward) / stb.ms_forward}
    except Exception as exc:  # reported beside the 20-checkpoint figures, which stand alone
        larger = {"snapshots": budget, "error": f"{type(exc).__name__}: {exc}"}
    bt.close()
    if not np.all(np.isfinite(J)) or not np.all(np.isfinite(grads[kmin])):
        raise RuntimeError("non-finite objective or gradient")
    cells = sum(n * n for n in sizes)
    fwd_ms, rev_ms = st.ms_forward, st.ms_total - st.ms_forward
    # FP64 single-mesh check of the smallest instance
    mesh, bc, ref, q = insts[kmin]
    s = Solver(mesh, bc, ref, precision="fp64", **kw)
    s.set_state(q)
    j64, g64 = s.gradient(nsteps, snapshots=snapshots, kind="l2", target=targets[kmin])[:2]
    s.close()
    g32 = grads[kmin]
    # single-mesh adjoints of the first `compare` instances against one batched adjoint of them
    single_ms = 0.0
    for k in range(compare):
        mesh, bc, ref, q = insts[k]
        s = Solver(mesh, bc, ref, precision="fp32", **kw)
        s.set_state(q)
        single_ms += s.gradient(nsteps, snapshots=snapshots, kind="l2", target=targets[k])[4].ms_total
        s.close()
    sub = Batch(insts[:compare], precision="fp32", **kw)
    sub_ms = sub.gradient(nsteps, targets[:compare], snapshots=snapshots, want=[])[2].ms_total
    sub.close()
    what = "scalar-advection" if law == "scalar" else "Euler"
    return {"workload": f"{ninst} Gaussian-sum {what} instances, n x n with n in 128..1024, L2 loss after "
                        f"{nsteps} ssp34 steps, {snapshots} snapshots, FP32, one batched adjoint",
            "cells": cells, "forward_ms": fwd_ms, "reverse_ms": rev_ms, "wall_s": wall,
            "recompute_ms": st.ms_recompute, "kernel_launches": int(st.kernel_launches),
            "forward_cell_updates_per_s": cells * nsteps / (fwd_ms / 1e3),
            "adjoint_step_over_forward_step": rev_ms / fwd_ms,
            "replays": int(st.replays), "stage_tapes": int(st.stage_tapes),
            "larger_checkpoint_budget": larger,
            "through_autograd_function": fn,
            "fp64_check": {"instance": kmin, "cells": sizes[kmin] ** 2,
                           "J_rel_diff": abs(float(J[kmin]) - j64) / abs(j64),
                           "grad_max_rel_diff": float(np.abs(g32 - g64).max() / np.abs(g64).max())},
            "batched_vs_single_mesh": {"instances": compare, "cells": sum(n * n for n in sizes[:compare]),
                                       "single_mesh_ms": single_ms, "batched_ms": sub_ms,
                                       "speedup": single_ms / sub_ms}}


def job_rate(pg, ms: float, world: int, units_per_rank: float, device: str = "cuda"):
    """Whole-job throughput of a replicas-only run: every rank processed units_per_rank in
    its own ms; the job took the slowest rank's time (the max over ranks), in which all
    world x units_per_rank were processed.  Returns (units per second, max ms)."""
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    if pg is not None:
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
    ms = float(t.item())
    return world * units_per_rank / (ms / 1e3), ms


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def run_reference(args):
    world, rank, _ = dist_setup()
    if rank != 0:
        return 0
    steps = max(1, args.steps)
    cb = cpu_baseline(sample_s=min(8.0, 2.0 + 0.5 * steps), samples=3)
    v = cb["value"]
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": steps,
            "warmup": args.warmup, "ms_per_step": NR * NTH / v * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(), "impl": "reference", "cpu_baseline": cb,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_adjoint_only(args):
    """`--adjoint-only`: the config-4 adjoint measurement alone (for profiling its kernels),
    FP64, with `--adjoint-steps` steps and `--adjoint-snapshots` snapshots; prints one JSON
    line with that measurement and no headline."""
    import torch
    torch.cuda.set_device(0)
    out = measure_adjoint(args.adjoint_steps, args.adjoint_snapshots, precisions=("fp64",), compare_no_tapes=False)
    print(json.dumps({"adjoint_only": True, "adjoint": out}), flush=True)
    return 0


def run_steady_full(args):
    """`--steady-full`: configuration 2 converged on its full grid (measure_steady_full);
    prints one JSON line with that measurement and no headline."""
    import torch
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        out = measure_steady_full(stream, max_steps=args.steady_full_cap)
    print(json.dumps({"steady_full": True, "steady": out}), flush=True)
    return 0


def run_gpu(args):
    import torch

    from hyperboliconvergence_gb300 import cases
    from hyperboliconvergence_gb300.solver import Solver

    if args.adjoint_only:
        return run_adjoint_only(args)
    if args.steady_full:
        return run_steady_full(args)
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        pg = dist
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    mesh, bc, ref, q, species = cases.cylinder(NR, NTH, mach=MACH)
    s = Solver(mesh, bc, ref, flux=FLUX, limiter=LIMITER, rk=RKT, precision="fp64", dt=DTMODE, cfl=CFL,
               species=species, stream=stream.cuda_stream)
    s.set_state(q)
    ncell = NR * NTH

    def barrier():
        if pg is not None:
            pg.barrier()
        torch.cuda.synchronize()

    # the clock sampler runs from before the warm-up to the end of the timed region (20 ms
    # samples; its first sample is waited for, so that the samples cover both)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        clk.wait_first()
        # warm-up
        s.step_async(max(3, args.warmup))
        s.sync()
        barrier()
        launches0 = s.sync().kernel_launches
        barrier()
        ev0.record(stream)
        s.step_async(args.steps)
        ev1.record(stream)
        barrier()
    st = s.sync()
    launches = st.kernel_launches - launches0
    value, ms = job_rate(pg, ev0.elapsed_time(ev1), world, ncell * args.steps)
    ms_per_step = ms / args.steps

    # roofline of the dominant kernel (the fused stage kernel; the timed region
    # holds only stage kernels and two 8-byte memsets per step)
    stage_ms = ms / (args.steps * NSTAGES)
    alg_bytes = ALG_BYTES_PER_CELL_STAGE * ncell
    achieved = alg_bytes / (stage_ms / 1e3) / 1e9
    peak, peak_src = measured_peaks()
    tpc = profiled_traffic_per_cell()
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": None if tpc is None else tpc * ncell, "peak_source": peak_src,
            "kernel": "stage_kernel<16,16,double,ROE,128 threads>", "alg_bytes_per_launch": alg_bytes,
            "avg_launch_ms": stage_ms}

    # end to end through the C ABI with host buffers (hc_step_host): every step uploads the
    # state from pinned host memory, runs one RK step and downloads the result
    host_in = torch.from_numpy(np.ascontiguousarray(s.get_state())).pin_memory()
    host_out = torch.empty_like(host_in).pin_memory()
    in_np, out_np = host_in.numpy(), host_out.numpy()
    ke = max(3, min(args.steps, 20))
    for _ in range(2):
        s.step_host(in_np, out_np)
    barrier()
    t0 = time.perf_counter()
    for _ in range(ke):
        s.step_host(in_np, out_np)
    barrier()
    e2e_value, _ = job_rate(pg, (time.perf_counter() - t0) * 1e3, world, ncell * ke)
    e2e = {"value": e2e_value, "unit": UNIT,
           "h2d_bytes_per_step": int(host_in.numel() * 8), "d2h_bytes_per_step": int(host_out.numel() * 8),
           "steps": ke}

    if rank == 0:
        cfg = workload_config()
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": cfg, "roofline": roof, "e2e": e2e, "gpu_launches": int(launches),
                "clocks": clk.summary()}
        # the roof that binds the FP64 stage kernel: FP64 arithmetic, with the
        # algorithmic FLOPs of the oracle's operation tally (recorded in profiles/)
        fpc = profile_value("algorithmic_flops_per_cell_stage")
        if fpc is not None:
            try:
                pk = fp64_peak_tflops()
                ach = fpc * ncell / (stage_ms / 1e3) / 1e12
                line["fp64_roofline"] = {"bound": "fp64", "achieved": ach, "peak": pk, "unit": "TFLOP/s",
                                         "frac": ach / pk, "flops_per_cell_stage": fpc,
                                         "peak_source": "measured here: float64 GEMM 4096^3 (cuBLAS), best of 5"}
            except Exception as exc:  # reported, not fatal
                line["fp64_roofline"] = {"error": f"{type(exc).__name__}: {exc}"}
        if world == 1 and not args.no_cpu:
            line["cpu_baseline"] = cpu_baseline()
        extras = [] if args.no_extras else [e for e in args.extras.split(",") if e]
        if world == 1 and extras:
            s.close()
            for name, fn in (("fp32", lambda: measure_precision(stream, args.steps, "fp32")),
                             ("fp64_df", lambda: measure_precision(stream, args.steps, "fp64_df")),
                             ("batched", lambda: measure_batched(stream)),
                             ("variants", lambda: measure_variants(stream)),
                             ("developed", lambda: measure_developed(stream)),
                             ("vortex", lambda: measure_vortex(stream)),
                             ("steady", lambda: measure_steady(stream, args.steady_steps)),
                             ("adjoint", lambda: measure_adjoint(args.adjoint_steps, args.adjoint_snapshots)),
                             ("batched_adjoint", measure_batched_adjoint),
                             ("batched_adjoint_scalar", lambda: measure_batched_adjoint(law="scalar"))):
                if name in extras:
                    try:
                        line[name] = fn()
                    except Exception as exc:  # reported, not fatal: the headline stands alone
                        line[name] = {"error": f"{type(exc).__name__}: {exc}"}
        print(json.dumps(line), flush=True)
    s.close()
    if pg is not None:
        pg.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--adjoint-steps", type=int, default=400, help="RK steps of the adjoint measurement")
    ap.add_argument("--adjoint-snapshots", type=int, default=20, help="checkpoints of the adjoint measurement")
    ap.add_argument("--adjoint-only", action="store_true",
                    help="run only the FP64 adjoint measurement (no headline line), for profiling its kernels")
    ap.add_argument("--steady-full", action="store_true",
                    help="run only configuration 2 to a 1e-10 residual drop on its full grid (minutes; no headline)")
    ap.add_argument("--steady-full-cap", type=int, default=300000, help="step cap of --steady-full")
    ap.add_argument("--steady-steps", type=int, default=2000,
                    help="step cap of each run of the steady O-grid extra (residual drop target 1e-10)")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the FP32, double-float, batched and adjoint measurements beside the headline")
    ap.add_argument("--extras",
                    default="fp32,fp64_df,batched,variants,developed,vortex,steady,adjoint,batched_adjoint,"
                            "batched_adjoint_scalar",
                    help="comma-separated subset of fp32,fp64_df,batched,variants,developed,vortex,steady,adjoint,"
                         "batched_adjoint,batched_adjoint_scalar to measure beside the headline")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
