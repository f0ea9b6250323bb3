#!/usr/bin/env python3
"""Benchmark of the GB300 PIC particle loop (one JSON line on stdout).

Workload (default ``curved``): PICLas's "plain FP64 at scale" case -- 32^3 curved hexahedra
(interior nodes displaced by 0.05 h sin sin sin), N=3, 8M electrons (2 eV) + 8M ions (mass
ratio 1836, 0.1 eV), external B_z = 0.1 T, RefTracking, shape_function deposition with radius
1.5 h (alpha 2), dt = 5e-12 s.  One step = Deposition + InterpolateFieldToParticle +
Boris push + RefTracking over all particles, the field frozen (the HDG solve is not timed).
Inputs are seeded synthetic particles; the particle arrays (~1.3 GB) exceed the 129 MB L2,
so no flush is needed between timed steps.

``--impl reference`` times the reference algorithm on the host cores instead: the C
restatement of the Fortran loop (oracle/), OpenMP over particles, on a bounded sample of the
same workload (the PICLas binary itself cannot be built: no Fortran compiler, MPI or HDF5).

Multi-GPU: the loop does not shard across GPUs here (replicas only): each rank runs its own
instance with seed = rank; ``value`` sums the ranks' particle-steps over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "particle-steps/s, mixed vs FP64 on 1 GB300 at <=1e-6 rel rho error; HBM GB/s"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ----------------------------------------------------------------------------------------------
def make_workload(name: str, seed: int, n_override: int | None = None, cells: int | None = None,
                  periodic_tracing: bool = False, n_geo: int = 1, p_adaption: str | None = None,
                  walls: str | None = None, wall_bulge: float = 0.0):
    from piclas_gb300 import workloads
    from piclas_gb300.mesh import build_box_mesh, p_adaption_degrees
    kw = {} if cells is None else {"n_cells": cells}
    if name == "curved":
        if n_override is not None:
            kw["n_per_species"] = n_override // 2
        if periodic_tracing or n_geo > 1 or p_adaption or walls:
            # periodic_tracing: the reference's default periodic RefTracking (CartesianPeriodic = F), BC lists with
            # the periodic sides; n_geo: curved elements of that geometry degree; p_adaption: degrees 1..3 per
            # element; walls: a closed box with reflective walls (wall_bulge: bulged wall faces, bilinear sides at
            # NGeo = 1 and curved Bezier sides at NGeo > 1)
            nc = kw.pop("n_cells", 32)
            n_loc = p_adaption_degrees(nc, nc, nc, p_adaption, 1, 3, seed=seed) if p_adaption else None
            bc = (walls,) * 3 if walls else ("periodic",) * 3
            kw["mesh"] = build_box_mesh(nc, nc, nc, 3, perturb=0.05, periodic_tracing=periodic_tracing, n_geo=n_geo,
                                        n_loc=n_loc, bc=bc, wall_bulge=wall_bulge if walls else 0.0)
        w = workloads.curved_two_species(seed=seed, **kw)
        w.periodic_tracing = periodic_tracing
        w.walls, w.wall_bulge = walls, (wall_bulge if walls else 0.0)
        return w
    if name == "plasma_wave":
        if n_override is not None:
            kw["n_particles"] = n_override
        return workloads.plasma_wave(seed=seed, **kw)
    raise ValueError(name)


def workload_config(w, name):
    m = w.mesh
    if name == "curved":
        cells = round(m.n_elems ** (1.0 / 3.0))
        tag = "plain FP64 at scale: " if (cells == 32 and w.n == 16_000_000) else "profiling case of plain FP64 at scale: "
        trk = ("RefTracking (CartesianPeriodic = F: periodic sides traced as BC sides)"
               if getattr(w, "periodic_tracing", False) else "RefTracking (CartesianPeriodic/FastPeriodic)")
        walls = getattr(w, "walls", None)
        if walls:
            bulge = getattr(w, "wall_bulge", 0.0)
            side = ("planar" if bulge == 0.0 else "bilinear" if m.n_geo == 1 else "curved Bezier (clipping)")
            trk = f"RefTracking, {walls} walls all round ({side} wall sides, ParticleBCTracking)"
        geo = "curved hex" if m.n_geo == 1 else f"curved NGeo={m.n_geo} hex"
        deg = f"N={m.N}" if m.n_loc is None else f"N_loc random 1..{m.N} ({m.n_dofs} DOFs)"
        out = {"workload": f"{tag}{cells}^3 {geo}, {deg}, {w.n // 2} e- + {w.n - w.n // 2} ions, "
                           "B_z=0.1 T, RefTracking, shape_function r=1.5h, dt=5e-12",
               "elements": m.n_elems, "N": m.N, "particles": w.n, "deposition": "shape_function",
               "tracking": trk, "l2": "inputs larger than L2 (no flush)"}
        if m.n_geo > 1:
            out["n_geo"] = m.n_geo
        if m.n_loc is not None:
            out["p_adaption"] = "random 1..3"
        if walls:
            out["walls"] = walls
            out["wall_bulge"] = getattr(w, "wall_bulge", 0.0)
        return out
    cells = round(m.n_elems ** (1.0 / 3.0))
    return {"workload": f"plasma wave: {cells}^3 hex, N={m.N}, {w.n} e-, CVWM, TriaTracking, dt=1e-11",
            "elements": m.n_elems, "N": m.N, "particles": w.n, "deposition": "cell_volweight_mean",
            "tracking": "TriaTracking", "l2": "L2 flushed between timed steps"}


def algorithmic_bytes_per_step(w, mixed: bool) -> float:
    """B_step of the loop: Np(2 S_state + 2*4 + 1) + Ne nDOF (3*8 + 8) [+ nodes 2*4*8 for CVWM]."""
    from piclas_gb300 import capi
    s_state = (24 + 12) if mixed else 48
    if w.tracking == capi.PIC_TRACK_REFMAPPING:
        s_state += 24                                   # PartPosRef
    b = w.n * (2 * s_state + 2 * 4 + 1) + w.mesh.n_dofs * (3 * 8 + 8)
    if w.deposition == capi.PIC_DEPO_CVWM:
        b += w.mesh.n_nodes * (2 * 4 * 8)
    return float(b)


def dominant_kernel_bytes(w, mixed: bool) -> tuple[str, float]:
    """Name and algorithmic bytes of one launch of the dominant kernel."""
    from piclas_gb300 import capi
    if w.deposition == capi.PIC_DEPO_SHAPE_FUNCTION:
        # gather: each packed particle record read once, PartSource written once
        rec = 32 if mixed else 16 + 24 + 32
        if w.mesh.n_loc is not None:
            name = f"k_sf_gather5<Nloc,{int(mixed)},0,{int(w.sf_alpha == 2)}> (one launch per degree)"
        elif sf_gather_variant() == 5 and mixed and w.mesh.N == 3:
            name = f"k_sf_gather7<{int(w.sf_alpha == 2)}>"
        elif sf_gather_variant() == 5:
            name = f"k_sf_gather5<{w.mesh.N},{int(mixed)},0,{int(w.sf_alpha == 2)}>"
        else:
            name = f"k_sf_gather2<{w.mesh.N},{int(mixed)}>"
        return name, float(w.n * rec + w.mesh.n_dofs * 4 * 8)
    s_state = (24 + 12) if mixed else 48
    b = w.n * (2 * s_state + 2 * 4 + 1) + w.mesh.n_dofs * 3 * (4 if mixed else 8)
    b += w.mesh.n_nodes * 4 * 8
    return f"k_step_cvwm_tria<{w.mesh.N},{int(mixed)}>", float(b)


def sf_gather_variant() -> int:
    """Compile-time shape-function gather variant of the loaded library (from pic_version)."""
    from piclas_gb300 import load_library
    v = load_library().pic_version().decode()
    try:
        return int(v.split("sf gather")[1].strip(" )"))
    except Exception:
        return 5


def sf_hits_per_launch(w) -> float:
    """Expected (particle, DOF) pairs with r <= R: particles x DOF density x sphere volume."""
    vol = float(np.prod(np.asarray(w.mesh.hi) - np.asarray(w.mesh.lo)))
    dof_density = w.mesh.n_dofs / vol
    return w.n * dof_density * 4.0 / 3.0 * math.pi * w.sf_radius ** 3


def compute_roofline(w, mixed: bool, avg_ms: float, fma_peak: float | None):
    """The shape-function gather is bound by arithmetic, not by HBM: in FP64 by GB300's FP64 pipe, in the mixed
    variant by instruction issue (FP32 arithmetic plus the culling around it).  Achieved = the reference's 19
    FLOP per (particle, DOF) hit (r^2: 3 sub, 3 mul, 2 add; 1 - r^2/R^2: 2; the square: 1; 4 x (mul, add)) x hits
    per launch / launch time; peak = the FMA rate of that precision measured in the same run
    (pic_fp64_fma_rate / pic_fp32_fma_rate; nominal 1.25 TFLOP/s FP64 or SMs x 128 lanes x 2 x 2.07 GHz FP32
    if the probe failed)."""
    from piclas_gb300 import capi
    if w.deposition != capi.PIC_DEPO_SHAPE_FUNCTION:
        return None
    hits = sf_hits_per_launch(w)
    flops = 19.0 * hits
    achieved = flops / (avg_ms / 1e3) / 1e9
    nominal = 152 * 128 * 2 * 2.07 if mixed else 1250.0
    peak, kind = (fma_peak, "measured (pic_fp32_fma_rate)" if mixed else "measured (pic_fp64_fma_rate)") \
        if fma_peak else (nominal, "nominal")
    out = {"bound": "fp32-issue" if mixed else "fp64", "achieved": achieved, "peak": peak, "unit": "GFLOP/s",
           "frac": achieved / peak, "peak_kind": kind, "nominal_peak": nominal, "hits_per_launch": hits,
           "flops_per_hit": 19, "hits_per_s": hits / (avg_ms / 1e3)}
    kname = dominant_kernel_bytes(w, mixed)[0]
    ncu = read_ncu_summary(f"{kname} @ 16^3 curved, 2M particles")
    if ncu:
        out["ncu_16cube"] = ncu
    pipe = read_ncu_fp64(f"{kname} @ 16^3 curved, 2M particles")
    if pipe and not mixed:
        out["ncu_16cube"] = pipe
        out["note"] = ("achieved counts the reference's 19 FLOP per (particle, DOF) hit; the kernel sums the particles "
                       "whose kernel covers every DOF of the target (or of a DOF half) as moments, fewer FP64 "
                       "operations than per hit, so frac can pass 1; the hardware figure is the FP64 pipe busy share")
    return out


def read_ncu_summary(key: str):
    """Issue-slot and instruction figures of a committed ncu capture (profiles/ncu_traffic.txt, second table:
    kernel @ case | issue slots busy | inst. executed per hit | candidates per hit)."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    try:
        for line in open(p):
            if line.startswith("|") and line.count("|") == 5:
                cells = [c.strip() for c in line.strip().strip("|").split("|")]
                if cells[0] == key:
                    return {"issue_slots_busy": float(cells[1]), "inst_per_hit": float(cells[2]),
                            "candidates_per_hit": float(cells[3])}
    except Exception:
        pass
    return None


def read_ncu_fp64(key: str):
    """FP64-pipe figures of a committed ncu capture (profiles/ncu_traffic.txt, third table, rows keyed
    "<kernel> @ <case>, FP64 pipe": busy share of active cycles (%) | lanes active of 32 | hits through moments (%))."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    try:
        for line in open(p):
            if line.startswith("|") and line.count("|") == 5:
                cells = [c.strip() for c in line.strip().strip("|").split("|")]
                if cells[0] == key + ", FP64 pipe":
                    return {"fp64_pipe_busy_pct": float(cells[1]), "lanes_active_of_32": float(cells[2]),
                            "hits_through_moments_pct": float(cells[3])}
    except Exception:
        pass
    return None


def hbm_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def read_traffic(key: str):
    """DRAM bytes per launch from the committed ncu summary (profiles/ncu_traffic.txt): the row whose
    first cell is ``key`` ("kernel @ workload"), last cell = bytes per full-size launch."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    try:
        for line in open(p):
            if line.startswith("|"):
                cells = [c.strip() for c in line.strip().strip("|").split("|")]
                if cells and cells[0] == key:
                    return float(cells[-1])
    except Exception:
        pass
    return None


def replica_rate(n_local: int, steps: int, seconds_local: float, dist=None, device: str = "cpu"):
    """Whole-job particle-steps/s of independent replicas (one per rank, no data-path collective):
    particles summed over the ranks, time of the slowest rank.  Returns (rate, slowest seconds)."""
    if dist is None:
        return n_local * steps / seconds_local, seconds_local
    import torch
    t = torch.tensor([seconds_local], dtype=torch.float64, device=device)
    n = torch.tensor([float(n_local)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(n, op=dist.ReduceOp.SUM)
    return float(n.item()) * steps / float(t.item()), float(t.item())


class ClockSampler:
    """nvidia-smi clock / throttle samples while the timed region runs."""

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.index), "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            if len(r) >= 9:
                for k, nm in enumerate(names):
                    if r[5 + k].lower().startswith("active"):
                        reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------------------------------------
def cpu_reference_run(name: str, steps: int, warmup: int, target_s: float = 15.0, nthreads: int | None = None,
                      mesh_kw: dict | None = None):
    """Time the reference algorithm (oracle, OpenMP) on a bounded sample of the workload: the full mesh
    with as many particles as fit ~target_s seconds per step (at most the full particle count).  The
    per-step cost is a fixed part (zeroing PartSource, per-thread accumulators and their reduction) plus
    a per-particle part; two probe sizes fit both, so that the sample is sized for the target time."""
    import oracle
    from piclas_gb300 import capi, workloads
    oracle.build()
    oracle.set_timing_build(True)     # -O3 with FMA contraction, as the reference's release build
    nthreads = nthreads or max(1, os.cpu_count() or 1)
    w = make_workload(name, seed=0, n_override=20000, **(mesh_kw or {}))
    ms = capi.MeshStruct(w.mesh)
    cfg = w.config()
    n_full = 16_000_000 if name == "curved" else 200_000

    def sample(n):
        if name == "curved":
            return workloads.curved_two_species(n_per_species=max(n // 2, 1), seed=0, mesh=w.mesh)
        return workloads.plasma_wave(n_particles=n, seed=0, mesh=w.mesh)

    def run(wk, nsteps):
        st = oracle.OracleState(wk.part_state, wk.elem, wk.part_species)
        if wk.tracking == capi.PIC_TRACK_REFMAPPING:
            oracle.map_particles(cfg, ms, st, nthreads)
        PS = np.zeros(wk.mesh.dof_shape(4))
        t0 = time.perf_counter()
        oracle.step(cfg, ms, wk.e_dof, st, wk.dt, nsteps, PS, nthreads)
        return time.perf_counter() - t0

    n1, n2 = 20000, min(100000, n_full)
    run(w, 1)                      # first run pays thread start-up and page faults
    t1 = run(w, 1)
    t2 = run(sample(n2), 1) if n2 > n1 else t1
    per = max((t2 - t1) / max(n2 - n1, 1), 1e-9)
    fixed = max(t1 - per * n1, 0.0)
    n_sample = int(min(max((target_s - fixed) / per, n1), n_full))
    if n_sample == n_full:
        # the whole workload fits: time more steps instead (at most 1000) so the sample lasts ~target_s
        steps = int(min(max(steps, target_s / max(fixed + per * n_full, 1e-6)), 1000))
    ws = sample(n_sample)
    if warmup > 0:
        run(ws, 1)
    t = run(ws, steps)
    oracle.set_timing_build(False)
    value = ws.n * steps / t
    return {"value": value, "unit": "particle-steps/s", "cores": nthreads, "kind": "port",
            "sample": f"{ws.n} of {n_full} particles x {steps} steps on the full {w.mesh.nx}^3 mesh "
                      f"(C restatement of the reference loop built -O3 like the reference's release build, "
                      f"OpenMP {nthreads} threads, {t:.1f} s; fitted per step {fixed:.2f} s + "
                      f"{per * 1e6:.2f} us/particle)"}


def cpu_baselines(name: str, target_s: float, mesh_kw: dict | None = None):
    """All host cores (the reported baseline) and one core (the reference itself runs one rank per core)."""
    allc = cpu_reference_run(name, steps=1, warmup=0, target_s=target_s, mesh_kw=mesh_kw)
    try:
        one = cpu_reference_run(name, steps=1, warmup=0, target_s=target_s * 0.6, nthreads=1, mesh_kw=mesh_kw)
        allc["one_core"] = {"value": one["value"], "cores": 1, "sample": one["sample"]}
    except Exception as ex:
        allc["one_core"] = {"error": repr(ex)}
    return allc


def mesh_kwargs(args):
    """The mesh variant flags of a curved-workload run (periodic BC tracing, NGeo, p-adaption)."""
    if args.workload != "curved":
        return {}
    return {"periodic_tracing": args.periodic_tracing, "n_geo": args.ngeo, "p_adaption": args.p_adaption,
            "walls": args.walls, "wall_bulge": args.wall_bulge}


# ----------------------------------------------------------------------------------------------
def run_gpu(args, rank, world, local_rank):
    import torch
    from piclas_gb300 import ParticleLoop, capi, load_library
    torch.cuda.set_device(local_rank)
    load_library(build_if_missing=True)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))

    mixed = args.precision == "mixed"
    prec = capi.PIC_PREC_MIXED if mixed else capi.PIC_PREC_FP64
    t0 = time.time()
    w = make_workload(args.workload, seed=rank, n_override=args.particles, cells=args.cells,
                      **mesh_kwargs(args))
    log(f"[rank {rank}] workload {w.name} built in {time.time() - t0:.1f}s")
    cfg = w.config(precision=prec, sort_interval=args.sort_interval)
    loop = ParticleLoop(cfg, w.mesh)
    loop.set_field(w.e_dof)
    loop.upload_particles(w.part_state, w.elem, w.part_species)
    stream = torch.cuda.ExternalStream(loop.stream_ptr)
    flush = None
    l2_flush = args.workload == "plasma_wave"
    if l2_flush:
        flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    # warm-up (the L2-flush kernel too, so its first-launch module load stays out of the timed region)
    loop.time_step(w.dt, args.warmup)
    if flush is not None:
        with torch.cuda.stream(stream):
            flush.fill_(0.5)
        torch.cuda.synchronize()
    loop.synchronize()

    def timed(nsteps):
        evs = []
        launches0 = loop.launch_count
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        loop.synchronize()
        if not l2_flush:
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            loop.time_step(w.dt, nsteps)
            b.record(stream)
            b.synchronize()
            ms = a.elapsed_time(b)
        else:
            ms = 0.0
            for _ in range(nsteps):
                with torch.cuda.stream(stream):
                    flush.fill_(1.0)
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(stream)
                loop.time_step(w.dt, 1)
                b.record(stream)
                b.synchronize()
                ms += a.elapsed_time(b)
        loop.synchronize()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        return ms, loop.launch_count - launches0

    with ClockSampler(local_rank) as clk:
        ms, launches = timed(args.steps)
    value, ms = replica_rate(w.n, args.steps, ms / 1e3, dist, "cuda")
    ms *= 1e3
    st = loop.status()

    # dominant kernel, timed live with CUDA events on the library's stream
    loop.profile(True)
    loop.time_step(w.dt, args.steps)
    prof = loop.profile_read()
    loop.profile(False)
    kname, kbytes = dominant_kernel_bytes(w, mixed)
    try:
        fma_peak = loop.fp32_fma_rate() if mixed else loop.fp64_fma_rate()
    except Exception:
        fma_peak = None
    dom = prof["deposit_main"]
    # a p-adapted mesh gathers with one launch per degree: the gather of a step is all of them
    avg_ms = dom["ms"] / max(dom["launches"] if w.mesh.n_loc is None else args.steps, 1)
    peak, peak_kind = hbm_peak()
    achieved = kbytes / (avg_ms / 1e3) / 1e9
    default_size = args.cells is None and args.particles is None
    traffic = read_traffic(f"{kname} @ {args.workload}") if default_size else None
    comp = compute_roofline(w, mixed, avg_ms, fma_peak)
    share = dom["ms"] / max(sum(v["ms"] for v in prof.values()), 1e-9)
    hbm = {"achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
           "algorithmic_bytes": kbytes, "traffic": traffic}
    if comp is not None:
        # the kernel's own bound: FP64 pipe (FP64) or instruction issue (mixed); HBM figures beside it
        roof = {"kernel": kname, "bound": comp["bound"], "achieved": comp["achieved"], "peak": comp["peak"],
                "unit": comp["unit"], "frac": comp["frac"], "traffic": traffic, "peak_kind": comp["peak_kind"],
                "avg_launch_ms": avg_ms, "share": share, "hbm": hbm}
        for extra in ("ncu_16cube", "note"):
            if extra in comp:
                roof[extra] = comp[extra]
    else:
        roof = {"kernel": kname, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind, "avg_launch_ms": avg_ms,
                "share": share, "algorithmic_bytes": kbytes}

    # end-to-end through the C-ABI with host buffers: per step the HDG hand-over (E in, PartSource out)
    E_host = torch.from_numpy(np.ascontiguousarray(w.e_dof)).pin_memory()
    PS_host = torch.zeros(w.mesh.dof_shape(4), dtype=torch.float64).pin_memory()
    loop.synchronize()
    te0 = time.perf_counter()
    for _ in range(args.steps):
        loop.set_field_ptr(E_host.data_ptr())
        loop.time_step_ptr(w.dt, 1, PS_host.data_ptr())
    te = time.perf_counter() - te0
    e2e = {"value": replica_rate(w.n, args.steps, te, dist, "cuda")[0], "unit": "particle-steps/s",
           "h2d_bytes_per_step": int(E_host.numel() * 8), "d2h_bytes_per_step": int(PS_host.numel() * 8)}

    out = {
        "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if not mixed else "f32+f64",
        "data": "synthetic (seeded), frozen field",
        "config": dict(workload_config(w, args.workload), precision=args.precision, parallelism=f"replicas x{world}"),
        "gpu_launches": int(launches),
        "loop_hbm": {"bytes_per_step": algorithmic_bytes_per_step(w, mixed),
                     "achieved_gbs": algorithmic_bytes_per_step(w, mixed) * args.steps / (ms / 1e3) / 1e9},
        "roofline": roof,
        "phases_ms": {k: round(v["ms"] / args.steps, 4) for k, v in prof.items() if v["launches"]},
        "e2e": e2e,
        "status": st,
    }
    clocks = clk.summary()
    out["clocks"] = clocks
    loop.close()
    del E_host, PS_host

    if rank == 0 and world == 1 and not mixed:
        try:
            out["mixed"] = mixed_arm(args, w)
        except Exception as ex:
            out["mixed"] = {"error": repr(ex)}
    if rank == 0 and world == 1 and not args.no_extras:
        try:
            out["extras"] = extras(args, w)
        except Exception as ex:  # extras are informative only
            out["extras"] = {"error": repr(ex)}
    if rank == 0 and not args.no_cpu:
        try:
            out["cpu_baseline"] = cpu_baselines(args.workload, args.cpu_seconds, mesh_kwargs(args))
        except Exception as ex:
            out["cpu_baseline"] = {"error": repr(ex)}
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(out), flush=True)


def rho_species_scale(w, g):
    """max over DOFs of sum_s |rho_s|: each species of the state g deposited on its own (FP64).  Electrons and
    ions cancel in the summed rho; a precision error is measured against what the species deposit."""
    from piclas_gb300 import ParticleLoop, capi
    tot = np.zeros(w.mesh.dof_shape(4)[:-1])
    for s in np.unique(w.part_species):
        k = (w.part_species == s) & (g["inside"] == 1)
        loop = ParticleLoop(w.config(precision=capi.PIC_PREC_FP64), w.mesh)
        loop.upload_particles(g["part_state"][k], g["elem"][k], w.part_species[k], is_new=np.zeros(int(k.sum()), np.uint8))
        tot += np.abs(loop.deposition()[..., 3])
        loop.close()
    return float(tot.max())


def mixed_arm(args, w):
    """The mixed-precision variant on the same workload: particle-steps/s (CUDA events on the library's
    stream, the same warm-up and step count as the FP64 arm), the dominant kernel's issue-bound roofline,
    and the charge-density error against the FP64 arm after 2 steps from the same particles (max |d rho|
    over max sum_s |rho_s|, and over max |rho|) with the element mismatches."""
    import torch
    from piclas_gb300 import ParticleLoop, capi
    loop = ParticleLoop(w.config(precision=capi.PIC_PREC_MIXED, sort_interval=args.sort_interval), w.mesh)
    loop.set_field(w.e_dof)
    loop.upload_particles(w.part_state, w.elem, w.part_species)
    s = torch.cuda.ExternalStream(loop.stream_ptr)
    loop.time_step(w.dt, args.warmup)
    loop.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record(s)
    loop.time_step(w.dt, args.steps)
    b.record(s)
    b.synchronize()
    ms = a.elapsed_time(b)
    loop.profile(True)
    loop.time_step(w.dt, args.steps)
    prof = loop.profile_read()
    loop.profile(False)
    try:
        fp32_peak = loop.fp32_fma_rate()
    except Exception:
        fp32_peak = None
    loop.close()
    dom = prof["deposit_main"]
    avg_ms = dom["ms"] / max(dom["launches"] if w.mesh.n_loc is None else args.steps, 1)
    kname, kbytes = dominant_kernel_bytes(w, True)
    out = {"value": w.n * args.steps / (ms / 1e3), "unit": "particle-steps/s", "ms_per_step": ms / args.steps,
           "phases_ms": {k: round(v["ms"] / args.steps, 4) for k, v in prof.items() if v["launches"]},
           "roofline": dict(compute_roofline(w, True, avg_ms, fp32_peak) or {}, kernel=kname, avg_launch_ms=avg_ms,
                            hbm={"achieved": kbytes / (avg_ms / 1e3) / 1e9, "algorithmic_bytes": kbytes})}

    def two_steps(prec):
        lp = ParticleLoop(w.config(precision=prec), w.mesh)
        lp.set_field(w.e_dof)
        lp.upload_particles(w.part_state, w.elem, w.part_species)
        PS = np.zeros(w.mesh.dof_shape(4))
        lp.time_step(w.dt, 2, PS)
        g = lp.download_particles()
        lp.close()
        return PS, g

    ps64, g64 = two_steps(capi.PIC_PREC_FP64)
    ps32, g32 = two_steps(capi.PIC_PREC_MIXED)
    d = float(np.max(np.abs(ps32[..., 3] - ps64[..., 3])))
    out["rho_rel_err_vs_fp64"] = d / rho_species_scale(w, g64)
    out["rho_rel_err_vs_fp64_of_max_rho"] = d / float(np.max(np.abs(ps64[..., 3])))
    out["elem_mismatch"] = int((g32["elem"] != g64["elem"]).sum())
    return out


def extras(args, w_main):
    """The plasma-wave pair (FP64 / mixed), its per-step mixed error, the 32-instance batch, the adjoint and
    the HDG solve."""
    import torch
    from piclas_gb300 import ParticleLoop, capi, workloads
    res = {}

    def rate(w, prec, steps, flush_l2):
        loop = ParticleLoop(w.config(precision=prec, sort_interval=args.sort_interval), w.mesh)
        loop.set_field(w.e_dof)
        loop.upload_particles(w.part_state, w.elem, w.part_species)
        s = torch.cuda.ExternalStream(loop.stream_ptr)
        loop.time_step(w.dt, 3)
        loop.synchronize()
        buf = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda") if flush_l2 else None
        tot = 0.0
        for _ in range(steps):
            if buf is not None:
                with torch.cuda.stream(s):
                    buf.fill_(2.0)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(s)
            loop.time_step(w.dt, 1)
            b.record(s)
            b.synchronize()
            tot += a.elapsed_time(b)
        loop.close()
        return w.n * steps / (tot / 1e3), tot / steps

    def rho_after_one_step(w, prec):
        loop = ParticleLoop(w.config(precision=prec), w.mesh)
        loop.set_field(w.e_dof)
        loop.upload_particles(w.part_state, w.elem, w.part_species)
        PS = np.zeros(w.mesh.dof_shape(4))
        loop.time_step(w.dt, 2, PS)
        g = loop.download_particles()
        loop.close()
        return PS, g

    # plasma wave (the reference's CPU-runnable case) in FP64 and mixed, L2 flushed between steps
    pw = workloads.plasma_wave()
    v64, ms64 = rate(pw, capi.PIC_PREC_FP64, 20, True)
    v32, ms32 = rate(pw, capi.PIC_PREC_MIXED, 20, True)
    ps64, g64 = rho_after_one_step(pw, capi.PIC_PREC_FP64)
    ps32, g32 = rho_after_one_step(pw, capi.PIC_PREC_MIXED)
    res["plasma_wave"] = {"fp64": {"value": v64, "ms_per_step": ms64}, "mixed": {"value": v32, "ms_per_step": ms32},
                          "mixed_over_fp64": v32 / v64,
                          "rho_rel_err_vs_fp64": float(np.max(np.abs(ps32[..., 3] - ps64[..., 3])) /
                                                       np.max(np.abs(ps64[..., 3]))),
                          "elem_mismatch": int((g32["elem"] != g64["elem"]).sum())}
    # mixed precision on the plasma wave: error vs FP64 after every one of the 100 steps
    from piclas_gb300 import precision_report
    res["plasma_wave_mixed_per_step"] = precision_report.summarize(
        precision_report.mixed_vs_fp64_per_step(pw, pw.nsteps))
    res["batch"] = batch_summary(batch_run(args))
    res["adjoint"] = adjoint_timing()
    res["hdg"] = hdg_timing()
    return res


def hdg_timing(cells=(8, 32), reps: int = 3, self_consistent: bool = True, cg_kernel: int = 0):
    """HDG Poisson solve (HDGLinear: RHS, CG_solver, PostProcessGradientHDG; Elem_Mat once at init) on periodic
    boxes of 8^3 (the plasma-wave mesh) and 32^3 (the curved workload's mesh) hexahedra, N = 3, PrecondType 2,
    epsCG 1e-6 relative to the first residual, each solve from lambda = 0.  The source is the periodic
    manufactured case phi = sin(2pi x+1) sin(2pi y+2) sin(2pi z+3).  Reported: init time, solve time,
    CG iterations, and the Smat bytes streamed per iteration over the CG time (the matvec reads every
    element's 36 blocks once per iteration).  The oracle's single-threaded solve of the 8^3 case is timed
    beside it.  Then the self-consistent plasma wave (200k electrons + 200k resting ions, CVWM,
    TriaTracking, one solve per step from the previous lambda) in FP64 and mixed."""
    import torch
    from piclas_gb300 import ParticleLoop, capi, workloads
    from piclas_gb300.hdg_mesh import build_hdg_mesh
    from piclas_gb300.mesh import build_box_mesh
    out = {}
    tp = 2.0 * np.pi

    def source(m):
        x = tp * m.elem_xgp
        phi = np.sin(x[..., 0] + 1.0) * np.sin(x[..., 1] + 2.0) * np.sin(x[..., 2] + 3.0)
        return (-3.0 * tp * tp * phi).reshape(m.n_elems, -1)

    for n in cells:
        m = build_box_mesh(n, n, n, 3, perturb=0.05 if n == 32 else 0.0)
        h = build_hdg_mesh(m)
        cfg = capi.make_config(3, capi.PIC_TRACK_TRIA, capi.PIC_DEPO_CVWM, capi.PIC_PREC_FP64,
                               [(-1.60217653e-19, 9.1093826e-31, 1.0)], 1)
        loop = ParticleLoop(cfg, m)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        loop.hdg_init(h, precond_type=2, eps_cg=1e-6, relative=True, max_iter_cg=5000, cg_kernel=cg_kernel)
        t_init = time.perf_counter() - t0
        src = source(m)
        zero = np.zeros((h.n_sides, 16))
        loop.hdg_set_lambda(zero)
        loop.hdg_solve(src, want_phi=False, want_e=False)                  # warm-up
        times, its = [], []
        for _ in range(reps):
            loop.hdg_set_lambda(zero)
            t0 = time.perf_counter()
            _, _, st = loop.hdg_solve(src, want_phi=False, want_e=False)
            times.append(time.perf_counter() - t0)
            its.append(st["iterations"])
        tsol = float(np.median(times))
        # the matvec is FP64-bound: 36 blocks of 16x16 per element, one fused multiply-add per entry
        # (the 15 off-diagonal stored blocks are applied twice, S_ij and S_ij^T)
        flops = 2.0 * 36 * 16 * 16 * m.n_elems
        entry = {"mesh": f"{n}^3 hex, N=3, periodic", "elements": m.n_elems, "sides": h.n_sides,
                 "init_s": t_init, "solve_ms": tsol * 1e3, "cg_iterations": int(its[0]),
                 "ms_per_iteration": tsol * 1e3 / max(its[0], 1),
                 "matvec_fp64_gflops_lower_bound": flops * its[0] / tsol / 1e9}
        loop.close()
        if n == cells[0]:
            import oracle
            o = oracle.HdgOracle(m, h)
            t0 = time.perf_counter()
            _, _, it_o, _, _ = o.solve(src, precond_type=2, eps_cg=1e-6, relative=True, max_iter=5000)
            t_o = time.perf_counter() - t0
            entry["oracle_cpu"] = {"solve_ms": t_o * 1e3, "cg_iterations": it_o, "cores": 1,
                                   "kind": "port"}
        out[f"{n}cube"] = entry

    if not self_consistent:
        return out
    # self-consistent plasma wave: Deposition -> HDG -> push -> TriaTracking every step
    pw = workloads.plasma_wave()
    rng = np.random.default_rng(7)
    xi = rng.random((pw.n, 3)) * (pw.mesh.hi - pw.mesh.lo) + pw.mesh.lo
    q, mass, mpf = pw.species[0]
    w = workloads.Workload(**{**pw.__dict__, "species": [pw.species[0], (-q, 1836.0 * mass, mpf)],
                              "part_state": np.concatenate([pw.part_state, np.concatenate([xi, np.zeros((pw.n, 3))], 1)]),
                              "elem": np.concatenate([pw.elem, workloads._elem_of_uniform(pw.mesh, xi)]).astype(np.int32),
                              "part_species": np.concatenate([pw.part_species, np.full(pw.n, 2, np.int32)])})
    h = build_hdg_mesh(w.mesh)
    sc = {"workload": "plasma wave 8^3 N=3, 200k e- + 200k ions, CVWM, TriaTracking, HDG every step "
                      "(PrecondType 2, epsCG 1e-6 relative, warm start)", "particles": w.n}
    for name, prec in (("fp64", capi.PIC_PREC_FP64), ("mixed", capi.PIC_PREC_MIXED)):
        loop = ParticleLoop(w.config(precision=prec), w.mesh)
        loop.upload_particles(w.part_state, w.elem, w.part_species)
        loop.hdg_init(h, precond_type=2, eps_cg=1e-6, relative=True, max_iter_cg=5000, solve_in_step=True)
        loop.time_step(w.dt, 3)
        loop.synchronize()
        loop.profile(True)
        steps = 20
        t0 = time.perf_counter()
        loop.time_step(w.dt, steps)
        loop.synchronize()
        t = time.perf_counter() - t0
        prof = loop.profile_read()
        loop.profile(False)
        sc[name] = {"particle_steps_per_s": w.n * steps / t, "ms_per_step": t * 1e3 / steps,
                    "hdg_ms_per_step": prof["hdg"]["ms"] / steps}
        loop.close()
    out["self_consistent_plasma_wave"] = sc
    return out


def adjoint_timing():
    """The differentiable loop (16^3, N=2, 1M electrons, B_z = 0.05 T, 50 steps, checkpoint every 10): wall
    time of one pic_adjoint_run (forward, recomputed segments and reverse pass) in FP64 and FP32."""
    import torch
    from piclas_gb300 import ParticleLoop, capi, workloads
    w = workloads.differentiable_loop()
    loop = ParticleLoop(w.config(), w.mesh)
    loop.set_field(w.e_dof)
    loop.upload_particles(w.part_state, w.elem, w.part_species, is_new=np.zeros(w.n, np.uint8))
    out = {"workload": "16^3 linear hex, N=2, 1M e-, 50 push+deposit steps, checkpoint 10", "particles": w.n}
    for name, prec in (("fp64", capi.PIC_PREC_FP64), ("fp32", capi.PIC_PREC_MIXED)):
        loop.adjoint(w.nsteps, w.dt, w.info["rho_target"], w.info["rho_scale"], precision=prec)   # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        L, gv, gb = loop.adjoint(w.nsteps, w.dt, w.info["rho_target"], w.info["rho_scale"], precision=prec)
        t = time.perf_counter() - t0
        out[name] = {"seconds": t, "particle_steps_per_s": w.n * w.nsteps / t, "loss": L, "dL_dB": gb}
    loop.close()
    return out


def batch_run(args):
    """32 independent plasma-wave instances (meshes {4,8,12,16}^3, N=3, 1e4..2e6 particles log-uniform,
    amplitude U[0.005,0.05], 100 steps), each run and timed separately in mixed precision (CUDA events on its
    own stream); the FP64 run of the same instance gives the charge-density error.  Then the 32 mixed
    instances again, all at once: each context enqueues its 100 steps on its own stream and the wall time
    from the first launch to the last completion gives the aggregate (contexts carry their own constants,
    so they run side by side)."""
    import torch
    from piclas_gb300 import ParticleLoop, capi, load_library, workloads
    load_library(build_if_missing=True)
    inst = workloads.batch_instances(32)
    out = []
    tot_ps, tot_ms = 0.0, 0.0
    ws = []
    for k, p in enumerate(inst):
        w = workloads.plasma_wave(n_cells=p["n_cells"], N=3, n_particles=p["n_particles"], amp=p["amp"],
                                  seed=p["seed"], nsteps=p["nsteps"])
        ws.append(w)
        res = {}
        for prec in (capi.PIC_PREC_MIXED, capi.PIC_PREC_FP64):
            loop = ParticleLoop(w.config(precision=prec, sort_interval=args.sort_interval), w.mesh)
            loop.set_field(w.e_dof)
            loop.upload_particles(w.part_state, w.elem, w.part_species)
            s = torch.cuda.ExternalStream(loop.stream_ptr)
            PS = np.zeros(w.mesh.dof_shape(4))
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            loop.synchronize()
            a.record(s)
            loop.time_step(w.dt, w.nsteps)
            b.record(s)
            b.synchronize()
            ms = a.elapsed_time(b)
            loop.time_step(w.dt, 1, PS)
            st = loop.status()
            g = loop.download_particles()
            loop.close()
            res[prec] = (ms, PS, g, st)
        ms, PS32, g32, st = res[capi.PIC_PREC_MIXED]
        _, PS64, g64, _ = res[capi.PIC_PREC_FP64]
        err = float(np.max(np.abs(PS32[..., 3] - PS64[..., 3])) / np.max(np.abs(PS64[..., 3])))
        rate = w.n * w.nsteps / (ms / 1e3)
        tot_ps += w.n * w.nsteps
        tot_ms += ms
        out.append({"instance": k, "cells": p["n_cells"], "particles": w.n, "amp": round(p["amp"], 5),
                    "ms": round(ms, 3), "particle_steps_per_s": rate, "rho_rel_err_vs_fp64": err,
                    "elem_mismatch": int((g32["elem"] != g64["elem"]).sum()), "lost": st["n_lost"]})
        log(f"[batch] {k}: {p['n_cells']}^3 {w.n} particles {ms:.2f} ms  {rate:.3g} p-s/s  rho err {err:.2e}")
    # all 32 at once, one stream per context
    loops = []
    for w in ws:
        lp = ParticleLoop(w.config(precision=capi.PIC_PREC_MIXED, sort_interval=args.sort_interval), w.mesh)
        lp.set_field(w.e_dof)
        lp.upload_particles(w.part_state, w.elem, w.part_species)
        lp.time_step(w.dt, 3)
        loops.append(lp)
    for lp in loops:
        lp.synchronize()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for lp, w in zip(loops, ws):
        lp.time_step(w.dt, w.nsteps)
    for lp in loops:
        lp.synchronize()
    t_conc = time.perf_counter() - t0
    for lp in loops:
        lp.close()
    return {"instances": out, "sequential_ms": tot_ms, "particle_steps": tot_ps, "concurrent_s": t_conc}


def batch_summary(r):
    return {"workload": "batch of 32 mixed-precision plasma-wave instances (4^3..16^3, 1e4..2e6 particles, 100 steps)",
            "aggregate_particle_steps_per_s": r["particle_steps"] / (r["sequential_ms"] / 1e3),
            "concurrent_particle_steps_per_s": r["particle_steps"] / r["concurrent_s"],
            "concurrent_wall_s": r["concurrent_s"],
            "max_rho_rel_err": max(x["rho_rel_err_vs_fp64"] for x in r["instances"]),
            "elem_mismatch_total": sum(x["elem_mismatch"] for x in r["instances"]),
            "per_instance_particle_steps_per_s": [round(x["particle_steps_per_s"]) for x in r["instances"]],
            "per_instance_rho_rel_err": [x["rho_rel_err_vs_fp64"] for x in r["instances"]]}


def run_batch(args):
    r = batch_run(args)
    print(json.dumps(dict(batch_summary(r), metric=METRIC, instances=r["instances"])), flush=True)


def reference_config(args):
    """The config of this arm's line for the same flags (the reference computes in FP64 whatever the
    precision flag says)."""
    from types import SimpleNamespace as NS
    from piclas_gb300.mesh import p_adaption_degrees
    cells, n = {"curved": (32, 16_000_000), "plasma_wave": (8, 200_000)}.get(args.workload, (8, 200_000))
    n_loc = p_adaption_degrees(cells, cells, cells, args.p_adaption, 1, 3, seed=0) if args.p_adaption else None
    n_dofs = cells ** 3 * 64 if n_loc is None else int(((np.asarray(n_loc) + 1) ** 3).sum())
    walls = args.walls if args.workload == "curved" else None
    stand_in = NS(mesh=NS(n_elems=cells ** 3, N=3, n_geo=args.ngeo, n_loc=n_loc, n_dofs=n_dofs), n=n,
                  periodic_tracing=args.periodic_tracing, walls=walls, wall_bulge=args.wall_bulge if walls else 0.0)
    return dict(workload_config(stand_in, args.workload if args.workload == "curved" else "plasma_wave"),
                precision=args.precision, parallelism=f"replicas x{args.gpus}")


def run_reference(args, rank):
    if rank != 0:
        return
    nsteps = max(args.steps, 1)
    # each step a bounded sample; the whole run (probes, warm-up, steps) stays within about three minutes
    per_step = min(args.cpu_seconds, 150.0 / (nsteps + (1 if args.warmup > 0 else 0)))
    base = cpu_reference_run(args.workload, steps=nsteps, warmup=args.warmup, target_s=per_step,
                             mesh_kw=mesh_kwargs(args))
    out = {"metric": METRIC, "value": base["value"], "unit": "particle-steps/s", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded), frozen field",
           "impl": "reference", "config": reference_config(args),
           "cpu_baseline": base,
           "e2e": {"value": base["value"], "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="curved", choices=["curved", "plasma_wave", "batch", "hdg"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--sort-interval", type=int, default=10)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--particles", type=int, default=None, help="override the particle count (profiling cases)")
    ap.add_argument("--cells", type=int, default=None, help="override the elements per axis (profiling cases)")
    ap.add_argument("--ngeo", type=int, default=1, choices=[1, 2, 3, 4],
                    help="curved workload on elements of this geometry degree (NGeo > 1: curved elements)")
    ap.add_argument("--p-adaption", default=None, choices=["random", "half-half"],
                    help="curved workload with per-element degrees 1..3 (N_DG_Mapping)")
    ap.add_argument("--periodic-tracing", action="store_true",
                    help="RefTracking traces the periodic sides as BC sides (the reference's default CartesianPeriodic = F)")
    ap.add_argument("--walls", default=None, choices=["reflective"],
                    help="curved workload in a closed box with these walls all round (ParticleBCTracking)")
    ap.add_argument("--wall-bulge", type=float, default=0.0,
                    help="with --walls: bulge the wall faces inwards by this fraction of h (curved sides at NGeo > 1)")
    ap.add_argument("--hdg-cg-kernel", type=int, default=0, choices=[0, 1, 2],
                    help="HDG CG launch form: 0 auto, 1 kernel per phase (graph), 2 cooperative")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl != "reference":
        log("warm-up raised to 3 steps")
        args.warmup = 3
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if args.workload == "batch":
        if rank == 0:
            run_batch(args)
        return
    if args.workload == "hdg":
        # the HDG field solve alone (also the extras' "hdg" entry); --cells picks one mesh size
        if rank == 0:
            cells = (args.cells,) if args.cells else (8, 32)
            print(json.dumps({"hdg": hdg_timing(cells=cells, self_consistent=not args.no_extras,
                                                cg_kernel=args.hdg_cg_kernel)}), flush=True)
        return
    run_gpu(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
