"""Benchmark of the fvm2d hot path on GB300.

Workload (the large Euler case): NACA 0012 O-grids of 1024 x 384 vertices
(393,216 vertices, 784,384 triangles, 1,177,600 edges each), interior
vertices jittered by +-10% of the local spacing from per-mesh seeds,
M 0.8, AoA 1.25 deg, Roe flux with Green-Gauss MUSCL + van Albada limiter,
3-stage RK, CFL 1.0, local time stepping, freestream start.  FP32 state,
reconstruction, fluxes and RK stages; FP64 geometry, residual norm and
forces.  ``--meshes`` (default 8) independent meshes share one device arena
and every kernel launch (the batched path), so the working set (about
1 GB) is far larger than the 129 MB L2: no L2 flush is needed between
steps.

A step is one full iteration of main.f:44-62 over every mesh of the batch:
time step, three RK stages (gradients, fluxes, update), monitors.
value = meshes x vertices x 3 stages x steps / device time of the steps.

Also reported on the same line:
  e2e           the same solve driven through the C ABI with host buffers:
                state upload, iterations, RES.DAT rows and final state
                download all inside the timed region;
  roofline      the flux kernel (the dominant one): algorithmic bytes per
                launch / its CUDA-event time, against the measured HBM peak;
  cpu_baseline  the CPU oracle (the serial FP64 restatement of the
                reference, single thread) on one mesh of the same workload;
  vs_fp64_gpu   the plain FP64 single-mesh GPU path on the same workload;
  fluxes        FP32 batched throughput with KFVS and HLLC;
  serving       the request workload (512 seeded NACA 4-digit solves,
                Poisson arrivals at 20/s, 5k-400k vertices, 70% Euler / 30%
                laminar) through the continuous-batching service: converged
                solves/s, p50/p99 latency, how many solves reached the
                residual drop, hit the iteration cap or failed; the plain
                FP64 single-mesh path measured on a size-stratified sample
                of the same requests (strict and FMA builds), and the
                served lift/drag against those FP64 solves.
``--impl reference`` times the reference's CPU implementation (the oracle
port; no Fortran compiler exists on this machine or the GPU host, probed
and recorded in the line) on all host cores instead.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = ("vertex-RK-stage updates/s and converged solves/s, p50/p99 latency, vs FP64 GPU")
UNIT = "vertex-RK-stage updates/s"
NI, NR = 1024, 384
FLOW = dict(mach=0.8, aoa_deg=1.25, cfl=1.0, ilimit=1)
FLUX_CODES = {"roe": 1, "kfvs": 2, "hllc": 3}


def grid(seed: int, ni=NI, nr=NR):
    from fvm2d_gb300.ogrid import naca_ogrid
    return naca_ogrid(ni, nr, radius=20.0, first_spacing=5e-4, jitter=0.1, seed=seed)


def sweep_fu_bytes(np_, ne, s=4, g=8, i=4):
    """Algorithmic bytes of one flux+update pass over a mesh: reads edge
    2i and ds 2g per edge; prim 4s, qx/qy 8s, coord 2g, prim_old 4s, dt s,
    cvarea g per vertex; writes prim 4s per vertex."""
    return ne * (2 * i + 2 * g) + np_ * (4 * s + 8 * s + 2 * g + 4 * s + s + g + 4 * s)


def bytes_per_vertex_stage(np_, nt, ne, s=4, g=8):
    """P(36s + 19g/3) + 12T + E(8 + 2g), per vertex-stage."""
    return (np_ * (36 * s + 19 * g / 3) + 12 * nt + ne * (8 + 2 * g)) / np_


class ClockSampler:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self._t.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for k, n in enumerate(names):
                if f[5 + k].strip() == "Active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic():
    """DRAM bytes per flux-kernel launch per mesh from the committed ncu
    summary (None if absent)."""
    p = os.path.join(ROOT, "profiles", "flux_fp32_traffic.txt")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        for ln in f:
            if ln.startswith("dram_bytes_per_launch_per_vertex:"):
                return float(ln.split(":")[1])
    return None


def build_meshes(nmesh, rank):
    import fvm2d_gb300 as F
    from fvm2d_gb300.replicas import seed_for
    out = []
    for k in range(nmesh):
        g = grid(seed_for(rank, k))
        out.append(F.build_geometry(g.coord, g.elem, g.ptype))
    return out


def run_gpu(args):
    import torch

    import fvm2d_gb300 as F
    from fvm2d_gb300 import replicas
    from fvm2d_gb300.batch import Batch

    replicas.init()
    rank, local, size = replicas.world()
    torch.cuda.set_device(local)
    dev = torch.cuda.current_device()
    meshes = build_meshes(args.meshes, rank)
    P, T, E = meshes[0].np, meshes[0].nt, meshes[0].ne
    V = sum(m.np for m in meshes)

    def make_batch(flux, precision, ms):
        b = Batch(precision, vertices=sum(m.np for m in ms), meshes=len(ms))
        par = F.make_params(iflux=flux, precision=precision, bugcompat=0, **FLOW)
        slots = [b.add(par, m) for m in ms]
        return b, slots

    # ---- value: FP32 batch, Roe ------------------------------------------
    b, slots = make_batch(FLUX_CODES[args.flux], F.FP32, meshes)
    ext = torch.cuda.ExternalStream(b.stream())
    for s in slots:
        b.start(s, args.warmup + 2 * args.steps + 200)   # + the tuner's iterations
    b.step(args.warmup)
    b.sync()
    if args.form:             # a given form (profiling runs): no tuning
        b.set_form(args.form)
        tuned = {"choice": args.form, "ms_per_iter": None}
    else:
        tuned = b.tune(iters=5)   # ordinary iterations of the solves; untimed
    b.sync()
    b.step(1)           # instantiates the timed graph outside the timed region
    b.sync()
    n0 = b.launch_count()
    replicas.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        e0.record(ext)
        b.step(args.steps)
        e1.record(ext)
        b.sync()
        torch.cuda.synchronize()
    replicas.barrier()
    launches = b.launch_count() - n0
    ms_local = e0.elapsed_time(e1)
    ms = replicas.max_over_ranks(ms_local)
    # per-kernel CUDA events over a second pass of the same steps (reading
    # them needs a host sync after every iteration, kept out of `value`);
    # kernels one at a time (no overlapped chains), so each launch's time
    # is its own
    alone = {"split+overlap": "bulk", "split+overlap4": "bulk", "split+overlap8": "bulk",
             "fused+overlap": "fused", "pipe+overlap": "pipe",
             "pipe+overlap4": "pipe"}.get(b.form, b.form)
    b.set_form(alone)
    b.timing(True)
    b.step(1)
    b.sync()
    b.timing(True)      # resets the per-kernel accumulators
    b.step(args.steps)
    b.sync()
    kt = b.timing_read()
    b.timing(False)
    b.set_form(tuned["choice"])
    units = replicas.sum_over_ranks(V * 3 * args.steps)
    value = units / (ms / 1e3)
    polls = [b.poll(s) for s in slots]
    ok = all(p["status"] == 0 for p in polls)

    fused = kt.get("step", (0.0, 0))[1] > 0
    flux_ms, flux_n = kt["step"] if fused else kt["flux"]
    flux_avg_s = flux_ms / 1e3 / max(flux_n, 1)
    if fused:   # one pass does gradients, fluxes and the update
        alg_stage = sum(bytes_per_vertex_stage(m.np, m.nt, m.ne) * m.np for m in meshes)
        kname = (f"k_step<float, {FLUX_CODES[args.flux]}> (gradients + recon + {args.flux} "
                 "flux + gather + RK stage)")
    else:
        alg_stage = sum(sweep_fu_bytes(m.np, m.ne) for m in meshes)
        # the workload's meshes have math.f's constants: the build with them
        # compiled in (template code + 4)
        kname = (f"k_flux<float, {FLUX_CODES[args.flux] + 4}> (recon + {args.flux} flux + gather "
                 "+ RK stage; math.f constants compiled in)")
    # all launches of the pass together moved alg_stage bytes per stage (with
    # the overlapped chains each launch covers part of the meshes)
    alg_flux = alg_stage * 3 * args.steps / max(flux_n, 1)
    achieved = alg_flux / flux_avg_s / 1e9
    peak, peak_kind = measured_peaks()
    tr = None if fused else profile_traffic()
    roofline = {"bound": "hbm", "kernel": kname,
                "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": f"{peak_kind} hbm_gbs",
                "traffic": (round(tr * V, 0) if tr is not None else None),
                "algorithmic_bytes_per_launch": alg_flux,
                "avg_launch_ms": round(flux_avg_s * 1e3, 4),
                "events": f"CUDA events around every launch, over a second pass of "
                          f"{args.steps} steps ({flux_n} launches) in form '{alone}' (one "
                          "kernel at a time)",
                "kernel_ms_share": {k: round(v[0] / max(sum(x[0] for x in kt.values()), 1e-9), 4)
                                    for k, v in kt.items() if v[1]}}

    # the whole stage (gradient pass + flux pass + monitor) against the
    # per-vertex-stage byte model
    stage_bytes = sum(bytes_per_vertex_stage(m.np, m.nt, m.ne) * m.np for m in meshes)
    stage_gbs = stage_bytes * 3 * args.steps / (ms_local / 1e3) / 1e9
    stage_roofline = {"bound": "hbm", "achieved": round(stage_gbs, 1), "peak": peak,
                      "unit": "GB/s", "frac": round(stage_gbs / peak, 4),
                      "algorithmic_bytes_per_stage": round(stage_bytes, 0),
                      "what": "P(36s + 19g/3) + 12T + E(8 + 2g) bytes per stage over the "
                              "device time of whole iterations"}

    # ---- e2e through the C ABI with host buffers -----------------------------
    # the driver's prim(4,np) arrays in pinned host memory (page-locked, as a
    # driver that keeps its state for device transfers allocates it), filled
    # before the timed region
    init, finals = [], []
    for m in meshes:
        par = F.make_params(precision=F.FP32, **FLOW)
        prim = torch.empty((m.np, 4), dtype=torch.float64, pin_memory=True).numpy()
        prim[:] = [par.r_inf, par.u_inf, par.v_inf, par.p_inf]
        init.append(prim)
        out = torch.empty((m.np, 4), dtype=torch.float64, pin_memory=True).numpy()
        out[:] = 0.0
        finals.append(out)
    b.sync()
    replicas.barrier()
    t0 = time.perf_counter()
    for s, prim in zip(slots, init):
        b.set_state(s, prim)
        b.start(s, args.steps)
    rows = 0
    drained = [0] * len(slots)
    done_steps = 0
    depth = 512
    while done_steps < args.steps:
        k = min(depth, args.steps - done_steps)
        b.step(k)
        done_steps += k
        for j, s in enumerate(slots):      # RES.DAT rows of this chunk
            st = b.poll(s)
            n = st["niter"] - drained[j]
            if n > 0:
                rows += len(b.history(s, drained[j], n)["fres"])
                drained[j] = st["niter"]
    for s, out in zip(slots, finals):     # the solution (prim) of each solve
        b.get_state(s, fields=("prim",), out={"prim": out})
    b.sync()
    e2e_s = replicas.max_over_ranks(time.perf_counter() - t0)
    e2e_value = replicas.sum_over_ranks(V * 3 * args.steps) / e2e_s
    # FP64 driver-order arrays cross the link (permuted and converted on the
    # device): prim in, prim out; RES.DAT rows; the per-mesh control records
    h2d = V * 8 * 4 + len(slots) * 96 * 2
    d2h = V * 8 * 4 + rows * 36 + len(slots) * 96 * 3
    e2e = {"value": e2e_value, "unit": UNIT,
           "h2d_bytes_per_step": round(h2d / args.steps, 1),
           "d2h_bytes_per_step": round(d2h / args.steps, 1),
           "what": "fvm_batch_set_state (pinned host FP64 prim -> device, permuted and "
                   "converted there) + start + steps + RES.DAT rows + fvm_batch_get_state "
                   "(into pinned host arrays), wall clock"}
    b.close()

    extra = {}
    if rank == 0 and not args.quick:
        # FP64 plain single-mesh GPU path on the same workload
        b64, s64 = make_batch(FLUX_CODES[args.flux], F.FP64, meshes[:1])
        n64 = max(5, args.steps // 20)
        b64.start(s64[0], n64 + 3)
        b64.step(2)
        b64.sync()
        ext64 = torch.cuda.ExternalStream(b64.stream())
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record(ext64)
        b64.step(n64)
        f1.record(ext64)
        b64.sync()
        v64 = P * 3 * n64 / (f0.elapsed_time(f1) / 1e3)
        b64.close()
        extra["vs_fp64_gpu"] = {"value": v64, "unit": UNIT,
                                "ratio": value / v64 / size,
                                "what": "FP64 single-mesh path (no FMA contraction), same mesh, "
                                        f"{n64} iterations"}
        fl = {}
        for name in ("kfvs", "hllc"):
            if name == args.flux:
                continue
            bf, sf = make_batch(FLUX_CODES[name], F.FP32, meshes)
            for s in sf:
                bf.start(s, args.steps + 10)
            bf.step(3)
            bf.sync()
            extf = torch.cuda.ExternalStream(bf.stream())
            g0 = torch.cuda.Event(enable_timing=True)
            g1 = torch.cuda.Event(enable_timing=True)
            nst = max(10, args.steps // 5)
            g0.record(extf)
            bf.step(nst)
            g1.record(extf)
            bf.sync()
            fl[name] = V * 3 * nst / (g0.elapsed_time(g1) / 1e3)
            bf.close()
        extra["fluxes"] = fl
        # CPU oracle, single thread, bounded sample on one mesh of the workload
        extra["cpu_baseline"] = cpu_baseline(meshes, args)
        # the serving half of the metric: converged solves/s and latency of
        # the request workload against the FP64 path measured on a sample
        if size == 1:
            extra["serving"] = serving(args)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": size,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32", "data": "synthetic",
                "config": {"workload": f"naca0012 O-grid {NI}x{NR} jittered +-10%, Euler "
                                       f"M0.8 AoA1.25, {args.flux} + limiter, RK3, CFL 1",
                           "meshes_per_gpu": args.meshes, "vertices_per_mesh": P,
                           "triangles_per_mesh": T, "edges_per_mesh": E,
                           "arithmetic": "FP32 state/flux/RK; FP64 geometry, norms, forces",
                           "l2": f"inputs larger than L2 (arena {V} vertices, "
                                 f"~{bytes_per_vertex_stage(P, T, E) * V / 1e9:.2f} GB "
                                 "touched per stage > 129 MB L2); no flush",
                           "parallelism": f"replicas x{size} (no data-path collective)",
                           "autotuner": tuned},
                "roofline": roofline, "stage_roofline": stage_roofline, "e2e": e2e,
                "clocks": clk.summary(),
                "gpu_launches": launches, "all_solves_ok": ok,
                "bytes_per_vertex_stage": round(bytes_per_vertex_stage(P, T, E), 1)}
        line.update(extra)
        print(json.dumps(line), flush=True)
    replicas.finish()


def oracle_rate(nthreads, ni, nr, iters, seeds):
    """Vertex-stages/s of the oracle, nthreads independent solves at once."""
    from oracle import oracle
    grids = [grid(s, ni, nr) for s in seeds[:nthreads]]
    orcs = [oracle.Oracle(g.coord, g.elem, g.ptype, iflux=1, **FLOW) for g in grids]
    for o in orcs:
        o.iterate(1)
    times = [0.0] * nthreads

    def work(k):
        t = time.perf_counter()
        orcs[k].iterate(iters)
        times[k] = time.perf_counter() - t
    t0 = time.perf_counter()
    th = [threading.Thread(target=work, args=(k,)) for k in range(nthreads)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    wall = time.perf_counter() - t0
    return nthreads * grids[0].np * 3 * iters / wall, wall


def cpu_baseline(meshes, args):
    from oracle import oracle
    oracle.build()
    iters = 40
    rate, wall = oracle_rate(1, NI, NR, iters, [2])
    return {"value": rate, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{iters} iterations of one {NI}x{NR} mesh of the same workload, "
                      f"serial FP64 oracle (gcc -O3 -ffp-contract=off), {wall:.1f} s"}


def fortran_probe():
    """Whether a Fortran compiler exists on this machine (the reference is
    Fortran 77 built with gfortran -O3); recorded in the reference line."""
    import shutil
    found = {}
    for c in ("gfortran", "f95", "f77", "flang", "flang-new", "lfortran"):
        path = shutil.which(c)
        if path:
            try:
                v = subprocess.run([path, "--version"], capture_output=True, text=True,
                                   timeout=30).stdout.splitlines()[:1]
            except (OSError, subprocess.TimeoutExpired):
                v = []
            found[c] = {"path": path, "version": v[0] if v else None}
    return found


def run_reference(args):
    """The reference's CPU implementation of the path: the oracle port (the
    Fortran reference cannot be compiled: no Fortran compiler on this
    machine, see the line's `fortran` record), one independent solve per
    host core."""
    from fvm2d_gb300 import replicas
    rank, local, size = replicas.world()
    if size > 1:
        replicas.init("gloo")
        if rank != 0:
            replicas.finish()
            return
    from oracle import oracle
    oracle.build()
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    # each step: one iteration per core, on the workload's 1024 x 384 mesh
    # when the run stays within a few minutes (about 0.45 s per iteration on
    # one core), else on a smaller mesh of the same family as the sample
    n_it = args.steps + args.warmup
    ni, nr = (NI, NR) if n_it <= 300 else ((512, 192) if n_it <= 1600 else (256, 96))
    seeds = list(range(2, 2 + cores))
    from fvm2d_gb300.ogrid import naca_ogrid
    grids = [naca_ogrid(ni, nr, radius=20.0, first_spacing=5e-4, jitter=0.1, seed=s)
             for s in seeds]
    orcs = [oracle.Oracle(g.coord, g.elem, g.ptype, iflux=FLUX_CODES[args.flux], bugcompat=0,
                          **FLOW) for g in grids]

    def run_steps(n):
        def work(k):
            orcs[k].iterate(n)
        th = [threading.Thread(target=work, args=(k,)) for k in range(cores)]
        for t in th:
            t.start()
        for t in th:
            t.join()
    run_steps(args.warmup)
    t0 = time.perf_counter()
    run_steps(args.steps)
    wall = time.perf_counter() - t0
    value = cores * grids[0].np * 3 * args.steps / wall
    sample = (f"{cores} concurrent serial FP64 oracle solves (one per core), {ni}x{nr} jittered "
              f"O-grid each, same flow and scheme, 1 iteration per step per core")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": size, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": f"naca0012 O-grid {NI}x{NR} jittered +-10%, Euler "
                                   f"M0.8 AoA1.25, {args.flux} + limiter, RK3, CFL 1",
                       "sample": f"{ni}x{nr} meshes of the same family, one per core",
                       "vertices_per_mesh": grids[0].np,
                       "parallelism": f"{cores} host threads"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": sample},
            "fortran": fortran_probe() or "no Fortran compiler on PATH (gfortran, f95, f77, "
                                          "flang, flang-new, lfortran probed)",
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    replicas.finish()


def fp64_solves(reqs, max_iter, minres):
    """The plain FP64 single-mesh path, one solve at a time: for each request
    a handle is created from its grid (upload, renumbering, device
    structures) and fvm_gpu_iterate runs it to its own stop (residual drop
    or iteration cap).  Wall seconds of create + iterate per solve, with the
    mean lift and drag of its last Result.TAIL iterations."""
    import numpy as np

    import fvm2d_gb300 as F
    from fvm2d_gb300 import serve
    out = []
    for req in reqs:
        g = serve.grid_for(req)
        mesh = F.build_geometry(g.coord, g.elem, g.ptype)
        par = serve.params_for(req, F.FP64)
        t0 = time.perf_counter()
        s = F.Solver(par, mesh)
        st, h = s.iterate(max_iter, minres, raise_on_error=False)
        dt = time.perf_counter() - t0
        s.close()
        k = min(serve.Result.TAIL, len(h["cl"]))
        out.append({"rid": req.rid, "vertices": mesh.np, "laminar": req.laminar,
                    "seconds": dt, "status": int(st), "iterations": int(len(h["fres"])),
                    "fres": float(h["fres"][-1]) if len(h["fres"]) else None,
                    "cl_tail": float(np.mean(h["cl"][-k:])) if k else None,
                    "cd_tail": float(np.mean(h["cd"][-k:])) if k else None})
    return out


def fp64_solves_subprocess(rids, args, variant):
    """fp64_solves in a child process that loads the given library variant."""
    env = dict(os.environ, FVM_LIB_VARIANT=variant)
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--mode", "fp64-solves",
           "--rids", ",".join(str(r) for r in rids), "--requests", str(args.requests),
           "--rate", str(args.rate), "--seed", str(args.seed), "--max-iter", str(args.max_iter),
           "--minres", str(args.minres)]
    r = subprocess.run(cmd, capture_output=True, text=True, env=env, timeout=1800)
    if r.returncode != 0:
        raise RuntimeError(f"fp64 solves ({variant}) failed: {r.stderr[-2000:]}")
    return json.loads(r.stdout.strip().splitlines()[-1])["solves"]


def run_fp64_solves(args):
    """--mode fp64-solves: fp64_solves on the given requests of the workload."""
    from fvm2d_gb300 import serve
    reqs = {r.rid: r for r in serve.generate_requests(n=args.requests, rate=args.rate,
                                                      seed=args.seed)}
    pick = [reqs[int(x)] for x in args.rids.split(",") if x]
    print(json.dumps({"mode": "fp64-solves", "library": os.environ.get("FVM_LIB_VARIANT", ""),
                      "solves": fp64_solves(pick, args.max_iter, args.minres)}), flush=True)


def serving(args):
    """Batched FP32 serving of the request workload (the native continuous-
    batching service), and the plain FP64 single-mesh path measured on a
    sample of the same requests, in the strict build (no FMA contraction,
    bitwise the reference's arithmetic) and the FMA build."""
    from fvm2d_gb300 import serve
    reqs = serve.generate_requests(n=args.requests, rate=args.rate, seed=args.seed)
    cls = serve.NativeServer if args.service == "native" else serve.Server
    srv = cls(vertices=args.arena_vertices, meshes=512, chunk=args.chunk,
              workers=args.workers, max_iter=args.max_iter, minres=args.minres,
              tune_every=args.tune_every)
    res, stats = srv.run(reqs)
    srv.close()
    by_rid = {r.rid: r for r in reqs}
    done = sorted((r for r in res if r.status == 0), key=lambda r: r.npts)
    k = min(args.fp64_sample, len(done))
    # stratified by grid size: the completed requests at the quantiles (2i+1)/2k
    sample = [done[int((2 * i + 1) * len(done) / (2 * k))] for i in range(k)]
    strict = fp64_solves([by_rid[r.rid] for r in sample], args.max_iter, args.minres)
    fma = fp64_solves_subprocess([r.rid for r in sample], args, "fp64fma")
    solves_s = stats["solves_per_s"]
    out = {"metric": "converged solves/s", "value": solves_s, "unit": "converged solves/s",
           "workload": f"{args.requests} NACA 4-digit requests, Poisson {args.rate}/s, "
                       "5k-400k vertices log-uniform, 70% Euler / 30% laminar NS, stop at drop "
                       f"{args.minres} or {args.max_iter} iterations, FP32 state",
           "latency_s": {"p50": stats["p50_latency_s"], "p99": stats["p99_latency_s"]},
           "solves": {"requests": stats["requests"], "reached_drop": stats["reached_minres"],
                      "hit_iteration_cap": stats["iteration_cap"],
                      "failed": len(stats["failures"]), "failures": stats["failures"]},
           "makespan_s": stats["makespan_s"],
           "vertex_stage_updates_per_s": stats["vertex_stage_updates_per_s"],
           "service_thread_s": stats.get("service_thread"),
           "arena_vertices": args.arena_vertices, "chunk": args.chunk,
           "tune_every_steps": args.tune_every}
    vs = {}
    for name, runs in (("fp64_strict", strict), ("fp64_fma", fma)):
        t = sum(x["seconds"] for x in runs)
        sps = len(runs) / t if t > 0 else None
        vs[name] = {"solves_per_s": sps, "ratio": solves_s / sps if sps else None,
                    "sample_seconds": [round(x["seconds"], 3) for x in runs],
                    "sample_iterations": [x["iterations"] for x in runs],
                    "sample_status": [x["status"] for x in runs]}
    vs["what"] = ("plain FP64 single-mesh path (fvm_gpu_create + fvm_gpu_iterate to the "
                  "request's own stop), one solve at a time, wall clock, on the served requests "
                  f"at the size quantiles (2i+1)/{2 * k}; solves/s = sample size / total seconds; "
                  "fp64_strict: no FMA contraction (bitwise the reference's arithmetic), "
                  "fp64_fma: the same kernels with FMA contraction")
    vs["sample"] = [{"rid": r.rid, "vertices": r.npts, "laminar": r.laminar} for r in sample]
    out["vs_fp64_gpu"] = vs
    rows = []
    for r, x in zip(sample, strict):
        dcl = abs(r.cl_tail - x["cl_tail"])
        dcd = abs(r.cd_tail - x["cd_tail"])
        rows.append({"rid": r.rid, "vertices": r.npts, "laminar": r.laminar,
                     "iterations32": r.niter, "iterations64": x["iterations"],
                     "status64": x["status"], "abs_dcl_tail": dcl, "abs_dcd_tail": dcd,
                     "within_target": bool(dcl <= 1e-4 and dcd <= 2e-5)})
    out["accuracy_vs_fp64"] = {
        "what": f"mean cl, cd over the last {serve.Result.TAIL} iterations, served FP32 vs "
                "the same request's FP64 strict solve", "target": {"cl": 1e-4, "cd": 2e-5},
        "solves": rows, "within_target": sum(x["within_target"] for x in rows)}
    return out


def run_serve(args):
    """--mode serve: the serving measurement alone, as one JSON line."""
    import torch
    torch.cuda.init()
    out = serving(args)
    out.update({"mode": "serve", "higher_is_better": True, "n_gpus": 1, "dtype": "f32",
                "data": "synthetic", "vs_baseline": None})
    print(json.dumps(out), flush=True)


ACCURACY_CASES = [
    # (name, workload grid, flow, iterations; see STOP_RULES for --stop-rules)
    ("config1 euler 160x48 roe", "euler_160x48", dict(mach=0.8, aoa_deg=1.25, cfl=1.0, iflux=1), 2000),
    ("config2 euler 1024x384 roe", "euler_1024x384", dict(mach=0.8, aoa_deg=1.25, cfl=1.0, iflux=1), 2000),
    ("config2 euler 1024x384 kfvs", "euler_1024x384", dict(mach=0.8, aoa_deg=1.25, cfl=1.0, iflux=2), 2000),
    ("config2 euler 1024x384 hllc", "euler_1024x384", dict(mach=0.8, aoa_deg=1.25, cfl=1.0, iflux=3), 2000),
    ("config3 laminar 512x192 roe", "laminar_512x192",
     dict(iflow=2, mach=0.5, aoa_deg=0.0, rey=5000.0, cfl=0.8, iflux=1), 2000),
    ("config4 rans-sa 768x256 hllc", "rans_768x256",
     dict(iflow=3, mach=0.7, aoa_deg=2.0, rey=6.5e6, cfl=0.5, iflux=3, nut_ratio=3.0), 1000),
]


# The single-mesh workloads' own stop rules, as (iteration cap, residual drop):
# 160x48 2000 iterations; 1024x384 5000 iterations or a drop of 1e-8; 512x192
# laminar a drop of 1e-7 (no cap given: 5000 here); 768x256 RANS-SA 20000
# iterations or a drop of 1e-6.
STOP_RULES = [(2000, 0.0), (5000, 1e-8), (5000, 1e-8), (5000, 1e-8), (5000, 1e-7), (20000, 1e-6)]


def run_accuracy(args):
    """FP32 against FP64 (whose arithmetic equals the serial FP64 oracle's)
    on the four single-mesh configurations: residual history, cl/cd (final
    and mean of the last 256 iterations) and wall Cp after the same number
    of iterations."""
    import numpy as np

    import fvm2d_gb300 as F
    from fvm2d_gb300 import results
    from fvm2d_gb300.batch import Batch
    from fvm2d_gb300.ogrid import workload_grid
    meshes, flows = [], []
    for name, wl, flow, n in ACCURACY_CASES:
        g = workload_grid(wl)
        meshes.append(F.build_geometry(g.coord, g.elem, g.ptype,
                                       wall_distance=flow.get("iflow", 1) == 3, bugcompat=0))
        flows.append(flow)
    out = {}
    runs = {}
    for prec in (F.FP64, F.FP32):
        b = Batch(prec, vertices=sum(m.np for m in meshes), meshes=len(meshes), viscous=True)
        pars = [F.make_params(precision=prec, bugcompat=0, **f) for f in flows]
        slots = [b.add(p, m) for p, m in zip(pars, meshes)]
        if args.stop_rules:
            nmax = [r[0] for r in STOP_RULES]
            drops = [r[1] for r in STOP_RULES]
        else:
            nmax = [c[3] for c in ACCURACY_CASES]
            drops = [0.0] * len(nmax)
        for s, n, dr in zip(slots, nmax, drops):
            b.start(s, n, dr)
        hist = [dict(fres=[], cl=[], cd=[]) for _ in slots]
        done = [0] * len(slots)
        t0 = time.perf_counter()
        while any(d < n for d, n in zip(done, nmax)):
            b.step(500)
            for j, s in enumerate(slots):
                q = b.poll(s)
                if q["niter"] > done[j]:
                    h = b.history(s, done[j], q["niter"] - done[j])
                    for k in ("fres", "cl", "cd"):
                        hist[j][k].append(h[k])
                    done[j] = q["niter"]
                if not q["active"] and q["niter"] < nmax[j]:
                    nmax[j] = q["niter"]          # stopped (status in poll)
        wall = time.perf_counter() - t0
        runs[prec] = []
        for j, s in enumerate(slots):
            q = b.poll(s)
            st = b.get_state(s)
            h = {k: np.concatenate(v) if v else np.zeros(0) for k, v in hist[j].items()}
            runs[prec].append(dict(poll=q, hist=h, wall=results.wall_table(
                meshes[j], st, pars[j], flows[j].get("iflow", 1))))
        b.close()
        out[f"wall_s_fp{64 if prec == F.FP64 else 32}"] = round(wall, 2)
    cases = []
    for j, (name, wl, flow, n) in enumerate(ACCURACY_CASES):
        r64, r32 = runs[F.FP64][j], runs[F.FP32][j]
        k = min(len(r64["hist"]["fres"]), len(r32["hist"]["fres"]))
        f64, f32 = r64["hist"]["fres"][:k], r32["hist"]["fres"][:k]
        tail = min(256, k)
        cases.append({
            "case": name, "vertices": meshes[j].np, "iterations": k,
            "iterations_fp64_fp32": [len(r64["hist"]["fres"]), len(r32["hist"]["fres"])],
            "status": [r64["poll"]["status"], r32["poll"]["status"]],
            "fres_final": [float(f64[-1]), float(f32[-1])] if k else None,
            "fres_max_rel_err": float(np.max(np.abs(f32 - f64) / np.abs(f64))) if k else None,
            "fres_log10_max_abs_diff": float(np.max(np.abs(np.log10(f32) - np.log10(f64)))) if k else None,
            "cl": [r64["poll"]["cl"], r32["poll"]["cl"]], "cd": [r64["poll"]["cd"], r32["poll"]["cd"]],
            "abs_err_cl": abs(r64["poll"]["cl"] - r32["poll"]["cl"]),
            "abs_err_cd": abs(r64["poll"]["cd"] - r32["poll"]["cd"]),
            "cl_tail": [float(np.mean(r64["hist"]["cl"][k - tail:k])),
                        float(np.mean(r32["hist"]["cl"][k - tail:k]))] if k else None,
            "cd_tail": [float(np.mean(r64["hist"]["cd"][k - tail:k])),
                        float(np.mean(r32["hist"]["cd"][k - tail:k]))] if k else None,
            "abs_err_cl_tail_mean": float(abs(np.mean(r64["hist"]["cl"][k - tail:k]) -
                                              np.mean(r32["hist"]["cl"][k - tail:k]))) if k else None,
            "abs_err_cd_tail_mean": float(abs(np.mean(r64["hist"]["cd"][k - tail:k]) -
                                              np.mean(r32["hist"]["cd"][k - tail:k]))) if k else None,
            "cp_max_abs_err": float(np.max(np.abs(r64["wall"]["cp"] - r32["wall"]["cp"]))),
        })
    out.update({"mode": "accuracy", "targets": {"cl": 1e-4, "cd": 2e-5},
                "what": "FP32 batch vs FP64 batch (bitwise the serial FP64 oracle's arithmetic), "
                        "same grids; " + ("each run to its workload's stop rule (STOP_RULES)"
                                          if args.stop_rules else "the same iteration counts"),
                "cases": cases})
    print(json.dumps(out), flush=True)


PROBE_FLOWS = {
    "euler": dict(mach=0.8, aoa_deg=1.25, cfl=1.0, iflux=1),
    "laminar": dict(iflow=2, mach=0.5, aoa_deg=0.0, rey=5000.0, cfl=0.8, iflux=1),
    "rans": dict(iflow=3, mach=0.7, aoa_deg=2.0, rey=6.5e6, cfl=0.5, iflux=3, nut_ratio=3.0),
}


def run_probe(args):
    """A few iterations of a batch of jittered ni x nr O-grid solves of one
    flow type (the flow parameters of the 512x192 laminar and 768x256 RANS-SA
    workloads), for profiling that flow's kernels under ncu; prints one JSON
    line with the wall time per iteration."""
    import fvm2d_gb300 as F
    from fvm2d_gb300.batch import Batch
    from fvm2d_gb300.ogrid import naca_ogrid
    prec = F.FP32 if args.precision == "fp32" else F.FP64
    flow = PROBE_FLOWS[args.flow]
    meshes = []
    for k in range(args.meshes):
        g = naca_ogrid(args.ni, args.nr, radius=20.0, first_spacing=5e-4, jitter=0.1, seed=2 + k)
        meshes.append(F.build_geometry(g.coord, g.elem, g.ptype,
                                       wall_distance=args.flow == "rans", bugcompat=0))
    b = Batch(prec, vertices=sum(m.np for m in meshes), meshes=args.meshes,
              viscous=args.flow != "euler")
    par = F.make_params(precision=prec, bugcompat=0, **flow)
    slots = [b.add(par, m) for m in meshes]
    for s in slots:
        b.start(s, args.warmup + args.steps + 25)
    b.set_form(args.form or "bulk")
    b.step(args.warmup)
    b.sync()
    t0 = time.perf_counter()
    b.step(args.steps)
    b.sync()
    dt = (time.perf_counter() - t0) / max(args.steps, 1)
    # per-kernel CUDA events over a few more iterations (one kernel at a
    # time: the events need a host sync after every iteration)
    b.timing(True)
    b.step(1)
    b.sync()
    b.timing(True)
    nk = min(args.steps, 20)
    b.step(nk)
    b.sync()
    kt = b.timing_read()
    b.timing(False)
    polls = [b.poll(s) for s in slots]
    out = {"mode": "probe", "flow": args.flow, "precision": args.precision,
           "meshes": args.meshes, "vertices_per_mesh": meshes[0].np, "form": args.form or "bulk",
           "iters": args.steps, "ms_per_iter": dt * 1e3, "status": [p["status"] for p in polls],
           "kernel_ms_per_iter": {k: round(v[0] / nk, 4) for k, v in kt.items() if v[1]},
           "kernel_launches_per_iter": {k: v[1] / nk for k, v in kt.items() if v[1]}}
    b.close()
    print(json.dumps(out), flush=True)


def main():
    from fvm2d_gb300.batch import Batch   # form names only: loads no library
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--meshes", type=int, default=8)
    ap.add_argument("--flux", choices=sorted(FLUX_CODES), default="roe")
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--quick", action="store_true", help="skip the side measurements")
    ap.add_argument("--form", default=None,
                    choices=list(Batch.TUNE_CANDIDATES),
                    help="use this form of the iteration instead of the autotuner's choice")
    ap.add_argument("--mode", choices=["throughput", "serve", "accuracy", "probe", "fp64-solves"],
                    default="throughput")
    ap.add_argument("--flow", choices=sorted(PROBE_FLOWS), default="euler",
                    help="probe: flow type of the batch")
    ap.add_argument("--ni", type=int, default=NI, help="probe: wall points per grid")
    ap.add_argument("--nr", type=int, default=NR, help="probe: radial points per grid")
    ap.add_argument("--precision", choices=["fp32", "fp64"], default="fp32",
                    help="probe: precision of the batch")
    ap.add_argument("--requests", type=int, default=512)
    ap.add_argument("--rate", type=float, default=20.0)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--arena-vertices", type=int, default=6_000_000)
    ap.add_argument("--chunk", type=int, default=100)
    ap.add_argument("--workers", type=int, default=8)
    ap.add_argument("--max-iter", type=int, default=5000)
    ap.add_argument("--minres", type=float, default=1e-6)
    ap.add_argument("--service", choices=["python", "native"], default="native",
                    help="serving loop: serve.Server (Python) or the C++ fvm_serve_* service")
    ap.add_argument("--tune-every", type=int, default=40,
                    help="serving: re-run the autotuner every N steps (0: never)")
    ap.add_argument("--fp64-sample", type=int, default=4,
                    help="serving: requests re-solved on the plain FP64 path")
    ap.add_argument("--rids", default="", help="fp64-solves: request ids")
    ap.add_argument("--stop-rules", action="store_true",
                    help="accuracy: run each case to its workload's stop rule (STOP_RULES)")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        run_reference(args)
    elif args.mode == "serve":
        from fvm2d_gb300 import build
        build.build()
        run_serve(args)
    elif args.mode == "accuracy":
        from fvm2d_gb300 import build
        build.build()
        run_accuracy(args)
    elif args.mode == "fp64-solves":
        from fvm2d_gb300 import build
        build.build()
        run_fp64_solves(args)
    elif args.mode == "probe":
        from fvm2d_gb300 import build
        build.build()
        run_probe(args)
    else:
        from fvm2d_gb300 import build
        build.build()
        run_gpu(args)


if __name__ == "__main__":
    main()
