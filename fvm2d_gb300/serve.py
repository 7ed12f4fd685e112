"""Continuous-batching service of steady airfoil solves on one GPU.

Requests arrive over time (seeded Poisson process).  Each names an airfoil
(NACA 4-digit thickness, camber and its position), a grid size, a flow
(Euler or laminar Navier-Stokes, Mach, angle of attack, Reynolds number).
The service:

* prepares each arrived request on host worker threads: O-grid, driver
  geometry (geometric.f chain), GPU dtlength, block layout (fvm_batch_prepare);
* admits prepared meshes into one device arena while it has room (the
  admission test is the arena's capacity in vertices, block entries and
  incidence entries, i.e. the HBM footprint; a refused mesh waits);
* advances every resident solve together, ``chunk`` iterations per step,
  all meshes in one launch per kernel (one CUDA graph per iteration);
* retires a solve when it reaches its residual drop or iteration cap
  (main.f:42), frees its arena ranges and admits the next.

So requests that arrive while others run join them on the device; no solve
waits for a batch boundary.  Latency is finish time minus arrival time.
"""
from __future__ import annotations

import collections
import concurrent.futures as cf
import dataclasses
import math
import time

import numpy as np

from . import _lib as L
from .batch import Batch, Prepared
from .ogrid import naca_ogrid
from .solver import build_geometry, make_params


@dataclasses.dataclass
class Request:
    rid: int
    arrival: float          # seconds after the start of the run
    thickness: float
    camber: float
    camber_pos: float
    npts: int               # requested vertex count
    laminar: bool
    mach: float
    aoa_deg: float
    rey: float
    seed: int


@dataclasses.dataclass
class Result:
    rid: int
    npts: int
    laminar: bool
    arrival: float
    admitted: float = math.nan
    finished: float = math.nan
    niter: int = 0
    fres: float = math.nan
    cl: float = math.nan
    cd: float = math.nan
    status: int = 0
    converged: bool = False
    cl_tail: float = math.nan   # mean cl, cd over the last TAIL iterations
    cd_tail: float = math.nan

    TAIL = 256

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


def generate_requests(n: int = 512, rate: float = 20.0, seed: int = 0, pmin: int = 5000,
                      pmax: int = 400000, laminar_frac: float = 0.3) -> list[Request]:
    """The serving workload: Poisson arrivals at ``rate`` per second; NACA
    4-digit thickness U[9,15]%, max camber U[0,4]% at U[30,50]% chord;
    vertex counts log-uniform in [pmin, pmax]; 70% Euler / 30% laminar with
    Re U[1e3,1e4]; Mach U[0.3,0.85]; angle of attack U[-3,5] degrees."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=n))
    t -= t[0]
    out = []
    for i in range(n):
        lam = rng.uniform() < laminar_frac
        out.append(Request(
            rid=i, arrival=float(t[i]), thickness=float(rng.uniform(0.09, 0.15)),
            camber=float(rng.uniform(0.0, 0.04)), camber_pos=float(rng.uniform(0.3, 0.5)),
            npts=int(round(math.exp(rng.uniform(math.log(pmin), math.log(pmax))))),
            laminar=bool(lam), mach=float(rng.uniform(0.3, 0.85)),
            aoa_deg=float(rng.uniform(-3.0, 5.0)),
            rey=float(rng.uniform(1e3, 1e4)) if lam else 0.0, seed=1000 + i))
    return out


def grid_for(req: Request):
    """O-grid with about ``npts`` vertices and ni:nr near 10:3."""
    ni = max(16, int(round(math.sqrt(req.npts * 10.0 / 3.0) / 2.0)) * 2)
    nr = max(8, int(round(req.npts / ni)))
    first = 2e-4 if req.laminar else 1e-3
    radius = 30.0 if req.laminar else 20.0
    first = min(first, 0.5 * radius / nr)
    return naca_ogrid(ni, nr, thickness=req.thickness, camber=req.camber,
                      camber_pos=req.camber_pos, radius=radius, first_spacing=first)


def params_for(req: Request, precision: int) -> L.FvmParams:
    if req.laminar:
        return make_params(iflow=L.LAMINAR, mach=req.mach, aoa_deg=req.aoa_deg, rey=req.rey,
                           cfl=0.8, precision=precision, bugcompat=0)
    return make_params(mach=req.mach, aoa_deg=req.aoa_deg, cfl=1.0, precision=precision,
                       bugcompat=0)


def prepare(req: Request, precision: int) -> Prepared:
    g = grid_for(req)
    m = build_geometry(g.coord, g.elem, g.ptype)
    return Prepared(params_for(req, precision), m)


class Server:
    def __init__(self, vertices: int = 6_000_000, meshes: int = 256, precision: int = L.FP32,
                 chunk: int = 50, workers: int = 8, max_iter: int = 5000, minres: float = 1e-6,
                 tune_every: int = 0, tune_iters: int = 10, **caps):
        self.batch = Batch(precision, vertices=vertices, meshes=meshes, viscous=True, **caps)
        self.precision = precision
        self.chunk = chunk
        # every tune_every steps the autotuner re-picks the form of the
        # iteration for the current mix (its iterations are ordinary ones)
        self.tune_every = tune_every
        self.tune_iters = tune_iters
        self.tunings = []
        self.workers = workers
        self.max_iter = max_iter
        self.minres = minres

    def close(self):
        self.batch.close()

    def run(self, requests: list[Request], log=None) -> tuple[list[Result], dict]:
        b = self.batch
        results = {r.rid: Result(rid=r.rid, npts=r.npts, laminar=r.laminar, arrival=r.arrival)
                   for r in requests}
        order = sorted(requests, key=lambda r: r.arrival)
        pool = cf.ThreadPoolExecutor(max_workers=self.workers)
        preparing = collections.deque()      # (req, future), arrival order
        ready = collections.deque()          # (req, Prepared)
        resident = {}                        # slot -> req
        nxt = 0
        done = 0
        steps = 0
        resident_vertices = []
        t0 = time.perf_counter()
        while done < len(order):
            now = time.perf_counter() - t0
            while nxt < len(order) and order[nxt].arrival <= now:
                preparing.append((order[nxt], pool.submit(prepare, order[nxt], self.precision)))
                nxt += 1
            while preparing and preparing[0][1].done():
                req, fut = preparing.popleft()
                ready.append((req, fut.result()))
            while ready:                                   # admission by footprint
                req, prep = ready[0]
                slot = b.add_prepared(prep)
                if slot is None:
                    if resident:
                        break                              # waits for room
                    # too large for an empty arena: refused with a status
                    ready.popleft()
                    prep.release()
                    r = results[req.rid]
                    r.admitted = r.finished = time.perf_counter() - t0
                    r.status = L.ERR_CAPACITY
                    done += 1
                    if log:
                        log(r)
                    continue
                ready.popleft()
                b.start(slot, self.max_iter, self.minres)
                resident[slot] = req
                results[req.rid].admitted = time.perf_counter() - t0
                results[req.rid].npts = b._meshes[slot].np     # the grid's actual size
            if not resident:
                if nxt < len(order) and not preparing and not ready:
                    time.sleep(max(0.0, min(0.01, order[nxt].arrival - now)))
                else:
                    time.sleep(0.001)
                continue
            if self.tune_every and steps % self.tune_every == 0:
                self.tunings.append(b.tune(self.tune_iters)["choice"])
            b.step(self.chunk)                             # all resident solves at once
            steps += 1
            resident_vertices.append(sum(b._meshes[s].np for s in resident))
            for slot in list(resident):
                p = b.poll(slot)
                if p["active"]:
                    continue
                req = resident.pop(slot)
                r = results[req.rid]
                r.finished = time.perf_counter() - t0
                r.niter, r.fres, r.cl, r.cd, r.status = (p["niter"], p["fres"], p["cl"],
                                                         p["cd"], p["status"])
                r.converged = p["status"] == 0 and p["fres"] <= self.minres
                if r.niter > 0:
                    k = min(Result.TAIL, r.niter)
                    h = b.history(slot, r.niter - k, k)
                    r.cl_tail, r.cd_tail = float(np.mean(h["cl"])), float(np.mean(h["cd"]))
                b.remove(slot)
                done += 1
                if log:
                    log(r)
        pool.shutdown()
        makespan = time.perf_counter() - t0
        res = [results[r.rid] for r in requests]
        lat = np.array([r.latency for r in res])
        ok = [r for r in res if r.status == 0]
        by_rid = {r.rid: r for r in requests}
        failures = [dict(rid=r.rid, status=r.status, niter=r.niter, npts=r.npts,
                         laminar=r.laminar, mach=by_rid[r.rid].mach,
                         aoa_deg=by_rid[r.rid].aoa_deg) for r in res if r.status != 0]
        stats = dict(requests=len(res), completed_ok=len(ok), failures=failures,
                     reached_minres=sum(r.converged for r in res),
                     iteration_cap=sum(r.status == 0 and not r.converged for r in res),
                     makespan_s=makespan, solves_per_s=len(ok) / makespan,
                     p50_latency_s=float(np.percentile(lat, 50)),
                     p99_latency_s=float(np.percentile(lat, 99)),
                     vertex_stage_updates=float(sum(r.npts * 3 * r.niter for r in res)),
                     mean_resident_vertices=float(np.mean(resident_vertices)) if resident_vertices else 0.0,
                     steps=steps, chunk=self.chunk,
                     tuner_choices={k: self.tunings.count(k) for k in set(self.tunings)})
        stats["vertex_stage_updates_per_s"] = stats["vertex_stage_updates"] / makespan
        return res, stats


class NativeServer:
    """The same service in native code (fvm_serve_* of the C ABI): a C++
    service thread owns the arena, admits, steps and retires; this class
    submits the arrivals (preparing them on a thread pool, since submit
    builds the block layout on the calling thread) and collects results."""

    def __init__(self, vertices: int = 6_000_000, meshes: int = 256, precision: int = L.FP32,
                 chunk: int = 50, workers: int = 8, max_iter: int = 5000, minres: float = 1e-6,
                 tune_every: int = 0, **caps):
        import ctypes as C
        c = L.FvmBatchCaps()
        c.vertices, c.meshes, c.viscous = int(vertices), int(meshes), 1
        for k, v in caps.items():
            setattr(c, k, int(v))
        h = C.c_void_p()
        L.check(L.lib().fvm_serve_create(precision, C.byref(c), chunk, tune_every, C.byref(h)),
                "fvm_serve_create")
        self.h = h
        self.precision = precision
        self.workers = workers
        self.max_iter = max_iter
        self.minres = minres
        self.chunk = chunk

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            L.lib().fvm_serve_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, params: L.FvmParams, mesh, keep_state: bool = False) -> int:
        import ctypes as C
        from .solver import MeshArrays
        m = mesh if isinstance(mesh, MeshArrays) else MeshArrays(mesh)
        ms = m.struct()
        t = C.c_int64(0)
        L.check(L.lib().fvm_serve_submit(self.h, C.byref(params), C.byref(ms), self.max_iter,
                                         self.minres, 1 if keep_state else 0, C.byref(t)),
                "fvm_serve_submit")
        return t.value

    def wait(self, ticket: int, timeout: float = 3600.0) -> bool:
        import ctypes as C
        st = C.c_int32(0)
        L.check(L.lib().fvm_serve_wait(self.h, ticket, timeout, C.byref(st)), "fvm_serve_wait")
        return st.value == 2

    def result(self, ticket: int) -> dict:
        import ctypes as C
        st, n = C.c_int32(), C.c_int32()
        f, cl, cd = C.c_double(), C.c_double(), C.c_double()
        tm = (C.c_double * 3)()
        tail = (C.c_double * 2)()
        L.check(L.lib().fvm_serve_result(self.h, ticket, C.byref(st), C.byref(n), C.byref(f),
                                         C.byref(cl), C.byref(cd), tail, tm), "fvm_serve_result")
        return dict(status=st.value, niter=n.value, fres=f.value, cl=cl.value, cd=cd.value,
                    cl_tail=tail[0], cd_tail=tail[1],
                    queued_s=tm[0], resident_s=tm[1], total_s=tm[2])

    def state(self, ticket: int, np_: int) -> dict:
        prim, nut = np.zeros((np_, 4)), np.zeros(np_)
        L.check(L.lib().fvm_serve_state(self.h, ticket, L.dptr(prim), L.dptr(nut)),
                "fvm_serve_state")
        return dict(prim=prim, nut=nut)

    def checkpoint(self, ticket: int):
        """Stops a running solve at the end of the current step, keeping
        its state (the ticket then finishes with status CHECKPOINTED)."""
        L.check(L.lib().fvm_serve_checkpoint(self.h, ticket), "fvm_serve_checkpoint")

    def checkpoint_read(self, ticket: int, np_: int) -> dict:
        """The kept state of a checkpointed solve (driver order) and its
        iteration count, from which fvm_serve_resume continues."""
        import ctypes as C
        prim, nut, mul, mu = np.zeros((np_, 4)), np.zeros(np_), np.zeros(np_), np.zeros(np_)
        it = C.c_int32(0)
        L.check(L.lib().fvm_serve_checkpoint_read(self.h, ticket, L.dptr(prim), L.dptr(nut),
                                                  L.dptr(mul), L.dptr(mu), C.byref(it)),
                "fvm_serve_checkpoint_read")
        return dict(prim=prim, nut=nut, mul=mul, mu=mu, iter=it.value)

    def resume(self, params: L.FvmParams, mesh, state: dict, nmax: int | None = None,
               keep_state: bool = False) -> int:
        """Queues a solve that starts from `state` (checkpoint_read's dict)
        at its iteration count, for up to nmax more iterations."""
        import ctypes as C
        from .solver import MeshArrays
        m = mesh if isinstance(mesh, MeshArrays) else MeshArrays(mesh)
        ms = m.struct()
        arr = {k: np.ascontiguousarray(state[k], dtype=np.float64)
               for k in ("prim", "nut", "mul", "mu")}
        t = C.c_int64(0)
        L.check(L.lib().fvm_serve_resume(self.h, C.byref(params), C.byref(ms),
                                         self.max_iter if nmax is None else int(nmax),
                                         self.minres, L.dptr(arr["prim"]), L.dptr(arr["nut"]),
                                         L.dptr(arr["mul"]), L.dptr(arr["mu"]),
                                         int(state["iter"]), 1 if keep_state else 0,
                                         C.byref(t)), "fvm_serve_resume")
        return t.value

    def stats(self) -> dict:
        import ctypes as C
        out = (C.c_int64 * 6)()
        L.check(L.lib().fvm_serve_stats(self.h, out), "fvm_serve_stats")
        return dict(zip(("submitted", "done", "queued", "running", "steps", "status"),
                        [int(x) for x in out]))

    def times(self) -> dict:
        """Seconds the service thread spent admitting between steps,
        tuning, stepping (launching and waiting for the GPU, including the
        admissions made beside a running step) and retiring."""
        import ctypes as C
        out = (C.c_double * 5)()
        L.check(L.lib().fvm_serve_times(self.h, out), "fvm_serve_times")
        return dict(zip(("admit_s", "tune_s", "step_s", "retire_s", "admit_beside_step_s"),
                        [float(x) for x in out]))

    def run(self, requests: list[Request]) -> tuple[list[Result], dict]:
        """The request workload: each request is submitted at its arrival
        time (grid generation and layout on the worker pool)."""
        results = {r.rid: Result(rid=r.rid, npts=r.npts, laminar=r.laminar, arrival=r.arrival)
                   for r in requests}
        t0 = time.perf_counter()

        def go(req):
            delay = req.arrival - (time.perf_counter() - t0)
            if delay > 0:
                time.sleep(delay)
            g = grid_for(req)
            m = build_geometry(g.coord, g.elem, g.ptype)
            results[req.rid].npts = m.np
            return self.submit(params_for(req, self.precision), m)

        order = sorted(requests, key=lambda r: r.arrival)
        with cf.ThreadPoolExecutor(max_workers=self.workers) as pool:
            tickets = list(pool.map(go, order))
        for req, t in zip(order, tickets):
            self.wait(t)
            q = self.result(t)
            r = results[req.rid]
            r.finished = r.arrival + q["total_s"]
            r.admitted = r.arrival + q["queued_s"]
            r.niter, r.fres, r.cl, r.cd, r.status = q["niter"], q["fres"], q["cl"], q["cd"], q["status"]
            r.cl_tail, r.cd_tail = q["cl_tail"], q["cd_tail"]
            r.converged = q["status"] == 0 and q["fres"] <= self.minres
        makespan = time.perf_counter() - t0
        res = [results[r.rid] for r in requests]
        ok = [r for r in res if r.status == 0]
        lat = np.array([r.latency for r in res])
        st = self.stats()
        stats = dict(requests=len(res), completed_ok=len(ok),
                     failures=[dict(rid=r.rid, status=r.status, niter=r.niter, npts=r.npts,
                                    laminar=r.laminar) for r in res if r.status != 0],
                     reached_minres=sum(r.converged for r in res),
                     iteration_cap=sum(r.status == 0 and not r.converged for r in res),
                     makespan_s=makespan, solves_per_s=len(ok) / makespan,
                     p50_latency_s=float(np.percentile(lat, 50)),
                     p99_latency_s=float(np.percentile(lat, 99)),
                     vertex_stage_updates=float(sum(r.npts * 3 * r.niter for r in res)),
                     steps=st["steps"], chunk=self.chunk, service="native",
                     service_thread=self.times())
        stats["vertex_stage_updates_per_s"] = stats["vertex_stage_updates"] / makespan
        return res, stats

