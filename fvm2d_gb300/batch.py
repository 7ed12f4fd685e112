"""Python side of the batch C ABI: many meshes resident in one device arena,
every kernel launched once per iteration for all of them (include/fvm_gpu.h,
fvm_batch_*).  ``Batch.add`` admits a mesh, ``start`` arms a solve,
``step`` enqueues iterations of every armed mesh, ``poll`` reports one."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from ._lib import check, dptr, iptr
from .solver import MeshArrays


def layout_stats(mesh) -> dict:
    """Block layout of a mesh after renumbering (host only)."""
    m = mesh if isinstance(mesh, MeshArrays) else MeshArrays(mesh)
    ms = m.struct()
    out = (C.c_int64 * 10)()
    check(L.lib().fvm_layout_stats(C.byref(ms), out), "fvm_layout_stats")
    keys = ["blocks", "edge_entries", "tri_entries", "max_slots", "max_tri", "boundary_entries",
            "max_tri2", "max_loc", "halo_entries", "layout_violations"]
    return dict(zip(keys, [int(x) for x in out]))


class Prepared:
    """A mesh whose block layout has been built on the host (thread safe,
    no device work); admit it with Batch.add_prepared."""

    def __init__(self, params: L.FvmParams, mesh):
        m = mesh if isinstance(mesh, MeshArrays) else MeshArrays(mesh)
        ms = m.struct()
        h = C.c_void_p()
        check(L.lib().fvm_batch_prepare(C.byref(params), C.byref(ms), C.byref(h)),
              "fvm_batch_prepare")
        self.h = h
        self.mesh = m
        self.np = m.np

    def nbytes(self, precision: int) -> int:
        return int(L.lib().fvm_prepared_bytes(self.h, precision))

    def release(self):
        if self.h is not None and self.h.value:
            L.lib().fvm_prepared_free(self.h)
        self.h = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


class Batch:
    def __init__(self, precision: int, vertices: int, meshes: int, viscous: bool = False,
                 **caps):
        c = L.FvmBatchCaps()
        c.vertices = int(vertices)
        c.meshes = int(meshes)
        c.viscous = 1 if viscous else 0
        for k, v in caps.items():
            setattr(c, k, int(v))
        h = C.c_void_p()
        check(L.lib().fvm_batch_create(precision, C.byref(c), C.byref(h)), "fvm_batch_create")
        self.h = h
        self.precision = precision
        self._meshes = {}
        gm = int(caps.get("grad_mode", 0)) or (3 if precision == L.FP32 else 1)
        ch = int(caps.get("overlap", 0))
        if int(caps.get("fused", 0)) > 0:
            self.form = "fused+overlap" if ch > 1 else "fused"
        elif ch > 1 and gm == 4:
            self.form = {2: "pipe+overlap", 4: "pipe+overlap4"}.get(ch, "pipe+overlap")
        elif ch > 1:
            self.form = {2: "split+overlap", 4: "split+overlap4", 8: "split+overlap8"}.get(
                ch, "split+overlap")
        else:
            self.form = {4: "pipe", 3: "bulk", 1: "loads", 2: "vertex"}[gm]

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            L.lib().fvm_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, params: L.FvmParams, mesh) -> int:
        m = mesh if isinstance(mesh, MeshArrays) else MeshArrays(mesh)
        ms = m.struct()
        slot = C.c_int32(-1)
        check(L.lib().fvm_batch_add(self.h, C.byref(params), C.byref(ms), C.byref(slot)),
              "fvm_batch_add")
        self._meshes[slot.value] = m
        return slot.value

    def try_add(self, params: L.FvmParams, mesh):
        """add() that returns None when the arena has no room."""
        try:
            return self.add(params, mesh)
        except L.FvmError as e:
            if e.status == L.ERR_CAPACITY:
                return None
            raise

    def add_prepared(self, prep: Prepared):
        """Upload a prepared mesh; returns its slot or None when the arena has
        no room (the prepared mesh is kept for a later try)."""
        slot = C.c_int32(-1)
        st = L.lib().fvm_batch_add_prepared(self.h, prep.h, C.byref(slot))
        if st == L.ERR_CAPACITY:
            return None
        check(st, "fvm_batch_add_prepared")
        prep.h = None          # taken by the batch
        self._meshes[slot.value] = prep.mesh
        return slot.value

    def remove(self, slot: int):
        check(L.lib().fvm_batch_remove(self.h, slot), "fvm_batch_remove")
        self._meshes.pop(slot, None)

    def set_state(self, slot, prim, nut=None, mul=None, mu=None, iterlast=0):
        prim = np.ascontiguousarray(prim, dtype=np.float64)
        conv = [None if a is None else np.ascontiguousarray(a, dtype=np.float64)
                for a in (nut, mul, mu)]
        check(L.lib().fvm_batch_set_state(self.h, slot, dptr(prim), *[dptr(a) for a in conv],
                                          iterlast), "fvm_batch_set_state")

    STATE_FIELDS = ("prim", "nut", "mul", "mu", "qx", "qy")

    def get_state(self, slot, fields=STATE_FIELDS, out=None) -> dict:
        """The slot's state in driver order (FP64); `fields` limits the
        arrays read back (the others are passed to the C ABI as NULL).
        `out` may hold caller-owned C-contiguous float64 arrays (for example
        in pinned memory) for some of the fields; they are filled in place."""
        n = self._meshes[slot].np
        bad = set(fields) - set(self.STATE_FIELDS)
        if bad:
            raise ValueError(f"unknown state fields {sorted(bad)}")
        given = dict(out or {})
        out = {}
        for k in fields:
            shape = (n, 4) if k in ("prim", "qx", "qy") else (n,)
            a = given.get(k)
            if a is None:
                a = np.zeros(shape)
            elif (a.shape != shape or a.dtype != np.float64 or not a.flags.c_contiguous
                  or not a.flags.writeable):
                raise ValueError(f"out[{k!r}] must be a writeable C-contiguous float64 {shape}")
            out[k] = a
        ptr = [dptr(out[k]) if k in out else None for k in self.STATE_FIELDS]
        check(L.lib().fvm_batch_get_state(self.h, slot, *ptr), "fvm_batch_get_state")
        return out

    def start(self, slot, nmax: int, minres: float = 0.0):
        check(L.lib().fvm_batch_start(self.h, slot, nmax, minres), "fvm_batch_start")

    def step(self, niter: int = 1):
        check(L.lib().fvm_batch_step(self.h, niter), "fvm_batch_step")

    def sync(self):
        check(L.lib().fvm_batch_sync(self.h), "fvm_batch_sync")

    def poll(self, slot) -> dict:
        a, n, st, bad = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
        f, cl, cd = C.c_double(), C.c_double(), C.c_double()
        check(L.lib().fvm_batch_poll(self.h, slot, C.byref(a), C.byref(n), C.byref(f),
                                     C.byref(cl), C.byref(cd), C.byref(st), C.byref(bad)),
              "fvm_batch_poll")
        return dict(active=a.value, niter=n.value, fres=f.value, cl=cl.value, cd=cd.value,
                    status=st.value, bad_point=bad.value)

    def history(self, slot, first: int, count: int) -> dict:
        h = dict(fres=np.zeros(count), iresi=np.zeros(count, np.int32), fresi=np.zeros(count),
                 cl=np.zeros(count), cd=np.zeros(count))
        check(L.lib().fvm_batch_history(self.h, slot, first, count, dptr(h["fres"]),
                                        iptr(h["iresi"]), dptr(h["fresi"]), dptr(h["cl"]),
                                        dptr(h["cd"])), "fvm_batch_history")
        return h

    def stream(self) -> int:
        return L.lib().fvm_batch_stream(self.h) or 0

    def timing(self, on: bool):
        check(L.lib().fvm_batch_timing(self.h, 1 if on else 0), "fvm_batch_timing")

    def timing_read(self) -> dict:
        names = C.create_string_buffer(32 * 8)
        ms = (C.c_double * 8)()
        cnt = (C.c_int64 * 8)()
        n = C.c_int32()
        check(L.lib().fvm_batch_timing_read(self.h, 8, names, ms, cnt, C.byref(n)),
              "fvm_batch_timing_read")
        out = {}
        for k in range(n.value):
            nm = names.raw[32 * k:32 * (k + 1)].split(b"\0")[0].decode()
            out[nm] = (float(ms[k]), int(cnt[k]))
        return out

    def launch_count(self) -> int:
        return int(L.lib().fvm_batch_launch_count(self.h))

    TUNE_CANDIDATES = ("bulk", "loads", "vertex", "fused", "split+overlap", "fused+overlap",
                       "split+overlap4", "split+overlap8", "pipe", "pipe+overlap",
                       "pipe+overlap4")

    def set_form(self, name: str):
        """Set the form of the iteration to one of TUNE_CANDIDATES."""
        check(L.lib().fvm_batch_set_form(self.h, self.TUNE_CANDIDATES.index(name)),
              "fvm_batch_set_form")
        self.form = name

    def tune(self, iters: int = 10) -> dict:
        """Time each form of the iteration on the resident solves (ordinary
        iterations: every form gives the same bits) and keep the fastest.
        Returns {"choice": name, "ms_per_iter": {name: ms or None}}."""
        n = len(self.TUNE_CANDIDATES)
        ms = (C.c_double * n)()
        ch = C.c_int32(-1)
        check(L.lib().fvm_batch_tune(self.h, int(iters), n, ms, C.byref(ch)), "fvm_batch_tune")
        self.form = self.TUNE_CANDIDATES[ch.value]
        return {"choice": self.TUNE_CANDIDATES[ch.value],
                "ms_per_iter": {k: (float(ms[i]) if ms[i] > 0 else None)
                                for i, k in enumerate(self.TUNE_CANDIDATES)}}
