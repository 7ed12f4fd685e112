"""Host-side mirror of the reference's hot-path interface.

``Solver`` wraps one C-ABI handle (include/fvm_gpu.h) and exposes the
routines of the reference's iteration loop under their Fortran names
(main.f:44-62): ``save_old``, ``time_step``, ``residu``, ``update(irk)``,
``sa_model``, ``check_positivity``, ``clcd``, ``conres``, plus ``iterate``
which runs whole iterations on the GPU (one CUDA graph per iteration) and
returns the RES.DAT columns.  Errors mirror the reference's ``stop`` sites
as :class:`FvmError` with the same status codes as the C ABI.

``Geometry`` is the driver side: the geometric.f chain built on the host
(``fvm_geom_build``) with dtlength and wall_dist run as GPU kernels.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from ._lib import check, dptr, iptr


def make_params(*, iflow=L.INVISCID, mach=0.8, aoa_deg=1.25, rey=0.0, cfl=1.0, iflux=L.ROE,
                ilimit=1, vortex=0, xref=0.25, yref=0.0, cell_type=L.MEDIAN, nut_ratio=0.1,
                precision=L.FP64, bugcompat=1) -> L.FvmParams:
    """fvm_params from the fvm.inp inputs (read_input.f:20-66)."""
    p = L.FvmParams()
    check(L.lib().fvm_params_init(C.byref(p), iflow, mach, aoa_deg, rey, cfl, iflux, ilimit,
                                  vortex, xref, yref, cell_type, nut_ratio, precision,
                                  bugcompat), "fvm_params_init")
    return p


_MESH_INTS = ["np", "nt", "ne", "netot", "nsp", "nbe", "nswe1", "nswe2", "nffe1", "nffe2"]
_MESH_DBL = ["coord", "ds", "elarea", "cvarea", "mcarea", "drmin", "wd"]
_MESH_INT = ["elem", "ptype", "spts", "edge", "iedge", "beindx"]


class MeshArrays:
    """The fvm_mesh inputs as numpy arrays (driver order, 1-based indices)."""

    def __init__(self, d: dict):
        for k in _MESH_INTS:
            setattr(self, k, int(d[k]))
        for k in _MESH_DBL:
            v = d.get(k)
            setattr(self, k, None if v is None else np.ascontiguousarray(v, dtype=np.float64))
        for k in _MESH_INT:
            setattr(self, k, np.ascontiguousarray(d[k], dtype=np.int32))
        for k in ("dsb", "edneigh"):
            if k in d and d[k] is not None:
                setattr(self, k, np.asarray(d[k]))

    def struct(self) -> L.FvmMesh:
        m = L.FvmMesh()
        for k in _MESH_INTS:
            setattr(m, k, getattr(self, k))
        for k in _MESH_DBL:
            setattr(m, k, dptr(getattr(self, k)))
        for k in _MESH_INT:
            setattr(m, k, iptr(getattr(self, k)))
        return m

    def as_dict(self) -> dict:
        out = {k: getattr(self, k) for k in _MESH_INTS + _MESH_DBL + _MESH_INT}
        for k in ("dsb", "edneigh"):
            if hasattr(self, k):
                out[k] = getattr(self, k)
        return out


def build_geometry(coord, elem, ptype, *, cell_type=L.MEDIAN, wall_distance=False,
                   bugcompat=1, setup_on_gpu=True, chain_on_gpu=False) -> MeshArrays:
    """geometric.f:15-60 for a grid: host chain + GPU dtlength / wall_dist.

    With ``setup_on_gpu=False`` drmin and wd stay zero (host-only callers).
    With ``chain_on_gpu=True`` the chain itself runs on the GPU
    (fvm_gpu_geom_build: the same arrays bit for bit, drmin included).
    """
    coord = np.ascontiguousarray(coord, dtype=np.float64)
    elem = np.array(elem, dtype=np.int32, order="C", copy=True)   # oriented in place
    ptype = np.ascontiguousarray(ptype, dtype=np.int32)
    gp = C.POINTER(L.FvmGeom)()
    fn = "fvm_gpu_geom_build" if chain_on_gpu else "fvm_geom_build"
    check(getattr(L.lib(), fn)(coord.shape[0], elem.shape[0], dptr(coord), iptr(elem),
                               iptr(ptype), cell_type, C.byref(gp)), fn)
    try:
        g = gp.contents
        m = g.mesh
        d = {k: getattr(m, k) for k in _MESH_INTS}

        def darr(p, n):
            return np.ctypeslib.as_array(p, shape=(n,)).copy() if n else np.zeros(0)

        def iarr(p, n):
            return np.ctypeslib.as_array(p, shape=(n,)).copy() if n else np.zeros(0, np.int32)
        npt, nt, netot = m.np, m.nt, m.netot
        d.update(coord=coord, elem=elem, ptype=ptype,
                 spts=iarr(g.spts, m.nsp), edge=iarr(g.edge, 2 * netot).reshape(-1, 2),
                 edneigh=iarr(g.edneigh, 2 * netot).reshape(-1, 2),
                 iedge=iarr(g.iedge, m.ne), beindx=iarr(g.beindx, m.nbe),
                 ds=darr(g.ds, 2 * netot).reshape(-1, 2), dsb=darr(g.dsb, 2 * npt).reshape(-1, 2),
                 elarea=darr(g.elarea, nt), cvarea=darr(g.cvarea, npt),
                 mcarea=darr(g.mcarea, npt),
                 drmin=darr(g.drmin, npt) if chain_on_gpu else np.zeros(npt), wd=np.zeros(npt))
    finally:
        L.lib().fvm_geom_free(gp)
    if setup_on_gpu:
        if not chain_on_gpu:
            d["drmin"] = dtlength(d["coord"], d["elem"], d["elarea"])
        if wall_distance:
            d["wd"] = wall_dist(d["coord"], d["edge"], d["ptype"], bugcompat)
    return MeshArrays(d)


def dtlength(coord, elem, elarea) -> np.ndarray:
    """dtlength.f:6-47 on the GPU."""
    coord = np.ascontiguousarray(coord, dtype=np.float64)
    elem = np.ascontiguousarray(elem, dtype=np.int32)
    elarea = np.ascontiguousarray(elarea, dtype=np.float64)
    out = np.zeros(coord.shape[0])
    check(L.lib().fvm_gpu_dtlength(coord.shape[0], elem.shape[0], dptr(coord), iptr(elem),
                                   dptr(elarea), dptr(out)), "fvm_gpu_dtlength")
    return out


def wall_dist(coord, edge, ptype, bugcompat=1) -> np.ndarray:
    """wall_dist.f:16-61,87-92 on the GPU."""
    coord = np.ascontiguousarray(coord, dtype=np.float64)
    edge = np.ascontiguousarray(edge, dtype=np.int32)
    ptype = np.ascontiguousarray(ptype, dtype=np.int32)
    out = np.zeros(coord.shape[0])
    check(L.lib().fvm_gpu_wall_dist(coord.shape[0], edge.shape[0], dptr(coord), iptr(edge),
                                    iptr(ptype), bugcompat, dptr(out)), "fvm_gpu_wall_dist")
    return out


class Solver:
    """One mesh on the GPU behind the C ABI."""

    def __init__(self, params: L.FvmParams, mesh):
        self.params = params
        self.mesh = mesh if isinstance(mesh, MeshArrays) else MeshArrays(mesh)
        self._ms = self.mesh.struct()
        self.np = self.mesh.np
        h = C.c_void_p()
        check(L.lib().fvm_gpu_create(C.byref(params), C.byref(self._ms), C.byref(h)),
              "fvm_gpu_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            L.lib().fvm_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- state -------------------------------------------------------------
    def set_state(self, prim, nut=None, mul=None, mu=None, iterlast=0):
        prim = np.ascontiguousarray(prim, dtype=np.float64).reshape(self.np, 4)
        conv = [None if a is None else np.ascontiguousarray(a, dtype=np.float64)
                for a in (nut, mul, mu)]
        check(L.lib().fvm_gpu_set_state(self.h, dptr(prim), *[dptr(a) for a in conv],
                                        iterlast), "fvm_gpu_set_state")

    def get_state(self) -> dict:
        out = {k: np.zeros((self.np, 4)) for k in ("prim", "qx", "qy")}
        for k in ("nut", "mul", "mu"):
            out[k] = np.zeros(self.np)
        check(L.lib().fvm_gpu_get_state(self.h, dptr(out["prim"]), dptr(out["nut"]),
                                        dptr(out["mul"]), dptr(out["mu"]), dptr(out["qx"]),
                                        dptr(out["qy"])), "fvm_gpu_get_state")
        return out

    def residual(self) -> np.ndarray:
        r = np.zeros((self.np, 4))
        check(L.lib().fvm_gpu_get_residual(self.h, dptr(r)), "fvm_gpu_get_residual")
        return r

    def dt(self) -> np.ndarray:
        r = np.zeros(self.np)
        check(L.lib().fvm_gpu_get_dt(self.h, dptr(r)), "fvm_gpu_get_dt")
        return r

    def prim_old(self) -> np.ndarray:
        r = np.zeros((self.np, 4))
        check(L.lib().fvm_gpu_get_prim_old(self.h, dptr(r)), "fvm_gpu_get_prim_old")
        return r

    # ---- routines of main.f:44-62 -------------------------------------------
    def save_old(self):
        check(L.lib().fvm_gpu_save_old(self.h), "save_old")

    def time_step(self):
        check(L.lib().fvm_gpu_time_step(self.h), "time_step")

    def residu(self):
        check(L.lib().fvm_gpu_residu(self.h), "residu")

    def update(self, irk: int):
        check(L.lib().fvm_gpu_update(self.h, irk), "update")

    def sa_model(self):
        check(L.lib().fvm_gpu_sa_model(self.h), "sa_model")

    def gradient(self):
        """gradient.f: edge-based Green-Gauss gradients (read with get_state)."""
        check(L.lib().fvm_gpu_gradient(self.h), "fvm_gpu_gradient")

    def shockind(self):
        """shockind.f: zero the gradients where the shock indicator exceeds 1."""
        check(L.lib().fvm_gpu_shockind(self.h), "fvm_gpu_shockind")

    def limitgrad(self):
        check(L.lib().fvm_gpu_limitgrad(self.h), "limitgrad")

    def check_positivity(self) -> int:
        bad = C.c_int32(0)
        st = L.lib().fvm_gpu_check_positivity(self.h, C.byref(bad))
        if st not in (L.OK, L.ERR_NONPOSITIVE):
            check(st, "check_positivity")
        return bad.value

    def clcd(self):
        cl, cd = C.c_double(), C.c_double()
        check(L.lib().fvm_gpu_clcd(self.h, C.byref(cl), C.byref(cd)), "clcd")
        return cl.value, cd.value

    def conres(self, first: bool):
        f, fi, ir = C.c_double(), C.c_double(), C.c_int32()
        check(L.lib().fvm_gpu_conres(self.h, 1 if first else 0, C.byref(f), C.byref(fi),
                                     C.byref(ir)), "conres")
        return f.value, fi.value, ir.value

    def iterate(self, nmax: int, minres: float = 0.0, raise_on_error: bool = True):
        """Up to ``nmax`` iterations of main.f:44-62; returns (status, history)."""
        hf = np.zeros(nmax)
        hi = np.zeros(nmax, dtype=np.int32)
        hfi = np.zeros(nmax)
        hcl = np.zeros(nmax)
        hcd = np.zeros(nmax)
        n = C.c_int32(0)
        bad = C.c_int32(0)
        st = L.lib().fvm_gpu_iterate(self.h, nmax, minres, C.byref(n), dptr(hf), iptr(hi),
                                     dptr(hfi), dptr(hcl), dptr(hcd), C.byref(bad))
        k = n.value
        hist = dict(fres=hf[:k], iresi=hi[:k], fresi=hfi[:k], cl=hcl[:k], cd=hcd[:k],
                    bad_point=bad.value)
        if raise_on_error and st != L.OK:
            raise L.FvmError(st, f"iterate (after {k} iterations, bad point {bad.value})")
        return st, hist
