"""ctypes wrapper of the CPU oracle (test infrastructure).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs of
``bench.py`` (its cpu_baseline and the reference arm) import this module,
as the checker and the timed CPU implementation.  The oracle is a serial
FP64 C restatement of the reference's Fortran hot path (fvm_oracle.c);
``build()`` compiles it with the Makefile beside this file.  Parity is
unpinned by the reference, which ships no tests or vectors and cannot be
compiled here; tests/test_oracle.py pins it by answers derived from the
equations.
"""
from __future__ import annotations

import ctypes as C
import os
import platform
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", platform.machine(), "libfvm_oracle.so")

INVISCID, LAMINAR, TURBULENT = 1, 2, 3
ROE, KFVS, HLLC = 1, 2, 3
MEDIAN, BARTH = 1, 2


class OrcInput(C.Structure):
    _fields_ = [("iflow", C.c_int32), ("mach_inf", C.c_double), ("aoa_deg", C.c_double),
                ("rey", C.c_double), ("cfl", C.c_double), ("iterlast", C.c_int32),
                ("maxiter", C.c_int32), ("minres", C.c_double), ("iflux", C.c_int32),
                ("ilimit", C.c_int32), ("vortex", C.c_int32), ("xref", C.c_double),
                ("yref", C.c_double), ("cell_type", C.c_int32), ("nut_ratio", C.c_double),
                ("bugcompat", C.c_int32)]


_SCALAR_INTS = ["np", "nt", "ne", "netot", "nsp", "nfp", "nbe", "nswe1", "nswe2", "nffe1",
                "nffe2", "iter", "iterlast", "iresi", "err", "err_point"]
_SCALAR_DBLS = ["fres", "fres1", "fresi", "cl", "cd", "dtglobal", "gamma", "gamma1",
                "gas_const", "pi", "prandtl", "prandtl_turb", "albada11", "albada12",
                "albada21", "albada22", "cb1", "cb2", "sigma_sa", "kolm", "cw1", "cw2",
                "cw3", "cv1", "cv2", "cv11", "cw31", "cw32", "kolm2", "cb2sig1", "cb2sig2",
                "mach_inf", "aoa_deg", "aoa", "rey", "cfl", "q_inf", "r_inf", "p_inf",
                "t_inf", "u_inf", "v_inf", "a_inf", "sconst", "nut_inf", "xref", "yref"]


class OrcScalars(C.Structure):
    _fields_ = ([(n, C.c_int32) for n in _SCALAR_INTS]
                + [(n, C.c_double) for n in _SCALAR_DBLS]
                + [("airk", C.c_double * 3), ("birk", C.c_double * 3)])


def build(quiet: bool = True) -> str:
    """Compile the oracle library (make -C oracle)."""
    out = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        vp, i32, dbl = C.c_void_p, C.c_int32, C.c_double
        pd, pi = C.POINTER(C.c_double), C.POINTER(C.c_int32)
        L.orc_create.restype = vp
        L.orc_create.argtypes = [C.POINTER(OrcInput), i32, i32, pd, pi, pi, pi]
        L.orc_destroy.argtypes = [vp]
        L.orc_get_scalars.argtypes = [vp, C.POINTER(OrcScalars)]
        L.orc_set_cl.argtypes = [vp, dbl]
        L.orc_darray.restype = pd
        L.orc_darray.argtypes = [vp, C.c_char_p, C.POINTER(C.c_int64)]
        L.orc_iarray.restype = pi
        L.orc_iarray.argtypes = [vp, C.c_char_p, C.POINTER(C.c_int64)]
        for n in ["orc_save_old", "orc_time_step", "orc_residu", "orc_sa_model",
                  "orc_limitgrad", "orc_clcd", "orc_gradient"]:
            getattr(L, n).argtypes = [vp]
        L.orc_shockind.argtypes = [vp, pd]
        L.orc_update.argtypes = [vp, i32]
        L.orc_check_positivity.argtypes = [vp]
        L.orc_check_positivity.restype = i32
        L.orc_conres.argtypes = [vp]
        L.orc_conres.restype = i32
        L.orc_iterate.argtypes = [vp, i32, dbl, pi, pd, pi, pd, pd, pd]
        L.orc_iterate.restype = i32
        L.orc_dtlength.argtypes = [i32, i32, pd, pi, pd, pd]
        L.orc_wall_dist.argtypes = [i32, i32, pd, pi, pi, i32, pd]
        L.orc_eval_flux.argtypes = [vp, i32, pd, pd, pd, pd]
        L.orc_eval_flux.restype = i32
        L.orc_limit_albada.argtypes = [dbl, dbl]
        L.orc_limit_albada.restype = dbl
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


class Oracle:
    """One solver instance: start-up of main.f:20-27 then the loop body."""

    def __init__(self, coord, elem, ptype, *, iflow=INVISCID, mach=0.8, aoa_deg=1.25,
                 rey=0.0, cfl=1.0, iflux=ROE, ilimit=1, vortex=0, xref=0.25, yref=0.0,
                 cell_type=MEDIAN, nut_ratio=0.1, bugcompat=1, iterlast=0):
        L = lib()
        self._coord = np.ascontiguousarray(coord, dtype=np.float64)
        self._elem = np.ascontiguousarray(elem, dtype=np.int32)
        self._ptype = np.ascontiguousarray(ptype, dtype=np.int32)
        self.inp = OrcInput(iflow=iflow, mach_inf=mach, aoa_deg=aoa_deg, rey=rey, cfl=cfl,
                            iterlast=iterlast, maxiter=10**9, minres=0.0, iflux=iflux,
                            ilimit=ilimit, vortex=vortex, xref=xref, yref=yref,
                            cell_type=cell_type, nut_ratio=nut_ratio, bugcompat=bugcompat)
        st = C.c_int32(0)
        h = L.orc_create(C.byref(self.inp), self._coord.shape[0], self._elem.shape[0],
                         _dp(self._coord), _ip(self._elem), _ip(self._ptype), C.byref(st))
        if not h:
            raise RuntimeError(f"oracle start-up stopped with status {st.value}")
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    # ---- views -----------------------------------------------------------
    def scalars(self) -> dict:
        s = OrcScalars()
        lib().orc_get_scalars(self.h, C.byref(s))
        d = {n: getattr(s, n) for n in _SCALAR_INTS + _SCALAR_DBLS}
        d["airk"] = list(s.airk)
        d["birk"] = list(s.birk)
        return d

    def d(self, name: str, shape2: int | None = None) -> np.ndarray:
        """Live view of a double array (shape [n, k] for k-component arrays)."""
        n = C.c_int64(0)
        p = lib().orc_darray(self.h, name.encode(), C.byref(n))
        if not p:
            raise KeyError(name)
        a = np.ctypeslib.as_array(p, shape=(max(n.value, 1),))[: n.value]
        comp = {"coord": 2, "prim": 4, "prim_old": 4, "qx": 4, "qy": 4, "res": 4, "ds": 2,
                "dsb": 2, "tcoord": 2}.get(name, shape2)
        return a.reshape(-1, comp) if comp else a

    def i(self, name: str) -> np.ndarray:
        n = C.c_int64(0)
        p = lib().orc_iarray(self.h, name.encode(), C.byref(n))
        if not p:
            raise KeyError(name)
        a = np.ctypeslib.as_array(p, shape=(max(n.value, 1),))[: n.value]
        comp = {"elem": 3, "edge": 2, "edneigh": 2}.get(name)
        return a.reshape(-1, comp) if comp else a

    def mesh_arrays(self) -> dict:
        """The fvm_mesh inputs of the C ABI, as produced by geometric()."""
        s = self.scalars()
        out = {k: s[k] for k in ["np", "nt", "ne", "netot", "nsp", "nbe", "nswe1",
                                  "nswe2", "nffe1", "nffe2"]}
        for k in ["coord", "ds", "dsb", "elarea", "cvarea", "mcarea", "drmin", "wd"]:
            out[k] = self.d(k).copy()
        for k in ["elem", "ptype", "spts", "edge", "edneigh", "iedge", "beindx"]:
            out[k] = self.i(k).copy()
        return out

    # ---- routines -----------------------------------------------------------
    def save_old(self):
        lib().orc_save_old(self.h)

    def time_step(self):
        lib().orc_time_step(self.h)

    def residu(self):
        lib().orc_residu(self.h)

    def update(self, irk: int):
        lib().orc_update(self.h, irk)

    def sa_model(self):
        lib().orc_sa_model(self.h)

    def limitgrad(self):
        lib().orc_limitgrad(self.h)

    def gradient(self):
        """gradient.f: edge-based Green-Gauss gradients into qx, qy."""
        lib().orc_gradient(self.h)

    def shockind(self):
        """shockind.f: returns the indicator per vertex; zeroes qx, qy where
        it exceeds 1."""
        ind = np.zeros(self.scalars()["np"])
        lib().orc_shockind(self.h, ind.ctypes.data_as(C.POINTER(C.c_double)))
        return ind

    def check_positivity(self) -> int:
        return lib().orc_check_positivity(self.h)

    def clcd(self):
        lib().orc_clcd(self.h)
        s = self.scalars()
        return s["cl"], s["cd"]

    def conres(self):
        st = lib().orc_conres(self.h)
        s = self.scalars()
        return st, s["fres"], s["fresi"], s["iresi"]

    def flux(self, iflux: int, ds, priml, primr):
        """One interior face flux; returns (status, flux[4])."""
        ds = np.ascontiguousarray(ds, dtype=np.float64)
        pl = np.ascontiguousarray(priml, dtype=np.float64)
        pr = np.ascontiguousarray(primr, dtype=np.float64)
        out = np.zeros(4)
        st = lib().orc_eval_flux(self.h, iflux, _dp(ds), _dp(pl), _dp(pr), _dp(out))
        return st, out

    def set_cl(self, cl: float):
        lib().orc_set_cl(self.h, cl)

    def iterate(self, nmax: int, minres: float = 0.0):
        hf = np.zeros(nmax)
        hi = np.zeros(nmax, dtype=np.int32)
        hfi = np.zeros(nmax)
        hcl = np.zeros(nmax)
        hcd = np.zeros(nmax)
        n = C.c_int32(0)
        st = lib().orc_iterate(self.h, nmax, minres, C.byref(n), _dp(hf), _ip(hi), _dp(hfi),
                               _dp(hcl), _dp(hcd))
        k = n.value
        return st, dict(fres=hf[:k], iresi=hi[:k], fresi=hfi[:k], cl=hcl[:k], cd=hcd[:k])


def dtlength(coord, elem, elarea):
    coord = np.ascontiguousarray(coord, dtype=np.float64)
    elem = np.ascontiguousarray(elem, dtype=np.int32)
    elarea = np.ascontiguousarray(elarea, dtype=np.float64)
    out = np.zeros(coord.shape[0])
    lib().orc_dtlength(coord.shape[0], elem.shape[0], _dp(coord), _ip(elem), _dp(elarea),
                       _dp(out))
    return out


def wall_dist(coord, edge, ptype, bugcompat=1):
    coord = np.ascontiguousarray(coord, dtype=np.float64)
    edge = np.ascontiguousarray(edge, dtype=np.int32)
    ptype = np.ascontiguousarray(ptype, dtype=np.int32)
    out = np.zeros(coord.shape[0])
    lib().orc_wall_dist(coord.shape[0], edge.shape[0], _dp(coord), _ip(edge), _ip(ptype),
                        bugcompat, _dp(out))
    return out


def limit_albada(ul: float, ur: float) -> float:
    return lib().orc_limit_albada(ul, ur)
