"""The allocation-free residual-norm entry point (fvm_gpu_conres_noalloc).

It exists for drivers that own all device memory themselves (OpenACC or
CUDA Fortran data regions, another framework's memory pool) and therefore
cannot let the library allocate: it works on the driver's own device
arrays and keeps its scratch in a static device array.  Checked here
through the C ABI against the allocating path (fvm_gpu_conres) on two calls
in a row: the first sets the normaliser, the second is normalised by it.
Kept in a file of its own that runs last."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from fvm2d_gb300 import _lib as L  # noqa: E402
from fvm2d_gb300.ogrid import naca_ogrid  # noqa: E402

RTOL = 1e-13   # the two paths sum the squares in different orders


def one_iteration(s):
    s.save_old()
    s.time_step()
    for irk in (1, 2, 3):
        s.residu()
        s.update(irk)


def noalloc(prim, prim_old, first, fres1):
    import torch
    dp = torch.from_numpy(np.ascontiguousarray(prim)).cuda()
    do = torch.from_numpy(np.ascontiguousarray(prim_old)).cuda()
    torch.cuda.synchronize()
    f1 = C.c_double(fres1)
    f, fi, ir = C.c_double(), C.c_double(), C.c_int32()
    st = L.lib().fvm_gpu_conres_noalloc(C.c_void_p(dp.data_ptr()), C.c_void_p(do.data_ptr()),
                                        prim.shape[0], 1 if first else 0, C.byref(f1),
                                        C.byref(f), C.byref(fi), C.byref(ir))
    return st, f1.value, f.value, fi.value, ir.value


def test_noalloc_conres_matches_handle(fvm_lib):
    g = naca_ogrid(64, 24, jitter=0.1, seed=4)
    s = fvm_lib.Solver(fvm_lib.make_params(), fvm_lib.build_geometry(g.coord, g.elem, g.ptype))
    s.iterate(3)
    one_iteration(s)
    f_h, fi_h, ir_h = s.conres(first=True)
    st, fres1, f, fi, ir = noalloc(s.get_state()["prim"], s.prim_old(), True, 0.0)
    assert st == L.OK and f == f_h == 1.0
    assert fi == fi_h and ir == ir_h
    d = s.get_state()["prim"][:, 0] - s.prim_old()[:, 0]
    assert abs(fres1 - np.sqrt(np.sum(d * d) / len(d))) <= RTOL * fres1
    one_iteration(s)
    f_h2, fi_h2, ir_h2 = s.conres(first=False)
    st, _, f2, fi2, ir2 = noalloc(s.get_state()["prim"], s.prim_old(), False, fres1)
    assert st == L.OK
    assert abs(f2 - f_h2) <= RTOL * f_h2
    assert fi2 == fi_h2 and ir2 == ir_h2


def test_noalloc_refuses_oversize_and_zero(fvm_lib):
    import torch
    small = torch.zeros((8, 4), dtype=torch.float64, device="cuda")
    f1 = C.c_double(0.0)
    f = C.c_double()
    too_many = (1 << 20) + 1
    st = L.lib().fvm_gpu_conres_noalloc(C.c_void_p(small.data_ptr()), C.c_void_p(small.data_ptr()),
                                        too_many, 1, C.byref(f1), C.byref(f), None, None)
    assert st == L.ERR_ARG
    st = L.lib().fvm_gpu_conres_noalloc(C.c_void_p(small.data_ptr()), C.c_void_p(small.data_ptr()),
                                        8, 1, C.byref(f1), C.byref(f), None, None)
    assert st == L.ERR_ZERO_FIRST_RES


def test_noalloc_nan_density_change_is_never_the_maximum(fvm_lib):
    """conres.f:17-21 compares |gra| > fresi, which is false for a NaN: a NaN
    density change makes fres NaN but fresi/iresi come from the finite
    points (first maximum on ties)."""
    rng = np.random.default_rng(9)
    n = 3000
    prim_old = rng.uniform(0.5, 1.5, (n, 4))
    prim = prim_old.copy()
    prim[:, 0] += rng.uniform(-1e-3, 1e-3, n)
    prim_old[700, 0] = prim_old[2500, 0] = 1.0
    prim[700, 0] = 1.0 + 2.0 ** -8                    # the largest finite change
    prim[2500, 0] = 1.0 - 2.0 ** -8                   # ties it exactly, later index
    prim[10, 0] = np.nan
    for first in (True, False):
        st, _, f, fi, ir = noalloc(prim, prim_old, first, 1.0)
        assert st == L.OK
        assert np.isnan(f)
        assert fi == 2.0 ** -8 and ir == 701
