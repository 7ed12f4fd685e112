"""GB300-native implementation of fvm2d's per-iteration hot path.

The product is the C-ABI library ``_build/libfvm2d_gb300.so`` (hand-written
CUDA for sm_103a + host runtime); this package is its Python host side:
``solver.Solver`` mirrors the reference routines, ``solver.build_geometry``
is the driver-side geometry, ``ogrid`` generates the benchmark grids.
"""
from ._lib import (BARTH, FP32, FP64, HLLC, INVISCID, KFVS, LAMINAR, MEDIAN, ROE,  # noqa: F401
                   TURBULENT, FvmError)
from .ogrid import naca_ogrid, workload_grid  # noqa: F401
from .solver import Solver, build_geometry, dtlength, make_params, wall_dist  # noqa: F401
