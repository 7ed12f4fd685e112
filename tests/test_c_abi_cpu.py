"""The C ABI from C: a driver program written against include/fvm_gpu.h
compiles as C11 with every warning an error, links against the built
library, and runs its host-only part here (parameters and the driver
geometry of a small grid).  The GPU calls are compiled and linked in a
function the program does not call (this host has no GPU); they use the
batch, serving and per-routine calls as a C or Fortran driver would."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from fvm2d_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <stdio.h>
#include <stdlib.h>
#include "fvm_gpu.h"

/* compiled and linked, not run: every call a batched or served driver makes */
void gpu_driver(const fvm_params *par, const fvm_mesh *mesh, double *prim, double *nut,
                double *mul, double *mu, double *qx, double *qy) {
  fvm_handle *h;
  int32_t niter, iresi[10];
  double fres[10], fresi[10], cl[10], cd[10];
  if (fvm_gpu_create(par, mesh, &h) == FVM_OK) {
    fvm_gpu_iterate(h, 10, 1e-6, &niter, fres, iresi, fresi, cl, cd, NULL);
    fvm_gpu_save_old(h);
    fvm_gpu_time_step(h);
    fvm_gpu_residu(h);
    fvm_gpu_update(h, 1);
    fvm_gpu_get_state(h, prim, nut, mul, mu, qx, qy);
    fvm_gpu_destroy(h);
  }
  fvm_batch_caps caps = {0};
  caps.vertices = 6000000; caps.meshes = 256; caps.viscous = 1;
  fvm_batch *b;
  if (fvm_batch_create(FVM_PREC_FP32, &caps, &b) == FVM_OK) {
    int32_t slot, active = 1, n, st, bad, form;
    double ms[16], f, l, d;
    fvm_batch_add(b, par, mesh, &slot);
    fvm_batch_start(b, slot, 5000, 1e-6);
    fvm_batch_tune(b, 5, 16, ms, &form);
    while (active) {
      fvm_batch_step(b, 50);
      fvm_batch_poll(b, slot, &active, &n, &f, &l, &d, &st, &bad);
    }
    fvm_batch_get_state(b, slot, prim, nut, mul, mu, qx, qy);
    fvm_batch_destroy(b);
  }
  fvm_server *srv;
  if (fvm_serve_create(FVM_PREC_FP32, &caps, 50, 40, &srv) == FVM_OK) {
    int64_t t, u, v;
    int32_t state, st, n, it;
    double f, l, d, tail[2], times[3];
    fvm_serve_submit(srv, par, mesh, 5000, 1e-6, 1, &t);
    fvm_serve_wait(srv, t, 600.0, &state);
    fvm_serve_result(srv, t, &st, &n, &f, &l, &d, tail, times);
    fvm_serve_state(srv, t, prim, nut);
    fvm_serve_release(srv, t);
    fvm_serve_submit(srv, par, mesh, 20000, 1e-6, 0, &u);
    fvm_serve_checkpoint(srv, u);
    fvm_serve_wait(srv, u, 1e9, &state);
    fvm_serve_checkpoint_read(srv, u, prim, nut, mul, mu, &it);
    fvm_serve_resume(srv, par, mesh, 20000 - it, 1e-6, prim, nut, mul, mu, it, 1, &v);
    fvm_serve_destroy(srv);
  }
}

int main(void) {
  /* a unit square of 3 x 3 points, two triangles per cell */
  double coord[18];
  int32_t elem[24], ptype[9];
  int k = 0;
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++) {
      coord[2 * (3 * j + i)] = i;
      coord[2 * (3 * j + i) + 1] = j;
      ptype[3 * j + i] = (i == 1 && j == 1) ? FVM_PT_INTERIOR : FVM_PT_FARFIELD;
    }
  for (int j = 0; j < 2; j++)
    for (int i = 0; i < 2; i++) {
      const int a = 3 * j + i + 1, bb = a + 1, c = a + 3, d = a + 4;
      elem[k++] = a; elem[k++] = bb; elem[k++] = d;
      elem[k++] = a; elem[k++] = d; elem[k++] = c;
    }
  fvm_params par;
  if (fvm_params_init(&par, FVM_INVISCID, 0.5, 1.0, 0.0, 1.0, FVM_FLUX_ROE, 1, 0, 0.25, 0.0,
                      FVM_CELL_MEDIAN, 3.0, FVM_PREC_FP64, 0) != FVM_OK) return 1;
  fvm_geom *g;
  const int32_t st = fvm_geom_build(9, 8, coord, elem, ptype, FVM_CELL_MEDIAN, &g);
  if (st != FVM_OK) { printf("geom %s\n", fvm_gpu_strerror(st)); return 2; }
  double area = 0.0;
  for (int i = 0; i < g->mesh.np; i++) area += g->cvarea[i];
  printf("np %d nt %d netot %d ne %d nbe %d area %.17g gamma %.17g\n", g->mesh.np, g->mesh.nt,
         g->mesh.netot, g->mesh.ne, g->mesh.nbe, area, par.gamma);
  fvm_geom_free(g);
  if (getenv("FVM_NEVER_SET_THIS")) gpu_driver(&par, NULL, NULL, NULL, NULL, NULL, NULL, NULL);
  return 0;
}
"""


@pytest.fixture(scope="module")
def built():
    B.build()
    return B.LIB


def test_c_driver_compiles_links_and_runs_host_part(built, tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    src = tmp_path / "driver.c"
    src.write_text(PROGRAM)
    exe = tmp_path / "driver"
    libdir = os.path.dirname(built)
    cmd = [cc, "-std=c11", "-Wall", "-Wextra", "-Werror", "-Wno-unused-parameter",
           "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
           "-L", libdir, "-lfvm2d_gb300", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    f = dict(zip(r.stdout.split()[0::2], r.stdout.split()[1::2]))
    # 9 points, 8 triangles, 16 edges, all kept; 8 boundary edges on the
    # farfield; the median dual areas tile the unit square... of side 2
    assert (int(f["np"]), int(f["nt"]), int(f["netot"]), int(f["ne"]), int(f["nbe"])) == \
        (9, 8, 16, 16, 8)
    assert abs(float(f["area"]) - 4.0) < 1e-12
    assert float(f["gamma"]) == 1.4
    assert np.isfinite(float(f["area"]))
