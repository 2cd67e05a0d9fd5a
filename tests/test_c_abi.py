"""The headers are plain C: a C99 program includes include/htr_rhs.h, links
libhtr_gb300.so and calls the host-side entry points (mixture builders,
argument checks).  No GPU is needed: htr_load_mixture reports
HTR_ERR_NO_DEVICE where there is none."""
import os
import shutil
import subprocess

import pytest

from htr_gb300 import runtime

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <stdio.h>
#include <string.h>
#include "htr_rhs.h"

int main(void) {
  htr_constpropmix_t cp;
  htr_airmix_t air;
  const double xi[HTR_AIR_NSPEC] = {0.79, 0.21, 0.0, 0.0, 0.0};
  htr_mixture_t h = NULL;
  htr_fluid_view v;
  htr_field cc;
  htr_rect3 r = {{0, 0, 0}, {3, 3, 3}};
  const double w[3] = {1.0, 1.0, 1.0};
  int st;
  memset(&v, 0, sizeof v);
  memset(&cc, 0, sizeof cc);
  if (htr_constpropmix_init(287.0, 1.4, 0.71, 1, 1e-3, 300.0, 0.7, &cp) != HTR_OK) return 2;
  if (htr_airmix_init(101325.0, 300.0, 1.0, xi, &air) != HTR_OK) return 3;
  st = htr_load_mixture(HTR_EOS_AIRMIX, &air, sizeof air, &h);
  printf("load %d\n", st);
  if (st == HTR_OK) htr_free_mixture(h);
  /* argument checks run before any device work */
  printf("metric %d\n", htr_InitializeMetric(NULL, cc, r, r, w, NULL));
  printf("bcstep %d\n", htr_rk3_step_bc_ws(&v, r, r, NULL, NULL, NULL, NULL, 0, NULL, NULL, NULL));
  printf("gamma %.3f\n", cp.gamma);
  return 0;
}
"""

# A C program that dumps the restart fields of a host-resident 6x5x4 grid as
# two tiles plus the master file, reads them back into zeroed arrays and
# compares.
RESTART_PROGRAM = r"""
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "htr_restart.h"

#define NX 6
#define NY 5
#define NZ 4
#define NS 5

static void bind(htr_field *f, double *p, int comps) {
  f->base = p;
  f->stride[0] = 8 * comps;
  f->stride[1] = 8 * comps * NX;
  f->stride[2] = 8 * comps * NX * NY;
}

int main(int argc, char **argv) {
  static const int comps[7] = {1, 1, 1, NS, 3, 3, 1};
  double *a[7], *b[7];
  htr_fluid_view va, vb;
  htr_field *fa[7] = {&va.rho, &va.pressure, &va.temperature, &va.MolarFracs, &va.velocity,
                      &va.dudtBoundary, &va.dTdtBoundary};
  htr_field *fb[7] = {&vb.rho, &vb.pressure, &vb.temperature, &vb.MolarFracs, &vb.velocity,
                      &vb.dudtBoundary, &vb.dTdtBoundary};
  htr_rect3 whole = {{0, 0, 0}, {NX - 1, NY - 1, NZ - 1}};
  htr_rect3 parts[2] = {{{0, 0, 0}, {2, NY - 1, NZ - 1}}, {{3, 0, 0}, {NX - 1, NY - 1, NZ - 1}}};
  const int64_t tiles[3] = {2, 1, 1};
  htr_restart_info info = {42, 0.5, 0.0}, back;
  htr_rect3 bounds, got[2];
  int64_t nt[3];
  int i, k, st;
  if (argc < 2) return 9;
  memset(&va, 0, sizeof va);
  memset(&vb, 0, sizeof vb);
  for (k = 0; k < 7; k++) {
    size_t n = (size_t)NX * NY * NZ * comps[k];
    a[k] = malloc(n * sizeof(double));
    b[k] = calloc(n, sizeof(double));
    for (i = 0; i < (int)n; i++) a[k][i] = k * 1000.0 + i * 0.25;
    bind(fa[k], a[k], comps[k]);
    bind(fb[k], b[k], comps[k]);
  }
  for (k = 0; k < 2; k++)
    if ((st = htr_restart_write_tile(argv[1], &va, parts[k], NS, HTR_RESTART_HOST_VIEW, NULL)) != HTR_OK) {
      printf("write %d %s\n", st, htr_last_error());
      return 1;
    }
  if (htr_restart_write_master(argv[1], &info, whole, tiles, parts, NS, NULL, NULL) != HTR_OK) return 2;
  if (htr_restart_read_master(argv[1], &back, &bounds, nt, got, 2) != HTR_OK) return 3;
  for (k = 0; k < 2; k++)
    if (htr_restart_read_tile(argv[1], &vb, got[k], NS, HTR_RESTART_HOST_VIEW, NULL) != HTR_OK) return 4;
  for (k = 0; k < 7; k++)
    if (memcmp(a[k], b[k], (size_t)NX * NY * NZ * comps[k] * sizeof(double)) != 0) return 5;
  printf("timeStep %ld tiles %ld\n", (long)back.timeStep, (long)(nt[0] * nt[1] * nt[2]));
  return 0;
}
"""


def test_c_program_writes_and_reads_a_restart(tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("no host compiler")
    if not os.path.exists(runtime.LIB_PATH):
        pytest.skip("CUDA library not built")
    src = tmp_path / "r.c"
    src.write_text(RESTART_PROGRAM)
    exe = tmp_path / "r"
    libdir = os.path.dirname(runtime.LIB_PATH)
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                    "-L", libdir, "-l:" + os.path.basename(runtime.LIB_PATH), "-Wl,-rpath," + libdir], check=True)
    d = tmp_path / "restart"
    d.mkdir()
    r = subprocess.run([str(exe), str(d)], capture_output=True, text=True)
    assert r.returncode == 0, (r.returncode, r.stdout)
    assert r.stdout.split() == ["timeStep", "42", "tiles", "2"]
    assert sorted(os.listdir(d)) == ["0,0,0-2,4,3.hdf", "3,0,0-5,4,3.hdf", "master.hdf"]


def test_headers_compile_as_c_and_cxx(tmp_path):
    if shutil.which("gcc") is None or shutil.which("g++") is None:
        pytest.skip("no host compiler")
    src = tmp_path / "t.c"
    src.write_text(PROGRAM)
    inc = os.path.join(ROOT, "include")
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I", inc, str(src)], check=True)
    rst = tmp_path / "r.c"
    rst.write_text(RESTART_PROGRAM)
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I", inc, str(rst)], check=True)
    cxx = tmp_path / "t.cpp"
    cxx.write_text('#include "htr_rhs.h"\n#include "htr_restart.h"\nint main() { return 0; }\n')
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-fsyntax-only", "-I", inc, str(cxx)], check=True)


def test_c_program_calls_the_library(tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("no host compiler")
    if not os.path.exists(runtime.LIB_PATH):
        pytest.skip("CUDA library not built")
    src = tmp_path / "t.c"
    src.write_text(PROGRAM)
    exe = tmp_path / "t"
    libdir = os.path.dirname(runtime.LIB_PATH)
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                    "-L", libdir, "-l:" + os.path.basename(runtime.LIB_PATH), "-Wl,-rpath," + libdir], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    vals = dict(line.split() for line in out if line)
    assert vals["load"] in ("0", "6")  # HTR_OK on a GB300, HTR_ERR_NO_DEVICE elsewhere
    assert vals["metric"] == "1" and vals["bcstep"] == "1"  # HTR_ERR_ARGUMENT
    assert vals["gamma"] == "1.400"
