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


def test_headers_compile_as_c_and_cxx(tmp_path):
    if shutil.which("gcc") is None or shutil.which("g++") is None:
        pytest.skip("no host compiler")
    src = tmp_path / "t.c"
    src.write_text(PROGRAM)
    inc = os.path.join(ROOT, "include")
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I", inc, str(src)], check=True)
    cxx = tmp_path / "t.cpp"
    cxx.write_text('#include "htr_rhs.h"\nint main() { return 0; }\n')
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
