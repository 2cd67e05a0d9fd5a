"""Double-float arithmetic of the transport properties
(htr-solver_gb300/csrc/dfloat.cuh): the operations, compiled for the host
from the same header (the device uses explicitly rounded intrinsics, the host
the same IEEE float operations), stay within their error bounds against
double arithmetic on two million random operands each.  Bounds in units of
u^2 = 2^-48: addition 3 (Joldes, Muller, Popescu 2017, AccurateDWPlusDW; the sloppy
algorithm on operands of one sign too),
multiplication 4 (DWTimesDW3), by a float 2 (DWTimesFP3); division,
reciprocal and square root (one Newton correction) 10.  The integer-pipe
conversion from double keeps 2^-48 (2^-23 below 2^-74, 0 below 2^-126), and
the conversion back equals the conversion instructions' result; the
round-to-nearest conversion to float equals the conversion instruction's
(ties included) over float's normal range."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "htr-solver_gb300", "csrc")


def test_dfloat_error_bounds(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "dfloat_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I" + CSRC,
                    os.path.join(HERE, "dfloat_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()
    err = {out[i]: float(out[i + 1]) for i in range(0, len(out), 2)}
    print(err)
    bounds = dict(add=3, addpos=3, same=3, mul=4, mulf=2, div=10, rcp=10, sqrt=10, conv=0.5, bits=1.0,
                  bits_small=2.0 ** -23)
    for k, b in bounds.items():
        assert err[k] <= b, (k, err[k], b)
    assert err["bits_back_mismatch"] == 0
    assert err["round_mismatch"] == 0
    assert err["zero"] == 1
