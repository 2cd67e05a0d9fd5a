"""The table-driven exponential of the explicit chemistry sources
(htr-solver_gb300/csrc/fastexp.cuh, Tang's method): its table and reduction
constants are the correctly rounded values (CPU, exact decimal arithmetic),
and on the GPU its results agree with CUDA's exp within one ulp over the
argument range of the Arrhenius rates and equilibrium constants, with the
library's exp taking over at |x| >= 700."""
import ctypes as C
import decimal
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "htr-solver_gb300", "csrc")
HEADER = os.path.join(CSRC, "fastexp.cuh")


def _header():
    with open(HEADER) as f:
        return f.read()


def _exact(expr, prec=60):
    with decimal.localcontext() as ctx:
        ctx.prec = prec
        return expr()


def test_table_is_correctly_rounded():
    src = _header()
    body = src[src.index("kExp2Frac[64] = {"):]
    body = body[:body.index("};")]
    vals = [float.fromhex(h) for h in re.findall(r"0x[0-9a-f.]+p[+-]\d+", body)]
    assert len(vals) == 64
    for j, v in enumerate(vals):
        want = _exact(lambda: decimal.Decimal(2) ** (decimal.Decimal(j) / 64))
        assert v == float(want), j  # float(Decimal) rounds to nearest


def test_reduction_constants():
    src = _header()
    inv = float.fromhex("0x1.71547652b82fep+6")
    l1 = float.fromhex("0x1.62e42fefa39efp-7")
    l2 = float.fromhex("0x1.abc9e3b39803fp-62")
    for h in ("0x1.71547652b82fep+6", "0x1.62e42fefa39efp-7", "0x1.abc9e3b39803fp-62"):
        assert h in src
    ln2 = _exact(lambda: decimal.Decimal(2).ln())
    assert inv == float(_exact(lambda: 64 / ln2))
    step = _exact(lambda: ln2 / 64)
    assert l1 == float(step)
    assert l2 == float(_exact(lambda: step - decimal.Decimal(l1)))


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    nvcc = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    out = str(tmp_path_factory.mktemp("fastexp") / "libfastexp_check.so")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-shared",
                    "-Xcompiler", "-fPIC", "-I" + CSRC, "-I" + os.path.join(os.path.dirname(HERE), "include"),
                    os.path.join(HERE, "fastexp_check.cu"), "-o", out], check=True)
    lib = C.CDLL(out)
    lib.fastexp_check.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
    return lib


@pytest.mark.gpu
def test_matches_the_math_library(checker):
    rng = np.random.Generator(np.random.PCG64(5))
    x = np.concatenate([
        rng.uniform(-700, 700, 1 << 20),
        rng.uniform(-1, 1, 1 << 16),
        rng.uniform(-1e-3, 1e-3, 1 << 12),
        np.linspace(-699.999, 699.999, 4001),
        # around the table's breakpoints k ln2/64 and the fallback threshold
        np.arange(-4000, 4000) * (np.log(2) / 64) + 1e-13,
        np.arange(-4000, 4000) * (np.log(2) / 64) - 1e-13,
        np.array([0.0, -0.0, 699.9999999, -699.9999999, 700.0, -700.0, 710.0, -745.0, -800.0]),
    ])
    fast = np.empty_like(x)
    ref = np.empty_like(x)
    assert checker.fastexp_check(x.ctypes.data, fast.ctypes.data, ref.ctypes.data, len(x)) == 0
    big = np.abs(x) >= 700
    assert np.array_equal(fast[big], ref[big])
    ulp = np.spacing(np.abs(ref[~big]))
    err = np.abs(fast[~big] - ref[~big]) / ulp
    print(f"max |exp_table - exp| = {err.max():.2f} ulp over {err.size} arguments; "
          f"{np.mean(err > 0):.3%} differ")
    assert err.max() <= 1.0
    rel = np.abs(fast[~big] / ref[~big] - 1.0)
    assert rel.max() < 2.3e-16
