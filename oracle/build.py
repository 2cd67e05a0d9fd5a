"""Builds the CPU oracles (test infrastructure only).

* oracle/_build/libhtroracle.so   the from-scratch C++ port (oracle/port/)
* oracle/_ref/libhtrref_<EOS>.so  the reference's own CPU task code, built
                                  by oracle/ref/Makefile from the reference
                                  sources, only where those sources exist.

Both are compiled without FMA contraction (-ffp-contract=off) so that x86-64
and aarch64 hosts produce the same bits.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def ref_src():
    """The reference's src/ directory: $HTR_REF_SRC, else src/ of a checkout of
    the reference named `reference` beside this repository."""
    env = os.environ.get("HTR_REF_SRC")
    if env:
        return env
    return os.path.join(os.path.dirname(ROOT), "reference", "src")


def _newer(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_port(force=False):
    out_dir = os.path.join(HERE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "libhtroracle.so")
    port = os.path.join(HERE, "port")
    srcs = sorted(os.path.join(port, f) for f in os.listdir(port) if f.endswith(".cpp"))
    deps = srcs + sorted(os.path.join(port, f) for f in os.listdir(port) if f.endswith(".hpp"))
    deps += [os.path.join(ROOT, "include", h) for h in ("htr_rhs.h", "htr_mix.h")]
    if not force and not _newer(out, deps):
        return out
    cxx = os.environ.get("CXX", "g++")
    cmd = [cxx, "-std=c++17", "-O3", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off",
           "-I" + os.path.join(ROOT, "include"), "-o", out] + srcs
    subprocess.run(cmd, check=True)
    return out


def build_ref(force=False):
    """Build the reference oracle if its sources are present; return True if built."""
    src = ref_src()
    if not os.path.isdir(src) or shutil.which("make") is None:
        return False
    jobs = str(max(1, min(16, os.cpu_count() or 1)))
    cmd = ["make", "-s", "-C", os.path.join(HERE, "ref"), "-j", jobs, "REF_SRC=" + os.path.abspath(src)]
    if force:
        cmd.insert(1, "-B")
    subprocess.run(cmd, check=True)
    return True


def build_all(force=False):
    build_port(force)
    build_ref(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
