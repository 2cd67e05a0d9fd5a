"""Builds libhtr_gb300.so (CUDA, sm_103a) in-tree under htr-solver_gb300/_build/.

Translation units that evaluate TENO selections or shock sensors
(euler.cu, sensor.cu, stage_euler.cu), the grid metrics (metric.cu) and the
implicit chemistry solver (implicit_chem.cu) are compiled with -fmad=false
so every floating-point operation is rounded exactly as the reference's CPU
build rounds it; the others keep FMA contraction.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libhtr_gb300.so")
# the benchmark's FP64 peak probe, a library of its own (not the product)
PROBE_SRC = os.path.join(HERE, "probe", "fp64_probe.cu")
PROBE_LIB = os.path.join(OUT_DIR, "libhtr_probe.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
EXACT_TUS = {"euler.cu", "sensor.cu", "stage_euler.cu", "metric.cu", "implicit_chem.cu"}


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _sources():
    # CUDA translation units and host-only C++ (compiled by nvcc's host compiler)
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    root = os.path.dirname(HERE)
    files += [os.path.join(root, "include", h) for h in os.listdir(os.path.join(root, "include"))]
    files.append(os.path.abspath(__file__))
    return files


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = _deps()
    if not force and not _stale(LIB, deps):
        return LIB
    root = os.path.dirname(HERE)
    base = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
            "--expt-relaxed-constexpr", "-I" + os.path.join(root, "include"), "-I" + CSRC]
    if verbose:
        base += ["-Xptxas", "-v"]

    def compile_one(src):
        obj = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
        cmd = base + (["-fmad=false"] if src in EXACT_TUS else []) + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        return obj, r.stderr

    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        results = list(ex.map(compile_one, srcs))
    if verbose:
        for _, err in results:
            print(err)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    subprocess.run([nvcc(), *ARCH, "-shared", "-o", tmp] + objs, check=True)
    os.replace(tmp, LIB)
    return LIB


def build_probe(force=False):
    """libhtr_probe.so: the benchmark's FP64 rate probe."""
    os.makedirs(OUT_DIR, exist_ok=True)
    root = os.path.dirname(HERE)
    if not force and not _stale(PROBE_LIB, [PROBE_SRC, os.path.abspath(__file__)]):
        return PROBE_LIB
    tmp = PROBE_LIB + ".tmp"
    subprocess.run([nvcc(), *ARCH, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
                    "-I" + os.path.join(root, "include"), PROBE_SRC, "-o", tmp], check=True)
    os.replace(tmp, PROBE_LIB)
    return PROBE_LIB


def build_all(root, force=False):
    """Package library, the benchmark's probe, and the CPU checkers used by the tests."""
    build(force=force)
    build_probe(force=force)
    import importlib.util
    spec = importlib.util.spec_from_file_location("_htr_oracle_build", os.path.join(root, "oracle", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build_all(force=force)
