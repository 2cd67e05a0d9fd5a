"""Speed of the oracle port against the reference's compiled CPU tasks on the
same machine (test infrastructure: it times the two CPU oracles, nothing of
the product).

Both run one SSP-RK3 step of the same seeded 5-species air box (hybrid
scheme, diffusion, explicit chemistry) through the oracle driver, with the
same number of OpenMP threads, alternating port and reference `--reps`
times; prints the cell-updates/s of each and the median and spread of the
per-pair ratio port / reference as one JSON line.

    python oracle/speed.py [--n 48] [--reps 9] [--threads N]

Needs the compiled reference (oracle/_ref, built where the reference sources
are present).
"""
import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=48)
    ap.add_argument("--reps", type=int, default=9)
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    args = ap.parse_args()
    os.environ["OMP_NUM_THREADS"] = str(args.threads)
    import __graft_entry__
    __graft_entry__.load_package()
    import numpy as np

    import oracle
    from htr_gb300 import abi, workloads
    eos = abi.HTR_EOS_AIRMIX
    ref = oracle.ref_lib(eos)
    if ref is None:
        print(json.dumps({"error": "the compiled reference is not built here"}))
        return 1
    port = oracle.port_lib()
    port.htr_oracle_set_threads(args.threads)
    libs = {"port": port, "reference": ref}
    states = {}
    for name, lib in libs.items():
        fl = workloads.air_box(args.n, seed=1234)
        h = oracle.load_mixture(lib, eos, workloads.make_mixture_struct(lib, eos, fl.meta["mix"]))
        workloads.derive_state(lib, fl, h)
        states[name] = (fl, h)
    dt = 1e-9
    for name, lib in libs.items():  # warm-up
        fl, h = states[name]
        oracle.step(lib, fl.copy(), h, dt=dt, chemistry=True)
    rates = {"port": [], "reference": []}
    for _ in range(args.reps):
        for name, lib in libs.items():
            fl, h = states[name]
            f = fl.copy()
            t0 = time.perf_counter()
            oracle.step(lib, f, h, dt=dt, chemistry=True)
            rates[name].append(3.0 * f.ncells / (time.perf_counter() - t0))
    ratio = np.array(rates["port"]) / np.array(rates["reference"])
    print(json.dumps({"grid": [args.n] * 3, "threads": args.threads, "reps": args.reps,
                      "port_cell_updates_per_s": float(np.median(rates["port"])),
                      "reference_cell_updates_per_s": float(np.median(rates["reference"])),
                      "ratio_port_over_reference_median": float(np.median(ratio)),
                      "ratio_min": float(ratio.min()), "ratio_max": float(ratio.max())}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
