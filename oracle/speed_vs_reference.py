"""How fast the oracle port is next to the reference's own code (test infrastructure).

The benchmark's CPU baseline runs the port (oracle/nbpg_oracle.cpp) because the reference's sources
do not reach the GPU host.  This script, run where the reference harness is built
(oracle/_ref/libnbpg_ref.so), times on the same inputs and thread count the port's strict search and
the reference's own qsearchAll (beamSearch.h:257-303, scratch allocation inside the timed call as in
check_nn_recall.h:74-76), checks that their ids agree, and prints one JSON line.

    python oracle/speed_vs_reference.py [--n 200000] [--nq 2000] [--threads 0] [--reps 5]
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
# run as a script, this directory comes first on the path and would shadow the package
sys.path = [ROOT] + [p for p in sys.path if os.path.abspath(p or ".") not in (HERE, ROOT)]


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=200_000)
    ap.add_argument("--nq", type=int, default=2_000)
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--reps", type=int, default=5)
    args = ap.parse_args()
    from nbpg_gb300 import synth
    from oracle.oracle import oracle, reference
    O, R = oracle(), reference()
    if R is None:
        sys.exit("the reference harness is not built here (oracle/Makefile: make ref)")
    threads = args.threads or os.cpu_count() or 1
    base, q = synth.u8_mixture(args.n, args.nq, dim=128, n_centres=1000)
    t = time.perf_counter()
    g, _, _, _ = O.build_graph("u8", "l2", base, R=64, L=100, VL=140, num_split=4, num_passes=2,
                               dynamic_prune=True, min_alpha=1.05, max_alpha=1.1, sp_seed=0, threads=threads)
    out = {"n_base": args.n, "n_query": args.nq, "threads": threads, "build_s_port": time.perf_counter() - t,
           "search": {}}
    for L in (19, 50, 100):
        port, ref = [], []
        for _ in range(args.reps):
            t = time.perf_counter()
            oi = O.search("u8", "l2", base, g, q, L=L, k=10, cut=1.35, threads=threads)[0]
            port.append(time.perf_counter() - t)
            ri, sec = R.qsearch_all("u8", "l2", base, g, q, L=L, k=10, cut=1.35, threads=threads)
            ref.append(sec)
        out["search"][f"L{L}"] = {"port_qps": args.nq / float(np.median(port)),
                                  "reference_qsearchAll_qps": args.nq / float(np.median(ref)),
                                  "port_over_reference": float(np.median(ref) / np.median(port)),
                                  "ids_equal": bool(np.array_equal(oi, ri))}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
