"""Record the oracle's FP64 Jacobi-PCG iteration count to 1e-10 for a bench
configuration into oracle/iterations.json.

TEST INFRASTRUCTURE ONLY.  bench.py's reference arm and cpu_baseline leg time
a bounded sample of oracle iterations and scale it by this count, so that a
default bench run does not spend ten minutes in a full CPU solve.

    python oracle/count_iterations.py c2
"""
from __future__ import annotations

import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import bench  # noqa: E402
from oracle import oracle as orc  # noqa: E402


def main(config: str) -> None:
    t0 = time.time()
    _, m, mask, h1c, h2, f, dinv = bench.setup_cpu_case(bench.CONFIGS[config])
    t1 = time.time()
    _, it, r0, r1 = orc.cg(m, f, h1c=h1c, h2=h2, mask=mask, dinv=dinv, rtol=bench.RTOL, max_iter=20000)
    t2 = time.time()
    path = os.path.join(HERE, "iterations.json")
    rec = json.load(open(path)) if os.path.exists(path) else {}
    rec[config] = {"iters": int(it), "res_start": r0, "res_final": r1, "setup_s": round(t1 - t0, 2),
                   "solve_s": round(t2 - t1, 2), "threads": orc.num_threads()}
    with open(path, "w") as fh:
        json.dump(rec, fh, indent=1)
        fh.write("\n")
    print(json.dumps(rec[config]))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "c2")
