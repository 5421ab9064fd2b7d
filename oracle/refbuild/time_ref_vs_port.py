"""Times the reference's own Nesterov loop (oracle/_ref/ref_driver, built from
the reference sources) against the oracle restatement on the same netlist,
one thread each, on this host.

TEST INFRASTRUCTURE ONLY: it records which CPU arm is faster.  The
reference build needs the reference sources, so it runs where they are (not
on the GPU host).

    python oracle/refbuild/time_ref_vs_port.py [--workload NAME ...] [--warm 3] [--steps 5]

Per-iteration time = (wall(warm + steps iterations) - wall(warm iterations))
/ steps for the reference build (each a separate process from the centred
placement, so setup cancels), and the oracle's nesterov_run(steps) after
nesterov_run(warm) in one process.  Prints one JSON line per workload.
"""

from __future__ import annotations

import argparse
import json
import os
import platform
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, HERE):
    if p not in sys.path:
        sys.path.insert(0, p)

import refnet  # noqa: E402
from replace_gb300 import netlist as N  # noqa: E402


def ref_wall(net, td, bins, iters):
    t0 = time.perf_counter()
    r = subprocess.run([refnet.DRIVER, "place", net, "--density", str(td), "--bins", str(bins),
                        "--maxiter", str(iters)], capture_output=True, text=True)
    if r.returncode not in (0, 3, 4):
        raise RuntimeError(r.stdout + r.stderr)
    return time.perf_counter() - t0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", action="append", default=None)
    ap.add_argument("--warm", type=int, default=3)
    ap.add_argument("--steps", type=int, default=5)
    args = ap.parse_args()
    if not refnet.available():
        raise SystemExit("reference build unavailable (oracle/_ref)")
    from oracle import oracle as O
    for name in args.workload or ["200k_cells_40macros_512bins", "1m_cells_1024bins"]:
        nl, td, bins = N.generate_workload(name, seed=1)
        with tempfile.TemporaryDirectory() as d:
            net = os.path.join(d, "net.txt")
            refnet.write_refnet(nl, net)
            a = ref_wall(net, td, bins, args.warm)
            b = ref_wall(net, td, bins, args.warm + args.steps)
        ref_s = (b - a) / args.steps
        o = O.Oracle(nl, target_density=td, bin_grid_cnt_x=bins, bin_grid_cnt_y=bins,
                     initial_place_max_iter=0)
        o.initial_place()
        o.nesterov_init()
        o.nesterov_run(args.warm)
        t0 = time.perf_counter()
        o.nesterov_run(args.steps)
        port_s = (time.perf_counter() - t0) / args.steps
        print(json.dumps({"workload": name, "reference_s_per_iter": ref_s, "port_s_per_iter": port_s,
                          "faster": "port" if port_s < ref_s else "reference",
                          "host": f"{platform.machine()} {os.cpu_count()} threads, one used",
                          "warm": args.warm, "steps": args.steps}), flush=True)


if __name__ == "__main__":
    main()
