"""Golden records of the reference at the benchmark sizes.

Run where the reference tree is available (it is read, never modified):

    python tests/golden/make_golden_scale.py [--ref /path/to/RePlAce] [--workload NAME ...]

(default: $REPLACE_REFERENCE_ROOT, else the build container's copy).  It
builds the reference's unchanged placement sources with oracle/refbuild
(outputs in oracle/_ref/, git-ignored) and, for each workload of
scale_cases.SCALE_WORKLOADS (the generator's 200k-cell / 40-macro / 512-bin
and 1M-cell / 1024-bin netlists), records:

* scale_eval_<workload>.npz   digests (scale_cases.eval_digest) of one
                              reference NesterovBase evaluation at the seeded
                              centres of scale_cases.eval_coords, with the
                              HPWL, overflow area and sumPhi it reports
* scale_place_<workload>.npz  the reference's own NesterovPlace run without
                              initial place (every movable instance at the
                              core centre, as InitialPlace::placeInstsCenter
                              leaves them): logged (iteration, overflow,
                              HPWL), final overflow and HPWL, exit code and
                              the run's wall time on this host

The netlists themselves are regenerated from the seeded generator by the
tests, so they are not stored.
"""

from __future__ import annotations

import argparse
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "oracle", "refbuild"), HERE):
    if p not in sys.path:
        sys.path.insert(0, p)

from replace_gb300 import netlist as N  # noqa: E402
import scale_cases as S  # noqa: E402
from make_golden import parse_log  # noqa: E402


def oracle_drect(nl, td, bins):
    """Initial gcell density rectangles (centre placement) from the oracle,
    which is bit-exact with the reference on them."""
    from oracle import oracle as O
    o = O.Oracle(nl, target_density=td, bin_grid_cnt_x=bins, bin_grid_cnt_y=bins,
                 initial_place_max_iter=0)
    o.initial_place()
    assert o.nesterov_base() == 0
    drect, _, _ = o.gcells()
    return drect, o.info.n_gcells


def main():
    import refnet
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=refnet.default_ref_root())
    ap.add_argument("--workload", action="append", default=None)
    ap.add_argument("--skip-place", action="store_true")
    args = ap.parse_args()
    if not refnet.build(args.ref):
        raise SystemExit("reference build unavailable")
    for name in args.workload or list(S.SCALE_WORKLOADS):
        nl, td, bins = N.generate_workload(name, seed=S.SCALE_WORKLOADS[name])
        drect, ng = oracle_drect(nl, td, bins)
        xy = S.eval_coords(nl.core, drect)
        t0 = time.time()
        ev = refnet.run_eval(nl, coords=xy, density=td, bins=bins)
        t_eval = time.time() - t0
        grid = ev["grid"]
        assert int(ev["scalars"][5]) == ng, "gcell count differs from the oracle's"
        dig = S.eval_digest(ev, ng, int(grid[0]) * int(grid[1]))
        np.savez_compressed(os.path.join(HERE, f"scale_eval_{name}.npz"), grid=grid,
                            hpwl=np.array(int(ev["scalars"][1]), np.int64),
                            overflow_area=np.array(int(ev["scalars"][0]), np.int64),
                            sum_phi=np.array(float(ev["fscalars"][0])),
                            wl_coef=np.array(float(ev["fscalars"][1])), n_gcells=np.array(ng),
                            seconds=np.array(t_eval), **dig)
        print(name, "eval", f"{t_eval:.1f}s", flush=True)
        if args.skip_place:
            continue
        t0 = time.time()
        rc, log, _ = refnet.run_place(nl, density=td, bins=bins)
        wall = time.time() - t0
        its, ovf, hp, fin, fh = parse_log(log)
        np.savez_compressed(os.path.join(HERE, f"scale_place_{name}.npz"), rc=np.array(rc),
                            iters=its, overflow=ovf, hpwl=hp, final_overflow=np.array(fin),
                            final_hpwl=np.array(fh), seconds=np.array(wall),
                            host=np.array(f"{platform.machine()} {os.cpu_count()} threads"),
                            opts=np.array(repr(dict(density=td, bins=bins))))
        print(name, "place", rc, its[-1] if len(its) else None, fin, fh, f"{wall:.0f}s", flush=True)


if __name__ == "__main__":
    main()
