"""Generates the golden fixtures in this directory from the reference's own code.

Run where the reference tree is available (it is read, never modified):

    python tests/golden/make_golden.py [--ref /path/to/RePlAce]

(default: $REPLACE_REFERENCE_ROOT, else the build container's copy)

It builds the reference's unchanged placement sources with oracle/refbuild
(outputs in oracle/_ref/, git-ignored), then records for each case:

* netlist_<case>.npz   the flattened netlist (from the reference's regression
                       LEF/DEF, or the seeded synthetic generator)
* eval_<case>.npz      one NesterovBase evaluation at seeded random gcell
                       centres: bin areas, density, phi, field, per-gcell WA
                       and density gradients, overflow area, HPWL
* place_<case>.npz     the Nesterov run: logged (iteration, overflow, HPWL),
                       exit code, final overflow and HPWL, final locations
* ip_<case>.npz        for designs placed with the initial place (simple03,
                       simple04): the rounds and Nesterov lines the
                       reference logged in test/<case>.ok (its initial place
                       needs Eigen, so it is not rebuilt here)
* defok_<case>.npz     the COMPONENTS section of the reference's regression
                       output test/<case>.defok (what its write_def produced
                       after global_placement): per component its location,
                       status and orientation, in DEF order
"""

from __future__ import annotations

import argparse
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle", "refbuild"))

from replace_gb300 import netlist as N  # noqa: E402

# regression designs and their global_placement flags (test/<case>.tcl)
LEFDEF_CASES = {
    "simple01": dict(density=0.7, idp=0.01),
    "simple02": dict(density=0.6, idp=0.01),
    "core01": dict(density=0.6, idp=0.01),
    "ar01": dict(density=0.6, idp=0.01),
    "ar02": dict(density=0.6, idp=0.01),
    "incremental01": dict(density=0.7, idp=0.1, incremental=True),
    "diverge01": dict(density=0.7, idp=100),
}
EVAL_CASES = ["simple01", "simple02", "ar01", "syn10k_b128", "syn_macro", "syn_fixed"]
PLACE_CASES = list(LEFDEF_CASES) + ["syn10k_b128", "syn_macro", "syn_fixed"]
# designs run with the initial place (netlists only: the reference's IP needs
# Eigen and does not build here; its logged rounds are in test/<case>.ok)
IP_CASES = ["simple03", "simple04"]


def synthetic(name):
    """Synthetic cases: (netlist, options)."""
    if name == "syn10k_b128":
        return N.generate(10_000, 10_500, seed=1), dict(density=0.7, bins=128)
    if name in ("syn_macro", "syn_fixed"):
        nl = N.generate(3_000, 3_150, n_io=100, n_macros=6, seed=3, macro_rows=(10, 20))
        if name == "syn_fixed":
            # fix two macros at chosen places: their pins become fixed pins
            h = nl.inst_uy - nl.inst_ly
            macros = np.nonzero(h > 6 * N.ROW_H)[0][:2]
            c = nl.core
            for k, i in enumerate(macros):
                w = nl.inst_ux[i] - nl.inst_lx[i]
                x = c[0] + (c[2] - c[0]) // 4 + k * (c[2] - c[0]) // 3
                y = c[1] + (c[3] - c[1]) // 3
                nl.inst_lx[i], nl.inst_ux[i] = x, x + w
                nl.inst_ly[i], nl.inst_uy[i] = y, y + h[i]
                nl.inst_kind[i] = N.INST_FIXED
            nl._update_pins()
        return nl, dict(density=0.7)
    raise KeyError(name)


def case_netlist(name, ref_root):
    if name in LEFDEF_CASES:
        t = os.path.join(ref_root, "test")
        return N.read(os.path.join(t, "nangate45.lef"), os.path.join(t, name + ".def")), \
            dict(LEFDEF_CASES[name])
    return synthetic(name)


def parse_log(log):
    its, ovf, hp = [], [], []
    for l in log.splitlines():
        m = re.match(r"\[NesterovSolve\] Iter: (\d+) overflow: (\S+) HPWL: (\d+)", l)
        if m:
            its.append(int(m.group(1))); ovf.append(float(m.group(2))); hp.append(int(m.group(3)))
    fin = re.search(r"Finished with Overflow: (\S+)", log)
    fh = re.search(r"\[REF\] FinalHPWL (\d+)", log)
    return (np.array(its, np.int32), np.array(ovf, np.float64), np.array(hp, np.int64),
            float(fin.group(1)) if fin else float("nan"), int(fh.group(1)) if fh else -1)


STATUS_CODES = {"UNPLACED": 0, "PLACED": 1, "FIXED": 2, "COVER": 3}


def save_defok(ref_root, name):
    from replace_gb300 import lefdef
    d = lefdef.read_def(os.path.join(ref_root, "test", name + ".defok"))
    np.savez_compressed(os.path.join(HERE, f"defok_{name}.npz"),
                        x=np.array([c.x for c in d.components], np.int32),
                        y=np.array([c.y for c in d.components], np.int32),
                        status=np.array([STATUS_CODES[c.status] for c in d.components], np.int8),
                        orient=np.array([c.orient for c in d.components]),
                        master=np.array([c.master for c in d.components]),
                        name=np.array([c.name for c in d.components]))


def main():
    ap = argparse.ArgumentParser()
    import refnet
    ap.add_argument("--ref", default=refnet.default_ref_root())
    ap.add_argument("--only-defok", action="store_true",
                    help="write only the defok_<case>.npz fixtures")
    args = ap.parse_args()
    for name in LEFDEF_CASES:
        save_defok(args.ref, name)
    if args.only_defok:
        return
    if not refnet.build(args.ref):
        raise SystemExit("reference build unavailable")
    t = os.path.join(args.ref, "test")
    for name in IP_CASES:
        nl = N.read(os.path.join(t, "nangate45.lef"), os.path.join(t, name + ".def"))
        N.save_npz(nl, os.path.join(HERE, f"netlist_{name}.npz"))
        rounds = []
        for l in open(os.path.join(t, name + ".ok")):
            m = re.match(r"\[InitialPlace\]\s+Iter: (\d+) CG Error: (\S+) HPWL: (\d+)", l)
            if m:
                rounds.append((int(m.group(1)), float(m.group(2)), int(m.group(3))))
        r = np.array(rounds, np.float64)
        its, ovf, hp, fin, _ = parse_log(open(os.path.join(t, name + ".ok")).read())
        np.savez_compressed(os.path.join(HERE, f"ip_{name}.npz"), iter=r[:, 0].astype(np.int32),
                            cg_error=r[:, 1], hpwl=r[:, 2].astype(np.int64),
                            nesterov_iters=its, nesterov_overflow=ovf, nesterov_hpwl=hp,
                            final_overflow=np.array(fin))
        print(name, "ok")
    for name in sorted(set(EVAL_CASES) | set(PLACE_CASES)):
        nl, opts = case_netlist(name, args.ref)
        N.save_npz(nl, os.path.join(HERE, f"netlist_{name}.npz"))
        if name in EVAL_CASES:
            o = {k: v for k, v in opts.items() if k in ("density", "bins", "incremental")}
            r = refnet.run_eval(nl, seed=7, **o)
            np.savez_compressed(os.path.join(HERE, f"eval_{name}.npz"), **r)
        if name in PLACE_CASES:
            rc, log, xy = refnet.run_place(nl, **opts)
            its, ovf, hp, fin, fh = parse_log(log)
            np.savez_compressed(os.path.join(HERE, f"place_{name}.npz"), rc=np.array(rc),
                                iters=its, overflow=ovf, hpwl=hp, final_overflow=np.array(fin),
                                final_hpwl=np.array(fh),
                                lx=xy[:, 0] if xy is not None else np.zeros(0, np.int64),
                                ly=xy[:, 1] if xy is not None else np.zeros(0, np.int64),
                                opts=np.array(repr(opts)))
        print(name, "ok")


if __name__ == "__main__":
    main()
