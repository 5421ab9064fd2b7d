"""Runs the reference build (oracle/_ref/ref_driver) on a Netlist.

TEST INFRASTRUCTURE ONLY: used by tests/ and tests/golden/make_golden.py to
pin the oracle restatement against the reference's own code.  The reference
build exists only where the reference sources were available at build time.
"""

from __future__ import annotations

import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(os.path.dirname(HERE), "_ref")
DRIVER = os.path.join(REF_DIR, "ref_driver")


def default_ref_root() -> str:
    """Where the reference tree is read from: $REPLACE_REFERENCE_ROOT, else
    the build container's copy."""
    return os.environ.get("REPLACE_REFERENCE_ROOT", "/root/reference")


def available() -> bool:
    return os.path.exists(DRIVER)


def build(ref_root: str | None = None) -> bool:
    """Compile the reference build if the reference sources are present."""
    ref_root = ref_root or default_ref_root()
    if not os.path.isdir(os.path.join(ref_root, "src")):
        return available()
    r = subprocess.run(["make", "-s", "-C", HERE, f"REF={ref_root}", "-j8"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference build failed:\n" + r.stdout + r.stderr)
    return available()


def write_refnet(nl, path: str) -> None:
    """Write a Netlist in the driver's text format (real instances only: the
    reference creates the fragmented-row dummies itself from the rows)."""
    from replace_gb300.netlist import INST_DUMMY, INST_PLACE
    real = np.nonzero(nl.inst_kind != INST_DUMMY)[0]
    assert np.all(real == np.arange(len(real))), "dummies must follow real instances"
    key = np.zeros(nl.n_pins, np.int64)
    for i in range(nl.n_insts):
        s, e = nl.inst_pin_start[i], nl.inst_pin_start[i + 1]
        key[nl.inst_pins[s:e]] = np.arange(e - s)
    rows = nl.rows
    if not rows:
        c = nl.core
        sh = nl.site[1]
        rows = [(c[0], y, c[2], y + sh) for y in range(c[1], c[3], sh)]
    out = [f"REFNET 1", f"DBU {nl.dbu}", f"SITE {nl.site[0]} {nl.site[1]}",
           "DIE {} {} {} {}".format(*nl.die), f"ROWS {len(rows)}"]
    out += ["{} {} {} {}".format(*r) for r in rows]
    out.append(f"INSTS {len(real)}")
    w = nl.inst_ux - nl.inst_lx
    h = nl.inst_uy - nl.inst_ly
    for i in real:
        st = 0 if nl.inst_kind[i] == INST_PLACE else 1
        out.append(f"{nl.inst_lx[i]} {nl.inst_ly[i]} {w[i]} {h[i]} {w[i]} {h[i]} {st}")
    out.append(f"NETS {nl.n_nets}")
    for n in range(nl.n_nets):
        s, e = nl.net_start[n], nl.net_start[n + 1]
        pins = np.arange(s, e)
        it = pins[nl.pin_inst[pins] >= 0]
        bt = pins[nl.pin_inst[pins] < 0]
        out.append(f"0 {len(it)} {len(bt)}")
        for p in it:
            i = nl.pin_inst[p]
            c = w[i] // 2 + nl.pin_ox[p]
            d = h[i] // 2 + nl.pin_oy[p]
            out.append(f"{i} {key[p]} 1 {c} {d} {c} {d}")
        for p in bt:
            out.append(f"1 {nl.pin_x[p]} {nl.pin_y[p]} {nl.pin_x[p]} {nl.pin_y[p]}")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")


def _opt_args(opts: dict):
    args = []
    for k, v in opts.items():
        if v is True:
            args.append("--" + k)
        elif v is False or v is None:
            continue
        else:
            args += ["--" + k, str(v)]
    return args


def run_place(nl, **opts):
    """Run the reference Nesterov flow; returns (log text, final inst lx/ly)."""
    with tempfile.TemporaryDirectory() as td:
        net = os.path.join(td, "net.txt")
        pos = os.path.join(td, "pos.txt")
        write_refnet(nl, net)
        r = subprocess.run([DRIVER, "place", net, "--out-pos", pos] + _opt_args(opts),
                           capture_output=True, text=True)
        xy = None
        if os.path.exists(pos):
            xy = np.loadtxt(pos, dtype=np.int64, ndmin=2)
        return r.returncode, r.stdout, xy


def read_bin(path: str) -> dict:
    out = {}
    with open(path, "rb") as f:
        data = f.read()
    pos = 0
    while pos < len(data):
        nl = data.index(b"\n", pos)
        name, dt, n = data[pos:nl].decode().split()
        n = int(n)
        dtype = np.dtype(dt)
        start = nl + 1
        arr = np.frombuffer(data[start:start + n * dtype.itemsize], dtype=dtype).copy()
        out[name] = arr
        pos = start + n * dtype.itemsize + 1
    return out


def run_eval(nl, coords=None, **opts) -> dict:
    """One reference NesterovBase evaluation; see ref_driver.cpp (eval).
    `coords` (float32, x y per gcell) replaces the driver's seeded centres."""
    with tempfile.TemporaryDirectory() as td:
        net = os.path.join(td, "net.txt")
        out = os.path.join(td, "out.bin")
        write_refnet(nl, net)
        extra = []
        if coords is not None:
            cpath = os.path.join(td, "coords.bin")
            np.ascontiguousarray(coords, np.float32).tofile(cpath)
            extra = ["--coords", cpath]
        r = subprocess.run([DRIVER, "eval", net, out] + _opt_args(opts) + extra,
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(r.stdout + r.stderr)
        return read_bin(out)
