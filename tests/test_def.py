"""DEF write-back (lefdef.format_components / write_placement) and the
reference's regression outputs test/<case>.defok.

tests/golden/defok_<case>.npz holds the COMPONENTS section of the
reference's .defok files (make_golden.py): what its write_def produced after
global_placement.
"""

import os
import re

import numpy as np
import pytest

from conftest import GOLDEN, case, golden, params_of

DEFOK_CASES = ["simple01", "simple02", "core01", "ar01", "ar02", "incremental01"]


def _components(g, x=None, y=None):
    from replace_gb300 import lefdef
    x = g["x"] if x is None else x
    y = g["y"] if y is None else y
    st = {0: "UNPLACED", 1: "PLACED", 2: "FIXED", 3: "COVER"}
    return [lefdef.DefComponent(str(n), str(m), st[int(s)], int(a), int(b), str(o))
            for n, m, s, a, b, o in zip(g["name"], g["master"], g["status"], x, y, g["orient"])]


def _reparse(text, tmp_path):
    from replace_gb300 import lefdef
    p = os.path.join(tmp_path, "c.def")
    with open(p, "w") as f:
        f.write("VERSION 5.8 ;\nDESIGN t ;\nUNITS DISTANCE MICRONS 2000 ;\n" + text + "END DESIGN\n")
    return lefdef.read_def(p).components


@pytest.mark.parametrize("name", DEFOK_CASES)
def test_reference_build_reproduces_defok(name):
    """The reference build's final locations (place_<case>.npz, from its own
    NesterovPlace::updateDb) are the .defok's, bit for bit: the golden runs
    are the reference's regression results."""
    g = golden(f"defok_{name}.npz")
    ref = golden(f"place_{name}.npz")
    n = len(g["x"])
    assert np.array_equal(ref["lx"][:n], g["x"]) and np.array_equal(ref["ly"][:n], g["y"])


def test_components_round_trip(tmp_path):
    from replace_gb300 import lefdef
    g = golden("defok_simple01.npz")
    comps = _components(g)
    back = _reparse(lefdef.format_components(comps), str(tmp_path))
    assert [(c.name, c.master, c.status, c.x, c.y, c.orient) for c in back] == \
        [(c.name, c.master, c.status, c.x, c.y, c.orient) for c in comps]


def test_write_placement_matches_write_def():
    """write_placement on the reference's input DEF with the .defok's
    locations reproduces the .defok's COMPONENTS section byte for byte."""
    import refnet
    from replace_gb300 import lefdef
    t = os.path.join(refnet.default_ref_root(), "test")
    if not os.path.isdir(t):
        pytest.skip("reference test designs not present")
    import tempfile
    for name in DEFOK_CASES:
        g = golden(f"defok_{name}.npz")
        with tempfile.TemporaryDirectory() as td:
            out = os.path.join(td, "out.def")
            lefdef.write_placement(os.path.join(t, name + ".def"), out, g["x"], g["y"])
            a = open(out).read()
        b = open(os.path.join(t, name + ".defok")).read()
        sec = lambda s: re.search(r"^COMPONENTS.*?END COMPONENTS", s, re.M | re.S).group(0)
        assert sec(a) == sec(b), name


def _pin_hpwl(nl, lx, ly):
    """Pin HPWL (NesterovBase::getHpwl) of instance lower-left corners."""
    w = (nl.inst_ux - nl.inst_lx).astype(np.int64)
    h = (nl.inst_uy - nl.inst_ly).astype(np.int64)
    on = nl.pin_inst >= 0
    ii = np.where(on, nl.pin_inst, 0)
    px = np.where(on, lx[ii] + w[ii] // 2 + nl.pin_ox, nl.pin_x).astype(np.int64)
    py = np.where(on, ly[ii] + h[ii] // 2 + nl.pin_oy, nl.pin_y).astype(np.int64)
    s = nl.net_start[:-1]
    return int((np.maximum.reduceat(px, s) - np.minimum.reduceat(px, s)).sum() +
               (np.maximum.reduceat(py, s) - np.minimum.reduceat(py, s)).sum())


@pytest.mark.gpu
@pytest.mark.parametrize("name", DEFOK_CASES)
def test_gpu_placement_written_as_def(gpu_lib, tmp_path, name):
    """The GPU job's final locations written as a COMPONENTS section: same
    components, masters, order, orientation and status as the .defok, the
    locations read back unchanged, and the placement's pin HPWL within
    0.5 % of the .defok placement's."""
    from replace_gb300 import Placer, lefdef
    nl, opts = case(name)
    g = golden(f"defok_{name}.npz")
    p = Placer(nl, **params_of(opts))
    p.initial_place()
    p.nesterov_init()
    rc, st, _ = p.nesterov_run(0)
    lx, ly = p.inst_locations()
    p.close()
    n = len(g["x"])
    comps = lefdef.placed_components(_components(g, g["x"] * 0, g["y"] * 0), lx[:n], ly[:n])
    back = _reparse(lefdef.format_components(comps), str(tmp_path))
    assert [c.name for c in back] == [str(v) for v in g["name"]]
    assert [c.master for c in back] == [str(v) for v in g["master"]]
    assert [c.orient for c in back] == [str(v) for v in g["orient"]]
    assert all(c.status == "PLACED" for c in back)
    bx = np.array([c.x for c in back]); by = np.array([c.y for c in back])
    assert np.array_equal(bx, lx[:n]) and np.array_equal(by, ly[:n])
    full_x = lx.astype(np.int64).copy(); full_y = ly.astype(np.int64).copy()
    ref_x = full_x.copy(); ref_y = full_y.copy()
    ref_x[:n] = g["x"]; ref_y[:n] = g["y"]
    ours, theirs = _pin_hpwl(nl, full_x, full_y), _pin_hpwl(nl, ref_x, ref_y)
    assert abs(ours - theirs) <= 0.005 * theirs, (ours, theirs)
