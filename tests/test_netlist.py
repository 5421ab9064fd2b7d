"""Netlist construction: LEF/DEF reader, PlacerBase bookkeeping, generator."""

import os

import numpy as np
import pytest

import refnet
from conftest import GOLDEN, case
from replace_gb300 import netlist as N

REF_TEST = os.path.join(refnet.default_ref_root(), "test")


def test_regression_designs_counts():
    # numbers the reference prints for these designs (NumInstances, NumNets, NumPins)
    for name in ("simple01", "core01", "ar01", "ar02", "incremental01", "diverge01"):
        nl, _ = case(name)
        assert (nl.inst_kind == N.INST_PLACE).sum() == 294
        assert nl.n_nets == 364 and nl.n_pins == 1122
    nl, _ = case("simple02")
    assert (nl.inst_kind == N.INST_DUMMY).sum() == 1       # one fragmented row


def test_core_from_rows():
    assert case("simple01")[0].core == (0, 0, 61940, 61600)
    assert case("core01")[0].core == (2280, 2240, 70300, 69440)


@pytest.mark.skipif(not os.path.isdir(REF_TEST), reason="reference test designs not present")
def test_lefdef_reader_matches_fixture():
    for name in ("simple01", "simple02", "incremental01"):
        a = N.read(os.path.join(REF_TEST, "nangate45.lef"), os.path.join(REF_TEST, name + ".def"))
        b, _ = case(name)
        for k in ("inst_lx", "inst_ly", "inst_ux", "inst_uy", "inst_kind", "pin_inst", "pin_ox",
                  "pin_oy", "pin_x", "pin_y", "net_start", "inst_pin_start", "inst_pins"):
            assert np.array_equal(getattr(a, k), getattr(b, k)), (name, k)


def test_generator_deterministic_and_shaped():
    a = N.generate(2000, 2100, n_io=50, seed=5)
    b = N.generate(2000, 2100, n_io=50, seed=5)
    assert np.array_equal(a.pin_inst, b.pin_inst) and np.array_equal(a.pin_ox, b.pin_ox)
    deg = np.diff(a.net_start)
    assert deg.min() >= 2 and a.n_nets == 2100
    assert (a.pin_inst < 0).sum() == 50
    w = a.inst_ux - a.inst_lx
    assert np.all(w % 380 == 0) and w.min() >= 760 and w.max() <= 6080
    util = float(np.sum((a.inst_ux - a.inst_lx).astype(np.int64) * (a.inst_uy - a.inst_ly))) / (
        (a.core[2] - a.core[0]) * (a.core[3] - a.core[1]))
    assert 0.55 < util <= 0.60
    # pins of an instance are consistent with pin_inst
    for i in range(0, a.n_insts, 97):
        s, e = a.inst_pin_start[i], a.inst_pin_start[i + 1]
        assert np.all(a.pin_inst[a.inst_pins[s:e]] == i)


def test_npz_roundtrip(tmp_path):
    nl = N.generate(500, 520, n_io=10, n_macros=2, seed=2, macro_rows=(8, 12))
    p = tmp_path / "n.npz"
    N.save_npz(nl, str(p))
    m = N.load_npz(str(p))
    assert m.core == nl.core and m.rows == nl.rows
    assert np.array_equal(m.pin_x, nl.pin_x)
