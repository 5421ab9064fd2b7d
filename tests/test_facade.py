"""The compiled replace::Replace facade (include/replace/Replace.h,
replace_gb300/facade/) driven through OpenDB's interface.

The driver (tests/facade/facade_driver.cpp) reads a netlist into the
in-memory OpenDB stand-in and runs the facade's PlacerBase, Replace, or
InitialPlace / NesterovBase / NesterovPlace directly.

* CPU: the facade's PlacerBase, written in C++ against the OpenDB API,
  flattens each design into the same arrays as the Python flattening that
  reproduces the reference's PlacerBase (core, fragmented-row dummies,
  instance kinds, pin offsets, net and instance pin order, areas).
* GPU: placing through Replace, and through the three classes built from
  their Vars, writes the same locations into the database as the plain C
  ABI job (gpl_create ... gpl_get_inst_locations) with the same options,
  bit for bit; divergence exits with the reference's code after the
  write-back.
"""

import os
import subprocess
import sys
import tempfile

import numpy as np
import pytest

from conftest import ROOT, case, golden, params_of

sys.path.insert(0, os.path.join(ROOT, "tests", "facade"))

FLATTEN_CASES = ["simple01", "simple02", "core01", "ar01", "incremental01", "syn_macro", "syn_fixed"]


@pytest.fixture(scope="module")
def driver():
    import build_driver
    return build_driver.build()


def _run(driver, mode, nl, out, *opts):
    import refnet
    with tempfile.TemporaryDirectory() as td:
        net = os.path.join(td, "net.txt")
        refnet.write_refnet(nl, net)
        return subprocess.run([driver, mode, net, out] + [str(o) for o in opts],
                              capture_output=True, text=True, timeout=600)


@pytest.mark.parametrize("name", FLATTEN_CASES)
def test_placer_base_flattening(driver, name):
    import refnet
    from replace_gb300 import netlist as N
    nl, _ = case(name)
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "flat.bin")
        r = _run(driver, "flatten", nl, out)
        assert r.returncode == 0, r.stdout + r.stderr
        f = refnet.read_bin(out)
    assert tuple(f["geometry"][:4]) == tuple(nl.core)
    assert tuple(f["geometry"][4:]) == tuple(nl.site)
    for k in ("inst_lx", "inst_ly", "inst_ux", "inst_uy", "inst_kind", "pin_inst", "pin_ox",
              "pin_oy", "pin_x", "pin_y", "net_start", "inst_pin_start", "inst_pins"):
        assert np.array_equal(f[k], getattr(nl, k)), k
    # PlacerBase's area bookkeeping (place, non-place, standard-cell, macro)
    w = (nl.inst_ux - nl.inst_lx).astype(np.int64)
    h = (nl.inst_uy - nl.inst_ly).astype(np.int64)
    place = nl.inst_kind == N.INST_PLACE
    assert int(f["areas"][0]) == int((w * h)[place].sum())
    macro = place & (h > 6 * nl.site[1])
    assert int(f["areas"][3]) == int((w * h)[macro].sum())
    assert "[INFO] NumPlaceInstances = %d" % place.sum() in r.stdout


def _opts(opts):
    out = ["--density", opts.get("density", 0.7), "--idp", opts.get("idp", 0.00008)]
    if opts.get("bins"):
        out += ["--bins", opts["bins"]]
    if opts.get("incremental"):
        out += ["--incremental"]
    return out


def _locations(path):
    a = np.loadtxt(path, dtype=np.int64, ndmin=2)
    return a[:, 0], a[:, 1], a[:, 2]


@pytest.mark.gpu
@pytest.mark.parametrize("name,ip_iter", [("simple01", 0), ("syn_macro", 0), ("simple03", 5),
                                          ("syn10k_b128", 20)])
def test_replace_facade_matches_c_abi_job(gpu_lib, driver, name, ip_iter):
    from replace_gb300 import Placer
    nl, opts = case(name)
    kw = params_of(opts, initial_place_max_iter=ip_iter)
    p = Placer(nl, **kw)
    p.initial_place()
    p.nesterov_init()
    rc, st, _ = p.nesterov_run(0)
    lx, ly = p.inst_locations()
    p.close()
    place = nl.inst_kind == 0
    real = nl.inst_kind != 2
    with tempfile.TemporaryDirectory() as td:
        for mode in ("place", "components"):
            out = os.path.join(td, mode + ".txt")
            r = _run(driver, mode, nl, out, *_opts(opts), "--ip-iter", ip_iter)
            assert r.returncode == 0, r.stdout[-3000:] + r.stderr
            fx, fy, status = _locations(out)
            assert len(fx) == int(real.sum())
            assert np.array_equal(fx[place[real]], lx[place]), mode
            assert np.array_equal(fy[place[real]], ly[place]), mode
            assert np.all(status[place[real]] == 3), mode          # dbPlacementStatus::PLACED
    if name in ("simple01",):
        ref = golden(f"place_{name}.npz")
        assert abs(st.hpwl - int(ref["final_hpwl"])) <= 0.005 * int(ref["final_hpwl"])


@pytest.mark.gpu
def test_replace_facade_divergence_exits_with_reference_code(gpu_lib, driver):
    nl, opts = case("diverge01")
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "pos.txt")
        r = _run(driver, "place", nl, out, *_opts(opts), "--ip-iter", 0)
        assert r.returncode == 3, r.stdout[-2000:]
        assert "(REPL-3)" in r.stdout
