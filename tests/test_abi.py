"""The C ABI library: builds for sm_103a, loads, exports every declared entry
point, validates its inputs on the host (no GPU calls here)."""

import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT
from replace_gb300 import _abi, netlist as N


def declared_functions():
    src = open(os.path.join(ROOT, "include", "gpl.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gpl_[a-z0-9_]+)\s*\(", src)))


def test_library_builds_and_exports_all_symbols():
    from replace_gb300 import build
    path = build.build()
    lib = C.CDLL(path)
    names = declared_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n


def test_params_default_matches_reference_defaults():
    from replace_gb300 import load
    lib = load()
    p = _abi.Params()
    lib.gpl_params_default(C.byref(p))
    q = _abi.default_params()
    for f, _ in _abi.Params._fields_:
        assert getattr(p, f) == pytest.approx(getattr(q, f)), f
    # src/nesterovPlace.cpp:19-29 and src/replace.cpp:13-33
    assert p.max_back_track == 10 and p.initial_prev_coordi_update_coef == 100.0
    assert p.initial_place_max_fanout == 200 and p.reference_hpwl == 446000000.0


def test_invalid_netlists_are_rejected_before_any_device_work():
    from replace_gb300 import load
    lib = load()
    nl = N.generate(200, 210, n_io=5, seed=1)
    bad = nl.copy()
    bad.net_start = bad.net_start.copy()
    bad.net_start[-1] += 1                      # does not end at n_pins
    for net in (bad,):
        h = _abi.DescHolder(net)
        job = C.c_void_p()
        rc = lib.gpl_create(C.byref(h.desc), C.byref(_abi.default_params()), C.byref(job))
        assert rc == _abi.GPL_ERR_INVALID_ARG
        assert b"net_start" in lib.gpl_last_error()
    # utilisation above 100 %: the reference exits with code 1, here a status
    tight = nl.copy()
    tight.core = (0, 0, (nl.core[2] // 3), nl.core[3])
    h = _abi.DescHolder(tight)
    job = C.c_void_p()
    rc = lib.gpl_create(C.byref(h.desc), C.byref(_abi.default_params()), C.byref(job))
    assert rc == _abi.GPL_ERR_UTIL


def test_scatter_shape_parameters_are_checked():
    from replace_gb300 import load
    lib = load()
    nl = N.generate(200, 210, n_io=5, seed=1)
    h = _abi.DescHolder(nl)
    for kw in (dict(scatter_tile=48), dict(scatter_chunk=3000)):
        job = C.c_void_p()
        rc = lib.gpl_create(C.byref(h.desc), C.byref(_abi.default_params(**kw)), C.byref(job))
        assert rc == _abi.GPL_ERR_INVALID_ARG
        assert b"scatter" in lib.gpl_last_error()


def test_instance_pin_lists_must_cover_each_pin_once():
    """inst_pins (the instance pin order) must list every pin of every
    instance exactly once: a repeated or a missing pin is rejected."""
    from replace_gb300 import load
    lib = load()
    nl = N.generate(200, 210, n_io=5, seed=1)
    s, e = int(nl.inst_pin_start[3]), int(nl.inst_pin_start[4])
    assert e - s >= 2
    dup = nl.copy()
    dup.inst_pins = dup.inst_pins.copy()
    dup.inst_pins[s + 1] = dup.inst_pins[s]               # one pin twice, one missing
    short = nl.copy()
    short.inst_pin_start = short.inst_pin_start.copy()
    short.inst_pins = np.delete(short.inst_pins, s)       # one pin missing
    short.inst_pin_start[4:] -= 1
    for net, msg in ((dup, b"twice"), (short, b"every pin")):
        h = _abi.DescHolder(net)
        job = C.c_void_p()
        rc = lib.gpl_create(C.byref(h.desc), C.byref(_abi.default_params()), C.byref(job))
        assert rc == _abi.GPL_ERR_INVALID_ARG
        assert msg in lib.gpl_last_error()


def test_no_device_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from replace_gb300 import load
    lib = load()
    nl = N.generate(200, 210, n_io=5, seed=1)
    h = _abi.DescHolder(nl)
    job = C.c_void_p()
    rc = lib.gpl_create(C.byref(h.desc), C.byref(_abi.default_params()), C.byref(job))
    assert rc == _abi.GPL_ERR_NO_DEVICE
    assert b"no CPU fallback" in lib.gpl_last_error()


def test_server_parameters_and_missing_device():
    from replace_gb300 import load
    lib = load()
    p = _abi.ServerParams()
    lib.gpl_server_params_default(C.byref(p))
    assert p.max_active == 8 and p.chunk_iters == 64 and p.run_initial_place == 1
    h = C.c_void_p()
    bad = _abi.ServerParams(device=0, max_active=0, hbm_budget_bytes=0, chunk_iters=64,
                            run_initial_place=1)
    assert lib.gpl_server_create(C.byref(bad), C.byref(h)) == _abi.GPL_ERR_INVALID_ARG
    import torch
    if not torch.cuda.is_available():
        assert lib.gpl_server_create(C.byref(p), C.byref(h)) == _abi.GPL_ERR_NO_DEVICE
        assert b"no CPU fallback" in lib.gpl_last_error()


def test_job_batch_and_stream_generators():
    jobs = N.job_batch(n_jobs=4, seed=3, cells=(2_000, 4_000))
    assert len(jobs) == 4
    for nl, td in jobs:
        assert 2_000 <= int((nl.inst_kind == 0).sum()) <= 4_000 and 0.60 <= td <= 0.85
    spec = N.job_stream_spec(n_jobs=50, rate=2.0, seed=5)
    t = np.array([s["arrival_s"] for s in spec])
    assert np.all(np.diff(t) > 0)
    assert all(5_000 <= s["n_cells"] <= 500_000 for s in spec)
    assert 0 < sum(s["n_macros"] > 0 for s in spec) < 50


def test_large_netlist_checks_run_in_parallel_ranges():
    """Netlists of more than 65,536 pins are copied and checked by several
    host threads: a bad pin, a pin listed twice and a missing pin are still
    found wherever they are."""
    from replace_gb300 import load
    lib = load()
    nl = N.generate(30_000, 31_500, n_io=100, seed=2)
    assert nl.n_pins > (1 << 16)
    bad = nl.copy()
    bad.pin_inst = bad.pin_inst.copy()
    bad.pin_inst[nl.n_pins - 7] = nl.n_insts + 5          # out of range, near the end
    q = int(nl.inst_pin_start[20_000])
    assert int(nl.inst_pin_start[20_001]) - q >= 2
    dup = nl.copy()
    dup.inst_pins = dup.inst_pins.copy()
    dup.inst_pins[q + 1] = dup.inst_pins[q]
    for net, msg in ((bad, b"pin_inst out of range"), (dup, b"twice")):
        h = _abi.DescHolder(net)
        job = C.c_void_p()
        rc = lib.gpl_create(C.byref(h.desc), C.byref(_abi.default_params()), C.byref(job))
        assert rc == _abi.GPL_ERR_INVALID_ARG
        assert msg in lib.gpl_last_error()
    # the valid netlist passes the checks (and stops at the missing device here)
    import torch
    if not torch.cuda.is_available():
        h = _abi.DescHolder(nl)
        job = C.c_void_p()
        assert lib.gpl_create(C.byref(h.desc), C.byref(_abi.default_params()), C.byref(job)) == \
            _abi.GPL_ERR_NO_DEVICE


def test_batched_calls_validate_their_job_lists_on_the_host():
    """The batched entry points reject an empty or null job list before any
    device work (gpl_batch_initial_place, gpl_batch_nesterov_run)."""
    from replace_gb300 import load
    lib = load()
    launches = C.c_int64(-1)
    assert lib.gpl_batch_initial_place(None, 0, None, None, C.byref(launches)) == _abi.GPL_ERR_INVALID_ARG
    assert launches.value == 0
    assert b"no jobs" in lib.gpl_last_error()
    null_jobs = (C.c_void_p * 2)(None, None)
    assert lib.gpl_batch_initial_place(null_jobs, 2, None, None, None) == _abi.GPL_ERR_INVALID_ARG
    assert b"null job" in lib.gpl_last_error()
    assert lib.gpl_batch_nesterov_run(None, 0, 0, None, None, None) == _abi.GPL_ERR_INVALID_ARG
    assert lib.gpl_batch_nesterov_run(null_jobs, 2, 0, None, None, None) == _abi.GPL_ERR_INVALID_ARG
