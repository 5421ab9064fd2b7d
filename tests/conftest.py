"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on CPU."""

import ast
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, os.path.join(ROOT, "oracle", "refbuild")):
    if p not in sys.path:
        sys.path.insert(0, p)

from replace_gb300 import netlist as N  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def golden(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


def case(name):
    """(netlist, options) of a golden case."""
    nl = N.load_npz(os.path.join(GOLDEN, f"netlist_{name}.npz"))
    opts = {}
    p = os.path.join(GOLDEN, f"place_{name}.npz")
    if os.path.exists(p):
        opts = ast.literal_eval(str(np.load(p)["opts"]))
    elif name.startswith("syn10k_b128"):
        opts = dict(density=0.7, bins=128)
    else:
        opts = dict(density=0.7)
    return nl, opts


def params_of(opts, **extra):
    """gpl_params overrides equivalent to the reference driver options."""
    kw = dict(target_density=opts.get("density", 0.7),
              init_density_penalty=opts.get("idp", 0.00008),
              initial_place_max_iter=0,
              incremental_place_mode=1 if opts.get("incremental") else 0)
    if opts.get("bins"):
        kw["bin_grid_cnt_x"] = kw["bin_grid_cnt_y"] = opts["bins"]
    kw.update(extra)
    return kw


def rel_l2(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def gpu_lib():
    import replace_gb300
    try:
        import torch
        if not torch.cuda.is_available():
            pytest.skip("no CUDA device")
    except ImportError:
        pass
    return replace_gb300.load()
