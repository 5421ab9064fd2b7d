"""The oracle (CPU restatement) pinned against the reference's own code.

The golden fixtures were produced by the reference's unchanged placement
sources (tests/golden/make_golden.py); the oracle must reproduce their integer
results bit for bit and their floating-point results to within the FP64-vs-
FP32 transform difference.
"""

import numpy as np
import pytest

from conftest import case, golden, params_of, rel_l2

EVAL_CASES = ["simple01", "simple02", "ar01", "syn10k_b128", "syn_macro", "syn_fixed"]
PLACE_CASES = ["simple01", "simple02", "core01", "ar01", "ar02", "incremental01", "diverge01",
               "syn10k_b128", "syn_macro", "syn_fixed"]


@pytest.mark.parametrize("n", [2, 4, 8, 16, 64])
@pytest.mark.parametrize("kind", [0, 1, 2])
def test_transform_fft_matches_direct(oracle_mod, n, kind):
    a = np.random.default_rng(n + 10 * kind).standard_normal(n)
    d = oracle_mod.transform(kind, a, direct=True)
    f = oracle_mod.transform(kind, a, direct=False)
    assert np.max(np.abs(d - f)) <= 1e-12 * max(1.0, np.max(np.abs(d)))


def test_poisson_f64_matches_definition(oracle_mod):
    # FFT::doFFT by its definition (Ooura's ddct2d/ddsct2d/ddcst2d semantics)
    nx, ny, bsx, bsy = 8, 4, 3, 5
    rho = np.random.default_rng(3).random((ny, nx))
    i = np.arange(nx)[:, None]; u = np.arange(nx)[None, :]
    j = np.arange(ny)[:, None]; v = np.arange(ny)[None, :]
    cx = np.cos(np.pi * (i + 0.5) * u / nx)          # [i, u]
    cy = np.cos(np.pi * (j + 0.5) * v / ny)          # [j, v]
    A = cy.T @ rho @ cx                               # [v, u] = sum rho[j,i] cy[j,v] cx[i,u]
    A[:, 0] *= 0.5; A[0, :] *= 0.5; A *= 4.0 / nx / ny
    wx = (np.pi * np.arange(nx) / nx).astype(np.float32).astype(np.float64)
    wy = (np.pi * np.arange(ny) / ny * bsy / bsx).astype(np.float32).astype(np.float64)
    den = (wx[None, :].astype(np.float32) ** 2 + wy[:, None].astype(np.float32) ** 2).astype(np.float64)
    den[0, 0] = 1.0
    P = A / den; P[0, 0] = 0.0
    icx = np.cos(np.pi * u.T * (i.T + 0.5) / nx)      # [u, i]
    icy = np.cos(np.pi * v.T * (j.T + 0.5) / ny)      # [v, j]
    isx = np.sin(np.pi * u.T * (i.T + 0.5) / nx)
    isy = np.sin(np.pi * v.T * (j.T + 0.5) / ny)
    phi = icy.T @ P @ icx
    ex = icy.T @ (P * wx[None, :]) @ isx
    ey = isy.T @ (P * wy[:, None]) @ icx
    p2, ex2, ey2 = oracle_mod.poisson_f64(rho, nx, ny, bsx, bsy)
    for a, b in ((p2, phi), (ex2, ex), (ey2, ey)):
        assert np.max(np.abs(a - b)) <= 1e-7 * np.max(np.abs(b))


@pytest.mark.parametrize("name", EVAL_CASES)
def test_eval_matches_reference(oracle_mod, name):
    nl, opts = case(name)
    ref = golden(f"eval_{name}.npz")
    o = oracle_mod.Oracle(nl, **params_of(opts))
    assert o.create_status == 0
    o.initial_place()
    assert o.nesterov_base() == 0
    info = o.info
    assert info.n_gcells == int(ref["scalars"][5])
    assert [info.bin_cnt_x, info.bin_cnt_y, info.bin_size_x, info.bin_size_y] == list(ref["grid"])
    drect, scale, kind = o.gcells()
    gi = ref["ginfo"].reshape(-1, 9)
    assert np.array_equal(drect[:, 2] - drect[:, 0], gi[:, 6] - gi[:, 4])
    assert np.array_equal(drect[:, 3] - drect[:, 1], gi[:, 7] - gi[:, 5])
    assert np.array_equal(scale, ref["gscale"]) and np.array_equal(kind, gi[:, 8])
    wlc = float(ref["fscalars"][1])
    wl, dg, st, rs = o.eval(ref["coords"], wlc)
    b = o.bins()
    # integer work: bit-exact
    for k in ("inst_area", "filler_area", "nonplace_area", "density"):
        assert np.array_equal(b[k], ref[k]), k
    assert int(rs[0]) == int(ref["scalars"][0])            # float-accumulated overflow area
    assert st.hpwl == int(ref["scalars"][1])
    assert np.array_equal(wl.ravel(), ref["wl_grad"])      # same float operations and order
    # transforms: FP64 here vs Ooura FP32 in the reference
    for k in ("phi", "ex", "ey"):
        assert rel_l2(b[k], ref[k]) < 2e-6, k
    assert rel_l2(dg.ravel(), ref["density_grad"]) < 2e-6


@pytest.mark.parametrize("name", PLACE_CASES)
def test_nesterov_loop_matches_reference(oracle_mod, name):
    nl, opts = case(name)
    ref = golden(f"place_{name}.npz")
    o = oracle_mod.Oracle(nl, **params_of(opts))
    o.initial_place()
    rc = o.nesterov_init()
    rc2, st, lg = o.nesterov_run(0, log_capacity=4000)
    if int(ref["rc"]) != 0:
        assert rc2 == int(ref["rc"]) or rc == int(ref["rc"])
        return
    assert rc == 0 and rc2 == 0 and st.finished
    its = ref["iters"]
    # the first logged iteration is computed before transform rounding can
    # change any control decision: same overflow (6 digits) and HPWL
    assert abs(lg["overflow"][0] - ref["overflow"][0]) <= 5e-6
    assert abs(int(lg["hpwl"][0]) - int(ref["hpwl"][0])) <= 2e-5 * int(ref["hpwl"][0])
    # converged like the reference: overflow <= target, HPWL within 0.5 %
    assert st.overflow <= 0.1
    assert abs(st.hpwl - int(ref["final_hpwl"])) <= 0.005 * int(ref["final_hpwl"])
    assert abs(st.iterations - its[-1]) <= max(10, 0.1 * its[-1])


@pytest.mark.parametrize("name", ["simple03", "simple04"])
def test_initial_place_matches_reference_log(oracle_mod, name):
    """The reference logs PlacerBase::hpwl (instance and IO-pin boxes) at the
    start of each initial-place round, i.e. after the previous round's move
    (test/<case>.ok).  After k oracle rounds the HPWL must match round k+1."""
    nl, _ = case(name)
    ref = golden(f"ip_{name}.npz")
    assert nl.bbox_hpwl() == int(ref["hpwl"][0])          # the DEF positions
    for k in range(1, len(ref["hpwl"])):
        o = oracle_mod.Oracle(nl, target_density=0.7, initial_place_max_iter=k)
        rc, st = o.initial_place()
        assert rc == 0 and st.iterations == k
        lx, ly = o.inst_locations()
        h = nl.bbox_hpwl(lx, ly)
        assert abs(h - int(ref["hpwl"][k])) <= 1e-4 * int(ref["hpwl"][k]), (k, h)
        assert st.last_error < 1e-6


def test_net_weights_scale_pin_gradients(oracle_mod):
    """Per-net weights (GNet::customWeight): weight 1 everywhere is the
    unweighted gradient bit for bit, weight 2 doubles it exactly, and two
    complementary 0/1 weightings add up to the unweighted gradient; HPWL and
    the density gradient do not change."""
    nl, opts = case("simple02")
    ref = golden("eval_simple02.npz")
    o = oracle_mod.Oracle(nl, **params_of(opts))
    o.initial_place()
    assert o.nesterov_base() == 0
    wlc = float(ref["fscalars"][1])
    wl0, dg0, st0, _ = o.eval(ref["coords"], wlc)
    n = nl.n_nets
    o.set_net_weights(np.ones(n, np.float32))
    wl1, dg1, st1, _ = o.eval(ref["coords"], wlc)
    assert np.array_equal(wl1, wl0) and np.array_equal(dg1, dg0) and st1.hpwl == st0.hpwl
    o.set_net_weights(np.full(n, 2.0, np.float32))
    wl2, _, _, _ = o.eval(ref["coords"], wlc)
    assert np.array_equal(wl2, 2.0 * wl0)
    sel = np.random.default_rng(4).random(n) < 0.3
    o.set_net_weights(sel.astype(np.float32))
    wa, _, _, _ = o.eval(ref["coords"], wlc)
    o.set_net_weights((~sel).astype(np.float32))
    wb, dgb, stb, _ = o.eval(ref["coords"], wlc)
    assert rel_l2(wa + wb, wl0) < 1e-6
    assert np.array_equal(dgb, dg0) and stb.hpwl == st0.hpwl
    o.set_net_weights(None)
    wl3, _, _, _ = o.eval(ref["coords"], wlc)
    assert np.array_equal(wl3, wl0)


def test_cells_outside_the_core_are_clamped(oracle_mod):
    """Cells that stick out of the core (the reference reads outside its bins
    there) only touch in-core bins in the oracle, as on the GPU: with every
    centre on the core's corner the area lands in the bins around that
    corner, and repeated evaluations agree bit for bit."""
    nl, opts = case("simple02")
    o = oracle_mod.Oracle(nl, **params_of(opts))
    o.initial_place()
    assert o.nesterov_base() == 0
    n = o.info.n_gcells
    c = nl.core
    xy = np.empty(2 * n, np.float32)
    xy[0::2] = c[0]            # every centre on the core's lower-left corner
    xy[1::2] = c[1]
    _, _, st1, _ = o.eval(xy, 0.01)
    b1 = o.bins()
    _, _, st2, _ = o.eval(xy, 0.01)
    b2 = o.bins()
    assert np.array_equal(b1["inst_area"], b2["inst_area"])
    assert np.array_equal(b1["filler_area"], b2["filler_area"])
    # only the bins around the corner receive area
    nx = o.info.bin_cnt_x
    ia = b1["inst_area"].reshape(-1, nx) + b1["filler_area"].reshape(-1, nx)
    assert ia.sum() > 0 and ia[-1, :].sum() == 0 and ia[:, -1].sum() == 0


def test_eval_matches_reference_at_200k_cells(oracle_mod):
    """The oracle against the reference build at the 200k-cell / 40-macro /
    512-bin workload (digests in tests/golden/scale_eval_*.npz): bin areas,
    density and HPWL bit for bit, WA gradients within the float tolerance,
    field and density gradients within the FP64-vs-FP32 transform bar."""
    import os
    import sys
    from conftest import GOLDEN
    sys.path.insert(0, GOLDEN)
    import scale_cases as S
    from replace_gb300 import netlist as N
    name = "200k_cells_40macros_512bins"
    ref = golden(f"scale_eval_{name}.npz")
    nl, td, bins = N.generate_workload(name, seed=S.SCALE_WORKLOADS[name])
    o = oracle_mod.Oracle(nl, target_density=td, bin_grid_cnt_x=bins, bin_grid_cnt_y=bins,
                          initial_place_max_iter=0)
    o.initial_place()
    assert o.nesterov_base() == 0
    n = o.info.n_gcells
    assert n == int(ref["n_gcells"])
    drect, _, _ = o.gcells()
    xy = S.eval_coords(nl.core, drect)
    owl, odg, ost, _ = o.eval(xy, float(ref["wl_coef"]))
    dig = S.eval_digest(dict(o.bins(), wl_grad=owl, density_grad=odg), n, bins * bins)
    for k in ("inst_area_sha", "filler_area_sha", "nonplace_area_sha", "density_sha"):
        assert str(dig[k]) == str(ref[k]), k
    assert ost.hpwl == int(ref["hpwl"])
    assert rel_l2(dig["wl_grad_sample"], ref["wl_grad_sample"]) < 1e-5
    for k in ("phi", "ex", "ey", "density_grad"):
        assert rel_l2(dig[k + "_sample"], ref[k + "_sample"]) < 1e-4, k
