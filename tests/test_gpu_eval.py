"""GPU parity of one evaluation (scatter, Poisson, WA, gradients) through the C ABI.

Bars: integer work bit-exact (bin areas, bin density, HPWL); floating point
within 1e-4 relative L2 (measured values are ~1e-6); the overflow area, which
the GPU sums in FP64, within 1e-6 of the oracle's FP64 sum.
"""

import ctypes as C

import numpy as np
import pytest

from conftest import case, golden, params_of, rel_l2

pytestmark = pytest.mark.gpu

EVAL_CASES = ["simple01", "simple02", "ar01", "syn10k_b128", "syn_macro", "syn_fixed"]
TOL = 1e-4


@pytest.mark.parametrize("name", EVAL_CASES)
def test_eval_parity(gpu_lib, oracle_mod, name):
    from replace_gb300 import Placer
    nl, opts = case(name)
    ref = golden(f"eval_{name}.npz")
    p = Placer(nl, **params_of(opts))
    p.initial_place()
    o = oracle_mod.Oracle(nl, **params_of(opts))
    o.initial_place()
    o.nesterov_base()
    wlc = float(ref["fscalars"][1])
    wl, dg, st = p.eval(ref["coords"], wlc)
    owl, odg, ost, _ = o.eval(ref["coords"], wlc)
    info = o.info
    b = p.bins(info.bin_cnt_x, info.bin_cnt_y)
    for k in ("inst_area", "filler_area", "nonplace_area", "density"):
        assert np.array_equal(b[k], ref[k]), k
    assert st.hpwl == int(ref["scalars"][1]) == ost.hpwl
    assert abs(st.overflow_area_f64 - ost.overflow_area_f64) <= 1e-6 * max(ost.overflow_area_f64, 1.0)
    assert rel_l2(wl, ref["wl_grad"]) < TOL
    assert rel_l2(dg, odg) < TOL and rel_l2(dg, ref["density_grad"]) < TOL
    for k in ("phi", "ex", "ey"):
        assert rel_l2(b[k], ref[k]) < TOL, k
    assert abs(st.wire_length_grad_sum - ost.wire_length_grad_sum) <= TOL * ost.wire_length_grad_sum
    assert abs(st.density_grad_sum - ost.density_grad_sum) <= TOL * ost.density_grad_sum
    assert abs(st.sum_phi - ost.sum_phi) <= TOL * abs(ost.sum_phi)
    p.close()


def test_eval_deterministic_and_order_independent(gpu_lib):
    """Bin areas are int64 sums: identical across repeated runs, and the
    floating-point outputs are identical run to run (fixed reduction order)."""
    from replace_gb300 import Placer
    nl, opts = case("syn10k_b128")
    ref = golden("eval_syn10k_b128.npz")
    p = Placer(nl, **params_of(opts))
    p.initial_place()
    outs = []
    for _ in range(3):
        wl, dg, st = p.eval(ref["coords"], float(ref["fscalars"][1]))
        b = p.bins(128, 128)
        outs.append((wl.copy(), dg.copy(), b["inst_area"].copy(), b["ex"].copy(), st.overflow_area_f64))
    for o in outs[1:]:
        for x, y in zip(o[:4], outs[0][:4]):
            assert np.array_equal(x, y)
        assert o[4] == outs[0][4]


def test_eval_all_cells_on_one_bin(gpu_lib, oracle_mod):
    """Every cell at the core centre (the start of a run without initial
    place): maximal atomic contention, still bit-exact bin areas."""
    from replace_gb300 import Placer
    nl, opts = case("syn10k_b128")
    p = Placer(nl, **params_of(opts))
    p.initial_place()
    o = oracle_mod.Oracle(nl, **params_of(opts))
    o.initial_place()
    o.nesterov_base()
    n = o.info.n_gcells
    c = nl.core
    xy = np.tile(np.array([(c[0] + c[2]) / 2, (c[1] + c[3]) / 2], np.float32), (n, 1))
    wl, dg, st = p.eval(xy, 1e-4)
    owl, odg, ost, _ = o.eval(xy, 1e-4)
    b = p.bins(128, 128)
    ob = o.bins()
    assert np.array_equal(b["inst_area"], ob["inst_area"])
    assert np.array_equal(b["filler_area"], ob["filler_area"])
    assert st.hpwl == ost.hpwl


@pytest.mark.parametrize("nx,ny", [(2, 2), (4, 8), (16, 16), (64, 32), (128, 128), (256, 512), (512, 512),
                                   (1024, 1024)])
def test_poisson_solve_matches_fp64(gpu_lib, oracle_mod, nx, ny):
    """gpl_poisson_solve (FFT::doFFT semantics) vs the FP64 oracle."""
    import torch
    from replace_gb300 import poisson_solve
    rng = np.random.default_rng(nx * 7 + ny)
    rho = rng.random((ny, nx)).astype(np.float32) * 1.5
    bsx, bsy = 3901, 3877
    d = torch.from_numpy(rho).cuda()
    phi = torch.zeros_like(d); fx = torch.zeros_like(d); fy = torch.zeros_like(d)
    poisson_solve(d.data_ptr(), phi.data_ptr(), fx.data_ptr(), fy.data_ptr(), nx, ny, bsx, bsy,
                  torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    p64, x64, y64 = oracle_mod.poisson_f64(rho.astype(np.float64), nx, ny, bsx, bsy)
    assert rel_l2(phi.cpu().numpy(), p64) < 1e-5
    assert rel_l2(fx.cpu().numpy(), x64) < 1e-5
    assert rel_l2(fy.cpu().numpy(), y64) < 1e-5


@pytest.mark.parametrize("bins", [512, 1024])
def test_eval_parity_warp_form_grids(gpu_lib, oracle_mod, bins):
    """512 x 512 and 1024 x 1024 bin grids (the warp-per-pair FFT form of the
    Poisson passes, with the density from its own grid-wide kernel): bin
    areas and density bit-exact, overflow, potential, field and gradients
    against the FP64 oracle."""
    from replace_gb300 import Placer, netlist as N
    nl = N.generate(30_000, 31_500, n_io=300, seed=5)
    kw = dict(target_density=0.7, bin_grid_cnt_x=bins, bin_grid_cnt_y=bins, initial_place_max_iter=0)
    p = Placer(nl, **kw)
    p.initial_place()
    o = oracle_mod.Oracle(nl, **kw)
    o.initial_place()
    o.nesterov_base()
    n = o.info.n_gcells
    rng = np.random.default_rng(3)
    c = nl.core
    xy = np.empty(2 * n, np.float32)
    xy[0::2] = rng.uniform(c[0], c[2], n)
    xy[1::2] = rng.uniform(c[1], c[3], n)
    wl, dg, st = p.eval(xy, 0.01)
    owl, odg, ost, _ = o.eval(xy, 0.01)
    b = p.bins(bins, bins)
    ob = o.bins()
    for k in ("inst_area", "filler_area", "nonplace_area", "density"):
        assert np.array_equal(b[k], ob[k]), k
    assert st.hpwl == ost.hpwl
    assert abs(st.overflow_area_f64 - ost.overflow_area_f64) <= 1e-6 * max(ost.overflow_area_f64, 1.0)
    for k in ("phi", "ex", "ey"):
        assert rel_l2(b[k], ob[k]) < 1e-5, (k, rel_l2(b[k], ob[k]))
    assert rel_l2(dg, odg) < TOL and rel_l2(wl, owl) < TOL
    p.close()


def test_eval_parity_tensor_core_poisson(gpu_lib, oracle_mod):
    """The Poisson solve as tensor-core GEMMs (each value split into three
    bf16 terms, six products, smallest first; the density's mean taken out
    of the transformed operand): bin areas, density and HPWL are untouched
    and bit-exact; potential, field and density gradient within 1e-5 of the
    FP64 oracle (measured about 7e-7) and within 2e-4 of the reference's own
    FP32 transforms."""
    from replace_gb300 import Placer
    nl, opts = case("syn10k_b128")
    ref = golden("eval_syn10k_b128.npz")
    p = Placer(nl, **params_of(opts), poisson_path=2)
    p.initial_place()
    o = oracle_mod.Oracle(nl, **params_of(opts))
    o.initial_place()
    o.nesterov_base()
    wlc = float(ref["fscalars"][1])
    wl, dg, st = p.eval(ref["coords"], wlc)
    owl, odg, ost, _ = o.eval(ref["coords"], wlc)
    info = o.info
    b = p.bins(info.bin_cnt_x, info.bin_cnt_y)
    for k in ("inst_area", "filler_area", "nonplace_area", "density"):
        assert np.array_equal(b[k], ref[k]), k
    assert st.hpwl == ost.hpwl
    assert rel_l2(wl, ref["wl_grad"]) < TOL
    ob = o.bins()
    for k in ("phi", "ex", "ey"):
        assert rel_l2(b[k], ref[k]) < 2e-4, (k, rel_l2(b[k], ref[k]))
        assert rel_l2(b[k], ob[k]) < 1e-5, (k, rel_l2(b[k], ob[k]))
    assert rel_l2(dg, odg) < 1e-5
    p.close()


def test_eval_parity_tensor_core_poisson_1024(gpu_lib, oracle_mod):
    """The tensor-core Poisson form on a 1024 x 1024 grid: potential, field
    and density gradient within 2e-5 of the FP64 oracle (measured about
    5e-6; the tensor cores' fp32 accumulation over K = 6144 bounds it), the
    density gradient well inside the 1e-4 bar."""
    from replace_gb300 import Placer, netlist as N
    nl = N.generate(30_000, 31_500, n_io=300, seed=5)
    kw = dict(target_density=0.7, bin_grid_cnt_x=1024, bin_grid_cnt_y=1024, initial_place_max_iter=0)
    p = Placer(nl, **kw, poisson_path=2)
    p.initial_place()
    o = oracle_mod.Oracle(nl, **kw)
    o.initial_place()
    o.nesterov_base()
    n = o.info.n_gcells
    rng = np.random.default_rng(3)
    c = nl.core
    xy = np.empty(2 * n, np.float32)
    xy[0::2] = rng.uniform(c[0], c[2], n)
    xy[1::2] = rng.uniform(c[1], c[3], n)
    wl, dg, st = p.eval(xy, 0.01)
    owl, odg, ost, _ = o.eval(xy, 0.01)
    b = p.bins(1024, 1024)
    ob = o.bins()
    for k in ("inst_area", "filler_area", "density"):
        assert np.array_equal(b[k], ob[k]), k
    for k in ("phi", "ex", "ey"):
        assert rel_l2(b[k], ob[k]) < 2e-5, (k, rel_l2(b[k], ob[k]))
    assert rel_l2(dg, odg) < 2e-5, rel_l2(dg, odg)
    p.close()


@pytest.mark.parametrize("name", ["syn10k_b128", "syn_macro"])
def test_eval_net_weights(gpu_lib, oracle_mod, name):
    """Per-net weights (GNet::customWeight): the weighted WA gradient matches
    the oracle's; weight 1 is the unweighted result and weight 2 doubles it,
    both bit for bit; HPWL and the density gradient do not change; None
    switches the weights off again."""
    from replace_gb300 import Placer
    nl, opts = case(name)
    ref = golden(f"eval_{name}.npz")
    p = Placer(nl, **params_of(opts))
    p.initial_place()
    o = oracle_mod.Oracle(nl, **params_of(opts))
    o.initial_place()
    o.nesterov_base()
    wlc = float(ref["fscalars"][1])
    wl0, dg0, st0 = p.eval(ref["coords"], wlc)
    n = nl.n_nets
    w = np.random.default_rng(7).lognormal(0.0, 0.6, n).astype(np.float32)
    w[::11] = 0.0
    p.set_net_weights(w)
    o.set_net_weights(w)
    wl, dg, st = p.eval(ref["coords"], wlc)
    owl, _, _, _ = o.eval(ref["coords"], wlc)
    assert rel_l2(wl, owl) < TOL
    assert st.hpwl == st0.hpwl and np.array_equal(dg, dg0)
    p.set_net_weights(np.ones(n, np.float32))
    wl1, _, _ = p.eval(ref["coords"], wlc)
    assert np.array_equal(wl1, wl0)
    p.set_net_weights(np.full(n, 2.0, np.float32))
    wl2, _, _ = p.eval(ref["coords"], wlc)
    assert np.array_equal(wl2, 2.0 * wl0)
    p.set_net_weights(None)
    wl3, _, _ = p.eval(ref["coords"], wlc)
    assert np.array_equal(wl3, wl0)
    p.close()


def test_net_weights_are_checked(gpu_lib):
    from replace_gb300 import GplError, Placer, _abi
    nl, opts = case("simple01")
    p = Placer(nl, **params_of(opts))
    n = nl.n_nets
    for bad in (np.ones(n - 1, np.float32), np.full(n, -1.0, np.float32),
                np.full(n, np.nan, np.float32), np.full(n, np.inf, np.float32)):
        with pytest.raises(GplError) as e:
            p.set_net_weights(bad)
        assert e.value.status == _abi.GPL_ERR_INVALID_ARG
    p.close()
