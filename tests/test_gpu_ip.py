"""GPU initial place (B2B + BiCGSTAB) against the reference's logged rounds
(test/simple03.ok, simple04.ok) and the oracle; then the whole flow."""

import numpy as np
import pytest

from conftest import case, golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["simple03", "simple04"])
def test_initial_place_rounds_match_reference_log(gpu_lib, name):
    from replace_gb300 import Placer
    nl, _ = case(name)
    ref = golden(f"ip_{name}.npz")
    for k in range(1, len(ref["hpwl"])):
        p = Placer(nl, target_density=0.7, initial_place_max_iter=k)
        st = p.initial_place()
        assert st.iterations == k
        lx, ly = p.inst_locations()
        h = nl.bbox_hpwl(lx, ly)
        assert abs(h - int(ref["hpwl"][k])) <= 5e-4 * int(ref["hpwl"][k]), (k, h)
        assert st.last_error < 1e-5
        p.close()


def test_initial_place_matches_oracle_on_synthetic(gpu_lib, oracle_mod):
    from replace_gb300 import Placer
    nl, _ = case("syn10k_b128")
    p = Placer(nl, target_density=0.7, initial_place_max_iter=20)
    st = p.initial_place()
    o = oracle_mod.Oracle(nl, target_density=0.7, initial_place_max_iter=20)
    ost = o.initial_place()[1]
    lx, ly = p.inst_locations()
    olx, oly = o.inst_locations()
    h, oh = nl.bbox_hpwl(lx, ly), nl.bbox_hpwl(olx, oly)
    assert abs(h - oh) <= 5e-3 * oh
    assert st.iterations == ost.iterations
    # Here BiCGSTAB stops at its 100-iteration cap (as the reference's does)
    # with a relative residual near 1e-3: the near-singular translation mode
    # of the B2B system is left undetermined, so cells may be shifted as a
    # group; the residual reached must be comparable.
    assert ost.last_error > 1e-4
    assert st.last_error < 3 * ost.last_error


@pytest.mark.parametrize("name", ["simple03", "simple04"])
def test_full_flow_with_initial_place(gpu_lib, name):
    """global_placement with default options (initial place, then Nesterov)."""
    from replace_gb300 import global_placement
    nl, _ = case(name)
    ref = golden(f"ip_{name}.npz")
    r = global_placement(nl, density=0.7)
    st = r.np_stats
    assert st.finished and st.overflow <= 0.1
    lg = r.log
    # the initial place agrees with the reference to a few DBU per cell; the
    # first Nesterov step amplifies that (the oracle is 0.2 % off here too)
    assert abs(lg["overflow"][0] - ref["nesterov_overflow"][0]) <= 1e-2
    assert abs(int(lg["hpwl"][0]) - int(ref["nesterov_hpwl"][0])) <= 1e-2 * int(ref["nesterov_hpwl"][0])
    # the last logged reference line vs ours at the same iteration
    it = int(ref["nesterov_iters"][-1])
    if it <= len(lg["hpwl"]):
        assert abs(int(lg["hpwl"][it - 1]) - int(ref["nesterov_hpwl"][-1])) <= 0.005 * int(ref["nesterov_hpwl"][-1])


@pytest.mark.parametrize("name", ["simple03", "syn10k_b128"])
def test_cooperative_solve_agrees_with_phase_kernels(gpu_lib, name):
    """One cooperative launch per BiCGSTAB solve and one kernel per phase run
    the same phases on the same grid, but the phase kernels' SpMV gives each
    block a contiguous range of rows (the grid form strides them), so the
    dot products sum in another order: the same rounds, the HPWL within
    1e-3, comparable residuals."""
    from replace_gb300 import Placer
    nl, _ = case(name)
    out = []
    for mode in (2, 1):
        p = Placer(nl, target_density=0.7, initial_place_max_iter=8, ip_solver=mode)
        st = p.initial_place()
        lx, ly = p.inst_locations()
        out.append((st, nl.bbox_hpwl(lx, ly)))
        p.close()
    (a, ha), (b, hb) = out
    assert a.iterations == b.iterations and a.cooperative_rounds == a.iterations
    assert abs(ha - hb) <= 1e-3 * hb
    assert a.last_error < 3 * b.last_error + 1e-6 and b.last_error < 3 * a.last_error + 1e-6


def test_cluster_solve_agrees_with_grid_solve(gpu_lib):
    """The cluster-per-axis solve sums in another order than the grid forms:
    the same rounds and iteration counts, positions within a few DBU."""
    from replace_gb300 import Placer
    nl, _ = case("syn10k_b128")
    out = []
    for mode in (3, 1):
        p = Placer(nl, target_density=0.7, initial_place_max_iter=20, ip_solver=mode)
        st = p.initial_place()
        lx, ly = p.inst_locations()
        out.append((st, lx, ly, nl.bbox_hpwl(lx, ly)))
        p.close()
    (a, ax, ay, ha), (b, bx, by, hb) = out
    assert a.iterations == b.iterations and a.cooperative_rounds == a.iterations
    assert abs(ha - hb) <= 1e-3 * hb
    assert a.last_error < 3 * b.last_error and b.last_error < 3 * a.last_error


@pytest.mark.parametrize("name", ["simple03", "syn10k_b128"])
def test_device_loop_matches_host_loop(gpu_lib, name):
    """The rounds as one CUDA graph with conditional nodes (device_loop 1)
    take the host loop's decisions on the device: identical rounds, error,
    iteration counts and locations."""
    from replace_gb300 import Placer
    nl, _ = case(name)
    out = []
    for dl in (0, 1):
        p = Placer(nl, target_density=0.7, initial_place_max_iter=20, device_loop=dl)
        st = p.initial_place()
        out.append((st.iterations, st.last_error, st.solver_iters_x, st.solver_iters_y,
                    *p.inst_locations()))
        p.close()
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(np.asarray(a), np.asarray(b))
