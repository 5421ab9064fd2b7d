"""The batched form of the initial place (gpl_batch_initial_place): the B2B +
BiCGSTAB rounds of many jobs in lockstep, one launch per phase over a work
table of (job, block of the job's own launch, axis).

Each job's result -- rounds, last error, solver iterations, instance
locations -- must be bit-identical to gpl_initial_place on the job alone
with the kernel-per-phase solver: the batched kernels run the per-job
kernels' block bodies on the same blocks.
"""

import numpy as np
import pytest

from conftest import case
from replace_gb300 import netlist as N

pytestmark = pytest.mark.gpu


def _alone(nl, **kw):
    from replace_gb300 import Placer
    p = Placer(nl, ip_solver=1, **kw)
    st = p.initial_place()
    loc = p.inst_locations()
    p.close()
    return st, loc


def _same(st_b, loc_b, alone):
    st, loc = alone
    assert st_b.iterations == st.iterations
    assert st_b.last_error == st.last_error
    assert (st_b.solver_iters_x, st_b.solver_iters_y) == (st.solver_iters_x, st.solver_iters_y)
    assert np.array_equal(loc_b[0], loc[0]) and np.array_equal(loc_b[1], loc[1])


def test_batch_initial_place_matches_each_job_alone(gpu_lib):
    """Jobs of different sizes and stop rounds; one with movable macros, one
    with a lower solver-iteration cap, one incremental (not centred), one
    without initial-place rounds (centring only)."""
    from replace_gb300 import Placer, batch_initial_place
    jobs = [(nl, dict(target_density=td)) for nl, td in N.job_batch(n_jobs=8, seed=21, cells=(2_000, 12_000))]
    mac = N.generate(6_000, 6_300, n_io=100, n_macros=5, seed=9, macro_rows=(10, 16))
    jobs.append((mac, dict(target_density=0.75)))
    jobs.append((jobs[0][0], dict(target_density=0.7, initial_place_max_solver_iter=20)))
    jobs.append((jobs[1][0], dict(target_density=0.7, initial_place_max_iter=3)))
    jobs.append((jobs[2][0], dict(target_density=0.7, initial_place_max_iter=0)))
    nl_simple, _ = case("simple03")
    jobs.append((nl_simple, dict(target_density=0.7, incremental_place_mode=1)))
    ps = [Placer(nl, **kw) for nl, kw in jobs]
    stats, status, launches = batch_initial_place(ps)
    assert launches > 0
    assert all(s == 0 for s in status)
    locs = [p.inst_locations() for p in ps]
    for p in ps:
        p.close()
    for (nl, kw), st, loc in zip(jobs, stats, locs):
        _same(st, loc, _alone(nl, **kw))
    assert stats[-2].iterations == 0
    assert stats[-3].iterations == 3


def test_batch_initial_place_then_batched_loop(gpu_lib):
    """The whole batched flow (batched initial place, init, batched Nesterov
    loop) equals each job run alone through the plain job API."""
    from replace_gb300 import Placer, batch_initial_place, batch_nesterov_run
    jobs = N.job_batch(n_jobs=6, seed=33, cells=(2_000, 20_000))
    ps = [Placer(nl, target_density=td, poisson_path=1) for nl, td in jobs]
    batch_initial_place(ps)
    for p in ps:
        p.nesterov_init()
    stats, status, _ = batch_nesterov_run(ps)
    locs = [p.inst_locations() for p in ps]
    for p in ps:
        p.close()
    for (nl, td), st, s, loc in zip(jobs, stats, status, locs):
        p = Placer(nl, target_density=td, poisson_path=1)
        p.initial_place()
        p.nesterov_init()
        rc, st1, _ = p.nesterov_run(0, allow_divergence=True)
        lx, ly = p.inst_locations()
        p.close()
        assert s == rc and st.iterations == st1.iterations and st.hpwl == st1.hpwl
        assert np.array_equal(loc[0], lx) and np.array_equal(loc[1], ly)


def test_batch_initial_place_rejects(gpu_lib):
    from replace_gb300 import GplError, Placer, _abi, batch_initial_place
    nl, td = N.job_batch(n_jobs=1, seed=2, cells=(2_000, 3_000))[0]
    a = Placer(nl, target_density=td)
    b = Placer(nl, target_density=td)
    with pytest.raises(GplError) as e:
        batch_initial_place([a, a])
    assert e.value.status == _abi.GPL_ERR_INVALID_ARG
    b.initial_place()
    b.nesterov_init()
    with pytest.raises(GplError) as e:
        batch_initial_place([a, b])
    assert e.value.status == _abi.GPL_ERR_BAD_STATE
    a.close()
    b.close()
