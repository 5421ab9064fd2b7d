"""The batched form of the Nesterov loop (gpl_batch_nesterov_run): many jobs'
evaluations in one persistent launch per phase, driven by a work table.

Each job's result -- iterations, evaluations, final overflow and HPWL,
instance locations -- must be bit-identical to the same job run alone
through gpl_nesterov_run: the batched kernels run the per-job kernels' block
bodies on the same blocks.
"""

import numpy as np
import pytest

from replace_gb300 import netlist as N

pytestmark = pytest.mark.gpu


def _jobs(n=8, seed=21, cells=(2_000, 12_000)):
    return N.job_batch(n_jobs=n, seed=seed, cells=cells)


def _prepared(nl, td, **kw):
    from replace_gb300 import Placer
    p = Placer(nl, target_density=td, poisson_path=1, **kw)
    p.initial_place()
    p.nesterov_init()
    return p


def _alone(nl, td, weights=None, **kw):
    p = _prepared(nl, td, **kw)
    if weights is not None:
        p.set_net_weights(weights)
    rc, st, _ = p.nesterov_run(0, allow_divergence=True)
    lx, ly = p.inst_locations()
    p.close()
    return rc, st, lx, ly


def _same(st_b, status_b, loc_b, alone):
    rc, st, lx, ly = alone
    assert status_b == rc
    assert st_b.iterations == st.iterations and st_b.evaluations == st.evaluations
    assert st_b.hpwl == st.hpwl and st_b.overflow == st.overflow
    assert st_b.finished == st.finished
    assert np.array_equal(loc_b[0], lx) and np.array_equal(loc_b[1], ly)


def test_batch_matches_each_job_alone(gpu_lib):
    from replace_gb300 import batch_nesterov_run
    jobs = _jobs()
    ps = [_prepared(nl, td) for nl, td in jobs]
    stats, status, launches = batch_nesterov_run(ps)
    assert launches > 0
    locs = [p.inst_locations() for p in ps]
    for p in ps:
        p.close()
    for (nl, td), st, s, loc in zip(jobs, stats, status, locs):
        _same(st, s, loc, _alone(nl, td))
        assert st.finished and st.overflow <= 0.1


def test_batch_mixed_sizes_weights_macros_and_chunks(gpu_lib):
    """Jobs of different bin grids, one with per-net weights, one with
    movable macros (big-cell kernels), run in chunks of 25 iterations with
    the batch continuing where the last chunk stopped; then finished alone."""
    from replace_gb300 import batch_nesterov_run
    jobs = _jobs(n=4, seed=5, cells=(3_000, 30_000))
    mac = N.generate(6_000, 6_300, n_io=100, n_macros=5, seed=9, macro_rows=(10, 16))
    jobs.append((mac, 0.75))
    w = np.random.default_rng(3).lognormal(0.0, 0.5, jobs[1][0].n_nets).astype(np.float32)
    ps = [_prepared(nl, td) for nl, td in jobs]
    ps[1].set_net_weights(w)
    for _ in range(3):
        batch_nesterov_run(ps, max_iters=25)
    out = []
    for p in ps:
        rc, st, _ = p.nesterov_run(0, allow_divergence=True)   # the rest alone
        out.append((rc, st, p.inst_locations()))
        p.close()
    for k, ((nl, td), (rc, st, loc)) in enumerate(zip(jobs, out)):
        _same(st, rc, loc, _alone(nl, td, weights=w if k == 1 else None))


def test_batch_rejects_warp_form_grids(gpu_lib):
    from replace_gb300 import GplError, _abi, batch_nesterov_run
    nl = N.generate(20_000, 21_000, n_io=100, seed=2)
    ok = _prepared(*_jobs(n=1)[0])
    big = _prepared(nl, 0.7, bin_grid_cnt_x=512, bin_grid_cnt_y=512)
    with pytest.raises(GplError) as e:
        batch_nesterov_run([ok, big])
    assert e.value.status == _abi.GPL_ERR_INVALID_ARG
    with pytest.raises(GplError) as e:
        batch_nesterov_run([ok, ok])
    assert e.value.status == _abi.GPL_ERR_INVALID_ARG
    ok.close()
    big.close()


def test_batched_server_matches_alone_and_cancels(gpu_lib):
    """The server's batched mode: jobs join the running batch after their
    initialisation and leave it when their loop ends; every result equals
    the job run alone.  A job cancelled while it runs in the batch ends
    with the cancel code; the server shuts down with jobs still running."""
    from replace_gb300 import PlacementServer
    jobs = _jobs(n=10, seed=33, cells=(2_000, 20_000))
    with PlacementServer(max_active=6, batched=True) as srv:
        tickets = [srv.submit(nl, target_density=td, poisson_path=1) for nl, td in jobs]
        res = {r["ticket"]: r for r in srv.wait_all(600)}
        locs = {t: srv.locations(t, nl.n_insts) for t, (nl, _) in zip(tickets, jobs)}
    spans = sorted((res[t]["admit_s"], res[t]["finish_s"]) for t in tickets)
    assert any(spans[k + 1][0] < spans[k][1] for k in range(len(spans) - 1))
    for t, (nl, td) in zip(tickets, jobs):
        r = res[t]
        rc, st, lx, ly = _alone(nl, td)
        assert r["status"] == rc
        assert r["iterations"] == st.iterations and r["hpwl"] == st.hpwl and r["finished"] == st.finished
        assert np.array_equal(locs[t][0], lx) and np.array_equal(locs[t][1], ly)
    big = N.generate(40_000, 42_000, n_io=100, seed=4)
    with PlacementServer(max_active=3, batched=True) as srv:
        t = srv.submit(big, target_density=0.7, poisson_path=1)
        import time
        time.sleep(1.0)
        srv.cancel(t)
        r = srv.wait_all(600)[0]
        assert r["status"] in (0, 21)              # done before the cancel arrived, or cancelled
        srv.submit(big, target_density=0.7, poisson_path=1)   # left running at shutdown
