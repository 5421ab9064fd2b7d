"""Placement server (continuous batching on one GPU): each job's result is the
same alone and in the mix; admission respects the HBM budget; cancel and
rejection paths.

Jobs compared alone and in the mix pin the Poisson form (poisson_path 1):
the automatic choice times the FFT and tensor-core forms per job, and the
winner can differ with the load on the GPU."""

import numpy as np
import pytest

from replace_gb300 import _abi, netlist as N

pytestmark = pytest.mark.gpu


def small_batch(n=6, seed=11):
    return N.job_batch(n_jobs=n, seed=seed, cells=(2_000, 8_000))


def alone(nl, td):
    from replace_gb300 import Placer
    p = Placer(nl, target_density=td, poisson_path=1)
    p.initial_place()
    p.nesterov_init()
    rc, st, _ = p.nesterov_run(0)
    lx, ly = p.inst_locations()
    p.close()
    return rc, st, lx, ly


def test_results_are_the_same_alone_and_in_the_mix(gpu_lib):
    from replace_gb300 import PlacementServer
    jobs = small_batch()
    with PlacementServer(max_active=4) as srv:
        tickets = [srv.submit(nl, target_density=td, poisson_path=1) for nl, td in jobs]
        res = {r["ticket"]: r for r in srv.wait_all(600)}
        locs = {t: srv.locations(t, nl.n_insts) for t, (nl, _) in zip(tickets, jobs)}
    # several jobs were resident at once
    spans = sorted((res[t]["admit_s"], res[t]["finish_s"]) for t in tickets)
    assert any(spans[k + 1][0] < spans[k][1] for k in range(len(spans) - 1))
    for t, (nl, td) in zip(tickets, jobs):
        r = res[t]
        rc, st, lx, ly = alone(nl, td)
        assert r["status"] == rc == 0
        assert r["finished"] and r["overflow"] <= 0.1
        assert r["iterations"] == st.iterations
        assert r["hpwl"] == st.hpwl
        assert r["overflow"] == pytest.approx(st.overflow, abs=0.0)
        assert np.array_equal(locs[t][0], lx) and np.array_equal(locs[t][1], ly)


def test_admission_keeps_resident_footprints_within_budget(gpu_lib):
    from replace_gb300 import PlacementServer
    from replace_gb300 import GplError
    jobs = small_batch(5, seed=12)
    # a job larger than the whole budget is refused at submission
    with PlacementServer(max_active=4, hbm_budget_bytes=1) as tiny:
        with pytest.raises(GplError) as ei:
            tiny.submit(jobs[0][0], target_density=jobs[0][1])
        assert ei.value.status == _abi.GPL_ERR_OUT_OF_MEMORY
    with PlacementServer(max_active=4) as srv:
        for nl, td in jobs:
            srv.submit(nl, target_density=td)
        res = srv.wait_all(600)
    by = {r["ticket"]: r for r in res}
    # a budget that holds the largest job but not every pair of jobs
    bytes_ = sorted(r["device_bytes"] for r in res)
    budget = bytes_[-1] + bytes_[0] // 2
    with PlacementServer(max_active=4, hbm_budget_bytes=budget) as srv:
        tickets = [srv.submit(nl, target_density=td) for nl, td in jobs]
        res2 = {r["ticket"]: r for r in srv.wait_all(600)}
    for t in tickets:
        assert res2[t]["status"] == 0 and res2[t]["finished"]
    # at every admission instant the resident footprints fit the budget
    for t in tickets:
        a = res2[t]["admit_s"]
        live = [u for u in tickets if res2[u]["admit_s"] <= a < res2[u]["finish_s"]]
        assert sum(res2[u]["device_bytes"] for u in live) <= budget
    # same results as without the budget
    for t0, t1 in zip(sorted(by), tickets):
        assert by[t0]["hpwl"] == res2[t1]["hpwl"]


def test_cancel_queued_and_running_jobs(gpu_lib):
    import time
    from replace_gb300 import PlacementServer
    jobs = small_batch(3, seed=13)
    with PlacementServer(max_active=1, chunk_iters=8) as srv:
        ts = [srv.submit(nl, target_density=td) for nl, td in jobs]
        srv.cancel(ts[2])                       # still queued behind a single slot
        time.sleep(0.05)
        srv.cancel(ts[0])                       # admitted (or about to be): ends at a chunk boundary
        res = {r["ticket"]: r for r in srv.wait_all(600)}
    assert res[ts[2]]["status"] == _abi.GPL_ERR_CANCELLED
    assert res[ts[0]]["status"] in (_abi.GPL_ERR_CANCELLED, 0)
    assert res[ts[1]]["status"] == 0 and res[ts[1]]["finished"]


def test_invalid_netlist_is_rejected_at_submit(gpu_lib):
    from replace_gb300 import PlacementServer, GplError
    nl, td = small_batch(1, seed=14)[0]
    bad = nl.copy()
    bad.net_start = bad.net_start.copy()
    bad.net_start[-1] += 1
    with PlacementServer(max_active=2) as srv:
        with pytest.raises(GplError) as ei:
            srv.submit(bad, target_density=td)
        assert ei.value.status == _abi.GPL_ERR_INVALID_ARG
        assert srv.counts() == {"queued": 0, "running": 0, "ended": 0}


def test_weighted_jobs_match_alone(gpu_lib):
    """Per-net weights submitted with a job (gpl_server_submit_weighted) give
    the result of the same weighted job through the plain API; a weight
    array of the wrong length is rejected at submit."""
    from replace_gb300 import Placer, PlacementServer
    from replace_gb300._lib import GplError
    jobs = small_batch(n=3, seed=5)
    ws = [np.random.default_rng(k).lognormal(0.0, 0.5, nl.n_nets).astype(np.float32)
          for k, (nl, _) in enumerate(jobs)]
    with PlacementServer(max_active=2) as srv:
        tickets = [srv.submit(nl, target_density=td, net_weights=w, poisson_path=1)
                   for (nl, td), w in zip(jobs, ws)]
        res = {r["ticket"]: r for r in srv.wait_all(600)}
        locs = {t: srv.locations(t, nl.n_insts) for t, (nl, _) in zip(tickets, jobs)}
        with pytest.raises(GplError):
            srv.submit(jobs[0][0], target_density=jobs[0][1], net_weights=ws[0][:-1])
    for t, (nl, td), w in zip(tickets, jobs, ws):
        p = Placer(nl, target_density=td, poisson_path=1)
        p.set_net_weights(w)
        p.initial_place()
        p.nesterov_init()
        rc, st, _ = p.nesterov_run(0)
        lx, ly = p.inst_locations()
        p.close()
        r = res[t]
        assert r["status"] == rc == 0 and r["iterations"] == st.iterations and r["hpwl"] == st.hpwl
        assert np.array_equal(locs[t][0], lx) and np.array_equal(locs[t][1], ly)
