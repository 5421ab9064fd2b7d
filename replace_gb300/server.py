"""Placement server: continuous batching of independent placement jobs on one
GPU (gpl_server_* in include/gpl.h).

    with PlacementServer(max_active=8) as srv:
        t = srv.submit(netlist, target_density=0.7)
        for r in srv.wait_all():
            lx, ly = srv.locations(r["ticket"], netlist.n_insts)

Jobs are admitted in submission order as slots and HBM free up; admitted
jobs run concurrently on their own streams and retire when their Nesterov
loop ends.  With batched=True the admitted jobs' Nesterov loops run as one
batch (one launch per phase for all of them; jobs join and leave between
rounds).  A job's result does not depend on the other jobs in the mix.
"""

from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import _abi
from ._lib import check, load


def _result_dict(r: _abi.ServerResult) -> dict:
    return {
        "ticket": int(r.ticket), "status": int(r.status), "finished": bool(r.finished),
        "iterations": int(r.iterations), "ip_rounds": int(r.ip_rounds),
        "overflow": float(r.overflow), "n_insts": int(r.n_insts), "hpwl": int(r.hpwl),
        "device_bytes": int(r.device_bytes), "submit_s": float(r.submit_s),
        "admit_s": float(r.admit_s), "finish_s": float(r.finish_s),
        "latency_s": float(r.finish_s - r.submit_s), "message": r.message.decode(errors="replace"),
    }


class PlacementServer:
    def __init__(self, device: int = 0, max_active: int = 8, hbm_budget_bytes: int = 0,
                 chunk_iters: int = 64, run_initial_place: bool = True, blocking_sync: bool = True,
                 batched: bool = False):
        self.lib = load()
        p = _abi.ServerParams()
        self.lib.gpl_server_params_default(C.byref(p))
        p.device, p.max_active, p.hbm_budget_bytes = device, max_active, hbm_budget_bytes
        p.chunk_iters, p.run_initial_place = chunk_iters, 1 if run_initial_place else 0
        p.blocking_sync = 1 if blocking_sync else 0
        p.batched = 1 if batched else 0
        self.params = p
        h = C.c_void_p()
        check(self.lib.gpl_server_create(C.byref(p), C.byref(h)))
        self.h = h
        self.pending = set()

    def submit(self, netlist, params: _abi.Params | None = None, net_weights=None, **overrides) -> int:
        """Queue one placement job; returns its ticket.  The netlist (and the
        optional per-net weights, as Placer.set_net_weights) is copied."""
        prm = params if params is not None else _abi.default_params()
        for k, v in overrides.items():
            setattr(prm, k, v)
        prm.device = self.params.device
        holder = _abi.DescHolder(netlist)
        t = C.c_int64()
        if net_weights is None:
            check(self.lib.gpl_server_submit(self.h, C.byref(holder.desc), C.byref(prm), C.byref(t)))
        else:
            w = np.ascontiguousarray(net_weights, dtype=np.float32)
            check(self.lib.gpl_server_submit_weighted(self.h, C.byref(holder.desc), C.byref(prm),
                                                      w.ctypes.data_as(C.c_void_p), len(w), C.byref(t)))
        self.pending.add(int(t.value))
        return int(t.value)

    def poll(self, capacity: int = 64, wait_ms: int = 0) -> list[dict]:
        buf = (_abi.ServerResult * capacity)()
        n = self.lib.gpl_server_poll(self.h, buf, capacity, wait_ms)
        out = [_result_dict(buf[k]) for k in range(n)]
        for r in out:
            self.pending.discard(r["ticket"])
        return out

    def wait_all(self, timeout_s: float = 3600.0) -> list[dict]:
        """Results of every job submitted and not yet polled, in end order."""
        out = []
        t_end = time.monotonic() + timeout_s
        while self.pending and time.monotonic() < t_end:
            out += self.poll(64, 200)
        if self.pending:
            raise TimeoutError(f"{len(self.pending)} jobs still running")
        return out

    def locations(self, ticket: int, n_insts: int):
        lx = np.zeros(n_insts, np.int32)
        ly = np.zeros(n_insts, np.int32)
        check(self.lib.gpl_server_get_inst_locations(self.h, ticket, lx.ctypes.data, ly.ctypes.data))
        return lx, ly

    def release(self, ticket: int):
        check(self.lib.gpl_server_release(self.h, ticket))

    def cancel(self, ticket: int):
        check(self.lib.gpl_server_cancel(self.h, ticket))

    def counts(self):
        q, r, e = C.c_int32(), C.c_int32(), C.c_int32()
        self.lib.gpl_server_counts(self.h, C.byref(q), C.byref(r), C.byref(e))
        return {"queued": q.value, "running": r.value, "ended": e.value}

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.gpl_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
