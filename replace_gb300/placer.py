"""Host-side mirror of RePlAce's placement interface over the GB300 C ABI.

``Replace`` keeps the method names, argument meaning and defaults of
``replace::Replace`` (include/replace/Replace.h:23-94, src/replace.cpp:13-215);
``setNetlist`` stands in for ``setDb`` because OpenDB is not part of this
library.  ``Placer`` is the thinner per-job handle used by the tests and the
benchmark.  Errors raise ``GplError`` with the reference's codes (1 filler
area, 2/3/4 divergence) instead of exiting the process.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from ._lib import GplError, check, load


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Placer:
    """One placement job on the GPU (gpl_create ... gpl_destroy)."""

    def __init__(self, netlist, params: _abi.Params | None = None, **overrides):
        self.lib = load()
        self.netlist = netlist
        self.holder = _abi.DescHolder(netlist)
        self.params = params if params is not None else _abi.default_params(**overrides)
        if params is not None:
            for k, v in overrides.items():
                setattr(self.params, k, v)
        h = C.c_void_p()
        check(self.lib.gpl_create(C.byref(self.holder.desc), C.byref(self.params), C.byref(h)))
        self.h = h
        self.info = None

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.gpl_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_net_weights(self, weights=None):
        """Per-net weights in net order (GNet::setCustomWeight for every net,
        src/nesterovBase.cpp:264-266); None sets every weight back to 1.
        Allowed between nesterov_run calls."""
        if weights is None:
            check(self.lib.gpl_set_net_weights(self.h, None, 0))
            return
        self._net_w = np.ascontiguousarray(weights, dtype=np.float32)
        check(self.lib.gpl_set_net_weights(self.h, _p(self._net_w), len(self._net_w)))

    # -- stages ---------------------------------------------------------------
    def initial_place(self):
        st = _abi.IpStats()
        check(self.lib.gpl_initial_place(self.h, C.byref(st)))
        return st

    def nesterov_init(self, allow_divergence: bool = False):
        info = _abi.JobInfo()
        rc = self.lib.gpl_nesterov_init(self.h, C.byref(info))
        self.info = info
        check(rc, allow=(_abi.GPL_ERR_DIVERGED_INIT,) if allow_divergence else ())
        return rc

    def nesterov_run(self, max_iters: int = 0, log_capacity: int = 0, allow_divergence: bool = False):
        st = _abi.NesterovStats()
        lg = _abi.IterLogHolder(log_capacity) if log_capacity else None
        rc = self.lib.gpl_nesterov_run(self.h, max_iters, C.byref(st),
                                       C.byref(lg.log) if lg else None)
        div = (_abi.GPL_ERR_DIVERGED_INIT, _abi.GPL_ERR_DIVERGED_BACKTRACK,
               _abi.GPL_ERR_DIVERGED_PHI, _abi.GPL_ERR_DIVERGED_NAN)
        check(rc, allow=div if allow_divergence else ())
        return rc, st, (lg.arrays() if lg else None)

    # -- queries --------------------------------------------------------------
    def inst_locations(self):
        n = self.netlist.n_insts
        lx = np.zeros(n, np.int32)
        ly = np.zeros(n, np.int32)
        check(self.lib.gpl_get_inst_locations(self.h, _p(lx), _p(ly)))
        return lx, ly

    def gcell_coords(self):
        xy = np.zeros(2 * self.info.n_gcells, np.float32)
        check(self.lib.gpl_get_gcell_coords(self.h, _p(xy)))
        return xy.reshape(-1, 2)

    def gcells(self):
        if self.info is None:
            raise GplError(_abi.GPL_ERR_BAD_STATE, "call nesterov_init first")
        n = self.info.n_gcells
        drect = np.zeros(4 * n, np.int32)
        scale = np.zeros(n, np.float32)
        kind = np.zeros(n, np.uint8)
        check(self.lib.gpl_get_gcells(self.h, _p(drect), _p(scale), _p(kind)))
        return drect.reshape(-1, 4), scale, kind

    def eval(self, xy, wl_coef_x: float, wl_coef_y: float | None = None):
        """gpl_eval: WL and density gradients at the given gcell centres."""
        wl_coef_y = wl_coef_x if wl_coef_y is None else wl_coef_y
        xy = np.ascontiguousarray(xy, np.float32).reshape(-1)
        n = xy.size // 2
        wl = np.zeros(2 * n, np.float32)
        dg = np.zeros(2 * n, np.float32)
        st = _abi.EvalStats()
        check(self.lib.gpl_eval(self.h, _p(xy), wl_coef_x, wl_coef_y, _p(wl), _p(dg), C.byref(st)))
        return wl.reshape(-1, 2), dg.reshape(-1, 2), st

    def bins(self, nx: int, ny: int):
        nb = nx * ny
        out = dict(inst_area=np.zeros(nb, np.int64), filler_area=np.zeros(nb, np.int64),
                   nonplace_area=np.zeros(nb, np.int64), density=np.zeros(nb, np.float32),
                   phi=np.zeros(nb, np.float32), ex=np.zeros(nb, np.float32),
                   ey=np.zeros(nb, np.float32))
        check(self.lib.gpl_get_bins(self.h, *[_p(out[k]) for k in
                                              ("inst_area", "filler_area", "nonplace_area",
                                               "density", "phi", "ex", "ey")]))
        return out

    def kernel_times(self):
        cap = 16
        names = (C.c_char_p * cap)()
        ms = (C.c_double * cap)()
        launches = (C.c_int64 * cap)()
        n = self.lib.gpl_kernel_times(self.h, names, ms, launches, cap)
        return {names[i].decode(): (ms[i], launches[i]) for i in range(n)}

    def kernel_times_reset(self, enable: bool = True):
        self.lib.gpl_kernel_times_reset(self.h, 1 if enable else 0)

    def kernel_launches(self) -> int:
        return int(self.lib.gpl_kernel_launch_count(self.h))


def batch_nesterov_run(placers, max_iters: int = 0):
    """gpl_batch_nesterov_run: the Nesterov loops of several jobs (Placer
    objects after nesterov_init, one device, FFT Poisson form) in one
    batched launch per phase.  Returns ([NesterovStats], [status],
    kernel_launches); every job's result equals nesterov_run on it alone."""
    lib = load()
    n = len(placers)
    handles = (C.c_void_p * n)(*[p.h.value for p in placers])
    stats = (_abi.NesterovStats * n)()
    status = (C.c_int32 * n)()
    launches = C.c_int64(0)
    check(lib.gpl_batch_nesterov_run(handles, n, max_iters, stats, status, C.byref(launches)))
    return list(stats), list(status), int(launches.value)


def batch_initial_place(placers):
    """gpl_batch_initial_place: the initial places of several jobs (Placer
    objects before nesterov_init, one device) in lockstep rounds, one launch
    per phase for all of them.  Returns ([IpStats], [status],
    kernel_launches); every job's result equals initial_place on it alone
    (kernel-per-phase solver)."""
    lib = load()
    n = len(placers)
    handles = (C.c_void_p * n)(*[p.h.value for p in placers])
    stats = (_abi.IpStats * n)()
    status = (C.c_int32 * n)()
    launches = C.c_int64(0)
    check(lib.gpl_batch_initial_place(handles, n, stats, status, C.byref(launches)))
    return list(stats), list(status), int(launches.value)


def poisson_solve(density_dev_ptr: int, phi_dev_ptr: int, fx_dev_ptr: int, fy_dev_ptr: int,
                  nx: int, ny: int, bin_size_x: int, bin_size_y: int, stream: int = 0):
    """gpl_poisson_solve on device pointers (e.g. torch tensors' data_ptr())."""
    lib = load()
    check(lib.gpl_poisson_solve(nx, ny, bin_size_x, bin_size_y, C.c_void_p(density_dev_ptr),
                                C.c_void_p(phi_dev_ptr) if phi_dev_ptr else None,
                                C.c_void_p(fx_dev_ptr), C.c_void_p(fy_dev_ptr),
                                C.c_void_p(stream) if stream else None))


class Replace:
    """replace::Replace with the reference's setters and defaults.

    Defaults follow the C++ constructor (src/replace.cpp:13-33); note that the
    Tcl command ``global_placement`` sets the target density to 0.7
    (src/replace.tcl:17), as ``global_placement`` below does.
    """

    def __init__(self):
        self.reset()
        self._netlist = None
        self._placer = None
        self.log = []
        self.ip_stats = None
        self.np_stats = None

    def reset(self):
        # Replace::Replace() values (the reference's reset() uses others)
        self.initialPlaceMaxIter_ = 20
        self.initialPlaceMinDiffLength_ = 1500
        self.initialPlaceMaxSolverIter_ = 100
        self.initialPlaceMaxFanout_ = 200
        self.initialPlaceNetWeightScale_ = 800.0
        self.nesterovPlaceMaxIter_ = 2000
        self.binGridCntX_ = 0
        self.binGridCntY_ = 0
        self.overflow_ = 0.1
        self.density_ = 1.0
        self.initDensityPenalityFactor_ = 0.00008
        self.initWireLengthCoef_ = 0.25
        self.minPhiCoef_ = 0.95
        self.maxPhiCoef_ = 1.05
        self.referenceHpwl_ = 446000000.0
        self.incrementalPlaceMode_ = False
        self.verbose_ = 0
        self.device_ = 0
        self.netWeights_ = None

    # setDb(odb::dbDatabase*) counterpart
    def setNetlist(self, netlist):
        self._netlist = netlist
        self._placer = None

    def setInitialPlaceMaxIter(self, it): self.initialPlaceMaxIter_ = int(it)
    def setInitialPlaceMinDiffLength(self, l): self.initialPlaceMinDiffLength_ = int(l)
    def setInitialPlaceMaxSolverIter(self, it): self.initialPlaceMaxSolverIter_ = int(it)
    def setInitialPlaceMaxFanout(self, f): self.initialPlaceMaxFanout_ = int(f)
    def setInitialPlaceNetWeightScale(self, s): self.initialPlaceNetWeightScale_ = float(s)
    def setNesterovPlaceMaxIter(self, it): self.nesterovPlaceMaxIter_ = int(it)
    def setBinGridCntX(self, n): self.binGridCntX_ = int(n)
    def setBinGridCntY(self, n): self.binGridCntY_ = int(n)
    def setTargetDensity(self, d): self.density_ = float(d)
    def setTargetOverflow(self, o): self.overflow_ = float(o)
    def setInitDensityPenalityFactor(self, p): self.initDensityPenalityFactor_ = float(p)
    def setInitWireLengthCoef(self, c): self.initWireLengthCoef_ = float(c)
    def setMinPhiCoef(self, c): self.minPhiCoef_ = float(c)
    def setMaxPhiCoef(self, c): self.maxPhiCoef_ = float(c)
    def setReferenceHpwl(self, h): self.referenceHpwl_ = float(h)
    def setIncrementalPlaceMode(self, m): self.incrementalPlaceMode_ = bool(m)
    def setVerboseLevel(self, v): self.verbose_ = int(v)

    def setNetWeights(self, w):
        """GNet::setCustomWeight for every net (net order); None = all 1.
        Applies to the current job at once and to jobs made later."""
        self.netWeights_ = None if w is None else np.asarray(w, dtype=np.float32)
        if self._placer is not None:
            self._placer.set_net_weights(self.netWeights_)

    def _new_placer(self):
        p = Placer(self._netlist, self.params())
        if self.netWeights_ is not None:
            p.set_net_weights(self.netWeights_)
        return p

    def params(self) -> _abi.Params:
        return _abi.default_params(
            initial_place_max_iter=self.initialPlaceMaxIter_,
            initial_place_min_diff_length=self.initialPlaceMinDiffLength_,
            initial_place_max_solver_iter=self.initialPlaceMaxSolverIter_,
            initial_place_max_fanout=self.initialPlaceMaxFanout_,
            initial_place_net_weight_scale=self.initialPlaceNetWeightScale_,
            incremental_place_mode=1 if self.incrementalPlaceMode_ else 0,
            target_density=self.density_,
            bin_grid_cnt_x=self.binGridCntX_, bin_grid_cnt_y=self.binGridCntY_,
            nesterov_place_max_iter=self.nesterovPlaceMaxIter_,
            init_density_penalty=self.initDensityPenalityFactor_,
            init_wire_length_coef=self.initWireLengthCoef_,
            target_overflow=self.overflow_,
            min_phi_coef=self.minPhiCoef_, max_phi_coef=self.maxPhiCoef_,
            reference_hpwl=self.referenceHpwl_,
            verbose_level=self.verbose_, device=self.device_)

    def doInitialPlace(self):
        """Replace::doInitialPlace (src/replace.cpp:73-88): a new job (the
        reference builds a new PlacerBase here), then the initial place."""
        if self._netlist is None:
            raise GplError(_abi.GPL_ERR_BAD_STATE, "setNetlist first")
        self._placer = self._new_placer()
        self.ip_stats = self._placer.initial_place()
        return self.ip_stats

    def doNesterovPlace(self, log_capacity: int = 4096):
        """Replace::doNesterovPlace (src/replace.cpp:90-128)."""
        if self._placer is None:
            if self._netlist is None:
                raise GplError(_abi.GPL_ERR_BAD_STATE, "setNetlist first")
            self._placer = self._new_placer()
        self._placer.nesterov_init()
        rc, st, lg = self._placer.nesterov_run(0, log_capacity=log_capacity)
        self.np_stats = st
        self.log = lg
        return st

    def instLocations(self):
        """The locations NesterovPlace::updateDb writes (lower-left, DBU)."""
        return self._placer.inst_locations()


def global_placement(netlist, skip_initial_place=False, incremental=False, density=0.7,
                     bin_grid_count=None, init_density_penalty=None, init_wirelength_coef=None,
                     min_phi_coef=None, max_phi_coef=None, overflow=None,
                     initial_place_max_iter=None, initial_place_max_fanout=None,
                     verbose_level=None):
    """The ``global_placement`` Tcl command (src/replace.tcl:8-96) as a call."""
    r = Replace()
    r.setNetlist(netlist)
    r.setTargetDensity(density)
    if skip_initial_place:
        r.setInitialPlaceMaxIter(0)
    elif initial_place_max_iter is not None:
        r.setInitialPlaceMaxIter(initial_place_max_iter)
    if incremental:
        r.setInitialPlaceMaxIter(0)
        r.setIncrementalPlaceMode(True)
    if initial_place_max_fanout is not None:
        r.setInitialPlaceMaxFanout(initial_place_max_fanout)
    if min_phi_coef is not None:
        r.setMinPhiCoef(min_phi_coef)
    if max_phi_coef is not None:
        r.setMaxPhiCoef(max_phi_coef)
    if init_density_penalty is not None:
        r.setInitDensityPenalityFactor(init_density_penalty)
    if init_wirelength_coef is not None:
        r.setInitWireLengthCoef(init_wirelength_coef)
    if overflow is not None:
        r.setTargetOverflow(overflow)
    if verbose_level is not None:
        r.setVerboseLevel(verbose_level)
    if bin_grid_count is not None:
        r.setBinGridCntX(bin_grid_count)
        r.setBinGridCntY(bin_grid_count)
    r.doInitialPlace()
    r.doNesterovPlace()
    return r
