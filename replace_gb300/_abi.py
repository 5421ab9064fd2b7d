"""ctypes mirror of include/gpl.h (structures, status codes, array marshalling)."""

from __future__ import annotations

import ctypes as C

import numpy as np

GPL_OK = 0
GPL_ERR_FILLER_AREA = 1
GPL_ERR_DIVERGED_INIT = 2
GPL_ERR_DIVERGED_BACKTRACK = 3
GPL_ERR_DIVERGED_PHI = 4
GPL_ERR_UTIL = 5
GPL_ERR_DIVERGED_NAN = 6
GPL_ERR_INVALID_ARG = 16
GPL_ERR_CUDA = 17
GPL_ERR_OUT_OF_MEMORY = 18
GPL_ERR_BAD_STATE = 19
GPL_ERR_NO_DEVICE = 20
GPL_ERR_CANCELLED = 21

_i32p = C.POINTER(C.c_int32)
_u8p = C.POINTER(C.c_uint8)


class NetlistDesc(C.Structure):
    _fields_ = [
        ("core_lx", C.c_int32), ("core_ly", C.c_int32), ("core_ux", C.c_int32), ("core_uy", C.c_int32),
        ("site_w", C.c_int32), ("site_h", C.c_int32),
        ("n_insts", C.c_int32),
        ("inst_lx", _i32p), ("inst_ly", _i32p), ("inst_ux", _i32p), ("inst_uy", _i32p),
        ("inst_kind", _u8p),
        ("n_pins", C.c_int32),
        ("pin_inst", _i32p), ("pin_ox", _i32p), ("pin_oy", _i32p), ("pin_x", _i32p), ("pin_y", _i32p),
        ("n_nets", C.c_int32),
        ("net_start", _i32p),
        ("inst_pin_start", _i32p), ("inst_pins", _i32p),
    ]


class Params(C.Structure):
    _fields_ = [
        ("initial_place_max_iter", C.c_int32),
        ("initial_place_min_diff_length", C.c_int32),
        ("initial_place_max_solver_iter", C.c_int32),
        ("initial_place_max_fanout", C.c_int32),
        ("initial_place_net_weight_scale", C.c_float),
        ("incremental_place_mode", C.c_int32),
        ("target_density", C.c_float),
        ("bin_grid_cnt_x", C.c_int32),
        ("bin_grid_cnt_y", C.c_int32),
        ("min_wire_length_force_bar", C.c_float),
        ("nesterov_place_max_iter", C.c_int32),
        ("max_back_track", C.c_int32),
        ("init_density_penalty", C.c_float),
        ("init_wire_length_coef", C.c_float),
        ("target_overflow", C.c_float),
        ("min_phi_coef", C.c_float),
        ("max_phi_coef", C.c_float),
        ("min_preconditioner", C.c_float),
        ("initial_prev_coordi_update_coef", C.c_float),
        ("reference_hpwl", C.c_float),
        ("verbose_level", C.c_int32),
        ("device", C.c_int32),
        ("stream", C.c_void_p),
        ("use_graph", C.c_int32),
        ("ip_solver", C.c_int32),
        ("poisson_path", C.c_int32),
        ("scatter_tile", C.c_int32), ("scatter_chunk", C.c_int32),
        ("device_loop", C.c_int32),
    ]


class JobInfo(C.Structure):
    _fields_ = [
        ("n_place_insts", C.c_int32), ("n_gcells", C.c_int32), ("n_fillers", C.c_int32),
        ("bin_cnt_x", C.c_int32), ("bin_cnt_y", C.c_int32),
        ("bin_size_x", C.c_int32), ("bin_size_y", C.c_int32),
        ("filler_dx", C.c_int32), ("filler_dy", C.c_int32),
        ("place_insts_area", C.c_int64), ("std_insts_area", C.c_int64),
        ("macro_insts_area", C.c_int64), ("non_place_insts_area", C.c_int64),
        ("device_bytes", C.c_int64),
        ("poisson_path", C.c_int32), ("poisson_fft_us", C.c_float), ("poisson_gemm_us", C.c_float),
        ("scatter_tile", C.c_int32), ("scatter_chunk", C.c_int32), ("scatter_us", C.c_float),
    ]


class EvalStats(C.Structure):
    _fields_ = [
        ("overflow_area", C.c_int64), ("overflow_area_f64", C.c_double),
        ("hpwl", C.c_int64), ("sum_phi", C.c_double),
        ("wire_length_grad_sum", C.c_double), ("density_grad_sum", C.c_double),
    ]


class NesterovStats(C.Structure):
    _fields_ = [
        ("iterations", C.c_int32), ("evaluations", C.c_int32), ("finished", C.c_int32),
        ("status", C.c_int32), ("overflow", C.c_float), ("step_length", C.c_float),
        ("density_penalty", C.c_float), ("wire_length_coef", C.c_float), ("hpwl", C.c_int64),
    ]


class IterLog(C.Structure):
    _fields_ = [
        ("capacity", C.c_int32), ("count", C.c_int32),
        ("overflow", C.POINTER(C.c_float)), ("hpwl", C.POINTER(C.c_int64)),
        ("step_length", C.POINTER(C.c_float)), ("backtracks", C.POINTER(C.c_int32)),
    ]


class IpStats(C.Structure):
    _fields_ = [
        ("iterations", C.c_int32), ("last_error", C.c_float), ("last_hpwl", C.c_int64),
        ("solver_iters_x", C.c_int32), ("solver_iters_y", C.c_int32),
        ("cooperative_rounds", C.c_int32), ("pad", C.c_int32),
    ]


class ServerParams(C.Structure):
    _fields_ = [
        ("device", C.c_int32), ("max_active", C.c_int32), ("hbm_budget_bytes", C.c_int64),
        ("chunk_iters", C.c_int32), ("run_initial_place", C.c_int32),
        ("blocking_sync", C.c_int32), ("batched", C.c_int32),
    ]


class ServerResult(C.Structure):
    _fields_ = [
        ("ticket", C.c_int64), ("status", C.c_int32), ("finished", C.c_int32),
        ("iterations", C.c_int32), ("ip_rounds", C.c_int32), ("overflow", C.c_float),
        ("n_insts", C.c_int32), ("hpwl", C.c_int64), ("device_bytes", C.c_int64),
        ("submit_s", C.c_double), ("admit_s", C.c_double), ("finish_s", C.c_double),
        ("message", C.c_char * 160),
    ]


def ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


def default_params(**overrides) -> Params:
    """gpl_params_default() values (replace::Replace defaults), with overrides."""
    p = Params(
        initial_place_max_iter=20, initial_place_min_diff_length=1500,
        initial_place_max_solver_iter=100, initial_place_max_fanout=200,
        initial_place_net_weight_scale=800.0, incremental_place_mode=0,
        target_density=1.0, bin_grid_cnt_x=0, bin_grid_cnt_y=0,
        min_wire_length_force_bar=-300.0,
        nesterov_place_max_iter=2000, max_back_track=10,
        init_density_penalty=0.00008, init_wire_length_coef=0.25,
        target_overflow=0.1, min_phi_coef=0.95, max_phi_coef=1.05,
        min_preconditioner=1.0, initial_prev_coordi_update_coef=100.0,
        reference_hpwl=446000000.0, verbose_level=0, device=0, stream=None, use_graph=1,
        ip_solver=0, poisson_path=0, scatter_tile=0, scatter_chunk=0, device_loop=0,
    )
    for k, v in overrides.items():
        setattr(p, k, v)
    return p


class DescHolder:
    """Owns contiguous copies of a Netlist's arrays and the NetlistDesc
    pointing at them (keep this object alive while the descriptor is used)."""

    def __init__(self, nl):
        c = lambda a, t: np.ascontiguousarray(a, dtype=t)
        self.arrays = dict(
            inst_lx=c(nl.inst_lx, np.int32), inst_ly=c(nl.inst_ly, np.int32),
            inst_ux=c(nl.inst_ux, np.int32), inst_uy=c(nl.inst_uy, np.int32),
            inst_kind=c(nl.inst_kind, np.uint8),
            pin_inst=c(nl.pin_inst, np.int32), pin_ox=c(nl.pin_ox, np.int32),
            pin_oy=c(nl.pin_oy, np.int32), pin_x=c(nl.pin_x, np.int32),
            pin_y=c(nl.pin_y, np.int32), net_start=c(nl.net_start, np.int32),
            inst_pin_start=c(nl.inst_pin_start, np.int32), inst_pins=c(nl.inst_pins, np.int32),
        )
        a = self.arrays
        self.desc = NetlistDesc(
            core_lx=nl.core[0], core_ly=nl.core[1], core_ux=nl.core[2], core_uy=nl.core[3],
            site_w=nl.site[0], site_h=nl.site[1], n_insts=nl.n_insts,
            inst_lx=ptr(a["inst_lx"], C.c_int32), inst_ly=ptr(a["inst_ly"], C.c_int32),
            inst_ux=ptr(a["inst_ux"], C.c_int32), inst_uy=ptr(a["inst_uy"], C.c_int32),
            inst_kind=ptr(a["inst_kind"], C.c_uint8), n_pins=nl.n_pins,
            pin_inst=ptr(a["pin_inst"], C.c_int32), pin_ox=ptr(a["pin_ox"], C.c_int32),
            pin_oy=ptr(a["pin_oy"], C.c_int32), pin_x=ptr(a["pin_x"], C.c_int32),
            pin_y=ptr(a["pin_y"], C.c_int32), n_nets=nl.n_nets,
            net_start=ptr(a["net_start"], C.c_int32),
            inst_pin_start=ptr(a["inst_pin_start"], C.c_int32),
            inst_pins=ptr(a["inst_pins"], C.c_int32),
        )

    @property
    def nbytes(self) -> int:
        return int(sum(v.nbytes for v in self.arrays.values()))


class IterLogHolder:
    def __init__(self, capacity: int):
        self.overflow = np.zeros(capacity, np.float32)
        self.hpwl = np.zeros(capacity, np.int64)
        self.step_length = np.zeros(capacity, np.float32)
        self.backtracks = np.zeros(capacity, np.int32)
        self.log = IterLog(capacity=capacity, count=0,
                           overflow=ptr(self.overflow, C.c_float),
                           hpwl=ptr(self.hpwl, C.c_int64),
                           step_length=ptr(self.step_length, C.c_float),
                           backtracks=ptr(self.backtracks, C.c_int32))

    def arrays(self):
        n = self.log.count
        return dict(overflow=self.overflow[:n].copy(), hpwl=self.hpwl[:n].copy(),
                    step_length=self.step_length[:n].copy(),
                    backtracks=self.backtracks[:n].copy())
