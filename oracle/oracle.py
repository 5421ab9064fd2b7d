"""Python handle on the oracle (CPU restatement of RePlAce's placement path).

TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the product.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from replace_gb300 import _abi

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libgpl_oracle.so")
SRC = os.path.join(HERE, "gpl_oracle.cpp")


def build(force: bool = False) -> str:
    """Compile the oracle (g++, -ffp-contract=off so that x86 and Arm hosts
    evaluate the same float expressions)."""
    os.makedirs(BUILD, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "..", "include", "gpl.h"))):
        tmp = LIB + ".tmp"
        subprocess.check_call(["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-shared", "-fPIC",
                               "-o", tmp, SRC])
        os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        vp = C.c_void_p
        L.orc_create.restype = vp
        L.orc_create.argtypes = [C.POINTER(_abi.NetlistDesc), C.POINTER(_abi.Params), C.POINTER(C.c_int)]
        L.orc_destroy.argtypes = [vp]
        L.orc_set_net_weights.argtypes = [vp, vp, C.c_int64]
        L.orc_initial_place.argtypes = [vp, C.POINTER(_abi.IpStats)]
        L.orc_nesterov_base.argtypes = [vp, C.POINTER(_abi.JobInfo)]
        L.orc_nesterov_init.argtypes = [vp, C.POINTER(_abi.JobInfo)]
        L.orc_nesterov_run.argtypes = [vp, C.c_int, C.POINTER(_abi.NesterovStats), C.POINTER(_abi.IterLog)]
        L.orc_eval.argtypes = [vp, vp, C.c_float, C.c_float, vp, vp, C.POINTER(_abi.EvalStats), vp]
        L.orc_get_bins.argtypes = [vp] * 8
        L.orc_get_gcells.argtypes = [vp] * 4
        L.orc_get_gcell_coords.argtypes = [vp, vp]
        L.orc_get_inst_locations.argtypes = [vp, vp, vp]
        L.orc_get_pins.argtypes = [vp, vp, vp]
        L.orc_poisson_f64.argtypes = [C.c_int] * 4 + [vp] * 4
        L.orc_transform_direct.argtypes = [C.c_int, C.c_int, vp, vp]
        L.orc_transform_fft.argtypes = [C.c_int, C.c_int, vp, vp]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Oracle:
    """One placement job on the CPU oracle (mirrors replace_gb300.Placer)."""

    def __init__(self, netlist, params=None, **overrides):
        self.netlist = netlist
        self.holder = _abi.DescHolder(netlist)
        self.params = params if params is not None else _abi.default_params(**overrides)
        st = C.c_int(0)
        self.h = lib().orc_create(C.byref(self.holder.desc), C.byref(self.params), C.byref(st))
        self.create_status = st.value
        self.info = None

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def set_net_weights(self, weights=None):
        """Per-net weights in net order (None: every weight 1)."""
        if weights is None:
            rc = lib().orc_set_net_weights(self.h, None, 0)
        else:
            self._w = np.ascontiguousarray(weights, dtype=np.float32)
            rc = lib().orc_set_net_weights(self.h, _p(self._w), len(self._w))
        assert rc == 0, rc

    def initial_place(self):
        s = _abi.IpStats()
        rc = lib().orc_initial_place(self.h, C.byref(s))
        return rc, s

    def nesterov_base(self):
        info = _abi.JobInfo()
        rc = lib().orc_nesterov_base(self.h, C.byref(info))
        self.info = info
        return rc

    def nesterov_init(self):
        info = _abi.JobInfo()
        rc = lib().orc_nesterov_init(self.h, C.byref(info))
        self.info = info
        return rc

    def nesterov_run(self, max_iters=0, log_capacity=0):
        st = _abi.NesterovStats()
        lg = _abi.IterLogHolder(log_capacity) if log_capacity else None
        rc = lib().orc_nesterov_run(self.h, max_iters, C.byref(st),
                                    C.byref(lg.log) if lg else None)
        return rc, st, (lg.arrays() if lg else None)

    def eval(self, xy, wl_coef_x, wl_coef_y=None):
        wl_coef_y = wl_coef_x if wl_coef_y is None else wl_coef_y
        n = self.info.n_gcells
        xy = np.ascontiguousarray(xy, np.float32).reshape(-1)
        wl = np.zeros(2 * n, np.float32)
        dg = np.zeros(2 * n, np.float32)
        st = _abi.EvalStats()
        ref = np.zeros(4, np.float64)
        rc = lib().orc_eval(self.h, _p(xy), wl_coef_x, wl_coef_y, _p(wl), _p(dg), C.byref(st), _p(ref))
        assert rc == 0, rc
        return wl.reshape(-1, 2), dg.reshape(-1, 2), st, ref

    def bins(self):
        nb = self.info.bin_cnt_x * self.info.bin_cnt_y
        out = dict(inst_area=np.zeros(nb, np.int64), filler_area=np.zeros(nb, np.int64),
                   nonplace_area=np.zeros(nb, np.int64), density=np.zeros(nb, np.float32),
                   phi=np.zeros(nb, np.float32), ex=np.zeros(nb, np.float32),
                   ey=np.zeros(nb, np.float32))
        lib().orc_get_bins(self.h, *[_p(out[k]) for k in
                                     ("inst_area", "filler_area", "nonplace_area", "density",
                                      "phi", "ex", "ey")])
        return out

    def gcells(self):
        n = self.info.n_gcells
        drect = np.zeros(4 * n, np.int32)
        scale = np.zeros(n, np.float32)
        kind = np.zeros(n, np.uint8)
        lib().orc_get_gcells(self.h, _p(drect), _p(scale), _p(kind))
        return drect.reshape(-1, 4), scale, kind

    def gcell_coords(self):
        xy = np.zeros(2 * self.info.n_gcells, np.float32)
        lib().orc_get_gcell_coords(self.h, _p(xy))
        return xy.reshape(-1, 2)

    def inst_locations(self):
        n = self.netlist.n_insts
        lx = np.zeros(n, np.int32)
        ly = np.zeros(n, np.int32)
        lib().orc_get_inst_locations(self.h, _p(lx), _p(ly))
        return lx, ly

    def pins(self):
        n = self.netlist.n_pins
        x = np.zeros(n, np.int32)
        y = np.zeros(n, np.int32)
        lib().orc_get_pins(self.h, _p(x), _p(y))
        return x, y


def poisson_f64(density, nx, ny, bsx, bsy):
    """FFT::doFFT semantics in FP64; density is [ny, nx] (row-major by y)."""
    rho = np.ascontiguousarray(density, np.float64).reshape(-1)
    phi = np.zeros_like(rho); ex = np.zeros_like(rho); ey = np.zeros_like(rho)
    lib().orc_poisson_f64(nx, ny, bsx, bsy, _p(rho), _p(phi), _p(ex), _p(ey))
    return phi.reshape(ny, nx), ex.reshape(ny, nx), ey.reshape(ny, nx)


def transform(kind: int, a, direct: bool = False):
    a = np.ascontiguousarray(a, np.float64)
    out = np.zeros_like(a)
    fn = lib().orc_transform_direct if direct else lib().orc_transform_fft
    fn(kind, len(a), _p(a), _p(out))
    return out
