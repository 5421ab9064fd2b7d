"""Flat placement netlist (the host-side form the placer consumes).

``Netlist`` is the structure-of-arrays equivalent of RePlAce's ``PlacerBase``
(src/placerBase.h:233-312): instances with their bounding boxes and kinds,
pins with their offsets from the instance centre, and nets as a CSR list of
pins in net-major order.  It is built either from LEF/DEF
(``from_lefdef``, following ``PlacerBase::init`` src/placerBase.cpp:606-758 and
``initInstsForFragmentedRow`` :761-846) or by the seeded synthetic generator
(``generate``) that stands in for the public benchmark suites.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import lefdef

INST_PLACE = 0     # movable instance
INST_FIXED = 1     # fixed instance overlapping the core
INST_DUMMY = 2     # fragmented-row filler instance (always fixed)
INST_OUTSIDE = 3   # fixed instance outside the core (ignored by the placer)

INT_MAX = 2**31 - 1
INT_MIN = -2**31


def _cdiv(a, b):
    """C integer division (truncates toward zero) for ints or int arrays."""
    a = np.asarray(a, dtype=np.int64)
    q = np.abs(a) // b
    return np.where(a < 0, -q, q)


def _cdiv_int(a: int, b: int) -> int:
    q = abs(a) // b
    return -q if a < 0 else q


def _fast_mod(a: int, c: int) -> int:
    # fastModulo (src/placerBase.cpp:979-982): a % c only when a >= c
    return a % c if a >= c else a


@dataclass
class Netlist:
    core: tuple                     # (lx, ly, ux, uy) from the rows' bounding box
    die: tuple                      # (lx, ly, ux, uy)
    site: tuple                     # (width, height)
    dbu: int
    inst_lx: np.ndarray             # int32 [n_insts]
    inst_ly: np.ndarray
    inst_ux: np.ndarray
    inst_uy: np.ndarray
    inst_kind: np.ndarray           # uint8 [n_insts], INST_* above
    pin_inst: np.ndarray            # int32 [n_pins], -1 for IO ports
    pin_ox: np.ndarray              # int32 offset from the instance centre
    pin_oy: np.ndarray
    pin_x: np.ndarray               # int32 initial absolute pin centre
    pin_y: np.ndarray
    net_start: np.ndarray           # int32 [n_nets + 1]; pins are net-major
    inst_pin_start: np.ndarray      # int32 [n_insts + 1]
    inst_pins: np.ndarray           # int32 pin indices in instance pin order
    inst_names: list = field(default_factory=list)
    net_names: list = field(default_factory=list)
    rows: list = field(default_factory=list)     # row boxes (lx, ly, ux, uy)
    # IO pin boxes [n_pins, 4] (lx, ly, ux, uy); lx > ux marks "no box"
    # (component pins and unplaced IO pins)
    io_box: np.ndarray | None = None

    @property
    def n_insts(self):
        return len(self.inst_lx)

    @property
    def n_pins(self):
        return len(self.pin_inst)

    @property
    def n_nets(self):
        return len(self.net_start) - 1

    def place_indices(self):
        return np.nonzero(self.inst_kind == INST_PLACE)[0]

    def copy(self):
        kw = {}
        for k, v in self.__dict__.items():
            kw[k] = v.copy() if isinstance(v, np.ndarray) else (
                list(v) if isinstance(v, list) else v)
        return Netlist(**kw)

    def set_inst_locations(self, idx, lx, ly):
        """Move instances (lower-left) and their pins (PlacerBase semantics)."""
        idx = np.asarray(idx)
        dx = self.inst_ux[idx] - self.inst_lx[idx]
        dy = self.inst_uy[idx] - self.inst_ly[idx]
        self.inst_lx[idx] = lx
        self.inst_ly[idx] = ly
        self.inst_ux[idx] = lx + dx
        self.inst_uy[idx] = ly + dy
        self._update_pins()

    def _update_pins(self):
        # Pin::updateLocation (src/placerBase.cpp:408-412): centre + offset
        m = self.pin_inst >= 0
        inst = self.pin_inst[m]
        cx = _cdiv(self.inst_lx[inst].astype(np.int64) + self.inst_ux[inst], 2)
        cy = _cdiv(self.inst_ly[inst].astype(np.int64) + self.inst_uy[inst], 2)
        self.pin_x[m] = (cx + self.pin_ox[m]).astype(np.int32)
        self.pin_y[m] = (cy + self.pin_oy[m]).astype(np.int32)

    def bbox_hpwl(self, inst_lx=None, inst_ly=None):
        """PlacerBase::hpwl (src/placerBase.cpp:868-876, Net::updateBox
        :480-500): per net, the bounding box of its instances' boxes and its
        IO pins' boxes.  Instance lower-left corners may be given (their
        sizes are the netlist's)."""
        lx0 = self.inst_lx if inst_lx is None else np.asarray(inst_lx)
        ly0 = self.inst_ly if inst_ly is None else np.asarray(inst_ly)
        w = (self.inst_ux - self.inst_lx).astype(np.int64)
        h = (self.inst_uy - self.inst_ly).astype(np.int64)
        inst = self.pin_inst
        on = inst >= 0
        ii = np.where(on, inst, 0)
        box = np.empty((self.n_pins, 4), np.int64)
        box[:, 0] = np.where(on, lx0[ii], 0)
        box[:, 1] = np.where(on, ly0[ii], 0)
        box[:, 2] = np.where(on, lx0[ii] + w[ii], 0)
        box[:, 3] = np.where(on, ly0[ii] + h[ii], 0)
        io = self.io_box if self.io_box is not None else np.stack(
            [self.pin_x, self.pin_y, self.pin_x, self.pin_y], 1)
        valid = on | (io[:, 0] <= io[:, 2])
        box[~on] = io[~on]
        big = np.iinfo(np.int64).max // 4
        lo = np.where(valid[:, None], box, [big, big, -big, -big])
        starts = self.net_start[:-1]
        mnx = np.minimum.reduceat(lo[:, 0], starts)
        mny = np.minimum.reduceat(lo[:, 1], starts)
        mxx = np.maximum.reduceat(lo[:, 2], starts)
        mxy = np.maximum.reduceat(lo[:, 3], starts)
        return int(np.sum((mxx - mnx) + (mxy - mny)))


def _fragmented_row_dummies(core, site, rows, fixed_boxes):
    """initInstsForFragmentedRow (src/placerBase.cpp:761-846)."""
    sx, sy = site
    ncx = (core[2] - core[0]) // sx
    ncy = (core[3] - core[1]) // sy
    grid = np.zeros((ncy, ncx), dtype=np.uint8)   # 0 empty, 1 row, 2 fixed

    def rng(ll, uu, c0, s, hi):
        # getMinMaxIdx (src/placerBase.cpp:984-993), C integer semantics
        lo = _cdiv_int(ll - c0, s)
        d = uu - c0
        up = _cdiv_int(d, s) if _fast_mod(d, s) == 0 else _cdiv_int(d, s) + 1
        return max(0, lo), min(hi, up)

    for (lx, ly, ux, uy) in rows:
        a, b = rng(lx, ux, core[0], sx, ncx)
        c, d = rng(ly, uy, core[1], sy, ncy)
        grid[c:d, a:b] = 1
    for (lx, ly, ux, uy) in fixed_boxes:
        a, b = rng(lx, ux, core[0], sx, ncx)
        c, d = rng(ly, uy, core[1], sy, ncy)
        if a < b and c < d:
            grid[c:d, a:b] = 2
    out = []
    for j in range(ncy):
        i = 0
        while i < ncx:
            if grid[j, i] == 0:
                s = i
                while i < ncx and grid[j, i] == 0:
                    i += 1
                out.append((core[0] + sx * s, core[1] + sy * j,
                            core[0] + sx * i, core[1] + sy * (j + 1)))
            i += 1
    return out


def from_lefdef(lib: lefdef.LefLibrary, d: lefdef.DefDesign,
                reverse_net_iterms: bool = False) -> Netlist:
    """Build a Netlist from LEF/DEF following PlacerBase::init.

    ``reverse_net_iterms`` selects the order in which a net's component pins
    are listed (the order OpenDB's ``dbNet::getITerms`` iterates in).
    """
    rows = []
    site = None
    for r in d.rows:
        sw, sh = lib.sites[r.site]
        if site is None:
            site = (sw, sh)
        w = r.sx * (r.nx - 1) + sw if r.nx > 1 else sw
        h = r.sy * (r.ny - 1) + sh if r.ny > 1 else sh
        rows.append((r.x, r.y, r.x + w, r.y + h))
    core = (min(r[0] for r in rows), min(r[1] for r in rows),
            max(r[2] for r in rows), max(r[3] for r in rows))

    comp_idx = {c.name: k for k, c in enumerate(d.components)}
    n_real = len(d.components)
    lx = np.zeros(n_real, np.int64)
    ly = np.zeros(n_real, np.int64)
    ux = np.zeros(n_real, np.int64)
    uy = np.zeros(n_real, np.int64)
    kind = np.zeros(n_real, np.uint8)
    mw = np.zeros(n_real, np.int64)
    mh = np.zeros(n_real, np.int64)
    fixed_boxes = []
    for k, c in enumerate(d.components):
        m = lib.macros[c.master]
        mw[k], mh[k] = m.width, m.height
        w, h = (m.height, m.width) if c.orient in ("E", "W", "FE", "FW") else (m.width, m.height)
        lx[k], ly[k] = c.x, c.y
        ux[k], uy[k] = c.x + w, c.y + h
        if c.status in ("FIXED", "COVER", "LOCKED", "FIRM"):
            box = (lx[k], ly[k], ux[k], uy[k])
            fixed_boxes.append(box)
            ov = not (max(core[0], box[0]) >= min(core[2], box[2]) or
                      max(core[1], box[1]) >= min(core[3], box[3]))
            kind[k] = INST_FIXED if ov else INST_OUTSIDE
        else:
            kind[k] = INST_PLACE

    dummies = _fragmented_row_dummies(core, site, rows, fixed_boxes)
    nd = len(dummies)
    if nd:
        db = np.array(dummies, dtype=np.int64)
        lx = np.concatenate([lx, db[:, 0]]); ly = np.concatenate([ly, db[:, 1]])
        ux = np.concatenate([ux, db[:, 2]]); uy = np.concatenate([uy, db[:, 3]])
        kind = np.concatenate([kind, np.full(nd, INST_DUMMY, np.uint8)])

    # pins: per net (skipping POWER/GROUND/RESET), component pins then IO pins
    pin_by_name = {p.name: p for p in d.pins}
    io_by_net = {}
    for p in d.pins:
        if p.net is not None:
            io_by_net.setdefault(p.net, []).append(p)
    p_inst, p_ox, p_oy, p_x, p_y, p_key, p_box = [], [], [], [], [], [], []
    net_start = [0]
    net_names = []
    for net in d.nets:
        if net.use in ("POWER", "GROUND", "RESET"):
            continue
        conns = list(reversed(net.conns)) if reverse_net_iterms else net.conns
        for (cname, pname) in conns:
            k = comp_idx[cname]
            m = lib.macros[d.components[k].master]
            boxes = m.pins.get(pname, [])
            if boxes:
                oxl = min(b[0] for b in boxes); oyl = min(b[1] for b in boxes)
                oxh = max(b[2] for b in boxes); oyh = max(b[3] for b in boxes)
                ox = int(_cdiv(oxl + oxh, 2)) - int(_cdiv(m.width, 2))
                oy = int(_cdiv(oyl + oyh, 2)) - int(_cdiv(m.height, 2))
            else:
                ox = oy = 0
            p_inst.append(k)
            p_box.append((1, 1, 0, 0))
            p_ox.append(ox); p_oy.append(oy)
            p_x.append(int(lx[k]) + int(_cdiv(m.width, 2)) + ox)
            p_y.append(int(ly[k]) + int(_cdiv(m.height, 2)) + oy)
            p_key.append(m.pin_order.index(pname) if pname in m.pin_order else 0)
        ios = io_by_net.get(net.name, [])
        for p in ios:
            if p.box is None:
                x = y = 0   # (INT_MAX + INT_MIN) / 2 in the reference
            else:
                x = int(_cdiv(p.box[0] + p.box[2], 2))
                y = int(_cdiv(p.box[1] + p.box[3], 2))
            p_inst.append(-1); p_ox.append(0); p_oy.append(0)
            p_x.append(x); p_y.append(y); p_key.append(0)
            p_box.append(tuple(p.box) if p.box is not None else (1, 1, 0, 0))
        net_start.append(len(p_inst))
        net_names.append(net.name)

    n_insts = len(lx)
    pin_inst = np.array(p_inst, np.int32)
    key = np.array(p_key, np.int64)
    # instance pin order: master pin order (dbInst::getITerms)
    order = np.lexsort((key, pin_inst))
    order = order[pin_inst[order] >= 0]
    counts = np.bincount(pin_inst[order], minlength=n_insts)
    inst_pin_start = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)

    # OpenDB's block box covers the die area and every placed IO pin box
    die = list(d.die)
    for p in d.pins:
        if p.box is not None:
            die = [min(die[0], p.box[0]), min(die[1], p.box[1]),
                   max(die[2], p.box[2]), max(die[3], p.box[3])]
    return Netlist(
        core=core, die=tuple(die), site=site, dbu=d.dbu,
        inst_lx=lx.astype(np.int32), inst_ly=ly.astype(np.int32),
        inst_ux=ux.astype(np.int32), inst_uy=uy.astype(np.int32),
        inst_kind=kind,
        pin_inst=pin_inst,
        pin_ox=np.array(p_ox, np.int32), pin_oy=np.array(p_oy, np.int32),
        pin_x=np.array(p_x, np.int32), pin_y=np.array(p_y, np.int32),
        net_start=np.array(net_start, np.int32),
        inst_pin_start=inst_pin_start,
        inst_pins=order.astype(np.int32),
        inst_names=[c.name for c in d.components] + [f"dummy{k}" for k in range(nd)],
        net_names=net_names,
        rows=rows,
        io_box=np.array(p_box, np.int32).reshape(-1, 4),
    )


_NPZ_ARRAYS = ("inst_lx", "inst_ly", "inst_ux", "inst_uy", "inst_kind", "pin_inst", "pin_ox",
               "pin_oy", "pin_x", "pin_y", "net_start", "inst_pin_start", "inst_pins")


def save_npz(nl: Netlist, path: str) -> None:
    """Serialise a Netlist (arrays, core/die/site/dbu and row boxes)."""
    extra = {} if nl.io_box is None else {"io_box": nl.io_box}
    np.savez_compressed(
        path, core=np.array(nl.core, np.int64), die=np.array(nl.die, np.int64),
        site=np.array(nl.site, np.int64), dbu=np.array(nl.dbu),
        rows=np.array(nl.rows, np.int64).reshape(-1, 4),
        **{k: getattr(nl, k) for k in _NPZ_ARRAYS}, **extra)


def load_npz(path: str) -> Netlist:
    z = np.load(path)
    return Netlist(core=tuple(int(v) for v in z["core"]), die=tuple(int(v) for v in z["die"]),
                   site=tuple(int(v) for v in z["site"]), dbu=int(z["dbu"]),
                   rows=[tuple(int(v) for v in r) for r in z["rows"]],
                   io_box=z["io_box"].copy() if "io_box" in z.files else None,
                   **{k: z[k].copy() for k in _NPZ_ARRAYS})


def read(lef_paths, def_path, **kw) -> Netlist:
    return from_lefdef(lefdef.read_lef(lef_paths), lefdef.read_def(def_path), **kw)


# ---------------------------------------------------------------------------
# Seeded synthetic netlists
# ---------------------------------------------------------------------------

SITE_W = 380
ROW_H = 2800
DBU = 2000


def generate(n_cells: int, n_nets: int, n_io: int = 200, n_macros: int = 0,
             util: float = 0.60, seed: int = 1, window: int = 500,
             macro_rows=(20, 60)) -> Netlist:
    """Seeded synthetic flat standard-cell netlist.

    Cells are one row high (2800 DBU) and 380 x U{2..16} DBU wide; movable
    macros are squares of U{macro_rows} rows per side.  Net degrees are 2
    (60 %), 3 (15 %), U{4..10} (20 %) and U{11..50} (5 %); a net's pins are
    drawn from a window of +-``window`` instance indices around a random seed
    instance, with offsets uniform inside the instance.  ``n_io`` fixed IO
    pins lie uniformly on the die boundary, each joined to a random net.  The
    die equals the core: a square of whole rows and sites sized for ``util``.
    Movable instances start at the core's lower-left corner (unplaced).
    """
    rng = np.random.default_rng(seed)
    n_inst = n_cells + n_macros
    w = np.empty(n_inst, np.int64)
    h = np.empty(n_inst, np.int64)
    is_macro = np.zeros(n_inst, bool)
    if n_macros:
        macro_pos = rng.choice(n_inst, size=n_macros, replace=False)
        is_macro[macro_pos] = True
    cw = SITE_W * rng.integers(2, 17, size=n_inst)
    w[:] = cw
    h[:] = ROW_H
    if n_macros:
        side = ROW_H * rng.integers(macro_rows[0], macro_rows[1] + 1, size=n_macros)
        w[is_macro] = side
        h[is_macro] = side
    area = float(np.sum(w * h))
    side = np.sqrt(area / util)
    n_rows = int(np.ceil(side / ROW_H))
    n_sites = int(np.ceil(side / SITE_W))
    core = (0, 0, n_sites * SITE_W, n_rows * ROW_H)

    # net degrees
    u = rng.random(n_nets)
    deg = np.where(u < 0.60, 2,
          np.where(u < 0.75, 3,
          np.where(u < 0.95, rng.integers(4, 11, size=n_nets),
                   rng.integers(11, 51, size=n_nets)))).astype(np.int64)
    seeds = rng.integers(0, n_inst, size=n_nets)
    total = int(deg.sum())
    net_of_pin = np.repeat(np.arange(n_nets), deg)
    first = np.concatenate([[0], np.cumsum(deg)[:-1]])
    rank = np.arange(total) - np.repeat(first, deg)
    off = rng.integers(-window, window + 1, size=total)
    off[rank == 0] = 0                                  # seed instance itself
    # reflect at both ends of the index range (clipping would pile the pins
    # of every window that overhangs an end onto the first and last cells)
    cell = seeds[net_of_pin] + off
    cell = np.where(cell < 0, -cell, cell)
    cell = np.where(cell > n_inst - 1, 2 * (n_inst - 1) - cell, cell)
    cell = np.clip(cell, 0, n_inst - 1)
    pw = w[cell]
    ph = h[cell]
    ox = np.floor((rng.random(total) - 0.5) * pw).astype(np.int64)
    oy = np.floor((rng.random(total) - 0.5) * ph).astype(np.int64)

    # IO pins on the boundary, each appended to a random net
    io_net = rng.integers(0, n_nets, size=n_io)
    perim = 2 * (core[2] + core[3])
    t = rng.random(n_io) * perim
    iox = np.empty(n_io, np.int64)
    ioy = np.empty(n_io, np.int64)
    W, H = core[2], core[3]
    for k in range(n_io):
        s = t[k]
        if s < W:
            iox[k], ioy[k] = int(s), 0
        elif s < W + H:
            iox[k], ioy[k] = W, int(s - W)
        elif s < 2 * W + H:
            iox[k], ioy[k] = int(2 * W + H - s), H
        else:
            iox[k], ioy[k] = 0, int(perim - s)

    # merge: per net, its cell pins then its IO pins
    io_count = np.bincount(io_net, minlength=n_nets)
    full_deg = deg + io_count
    net_start = np.concatenate([[0], np.cumsum(full_deg)]).astype(np.int64)
    n_pins = int(net_start[-1])
    pin_inst = np.full(n_pins, -1, np.int64)
    pin_ox = np.zeros(n_pins, np.int64)
    pin_oy = np.zeros(n_pins, np.int64)
    pin_x = np.zeros(n_pins, np.int64)
    pin_y = np.zeros(n_pins, np.int64)
    dst = net_start[net_of_pin] + rank
    pin_inst[dst] = cell
    pin_ox[dst] = ox
    pin_oy[dst] = oy
    io_order = np.argsort(io_net, kind="stable")
    io_sorted_net = io_net[io_order]
    io_first = np.searchsorted(io_sorted_net, io_sorted_net, side="left")
    io_rank = np.arange(n_io) - io_first
    io_dst = net_start[io_sorted_net] + deg[io_sorted_net] + io_rank
    pin_x[io_dst] = iox[io_order]
    pin_y[io_dst] = ioy[io_order]

    lx = np.full(n_inst, core[0], np.int64)
    ly = np.full(n_inst, core[1], np.int64)
    nl = Netlist(
        core=core, die=core, site=(SITE_W, ROW_H), dbu=DBU,
        inst_lx=lx.astype(np.int32), inst_ly=ly.astype(np.int32),
        inst_ux=(lx + w).astype(np.int32), inst_uy=(ly + h).astype(np.int32),
        inst_kind=np.zeros(n_inst, np.uint8),
        pin_inst=pin_inst.astype(np.int32),
        pin_ox=pin_ox.astype(np.int32), pin_oy=pin_oy.astype(np.int32),
        pin_x=pin_x.astype(np.int32), pin_y=pin_y.astype(np.int32),
        net_start=net_start.astype(np.int32),
        inst_pin_start=np.zeros(n_inst + 1, np.int32),
        inst_pins=np.zeros(0, np.int32),
        rows=[(core[0], y, core[2], y + ROW_H) for y in range(core[1], core[3], ROW_H)],
    )
    m = nl.pin_inst >= 0
    pins = np.nonzero(m)[0]
    order = pins[np.argsort(nl.pin_inst[pins], kind="stable")]
    counts = np.bincount(nl.pin_inst[order], minlength=n_inst)
    nl.inst_pin_start = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
    nl.inst_pins = order.astype(np.int32)
    nl._update_pins()
    return nl


# Workload shapes named after what they are (cells / nets / bins).
WORKLOADS = {
    "10k_cells_128bins": dict(n_cells=10_000, n_nets=10_500, n_io=200, n_macros=0,
                              util=0.60, target_density=0.70, bins=128),
    "200k_cells_40macros_512bins": dict(n_cells=200_000, n_nets=210_000, n_io=200,
                                        n_macros=40, util=0.60, target_density=0.70,
                                        bins=512),
    "1m_cells_1024bins": dict(n_cells=1_000_000, n_nets=1_050_000, n_io=2_000,
                              n_macros=0, util=0.60, target_density=0.75, bins=1024),
    # the 1M workload's bin grid with 40 % of its cells: the case kernel
    # profiles are captured on (working set above L2, a few hundred MB)
    "400k_cells_1024bins": dict(n_cells=400_000, n_nets=420_000, n_io=1_000,
                                n_macros=0, util=0.60, target_density=0.75, bins=1024),
    # scale-out check beyond the headline size: 4x the cells on 4x the bins
    "4m_cells_2048bins": dict(n_cells=4_000_000, n_nets=4_200_000, n_io=4_000,
                              n_macros=0, util=0.60, target_density=0.75, bins=2048),
}


def generate_workload(name: str, seed: int = 1) -> tuple:
    """Return (netlist, target_density, bin_count) for a named workload."""
    cfg = dict(WORKLOADS[name])
    td = cfg.pop("target_density")
    bins = cfg.pop("bins")
    return generate(seed=seed, **cfg), td, bins


def job_batch(n_jobs: int = 64, seed: int = 4, cells=(2_000, 50_000), density=(0.60, 0.85)):
    """The batched form's instance set: n_jobs netlists from the same
    generator, cell counts log-uniform in `cells`, target densities uniform
    in `density`, bin grids left to the reference's bin-count rule.

    The generator's die is sized for 0.60 utilisation; a job whose target
    density is within 0.02 of that has (almost) no room for fillers and the
    reference stops with code 1, so such jobs are generated at utilisation
    target_density - 0.02 instead.  Returns a list of (netlist, td)."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_jobs):
        n = int(round(np.exp(rng.uniform(np.log(cells[0]), np.log(cells[1])))))
        td = float(rng.uniform(*density))
        util = min(0.60, td - 0.02)
        nl = generate(n_cells=n, n_nets=int(round(1.05 * n)), n_io=200, util=util,
                      seed=seed * 100_003 + k)
        out.append((nl, td))
    return out


def job_stream_spec(n_jobs: int = 500, rate: float = 2.0, seed: int = 5, cells=(5_000, 500_000),
                    density=(0.60, 0.90), macro_share: float = 0.10, macros=(10, 40)):
    """The serving form's request stream: Poisson arrivals at `rate` jobs/s,
    cell counts log-uniform in `cells`, target densities uniform in
    `density`, `macro_share` of the jobs mixed-size with a uniform number of
    macros in `macros`.  Returns a list of dicts (arrival_s, n_cells,
    n_macros, td, seed); `stream_job` builds a job's netlist."""
    rng = np.random.default_rng(seed)
    t = 0.0
    spec = []
    for k in range(n_jobs):
        t += float(rng.exponential(1.0 / rate))
        n = int(round(np.exp(rng.uniform(np.log(cells[0]), np.log(cells[1])))))
        td = float(rng.uniform(*density))
        nm = int(rng.integers(macros[0], macros[1] + 1)) if rng.random() < macro_share else 0
        spec.append({"arrival_s": t, "n_cells": n, "n_macros": nm, "td": td,
                     "seed": seed * 100_003 + k})
    return spec


def stream_job(s: dict) -> Netlist:
    """Netlist of one `job_stream_spec` entry (utilisation as in job_batch)."""
    util = min(0.60, s["td"] - 0.02)
    return generate(n_cells=s["n_cells"], n_nets=int(round(1.05 * s["n_cells"])), n_io=200,
                    n_macros=s["n_macros"], util=util, seed=s["seed"])
