"""Minimal LEF/DEF subset reader (and placement writer) for placement netlists.

Reads what global placement needs from a LEF library and a DEF design:

* LEF: database units, sites, macros (SIZE, per-pin port geometry from RECT and
  POLYGON statements, pin USE).
* DEF: units, die area, rows, components (master, status, location,
  orientation), IO pins (net, layer box, status, location, orientation) and
  nets (component pins, IO pins, USE).

The reader keeps OpenDB's conventions where they change placement results:
LEF coordinates are rounded to database units; an IO pin's box is its layer
rectangle transformed by the pin orientation and moved to the pin location
(the box OpenDB returns from ``dbBPin::getBox``); component pin offsets use the
master's pin geometry without the component orientation, as RePlAce does in
``Pin::updateCoordi(dbITerm*)`` (src/placerBase.cpp:330-376).

Writing back: ``format_components`` prints a COMPONENTS section the way
OpenDB's ``write_def`` does after ``global_placement`` (one line per
component, ``- name master + PLACED ( x y ) N ;``), and ``write_placement``
replaces the COMPONENTS section of an existing DEF with it, keeping every
other byte of the file.  The locations are those NesterovPlace::updateDb
writes into the database (src/nesterovPlace.cpp:585-595).
"""

from __future__ import annotations

import re
from dataclasses import dataclass, field

__all__ = [
    "LefMacro", "LefLibrary", "DefComponent", "DefPin", "DefNet", "DefRow",
    "DefDesign", "read_lef", "read_def", "transform_box", "format_components",
    "placed_components", "write_placement",
]


@dataclass
class LefMacro:
    name: str
    width: int = 0
    height: int = 0
    # pin name -> list of (xl, yl, xh, yh) boxes in master coordinates
    pins: dict = field(default_factory=dict)
    pin_use: dict = field(default_factory=dict)
    pin_order: list = field(default_factory=list)


@dataclass
class LefLibrary:
    dbu: int = 2000
    sites: dict = field(default_factory=dict)      # name -> (w, h) in DBU
    macros: dict = field(default_factory=dict)     # name -> LefMacro


@dataclass
class DefComponent:
    name: str
    master: str
    status: str = "UNPLACED"      # UNPLACED / PLACED / FIXED / COVER / ...
    x: int = 0
    y: int = 0
    orient: str = "N"


@dataclass
class DefPin:
    name: str
    net: str | None
    use: str = "SIGNAL"
    box: tuple | None = None      # absolute (xl, yl, xh, yh) or None if unplaced
    status: str = "UNPLACED"


@dataclass
class DefNet:
    name: str
    conns: list = field(default_factory=list)     # (component name, pin name)
    io_pins: list = field(default_factory=list)   # IO pin names
    use: str = "SIGNAL"


@dataclass
class DefRow:
    name: str
    site: str
    x: int
    y: int
    orient: str
    nx: int
    ny: int
    sx: int
    sy: int


@dataclass
class DefDesign:
    name: str = ""
    dbu: int = 2000
    die: tuple = (0, 0, 0, 0)
    rows: list = field(default_factory=list)
    components: list = field(default_factory=list)
    pins: list = field(default_factory=list)
    nets: list = field(default_factory=list)


def _tokens(text: str):
    # Strip comments, then split on whitespace; parentheses and semicolons
    # become their own tokens.
    text = re.sub(r"#[^\n]*", " ", text)
    text = text.replace("(", " ( ").replace(")", " ) ").replace(";", " ; ")
    return text.split()


def _dbu(v: str, dbu: int) -> int:
    # OpenDB rounds LEF micron values to the nearest database unit.
    f = float(v) * dbu
    return int(f + 0.5) if f >= 0 else -int(-f + 0.5)


def read_lef(paths) -> LefLibrary:
    """Read one or more LEF files into a LefLibrary."""
    if isinstance(paths, str):
        paths = [paths]
    lib = LefLibrary()
    for path in paths:
        with open(path) as f:
            toks = _tokens(f.read())
        i = 0
        n = len(toks)
        while i < n:
            t = toks[i]
            if t == "UNITS":
                while toks[i] != "END":
                    if toks[i] == "DATABASE" and toks[i + 1] == "MICRONS":
                        lib.dbu = int(float(toks[i + 2]))
                    i += 1
                i += 2
            elif t == "SITE":
                name = toks[i + 1]
                i += 2
                w = h = 0
                while not (toks[i] == "END" and toks[i + 1] == name):
                    if toks[i] == "SIZE":
                        w = _dbu(toks[i + 1], lib.dbu)
                        h = _dbu(toks[i + 3], lib.dbu)
                    i += 1
                lib.sites[name] = (w, h)
                i += 2
            elif t == "MACRO":
                i = _read_macro(toks, i, lib)
            elif t in ("LAYER", "VIA", "VIARULE", "NONDEFAULTRULE", "SPACING",
                       "PROPERTYDEFINITIONS"):
                # skip a named block up to its END <name>
                if t in ("SPACING", "PROPERTYDEFINITIONS"):
                    while toks[i] != "END" or toks[i + 1] != t:
                        i += 1
                    i += 2
                else:
                    name = toks[i + 1]
                    i += 2
                    while not (toks[i] == "END" and toks[i + 1] == name):
                        i += 1
                    i += 2
            else:
                i += 1
    return lib


def _read_macro(toks, i, lib):
    name = toks[i + 1]
    m = LefMacro(name)
    i += 2
    while not (toks[i] == "END" and toks[i + 1] == name):
        t = toks[i]
        if t == "SIZE":
            m.width = _dbu(toks[i + 1], lib.dbu)
            m.height = _dbu(toks[i + 3], lib.dbu)
            i += 4
        elif t == "PIN":
            pname = toks[i + 1]
            i += 2
            boxes = []
            use = "SIGNAL"
            while not (toks[i] == "END" and toks[i + 1] == pname):
                if toks[i] == "USE":
                    use = toks[i + 1].upper()
                    i += 2
                elif toks[i] == "RECT":
                    j = i + 1
                    if toks[j] == "MASK":
                        j += 2
                    xs = [_dbu(v, lib.dbu) for v in toks[j:j + 4]]
                    boxes.append((min(xs[0], xs[2]), min(xs[1], xs[3]),
                                  max(xs[0], xs[2]), max(xs[1], xs[3])))
                    i = j + 4
                elif toks[i] == "POLYGON":
                    j = i + 1
                    if toks[j] == "MASK":
                        j += 2
                    pts = []
                    while toks[j] != ";":
                        pts.append(_dbu(toks[j], lib.dbu))
                        j += 1
                    xs, ys = pts[0::2], pts[1::2]
                    # OpenDB splits a pin polygon into boxes whose union is the
                    # polygon; their common bounding box is the polygon's.
                    boxes.append((min(xs), min(ys), max(xs), max(ys)))
                    i = j
                else:
                    i += 1
            m.pins[pname] = boxes
            m.pin_use[pname] = use
            m.pin_order.append(pname)
            i += 2
        elif t == "OBS":
            while toks[i] != "END":
                i += 1
            i += 1
        else:
            i += 1
    lib.macros[name] = m
    return i + 2


# DEF orientation transforms (OpenDB dbTransform):
#   N=R0, S=R180, W=R90, E=R270, FN=MY, FS=MX, FW=MXR90, FE=MYR90
_ORIENT = {
    "N": lambda x, y: (x, y),
    "S": lambda x, y: (-x, -y),
    "W": lambda x, y: (-y, x),
    "E": lambda x, y: (y, -x),
    "FN": lambda x, y: (-x, y),
    "FS": lambda x, y: (x, -y),
    "FW": lambda x, y: (y, x),
    "FE": lambda x, y: (-y, -x),
}


def transform_box(box, orient, dx, dy):
    """Transform a box by a DEF orientation about the origin, then translate."""
    f = _ORIENT[orient]
    x0, y0 = f(box[0], box[1])
    x1, y1 = f(box[2], box[3])
    return (min(x0, x1) + dx, min(y0, y1) + dy,
            max(x0, x1) + dx, max(y0, y1) + dy)


def read_def(path) -> DefDesign:
    """Read the placement-relevant subset of a DEF file."""
    with open(path) as f:
        toks = _tokens(f.read())
    d = DefDesign()
    i = 0
    n = len(toks)
    while i < n:
        t = toks[i]
        if t == "DESIGN" and i + 2 < n and toks[i + 2] == ";":
            d.name = toks[i + 1]
            i += 3
        elif t == "UNITS" and toks[i + 1] == "DISTANCE":
            d.dbu = int(float(toks[i + 3]))
            i += 5
        elif t == "DIEAREA":
            pts = []
            j = i + 1
            while toks[j] != ";":
                if toks[j] == "(":
                    pts.append((int(toks[j + 1]), int(toks[j + 2])))
                    j += 4
                else:
                    j += 1
            xs = [p[0] for p in pts]
            ys = [p[1] for p in pts]
            d.die = (min(xs), min(ys), max(xs), max(ys))
            i = j + 1
        elif t == "ROW":
            name, site = toks[i + 1], toks[i + 2]
            x, y, orient = int(toks[i + 3]), int(toks[i + 4]), toks[i + 5]
            nx = ny = 1
            sx = sy = 0
            j = i + 6
            while toks[j] != ";":
                if toks[j] == "DO":
                    nx, ny = int(toks[j + 1]), int(toks[j + 3])
                    j += 4
                elif toks[j] == "STEP":
                    sx, sy = int(toks[j + 1]), int(toks[j + 2])
                    j += 3
                else:
                    j += 1
            d.rows.append(DefRow(name, site, x, y, orient, nx, ny, sx, sy))
            i = j + 1
        elif t == "COMPONENTS":
            i = _read_components(toks, i + 3, d)
        elif t == "PINS":
            i = _read_pins(toks, i + 3, d)
        elif t == "NETS":
            i = _read_nets(toks, i + 3, d, "NETS")
        elif t == "SPECIALNETS":
            while not (toks[i] == "END" and toks[i + 1] == "SPECIALNETS"):
                i += 1
            i += 2
        elif t in ("PROPERTYDEFINITIONS", "VIAS", "BLOCKAGES", "REGIONS",
                   "GROUPS", "NONDEFAULTRULES", "FILLS"):
            while not (toks[i] == "END" and toks[i + 1] == t):
                i += 1
            i += 2
        else:
            i += 1
    return d


def _read_components(toks, i, d):
    while not (toks[i] == "END" and toks[i + 1] == "COMPONENTS"):
        if toks[i] == "-":
            c = DefComponent(toks[i + 1], toks[i + 2])
            j = i + 3
            while toks[j] != ";":
                if toks[j] == "+" and toks[j + 1] in ("PLACED", "FIXED", "COVER"):
                    c.status = toks[j + 1]
                    c.x, c.y = int(toks[j + 3]), int(toks[j + 4])
                    c.orient = toks[j + 6]
                    j += 7
                elif toks[j] == "+" and toks[j + 1] == "UNPLACED":
                    c.status = "UNPLACED"
                    j += 2
                else:
                    j += 1
            d.components.append(c)
            i = j + 1
        else:
            i += 1
    return i + 2


def _read_pins(toks, i, d):
    while not (toks[i] == "END" and toks[i + 1] == "PINS"):
        if toks[i] == "-":
            name = toks[i + 1]
            net = None
            use = "SIGNAL"
            layer_box = None
            status = "UNPLACED"
            px = py = 0
            orient = "N"
            j = i + 2
            while toks[j] != ";":
                if toks[j] == "+" and toks[j + 1] == "NET":
                    net = toks[j + 2]
                    j += 3
                elif toks[j] == "+" and toks[j + 1] == "USE":
                    use = toks[j + 2].upper()
                    j += 3
                elif toks[j] == "+" and toks[j + 1] == "LAYER":
                    k = j + 3
                    if toks[k] in ("MASK", "SPACING", "DESIGNRULEWIDTH"):
                        k += 2
                    x0, y0 = int(toks[k + 1]), int(toks[k + 2])
                    x1, y1 = int(toks[k + 5]), int(toks[k + 6])
                    layer_box = (min(x0, x1), min(y0, y1), max(x0, x1), max(y0, y1))
                    j = k + 8
                elif toks[j] == "+" and toks[j + 1] in ("PLACED", "FIXED", "COVER"):
                    status = toks[j + 1]
                    px, py = int(toks[j + 3]), int(toks[j + 4])
                    orient = toks[j + 6]
                    j += 7
                else:
                    j += 1
            box = None
            if layer_box is not None and status != "UNPLACED":
                box = transform_box(layer_box, orient, px, py)
            d.pins.append(DefPin(name, net, use, box, status))
            i = j + 1
        else:
            i += 1
    return i + 2


def _read_nets(toks, i, d, section):
    while not (toks[i] == "END" and toks[i + 1] == section):
        if toks[i] == "-":
            net = DefNet(toks[i + 1])
            j = i + 2
            while toks[j] != ";":
                if toks[j] == "(":
                    a, b = toks[j + 1], toks[j + 2]
                    if a == "PIN":
                        net.io_pins.append(b)
                    elif a != "*":
                        net.conns.append((a, b))
                    j += 4
                elif toks[j] == "+" and toks[j + 1] == "USE":
                    net.use = toks[j + 2].upper()
                    j += 3
                elif toks[j] == "+":
                    # skip routing and other net attributes up to the next '+'
                    j += 2
                    while toks[j] not in ("+", ";"):
                        j += 1
                else:
                    j += 1
            d.nets.append(net)
            i = j + 1
        else:
            i += 1
    return i + 2


_FIXED_STATUS = ("FIXED", "COVER", "LOCKED", "FIRM")


def placed_components(components, lx, ly):
    """Components after placement: movable ones (not FIXED / COVER / LOCKED /
    FIRM) move to (lx[k], ly[k]) with status PLACED and keep their
    orientation (N when they had none); fixed ones are unchanged.  lx, ly are
    per component, in DEF order (the first len(components) instances of a
    Netlist read from that DEF)."""
    out = []
    for k, c in enumerate(components):
        if c.status in _FIXED_STATUS:
            out.append(DefComponent(c.name, c.master, c.status, c.x, c.y, c.orient))
        else:
            out.append(DefComponent(c.name, c.master, "PLACED", int(lx[k]), int(ly[k]),
                                    c.orient or "N"))
    return out


def format_components(components) -> str:
    """A COMPONENTS section as OpenDB's write_def prints it."""
    lines = [f"COMPONENTS {len(components)} ;"]
    for c in components:
        if c.status == "UNPLACED":
            lines.append(f"    - {c.name} {c.master} ;")
        else:
            lines.append(f"    - {c.name} {c.master} + {c.status} ( {c.x} {c.y} ) {c.orient} ;")
    lines.append("END COMPONENTS")
    return "\n".join(lines) + "\n"


def write_placement(def_in: str, def_out: str, lx, ly) -> None:
    """Copy DEF `def_in` to `def_out` with its COMPONENTS section replaced by
    the placed components (see placed_components)."""
    with open(def_in) as f:
        text = f.read()
    m = re.search(r"^[ \t]*COMPONENTS\b.*?^[ \t]*END[ \t]+COMPONENTS[^\n]*\n?", text,
                  re.MULTILINE | re.DOTALL)
    if m is None:
        raise ValueError(f"{def_in}: no COMPONENTS section")
    d = read_def(def_in)
    section = format_components(placed_components(d.components, lx, ly))
    with open(def_out, "w") as f:
        f.write(text[:m.start()] + section + text[m.end():])
