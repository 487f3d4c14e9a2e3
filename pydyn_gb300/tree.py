"""The region tree as one flat table.

TM5's dims_grid gives each region its shape, its corner coordinates and its refinement against
the globe; initexit derives from those where a child sits in its parent (the footprint), which
of its cells it updates itself (the scope), which of the parent's cells it covers (the `zoomed`
map) and where its edge ring lies (the `edge` map), and in which order each region runs the
operators (pydyn zoom/tree.py:53-191 transcribes that derivation).

Here every derived integer of a region is one row of `Zoom.table`, a NumPy structured array
indexed by region number (row 0 is the globe).  The step planner (pydyn_gb300.plan), the stream
scheduler (pydyn_gb300.schedule) and the device bodies read the rows; the per-region mappings
pydyn's bodies read (`children`, `ibeg` .. `jer`, `zoomed`, `edge`, `splitorderzoom`, `status`)
are views built from the table once.  Pure host geometry."""

import math
from typing import NamedTuple

import numpy as np

SPLITORDER = "xyzvsccsvzyx"  # TM5 dims.F90: the two half steps' operator order
N_OPERATORS = len(SPLITORDER) // 2
CFL_SPLITORDER = "xyzzyx"  # TM5 advectm_cfl.F90: Check_CFL's mass-only rehearsal
CFL_N_OPERATORS = 3

ROW = np.dtype([(name, np.int32) for name in (
    "parent", "depth", "im", "jm", "xr", "yr", "tr",  # shape, refinement relative to the parent
    "ibeg", "iend", "jbeg", "jend",  # footprint in the parent's cells (1-based, inclusive)
    "isr", "ier", "jsr", "jer",  # scope: the region's own cells it updates (1-based, inclusive)
    "xcyc", "touch_sp", "touch_np",
)])  # fmt: skip


def nint(x):
    """Fortran NINT: the nearest integer, halves away from zero."""
    whole = math.floor(abs(x) + 0.5)
    return whole if x >= 0 else -whole


class RedGrid:
    """A region's reduced grid: the latitude rows (1-based `jred`) whose x advection merges
    `clustsize` cells into one (pydyn redgrid.py:27-53).  `clust` is the cluster size of every
    row (1 on a uniform row), the form the x kernels take; `bands` lists (0-based row, cluster
    size, reduced cells)."""

    def __init__(self, im, jm, jred, clustsize):
        if len(jred) != len(clustsize):
            raise ValueError("redgrid: jred and clustsize differ in length")
        self.im, self.jm = im, jm
        self.clust = np.ones(jm, dtype=np.int32)
        for j, c in zip(jred, clustsize, strict=True):
            if im % c:
                raise ValueError(f"redgrid: clustsize {c} does not divide im = {im}")
            self.clust[j - 1] = c
        self.bands = [(j - 1, c, im // c) for j, c in zip(jred, clustsize, strict=True)]
        self.imred = im // self.clust.astype(int)

    @property
    def rows(self):
        return [row for row, _, _ in self.bands]


class Region(NamedTuple):
    """A region as dims_grid describes it: cells (im, jm), corners in degrees, refinements
    relative to the globe, the parent's number (0: the globe), whether it is cyclic in x and
    touches a pole, and an optional reduced grid.  Frozen: the tree's table is derived from it
    once."""

    name: str
    im: int
    jm: int
    xbeg: float = -180.0
    xend: float = 180.0
    ybeg: float = -90.0
    yend: float = 90.0
    xref: int = 1
    yref: int = 1
    zref: int = 1
    tref: int = 1
    parent: int = 0
    xcyc: int = 0
    touch_sp: int = 0
    touch_np: int = 0
    redgrid: object = None


def _expand_order(order, block, tref):
    """A child's operator order: every block of its parent's order done tref times over, the
    second, fourth ... time backwards (zoom_mode 1 of define_splitorderzoom)."""
    out = []
    for start in range(0, len(order), block):
        ops = order[start : start + block]
        out.extend(ops[:: 1 - 2 * (k % 2)] for k in range(tref))
    return "".join(out)


class Zoom:
    """The region tree.  Regions are numbered from 1; `table[r]` holds region r's derived
    integers, `g(r)` its Region."""

    def __init__(self, regions, lm, at=None, bt=None, splitorder=SPLITORDER):
        self.region = [None, *regions]
        self.nregions = len(regions)
        self.lm = lm
        self.at = np.zeros(lm + 1) if at is None else np.asarray(at, dtype=float)
        self.bt = np.zeros(lm + 1) if bt is None else np.asarray(bt, dtype=float)
        self.status = [0] * (self.nregions + 1)
        self.table = self._table()
        self._refuse_unsupported()
        t = self.table
        self.children = {r: [] for r in range(self.nregions + 1)}
        for c in range(2, self.nregions + 1):
            self.children[int(t["parent"][c])].append(c)
        for name in ("ibeg", "iend", "jbeg", "jend"):
            setattr(self, name, {r: int(t[name][r]) for r in range(2, self.nregions + 1)})
        self.lbeg = {r: 1 for r in range(2, self.nregions + 1)}
        self.lend = {r: lm for r in range(2, self.nregions + 1)}
        for name in ("isr", "ier", "jsr", "jer"):
            setattr(self, name, {r: int(t[name][r]) for r in self.regions()})
        self.zoomed, self.edge = {}, {}
        for r in self.regions():
            self.zoomed[r], self.edge[r] = self._paint(r)
        self.splitorderzoom = self.split_orders(splitorder, N_OPERATORS)

    def regions(self):
        return range(1, self.nregions + 1)

    def g(self, r):
        """Region r (r = 0: the globe, every refinement 1)."""
        return self.region[r] if r > 0 else Region("globe", self.region[1].im, self.region[1].jm)

    def ref(self, r, axis):
        """Region r's refinement against its parent along 'x', 'y', 'z' or 't'."""
        if axis == "z":
            return self.g(r).zref // self.g(self.g(r).parent).zref
        return int(self.table[axis + "r"][r])

    # -------------------------------------------------------------- the table
    def _table(self):
        t = np.zeros(self.nregions + 1, dtype=ROW)
        top = self.region[1]
        t[0] = (0, -1, top.im, top.jm, 1, 1, 1, 0, 0, 0, 0, 1, top.im, 1, top.jm, 1, 1, 1)
        # the globe's cell at refinement 1, in degrees: the footprints are counted in it
        cell_x = (top.xend - top.xbeg) / top.im * top.xref
        cell_y = (top.yend - top.ybeg) / top.jm * top.yref
        for r in self.regions():
            g = self.region[r]
            p = self.g(g.parent)
            if r > 1 and not 1 <= g.parent < r:
                raise ValueError(f"region {r}: its parent must be a region numbered before it")
            row = t[r]
            row["parent"], row["im"], row["jm"] = g.parent, g.im, g.jm
            row["depth"] = 0 if r == 1 else t["depth"][g.parent] + 1
            row["xr"], row["yr"], row["tr"] = g.xref // p.xref, g.yref // p.yref, g.tref // p.tref
            row["xcyc"], row["touch_sp"], row["touch_np"] = g.xcyc, g.touch_sp, g.touch_np
            if r == 1:
                row["isr"], row["ier"], row["jsr"], row["jer"] = 1, g.im, 1, g.jm
                continue
            # footprint: the parent cells between the child's corners (Fortran nint of the offset)
            px, py = cell_x / p.xref, cell_y / p.yref
            row["ibeg"] = nint((g.xbeg - p.xbeg) / px) + 1
            row["iend"] = nint((g.xend - p.xbeg) / px)
            row["jbeg"] = nint((g.ybeg - p.ybeg) / py) + 1
            row["jend"] = nint((g.yend - p.ybeg) / py)
            ncols = row["iend"] - row["ibeg"] + 1
            if row["iend"] <= row["ibeg"]:  # across the parent's dateline
                ncols += p.im
            if ncols * row["xr"] != g.im:
                raise ValueError(f"region {r}: {g.im} cells do not cover {ncols} parent columns at xref {row['xr']}")
            if (row["jend"] - row["jbeg"] + 1) * row["yr"] != g.jm:
                raise ValueError(f"region {r}: {g.jm} cells do not cover parent rows {row['jbeg']}..{row['jend']} "
                                 f"at yref {row['yr']}")  # fmt: skip
            # scope: all but the ring of one parent cell a side the region shares with its parent
            row["isr"], row["ier"] = (1, g.im) if g.xcyc else (row["xr"] + 1, g.im - row["xr"])
            row["jsr"] = 1 if g.touch_sp == 1 else row["yr"] + 1
            row["jer"] = g.jm if g.touch_np == 1 else g.jm - row["yr"]
        return t

    def _refuse_unsupported(self):
        """The trees the device bodies handle: a global region 1 and children inside their
        parent's interior, neither cyclic nor at a pole nor on a reduced grid."""
        top = self.region[1]
        if (top.xcyc, top.touch_sp, top.touch_np) != (1, 1, 1):
            raise NotImplementedError("region 1 must be global: cyclic and touching both poles")
        for r in range(2, self.nregions + 1):
            g, row = self.region[r], self.table[r]
            p = self.table[g.parent]
            if g.xcyc or g.touch_sp or g.touch_np:
                raise NotImplementedError(f"region {r}: cyclic or pole-touching children are not supported")
            if row["ibeg"] >= row["iend"]:
                raise NotImplementedError(f"region {r}: a child that crosses the dateline is not supported")
            if not (1 < row["ibeg"] and row["iend"] < p["im"] and 1 < row["jbeg"] and row["jend"] < p["jm"]):
                raise NotImplementedError(f"region {r}: its footprint touches its parent's boundary (the edge "
                                          "exchange would reach into the parent's halo)")  # fmt: skip
            if g.redgrid is not None:
                raise NotImplementedError(f"region {r}: a child on a reduced grid is not supported")
            if self.table["tr"][r] not in (1, 2, 4):
                raise ValueError(f"region {r}: its time refinement against its parent must be 1, 2 or 4")

    # -------------------------------------------------------------- maps and orders
    def _paint(self, r):
        """(zoomed, edge) of region r as 0-based (im, jm) int32 maps: a cell covered by a child's
        interior carries the child's number; a child's boundary columns of its footprint carry 1,
        its boundary rows 2 (3 at a corner); a child's own ring of one parent cell carries -1."""
        row = self.table[r]
        zoomed = np.full((row["im"], row["jm"]), r, dtype=np.int32)
        edge = np.zeros((row["im"], row["jm"]), dtype=np.int32)
        for c in self.children[r]:
            k = self.table[c]
            i0, i1, j0, j1 = k["ibeg"] - 1, k["iend"] - 1, k["jbeg"] - 1, k["jend"] - 1  # 0-based, inclusive
            inner_i = slice(None) if k["xcyc"] == 1 else slice(i0 + 1, i1)
            inner_j = slice(None if k["touch_sp"] == 1 else j0 + 1, None if k["touch_np"] == 1 else j1)
            zoomed[inner_i, inner_j] = c
            if k["xcyc"] != 1:
                edge[[i0, i1], j0 : j1 + 1] = 1
            for flag, j in ((k["touch_sp"], j0), (k["touch_np"], j1)):
                if flag != 1:
                    edge[i0 : i1 + 1, j] += 2
        if r > 1:
            xr, yr = row["xr"], row["yr"]
            if row["xcyc"] != 1:
                edge[:xr] = -1
                edge[row["im"] - xr :] = -1
            if row["touch_sp"] != 1:
                edge[:, :yr] = -1
            if row["touch_np"] != 1:
                edge[:, row["jm"] - yr :] = -1
        return zoomed, edge

    def split_orders(self, splitorder, n_operators):
        """{region: its operator order}: region 1 runs `splitorder`; a child expands its parent's
        order block by block (blocks of n_operators) by its time refinement."""
        order = {1: splitorder}
        for r in range(2, self.nregions + 1):
            order[r] = _expand_order(order[int(self.table["parent"][r])], n_operators, int(self.table["tr"][r]))
        return order

    # -------------------------------------------------------------- the physics' cells
    def scope(self, r):
        """Region r's scope as 0-based slices of an (im, jm) array."""
        return slice(self.isr[r] - 1, self.ier[r]), slice(self.jsr[r] - 1, self.jer[r])

    def owned(self, r):
        """(im, jm) bool: the scope's cells no child covers."""
        own = np.zeros((self.table["im"][r], self.table["jm"][r]), dtype=bool)
        own[self.scope(r)] = True
        return own & (self.zoomed[r] == r)
