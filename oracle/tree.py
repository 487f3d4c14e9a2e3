"""ORACLE -- test infrastructure.  A restatement of pydyn's region tree: the regions' dims_grid
parameters and what TM5's initexit derives from them (children, footprints, interior scopes, the
zoomed/edge maps, the per-region operator order), with the constructor and attribute names of
pydyn's zoom.Zoom (pydyn zoom/tree.py:53-191), and the reduced grid of a region (pydyn
redgrid.py:27-53).  The oracle's bodies read it; the product derives the same tree its own way
(pydyn_gb300.tree) and the tests compare the two."""

import math
from dataclasses import dataclass

import numpy as np

SPLITORDER = "xyzvsccsvzyx"  # dims.F90 splitorder (pydyn zoom/tree.py:18)
N_OPERATORS = len(SPLITORDER) // 2
CFL_SPLITORDER = "xyzzyx"  # advectm_cfl.F90 (pydyn zoom/check_cfl.py:38-39)
CFL_N_OPERATORS = 3


def nint(x):
    """Fortran nint: half away from zero (pydyn ops.py:78-80)."""
    return math.floor(abs(x) + 0.5) * (1 if x >= 0 else -1)


class RedGrid:
    """A region's reduced grid: latitude j (1-based in jred) advected in x as im / clustsize
    cluster cells (pydyn redgrid.py:27-53).  `clust` is the per-latitude cluster size (1 where
    the row is uniform), the form the device kernel takes."""

    def __init__(self, im, jm, jred, clustsize):
        self.im, self.jm = im, jm
        self.bands = []
        self.imred = np.full(jm, im, dtype=int)
        self.clust = np.ones(jm, dtype=np.int32)
        for j, c in zip(jred, clustsize, strict=True):
            if im % c:
                raise ValueError(f"redgrid: im={im} not a multiple of clustsize {c}")
            self.bands.append((j - 1, c, im // c))
            self.imred[j - 1] = im // c
            self.clust[j - 1] = c

    @property
    def rows(self):
        return [b[0] for b in self.bands]


@dataclass
class Region:
    """One region: refinements absolute (relative to the globe); parent 0 is the globe."""

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


class Zoom:
    """The region tree (regions numbered from 1).  Attributes as pydyn's: children, ibeg, iend,
    jbeg, jend, lbeg, lend, isr, ier, jsr, jer, zoomed, edge, splitorderzoom, status."""

    def __init__(self, regions, lm, at=None, bt=None, splitorder=SPLITORDER):
        self.region = [None, *regions]
        self.nregions = len(regions)
        self.lm = lm
        self.at = np.zeros(lm + 1) if at is None else np.asarray(at, dtype=float)
        self.bt = np.zeros(lm + 1) if bt is None else np.asarray(bt, dtype=float)
        self.status = [0] * (self.nregions + 1)
        self._geometry()
        self.zoomed, self.edge = {}, {}
        for r in self.regions():
            self.zoomed[r], self.edge[r] = self._maps(r)
        self.splitorderzoom = self.split_orders(splitorder, N_OPERATORS)
        self._check()

    def regions(self):
        return range(1, self.nregions + 1)

    def g(self, r):
        return self.region[r] if r > 0 else Region("globe", self.region[1].im, self.region[1].jm)

    def ref(self, r, axis):
        """Refinement of r relative to its parent along 'x', 'y', 'z' or 't' (integer division)."""
        g, p = self.g(r), self.g(self.g(r).parent)
        return getattr(g, axis + "ref") // getattr(p, axis + "ref")

    # initexit determine_children_etc (pydyn zoom/tree.py:93-129)
    def _geometry(self):
        n = self.nregions
        self.children = {r: [] for r in range(n + 1)}
        for r in range(2, n + 1):
            self.children[self.g(r).parent].append(r)
        self.ibeg, self.iend, self.jbeg, self.jend, self.lbeg, self.lend = {}, {}, {}, {}, {}, {}
        g1 = self.g(1)
        dx = (g1.xend - g1.xbeg) / g1.im * g1.xref
        dy = (g1.yend - g1.ybeg) / g1.jm * g1.yref
        for r in range(2, n + 1):
            g, p = self.g(r), self.g(self.g(r).parent)
            self.ibeg[r] = nint((g.xbeg - p.xbeg) / (dx / p.xref)) + 1
            self.jbeg[r] = nint((g.ybeg - p.ybeg) / (dy / p.yref)) + 1
            self.iend[r] = nint((g.xend - p.xbeg) / (dx / p.xref))
            self.jend[r] = nint((g.yend - p.ybeg) / (dy / p.yref))
            self.lbeg[r], self.lend[r] = 1, self.lm
            xr, yr = self.ref(r, "x"), self.ref(r, "y")
            icells = (self.iend[r] - self.ibeg[r] + 1 if self.iend[r] > self.ibeg[r]
                      else p.im - self.ibeg[r] + 1 + self.iend[r])  # fmt: skip
            if icells * xr != g.im:
                raise ValueError(f"region {r}: check xbeg/xend, im and ibeg/iend")
            if (self.jend[r] - self.jbeg[r] + 1) * yr != g.jm:
                raise ValueError(f"region {r}: check ybeg/yend, jm and jbeg/jend")
        self.isr, self.ier, self.jsr, self.jer = {1: 1}, {1: g1.im}, {1: 1}, {1: g1.jm}
        for r in range(2, n + 1):
            g, xr, yr = self.g(r), self.ref(r, "x"), self.ref(r, "y")
            self.isr[r], self.ier[r] = (1, g.im) if g.xcyc else (xr + 1, g.im - xr)
            self.jsr[r] = 1 if g.touch_sp == 1 else yr + 1
            self.jer[r] = g.jm if g.touch_np == 1 else g.jm - yr

    # initexit blank_zoom_region (pydyn zoom/tree.py:131-164): 0-based (im, jm) maps
    def _maps(self, r):
        g = self.g(r)
        zoomed = np.full((g.im, g.jm), r, dtype=np.int32)
        edge = np.zeros((g.im, g.jm), dtype=np.int32)
        for c in self.children[r]:
            gc = self.g(c)
            ib, ie, jb, je = self.ibeg[c], self.iend[c], self.jbeg[c], self.jend[c]
            i = np.arange(1, g.im + 1)[:, None]
            j = np.arange(1, g.jm + 1)[None, :]
            inside_i = (i > ib) & (i < ie) if gc.xcyc != 1 else np.ones_like(i, dtype=bool)
            inside_j = ((j > jb) | (gc.touch_sp == 1)) & ((j < je) | (gc.touch_np == 1))
            zoomed[inside_i & inside_j] = c
            if gc.xcyc != 1:
                edge[ib - 1, jb - 1 : je] = 1
                edge[ie - 1, jb - 1 : je] = 1
            if gc.touch_sp != 1:
                edge[ib - 1 : ie, jb - 1] += 2
            if gc.touch_np != 1:
                edge[ib - 1 : ie, je - 1] += 2
        if g.parent != 0:
            xr, yr = self.ref(r, "x"), self.ref(r, "y")
            if g.xcyc != 1:
                edge[:xr, :] = -1
                edge[g.im - xr :, :] = -1
            if g.touch_sp != 1:
                edge[:, :yr] = -1
            if g.touch_np != 1:
                edge[:, g.jm - yr :] = -1
        return zoomed, edge

    def split_orders(self, splitorder, n_operators):
        """define_splitorderzoom, zoom_mode 1: each child repeats its parent's blocks tref_
        times, the even copies reversed (pydyn zoom/tree.py:166-180, check_cfl.py:42-54)."""
        order = {1: splitorder}
        for r in range(2, self.nregions + 1):
            tref_ = self.ref(r, "t")
            if tref_ > 4 or tref_ == 3:
                raise ValueError(f"define_splitorderzoom: region {r}: tref_ = {tref_} not 1, 2 or 4")
            parent = order[self.g(r).parent]
            blocks = [parent[k : k + n_operators] for k in range(0, len(parent), n_operators)]
            order[r] = "".join(b if i % 2 == 1 else b[::-1] for b in blocks for i in range(1, tref_ + 1))
        return order

    def _check(self):
        g1 = self.g(1)
        if not (g1.xcyc == 1 and g1.touch_sp == 1 and g1.touch_np == 1):
            raise NotImplementedError("region 1 must be global: cyclic and touching both poles")
        for r in range(2, self.nregions + 1):
            g, p = self.g(r), self.g(self.g(r).parent)
            if g.xcyc or g.touch_sp or g.touch_np:
                raise NotImplementedError(f"region {r}: cyclic or pole-touching children are not supported")
            if self.ibeg[r] >= self.iend[r]:
                raise NotImplementedError(f"region {r}: a child across the dateline is not supported")
            if self.ibeg[r] <= 1 or self.iend[r] >= p.im:
                raise NotImplementedError(f"region {r}: put_xedges would read the parent's halo")
            if self.jbeg[r] <= 1 or self.jend[r] >= p.jm:
                raise NotImplementedError(f"region {r}: put_yedges would read the parent's halo")
            if g.redgrid is not None:
                raise NotImplementedError(f"region {r}: a reduced grid in a child is not supported")

    # the scopes of the physics (pydyn zoom/physics.py:17-28)
    def scope(self, r):
        """The interior scope isr:ier x jsr:jer as 0-based slices of an (im, jm) array."""
        return slice(self.isr[r] - 1, self.ier[r]), slice(self.jsr[r] - 1, self.jer[r])

    def owned(self, r):
        """(im, jm) bool: the scope's cells the region owns (zoomed == r)."""
        g = self.g(r)
        own = np.zeros((g.im, g.jm), dtype=bool)
        own[self.scope(r)] = True
        return own & (self.zoomed[r] == r)
