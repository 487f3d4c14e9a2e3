"""ORACLE -- test infrastructure.  The zoom exchange on host arrays (FA, Fortran bounds), one
statement per Fortran assignment, in the reference's evaluation order: pydyn
zoom/exchange.py:17-258 and zoom/massflow.py:334-428."""

import numpy as np

TRACERS = ("rm", "rxm", "rym", "rzm")


def _wide(zoom, r):
    g = zoom.g(r)
    return g.im // g.xref == zoom.g(1).im


def _fields(tracers, nt):
    """(name, tracer index or None) of the arrays an exchange statement touches."""
    out = [("m", None)]
    if tracers:
        out += [(q, n) for q in TRACERS for n in range(1, nt + 1)]
    return out


def _plane(fa, n):
    """The 3-d array of a field: m itself, or tracer n (1-based) of a 4-d tracer array."""
    return fa if n is None else _Sub(fa, n)


class _Sub:
    """Tracer n of a 4-d FA, addressed with the first three Fortran indices."""

    def __init__(self, fa, n):
        self.fa, self.n = fa, n

    def __getitem__(self, item):
        return self.fa[(*item, self.n)]

    def __setitem__(self, item, value):
        self.fa[(*item, self.n)] = value

    @property
    def data(self):
        return self.fa.data[..., self.n - self.fa.lower[3]]

    @property
    def lower(self):
        return self.fa.lower[:3]


def _gather(a, i, rows, levs):
    """a(i, rows(:), levs(:)) as an (len(rows), len(levs)) array (Fortran indices)."""
    d, lo = a.data, a.lower
    return d[i - lo[0]][np.ix_(np.asarray(rows) - lo[1], np.asarray(levs) - lo[2])]


def _gather_j(a, cols, j, levs):
    d, lo = a.data, a.lower
    return d[:, j - lo[1]][np.ix_(np.asarray(cols) - lo[0], np.asarray(levs) - lo[2])]


# ------------------------------------------------------------------ put_xedges / put_yedges
def put_xedges(zoom, st, region, tracers=True):
    for child in zoom.children[region]:
        if _wide(zoom, child):
            continue
        gc = zoom.g(child)
        xr, yr, zr = (zoom.ref(child, a) for a in "xyz")
        yzref, xyzref = 1.0 / (yr * zr), 1.0 / (xr * yr * zr)
        rows = [zoom.jbeg[child] + k // yr for k in range(gc.jm)]
        levs = [zoom.lbeg[child] + k // zr for k in range(zoom.lm)]
        ib, ie = zoom.ibeg[child], zoom.iend[child]
        for name, n in _fields(tracers, st.nt):
            p, c = _plane(st[region][name], n), _plane(st[child][name], n)
            inner = xyzref if name in ("m", "rm") else yzref
            west_out, west_in = _gather(p, ib - 1, rows, levs) * yzref, _gather(p, ib, rows, levs) * inner
            east_in, east_out = _gather(p, ie, rows, levs) * inner, _gather(p, ie + 1, rows, levs) * yzref
            c[0, 1 : gc.jm, 1 : zoom.lm] = west_out
            c[gc.im + 1, 1 : gc.jm, 1 : zoom.lm] = east_out
            for i in range(1, xr + 1):
                c[i, 1 : gc.jm, 1 : zoom.lm] = west_in
                c[gc.im + 1 - i, 1 : gc.jm, 1 : zoom.lm] = east_in


def put_yedges(zoom, st, region, tracers=True):
    im_p = zoom.g(region).im
    for child in zoom.children[region]:
        gc = zoom.g(child)
        xr, yr, zr = (zoom.ref(child, a) for a in "xyz")
        xzref, xyzref = 1.0 / (xr * zr), 1.0 / (xr * yr * zr)
        cols = [(zoom.ibeg[child] - 1 + k // xr) % im_p + 1 for k in range(gc.im)]
        levs = [zoom.lbeg[child] + k // zr for k in range(zoom.lm)]
        jb, je = zoom.jbeg[child], zoom.jend[child]
        for name, n in _fields(tracers, st.nt):
            p, c = _plane(st[region][name], n), _plane(st[child][name], n)
            inner = xyzref if name in ("m", "rm") else xzref
            south_out, south_in = _gather_j(p, cols, jb - 1, levs) * xzref, _gather_j(p, cols, jb, levs) * inner
            north_in, north_out = _gather_j(p, cols, je, levs) * inner, _gather_j(p, cols, je + 1, levs) * xzref
            c[1 : gc.im, 0, 1 : zoom.lm] = south_out
            c[1 : gc.im, gc.jm + 1, 1 : zoom.lm] = north_out
            for j in range(1, yr + 1):
                c[1 : gc.im, j, 1 : zoom.lm] = south_in
                c[1 : gc.im, gc.jm + 1 - j, 1 : zoom.lm] = north_in


# ------------------------------------------------------------------ compress / uncompress
def _running_sum(parts):
    acc = parts[0].copy()
    for p in parts[1:]:
        acc = acc + p
    return acc


def compress_xedges(zoom, st, region, js, je, ls, le, tracers=True):
    xr, g = zoom.ref(region, "x"), zoom.g(region)
    if xr == 1 or _wide(zoom, region):
        return
    im = g.im
    names = ["m"] + (list(TRACERS) if tracers else [])
    for name in names:
        for n in [None] if name == "m" else range(1, st.nt + 1):
            q = _plane(st[region][name], n)
            if name in ("m", "rm"):
                q[xr, js:je, ls:le] = _running_sum([q[i, js:je, ls:le] for i in range(1, xr + 1)])
                if name == "m":
                    q[xr - 1, js:je, ls:le] = q[0, js:je, ls:le]
                q[im - xr + 1, js:je, ls:le] = _running_sum([q[i, js:je, ls:le] for i in range(im - xr + 1, im + 1)])
                if name == "m":
                    q[im - xr + 2, js:je, ls:le] = q[im + 1, js:je, ls:le]
            if name != "m":
                q[xr - 1, js:je, ls:le] = q[0, js:je, ls:le]
                q[im - xr + 2, js:je, ls:le] = q[im + 1, js:je, ls:le]


def uncompress_xedges(zoom, st, region, js, je, ls, le, tracers=True):
    xr, g = zoom.ref(region, "x"), zoom.g(region)
    if xr == 1 or _wide(zoom, region):
        return
    im = g.im
    for name, n in _fields(tracers, st.nt):
        q = _plane(st[region][name], n)
        for lo, hi, edge in ((1, xr, xr), (im - xr + 1, im, im - xr + 1)):
            v = q[edge, js:je, ls:le].copy() / xr
            for i in range(lo, hi + 1):
                q[i, js:je, ls:le] = v


def compress_yedges(zoom, st, region, is_, ie, ls, le, tracers=True):
    yr, g = zoom.ref(region, "y"), zoom.g(region)
    if yr == 1 or region == 1:
        return
    jm = g.jm
    names = ["m"] + (list(TRACERS) if tracers else [])
    for name in names:
        for n in [None] if name == "m" else range(1, st.nt + 1):
            q = _plane(st[region][name], n)
            if name in ("m", "rm"):
                q[is_:ie, yr, ls:le] = _running_sum([q[is_:ie, j, ls:le] for j in range(1, yr + 1)])
                if name == "m":
                    q[is_:ie, yr - 1, ls:le] = q[is_:ie, 0, ls:le]
                q[is_:ie, jm - yr + 1, ls:le] = _running_sum([q[is_:ie, j, ls:le] for j in range(jm - yr + 1, jm + 1)])
                if name == "m":
                    q[is_:ie, jm - yr + 2, ls:le] = q[is_:ie, jm + 1, ls:le]
            if name != "m":
                q[is_:ie, yr - 1, ls:le] = q[is_:ie, 0, ls:le]
                q[is_:ie, jm - yr + 2, ls:le] = q[is_:ie, jm + 1, ls:le]


def uncompress_yedges(zoom, st, region, is_, ie, ls, le, tracers=True):
    yr, g = zoom.ref(region, "y"), zoom.g(region)
    if yr == 1 or region == 1:
        return
    jm = g.jm
    for name, n in _fields(tracers, st.nt):
        q = _plane(st[region][name], n)
        for lo, hi, edge in ((1, yr, yr), (jm - yr + 1, jm, jm - yr + 1)):
            v = q[is_:ie, edge, ls:le].copy() / yr
            for j in range(lo, hi + 1):
                q[is_:ie, j, ls:le] = v


# ------------------------------------------------------------------ mix_edges, update_parent
def mix_edges(zoom, st, region, tracers=True):
    g = zoom.g(region)
    xr, yr, zr = (zoom.ref(region, a) for a in "xyz")
    if zr != 1:
        raise ValueError("mix_edges: zooming in z direction not supported!")
    xedges = not (xr == 1 or _wide(zoom, region))
    if not xedges and region == 1:
        return
    ysp, ynp = g.touch_sp != 1, g.touch_np != 1
    imp, jmp = g.im // xr, g.jm // yr
    blocks = [(ip, jp) for ip in range(imp) for jp in range(jmp)
              if (xedges and ip in (0, imp - 1)) or (ysp and jp == 0) or (ynp and jp == jmp - 1)]  # fmt: skip
    for name, n in _fields(tracers, st.nt):
        q = _plane(st[region][name], n)
        for ip, jp in blocks:
            i0, j0 = ip * xr + 1, jp * yr + 1
            acc = np.zeros(zoom.lm)
            for b in range(yr):
                for a in range(xr):
                    acc = acc + q[i0 + a, j0 + b, 1 : zoom.lm] / (xr * yr)
            for b in range(yr):
                for a in range(xr):
                    q[i0 + a, j0 + b, 1 : zoom.lm] = acc


def update_parent(zoom, st, region, tracers=True):
    if region == 1:
        return
    g, parent = zoom.g(region), zoom.g(region).parent
    xr, yr, zr = (zoom.ref(region, a) for a in "xyz")
    if zr != 1:
        raise ValueError("update_parent: zooming in z direction not supported")
    imp, jmp, lm = g.im // xr, g.jm // yr, zoom.lm
    ib, jb = zoom.ibeg[region], zoom.jbeg[region]
    names = [("m", None)] + ([("rm", n) for n in range(1, st.nt + 1)] if tracers else [])
    for name, n in names:
        c, p = _plane(st[region][name], n), _plane(st[parent][name], n)
        for ip in range(imp):
            for jp in range(jmp):
                acc = np.zeros(lm)
                for a in range(xr):
                    for b in range(yr):
                        acc = acc + c[ip * xr + a + 1, jp * yr + b + 1, 1:lm]
                p[ib + ip, jb + jp, 1:lm] = acc


# ------------------------------------------------------------------ coarsen_block, coarsen_ambm
def coarsen_block(zoom, st, region):
    parent = zoom.g(region).parent
    g, f, p = zoom.g(region), st[region], st[parent]
    xr, yr, zr, tr = (zoom.ref(region, a) for a in "xyzt")
    if zr != 1:
        raise ValueError("coarsen_region: zooming in z direction not supported")
    imp, jmp, lm = g.im // xr, g.jm // yr, zoom.lm
    ib, jb, lb = zoom.ibeg[region], zoom.jbeg[region], zoom.lbeg[region]
    im_par = zoom.g(parent).im

    def wrap(i):
        return (i - 1) % im_par + 1

    levs = slice(lb, lb + lm - 1)
    for ip in range(imp + 1):  # am: child faces ip*xr, summed over the block's rows
        for jp in range(jmp):
            top = np.zeros(lm)
            for b in range(yr):
                top = top + f["am"][ip * xr, jp * yr + b + 1, 1:lm] * tr
            p["am"][wrap(ib - 1 + ip), jb + jp, levs] = top
    for ip in range(imp):  # bm: child faces 1 + jp*yr, summed over the block's columns
        for jp in range(jmp + 1):
            top = np.zeros(lm)
            for a in range(xr):
                top = top + f["bm"][ip * xr + a + 1, jp * yr + 1, 1:lm] * tr
            p["bm"][wrap(ib + ip), jb + jp, levs] = top
    for ip in range(imp):
        for jp in range(jmp):
            top = np.zeros(lm)  # cm: interfaces 1..lm, i outer / j inner
            for a in range(xr):
                for b in range(yr):
                    top = top + f["cm"][ip * xr + a + 1, jp * yr + b + 1, 1:lm] * tr
            p["cm"][wrap(ib + ip), jb + jp, levs] = top
            top = np.zeros(lm)  # m: j outer / i inner
            for b in range(yr):
                for a in range(xr):
                    top = top + f["m"][ip * xr + a + 1, jp * yr + b + 1, 1:lm]
            p["m"][wrap(ib + ip), jb + jp, levs] = top


def coarsen_ambm(zoom, st, region):
    am, bm = st[region]["am"], st[region]["bm"]
    for child in zoom.children[region]:
        gc = zoom.g(child)
        xr, yr, zr = (zoom.ref(child, a) for a in "xyz")
        ib, ie, jb, je = zoom.ibeg[child], zoom.iend[child], zoom.jbeg[child], zoom.jend[child]
        lb, le = zoom.lbeg[child], zoom.lend[child]
        amc, bmc = st[child]["am"], st[child]["bm"]
        if not _wide(zoom, child):
            for j in range(jb, je + 1):
                for lev in range(lb, le + 1):
                    jc, lc = (j - jb) * yr + 1, (lev - lb) * zr + 1
                    amc[xr - 1, jc : jc + yr - 1, lc : lc + zr - 1] = am[ib - 1, j, lev] / (yr * zr)
                    amc[gc.im - xr + 1, jc : jc + yr - 1, lc : lc + zr - 1] = am[ie, j, lev] / (yr * zr)
        for i in range(ib, ie + 1):
            for lev in range(lb, le + 1):
                ic, lc = (i - ib) * xr + 1, (lev - lb) * zr + 1
                if gc.touch_sp != 1:
                    bmc[ic : ic + xr - 1, yr, lc : lc + zr - 1] = bm[i, jb, lev] / (xr * zr)
                if gc.touch_np != 1:
                    bmc[ic : ic + xr - 1, gc.jm - yr + 2, lc : lc + zr - 1] = bm[i, je + 1, lev] / (xr * zr)
