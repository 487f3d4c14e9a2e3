"""ORACLE -- test infrastructure.  A restatement of pydyn's driver: the operator sequence of a
dynamic step and of Check_CFL on a region tree as pydyn runs it (pydyn zoom/steps.py:29-88,
zoom/advect.py:42-199, zoom/check_cfl.py:32-290, zoom/massflow.py:61-73 and 174-184, cfl.py:208-213),
calling the bodies through `st.lib` with pydyn's signatures and consuming their returns as
pydyn does: a mass-only body's return is the rehearsal's ok flag for its region, and the
rehearsal unwinds at the first failure.

It drives the oracle's host bodies (oracle.zoom) for the oracle's whole intervals, and the
device bodies (pydyn_gb300.zoom) in the tests that hold the device module to pydyn's body
contract.  The product plans its own sequence (pydyn_gb300.plan); the tests compare the two."""

from .tree import CFL_N_OPERATORS, CFL_SPLITORDER, N_OPERATORS, nint

__all__ = [
    "advect_x_zoom",
    "advect_y_zoom",
    "advect_z_zoom",
    "check_cfl_zoom",
    "coarsen_region",
    "do_steps",
    "new_valid_timestep",
    "proces_region",
    "setup_massflow",
    "step",
]


# ------------------------------------------------------------------ the scope of an advection call
def _block(zoom, region, status=None, order=None, n_ops=N_OPERATORS):
    """The operators of the current block of the region's order (advect*zoom's q), tref_."""
    tref_ = zoom.ref(region, "t")
    s = zoom.status[region] if status is None else status
    order = zoom.splitorderzoom[region] if order is None else order
    start = (s // (n_ops * tref_)) * n_ops * tref_
    return order[start : start + n_ops], tref_


def _second_half(zoom, region, status=None, n_ops=N_OPERATORS):
    """The coarse flux has crossed the interface already: mod(status, n_ops tref_) >= n_ops."""
    s = zoom.status[region] if status is None else status
    return s % (n_ops * zoom.ref(region, "t")) >= n_ops


def x_scope(zoom, region, block):
    """advectxzoom's rows (js, je): all when y comes before x, else inside the y refinement."""
    g = zoom.g(region)
    yr = 0 if region == 1 else zoom.ref(region, "y")
    x_seen, js, je = False, None, None
    for d in block:
        if d == "x":
            x_seen = True
        elif d == "y":
            if not x_seen:
                js, je = 1, g.jm
            else:
                js = 1 if g.touch_sp == 1 else yr + 1
                je = g.jm if g.touch_np == 1 else g.jm - yr
    return js, je


def y_scope(zoom, region, block):
    """advectyzoom's columns (is_, ie)."""
    g = zoom.g(region)
    xr = 0 if region == 1 else zoom.ref(region, "x")
    y_seen, is_, ie = False, None, None
    for d in block:
        if d == "x":
            is_, ie = (1, g.im) if (not y_seen or g.xcyc == 1) else (xr + 1, g.im - xr)
        elif d == "y":
            y_seen = True
    return is_, ie


def z_scope(zoom, region, block):
    """advectzzoom's (is_, ie, js, je): a direction's full range when it comes after z."""
    g = zoom.g(region)
    xr, yr = (0, 0) if region == 1 else (zoom.ref(region, "x"), zoom.ref(region, "y"))
    z_seen = False
    is_ = ie = js = je = None
    for d in block:
        if d == "x":
            is_, ie = (1, g.im) if (not z_seen or g.xcyc == 1) else (xr + 1, g.im - xr)
        elif d == "y":
            if not z_seen:
                js, je = 1, g.jm
            else:
                js = 1 if g.touch_sp == 1 else yr + 1
                je = g.jm if g.touch_np == 1 else g.jm - yr
        elif d == "z":
            z_seen = True
    return is_, ie, js, je


# ------------------------------------------------------------------ advect{x,y,z}zoom
def advect_x_zoom(zoom, st, region, limits=True, stats=None):
    lib = st.lib
    lib.put_xedges(zoom, st, region)
    block, _ = _block(zoom, region)
    js, je = x_scope(zoom, region, block)
    with lib.outer_x_faces_zeroed(zoom, st, region, _second_half(zoom, region)):
        if region == 1:
            lib._dynamu_region1(zoom, st, js, je, limits, stats)
        else:
            lib._dynamu_child(zoom, st, region, js, je, 1, zoom.lm, limits, stats)
            lib._uncompress_xedges(zoom, st, region, js, je, 1, zoom.lm)
            lib.mix_edges(zoom, st, region)


def advect_y_zoom(zoom, st, region, limits=True, stats=None):
    lib = st.lib
    lib.put_yedges(zoom, st, region)
    block, _ = _block(zoom, region)
    is_, ie = y_scope(zoom, region, block)
    with lib.outer_y_faces_zeroed(zoom, st, region, _second_half(zoom, region)):
        if region == 1:
            lib._dynamv_region1(zoom, st, limits, stats)
        else:
            lib._dynamv_child(zoom, st, region, is_, ie, 1, zoom.lm, limits, stats)
            lib._uncompress_yedges(zoom, st, region, is_, ie, 1, zoom.lm)
            lib.mix_edges(zoom, st, region)


def advect_z_zoom(zoom, st, region, limits=True, stats=None):
    lib = st.lib
    block, _ = _block(zoom, region)
    is_, ie, js, je = z_scope(zoom, region, block)
    if region == 1:
        lib._dynamw_region1(zoom, st, limits, stats)
    else:
        lib._dynamw_child(zoom, st, region, is_, ie, js, je, limits, stats)
        lib.mix_edges(zoom, st, region)


OPERATORS = {"x": advect_x_zoom, "y": advect_y_zoom, "z": advect_z_zoom}


# ------------------------------------------------------------------ do_steps, Proces_Region, step
def do_steps(zoom, st, region, conv, ndyn, limits=True, inverse="crout", stats=None, sources=None,
             chemistry=None):
    """modelIntegration do_steps: the region's next operators up to a block boundary (where the
    children's edges are refilled unless x was last), or to a z that follows a y."""
    lib, order = st.lib, zoom.splitorderzoom[region]
    for _ in range(N_OPERATORS):
        nxt = order[zoom.status[region]]
        if nxt in OPERATORS:
            OPERATORS[nxt](zoom, st, region, limits, stats=stats)
        elif nxt == "v":
            if conv is not None and conv.get(region) is not None:
                lib.convec_region(zoom, st, region, conv[region], ndyn, inverse)
        elif nxt == "s":
            if sources is not None:
                sources(zoom, st, region)
        elif nxt == "c":
            if chemistry is not None:
                chemistry(zoom, st, region)
        else:
            raise ValueError(f"do_steps: strange value in splitorderzoom: {nxt!r}")
        zoom.status[region] += 1
        s_now = zoom.status[region]
        if s_now % N_OPERATORS == 0:
            if nxt != "x":
                lib.put_xedges(zoom, st, region)
                lib.put_yedges(zoom, st, region)
            return
        if nxt == "z" and order[s_now - 2] == "y":
            return


def proces_region(zoom, st, region, conv, ndyn, **kw):
    """Proces_Region: tref_ passes of do_steps, the children run after the parent's xyz; then
    update_parent and m2phlb (m2phlb1 for region 1)."""
    for _ in range(zoom.ref(region, "t")):
        do_steps(zoom, st, region, conv, ndyn, **kw)
        for child in zoom.children[region]:
            proces_region(zoom, st, child, conv, ndyn, **kw)
        if zoom.status[region] % N_OPERATORS != 0:
            do_steps(zoom, st, region, conv, ndyn, **kw)
    if region != 1:
        st.lib.update_parent(zoom, st, region)
        st.lib.m2phlb(zoom, st, region)
    else:
        st.lib.m2phlb1(zoom, st, 1)


def step(zoom, st, conv, ndyn, **kw):
    """One ndyn step (fluxes already set): every region's status reset, Proces_Region(1) twice."""
    zoom.status = [0] * (zoom.nregions + 1)
    for _ in range(2):
        proces_region(zoom, st, 1, conv, ndyn, **kw)


# ------------------------------------------------------------------ Setup_MassFlow, coarsen_region
def coarsen_region(zoom, st, region):
    """zoom_tools coarsen_region: the parent's fluxes and mass over the child's footprint rebuilt
    from the child's, m2phlb of the parent, recursively up."""
    parent = zoom.g(region).parent
    if parent <= 0:
        return
    st.lib._coarsen_block(zoom, st, region)
    if parent != 1:
        st.lib.m2phlb(zoom, st, parent)
    else:
        st.lib.m2phlb1(zoom, st, parent)
    coarsen_region(zoom, st, parent)


def setup_massflow(zoom, st, ndyn):
    """Setup_MassFlow's region loop: dynam0 and coarsen_region region by region, then
    coarsen_ambm for every region."""
    for r in zoom.regions():
        st.lib.dynam0(zoom, st, r, ndyn)
        coarsen_region(zoom, st, r)
    for r in zoom.regions():
        st.lib.coarsen_ambm(zoom, st, r)


# ------------------------------------------------------------------ Check_CFL (pydyn zoom/check_cfl.py)
class _CFLRun:
    """advectm_cfl's module state for one Check_CFL: the CFL split order, the status counters and
    each region's ok flag (check_cfl.py:57-70)."""

    def __init__(self, zoom, caps=None):
        self.caps = caps
        self.order = zoom.split_orders(CFL_SPLITORDER, CFL_N_OPERATORS)
        self.status = [0] * (zoom.nregions + 1)
        self.ok = [True] * (zoom.nregions + 1)

    def all_ok(self):
        return all(self.ok[1:])


def _advectm(zoom, st, run, region, axis):
    """advectm{x,y,z}zoom (check_cfl.py:79-92, 140-153, 196-203): the body's return is the ok."""
    lib, lm = st.lib, zoom.lm
    s = run.status[region]
    block, _ = _block(zoom, region, s, run.order[region], CFL_N_OPERATORS)
    second = _second_half(zoom, region, s, CFL_N_OPERATORS)
    cap = {"x": 10, "y": 1, "z": 1}[axis] if run.caps is None else run.caps["xyz".index(axis)]
    if axis == "x":
        lib.put_xedges(zoom, st, region, tracers=False)
        js, je = x_scope(zoom, region, block)
        with lib.outer_x_faces_zeroed(zoom, st, region, second):
            if region == 1:
                ok = lib._dynamum_region1(zoom, st, js, je, cap)
            else:
                ok = lib._dynamum_child(zoom, st, region, js, je, 1, lm, cap)
            run.ok[region] = ok
    elif axis == "y":
        lib.put_yedges(zoom, st, region, tracers=False)
        is_, ie = y_scope(zoom, region, block)
        with lib.outer_y_faces_zeroed(zoom, st, region, second):
            if region == 1:
                ok = lib._dynamvm_region1(zoom, st, cap)
            else:
                ok = lib._dynamvm_child(zoom, st, region, is_, ie, 1, lm, cap)
            run.ok[region] = ok
    else:
        is_, ie, js, je = z_scope(zoom, region, block)
        run.ok[region] = lib._dynamwm(zoom, st, region, is_, ie, js, je, cap)
        if run.ok[region] and region != 1:
            lib.mix_edges(zoom, st, region, tracers=False)


def _cfl_do_steps(zoom, st, run, region):
    """do_steps of advectm_cfl (check_cfl.py:222-235): returns as soon as any region failed."""
    for _ in range(CFL_N_OPERATORS):
        _advectm(zoom, st, run, region, run.order[region][run.status[region]])
        if not run.all_ok():
            return
        run.status[region] += 1
        if run.status[region] % CFL_N_OPERATORS == 0:
            return


def determine_cfl_iter(zoom, st, run, region):
    """determine_cfl_iter (check_cfl.py:238-255): any failure unwinds back to Check_CFL."""
    run.ok[region] = True
    for _ in range(zoom.ref(region, "t")):
        _cfl_do_steps(zoom, st, run, region)
        if not run.ok[region]:
            return
        for child in zoom.children[region]:
            if not run.all_ok():
                break
            determine_cfl_iter(zoom, st, run, child)
        if run.status[region] % CFL_N_OPERATORS != 0 and run.all_ok():
            _cfl_do_steps(zoom, st, run, region)
            if not run.ok[region]:
                return
    if region != 1:
        st.lib.update_parent(zoom, st, region, tracers=False)


def new_valid_timestep(dtime, nread, cfl_outputstep, tref_max=1):
    """The largest dtime' < dtime dividing nread and cfl_outputstep, a multiple of 2 tref_max
    (pydyn cfl.py:208-213)."""
    for dt in range(dtime - 1, 0, -1):
        if nread % dt == 0 and cfl_outputstep % dt == 0 and dt % (2 * tref_max) == 0:
            return dt
    raise ValueError("new_valid_timestep: no valid time step")


def check_cfl_zoom(zoom, st, ndyn, n, nread, interpolate=None, max_iteration=100, caps=None):
    """Check_CFL on a region tree (check_cfl.py:258-290): for each of the n steps
    Setup_MassFlow (after `interpolate(zoom, st, i, ndyn)`) and the xyz / zyx mass-only
    rehearsals; on a failure m, am, bm, cm are restored, ndyn goes to the next valid step and
    the stored fluxes are scaled by ndyn_new / ndyn_old.  Returns (ndyn, n, iterations)."""
    tref_max = max(zoom.g(r).tref for r in zoom.regions())
    for iteration in range(1, max_iteration + 1):
        run = _CFLRun(zoom, caps)
        st.lib.save(st, "check_cfl", ("m", "am", "bm", "cm"))
        for i in range(1, n + 1):
            if interpolate is not None:
                interpolate(zoom, st, i, ndyn)
            setup_massflow(zoom, st, ndyn)
            determine_cfl_iter(zoom, st, run, 1)
            if run.all_ok():
                determine_cfl_iter(zoom, st, run, 1)
            if not run.all_ok():
                break
            run.status = [0] * (zoom.nregions + 1)
        st.lib.restore(st, "check_cfl")
        if run.all_ok():
            return ndyn, n, iteration
        ndyn_old = ndyn
        ndyn = new_valid_timestep(ndyn, nread, nread, tref_max)
        n = nint(float(n * ndyn_old) / float(ndyn))
        st.lib.scale(st, ("am", "bm", "cm"), float(ndyn) / float(ndyn_old))
    raise RuntimeError("check_cfl_zoom: exceeded maximum number of time steps")
