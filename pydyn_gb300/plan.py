"""The step planner: a region tree's operator sequence compiled once into a flat list of body
calls, replayed by every step.

TM5 runs a step by recursion over the tree with a position counter per region (modelIntegration
do_steps / Proces_Region; pydyn zoom/steps.py:29-88, zoom/advect.py:154-199): a region takes its
next block of operators, hands over to its children after its own x, y, z, and takes the block's
remaining operators after them.  None of that depends on the data -- sub-cycle counts and the
Check_CFL outcome are decided on the device -- so the sequence is a function of the tree alone.
`step_plan` walks it once into a tuple of `Call`s: the body of the device module (the names of
pydyn's zoom.host.BODIES), its region, its arguments (scopes resolved from the block's order),
and the region's position in its order when it runs.  `replay` issues them.  The eager step,
the captured CUDA graph and the stream scheduler all consume the same tuple, and no Python state
machine runs per step.

Check_CFL's mass-only rehearsal of one step (advectm_cfl.F90; pydyn zoom/check_cfl.py:32-256)
and Setup_MassFlow (pydyn zoom/massflow.py:61-73, 174-184) are planned the same way.  The planned
rehearsal does not stop at a failed operator: the failure is a device flag that every later
rehearsal kernel honours by doing nothing, read once per rehearsed step (`check_cfl`)."""

from typing import NamedTuple

from .tree import CFL_N_OPERATORS, CFL_SPLITORDER, N_OPERATORS, nint

# the run-time arguments of a step, filled in by replay
LIMITS, CONV, NDYN, INVERSE = "<limits>", "<conv>", "<ndyn>", "<inverse>"
CFL_CAPS = (10, 1, 1)  # Check_CFL's sub-cycle caps on x, y, z (cfl_max_nloop_{x,y,z})


class Call(NamedTuple):
    body: str  # a body of the device module, or "sources" / "chemistry" (the step's hooks)
    region: int
    args: tuple  # after (zoom, st); LIMITS, CONV, NDYN, INVERSE stand for the step's values
    status: int  # the region's position in its operator order when the call runs
    inner: tuple = ()  # calls made inside a context-manager body
    kw: tuple = ()  # keyword arguments, as (name, value) pairs


# ------------------------------------------------------------------ scopes
def _after(block, a, b):
    """Whether operator a comes after operator b in the block."""
    return a in block and b in block and block.index(a) > block.index(b)


def _inner_x(zoom, r):
    """The columns of region r inside its ring (all of them for a cyclic region)."""
    g, xr = zoom.g(r), zoom.ref(r, "x") if r != 1 else 0
    return (1, g.im) if g.xcyc == 1 else (xr + 1, g.im - xr)


def _inner_y(zoom, r):
    """The rows of region r inside its ring (a pole-touching side keeps its rows)."""
    g, yr = zoom.g(r), zoom.ref(r, "y") if r != 1 else 0
    return (1 if g.touch_sp == 1 else yr + 1), (g.jm if g.touch_np == 1 else g.jm - yr)


def scopes(zoom, r, block):
    """The cells each direction's advection updates in this block: x updates all rows unless y
    comes after it in the block (then only the rows inside the ring, whose halo rows y has yet
    to fill); y all columns unless x comes after it; z the inner columns / rows of a direction
    that comes after it.  Returns {'x': (js, je), 'y': (is, ie), 'z': (is, ie, js, je)}."""
    g = zoom.g(r)
    full_i, full_j = (1, g.im), (1, g.jm)
    out = {}
    if "x" in block:
        out["x"] = _inner_y(zoom, r) if _after(block, "y", "x") else full_j
    if "y" in block:
        out["y"] = _inner_x(zoom, r) if _after(block, "x", "y") else full_i
    if "z" in block:
        cols = _inner_x(zoom, r) if _after(block, "x", "z") else full_i
        rows = _inner_y(zoom, r) if _after(block, "y", "z") else full_j
        out["z"] = (*cols, *rows)
    return out


# ------------------------------------------------------------------ one operator's calls
def _advection(zoom, r, op, status, block, second, lm):
    """The calls of advect{x,y,z}zoom for region r."""
    sc = scopes(zoom, r, block)[op]
    if op == "x":
        if r == 1:
            inner = (Call("_dynamu_region1", 1, (*sc, LIMITS, None), status),)
        else:
            inner = (Call("_dynamu_child", r, (r, *sc, 1, lm, LIMITS, None), status),
                     Call("_uncompress_xedges", r, (r, *sc, 1, lm), status),
                     Call("mix_edges", r, (r,), status))  # fmt: skip
        return (Call("put_xedges", r, (r,), status),
                Call("outer_x_faces_zeroed", r, (r, second), status, inner))  # fmt: skip
    if op == "y":
        if r == 1:
            inner = (Call("_dynamv_region1", 1, (LIMITS, None), status),)
        else:
            inner = (Call("_dynamv_child", r, (r, *sc, 1, lm, LIMITS, None), status),
                     Call("_uncompress_yedges", r, (r, *sc, 1, lm), status),
                     Call("mix_edges", r, (r,), status))  # fmt: skip
        return (Call("put_yedges", r, (r,), status),
                Call("outer_y_faces_zeroed", r, (r, second), status, inner))  # fmt: skip
    if r == 1:
        return (Call("_dynamw_region1", 1, (LIMITS, None), status),)
    return (Call("_dynamw_child", r, (r, *sc, LIMITS, None), status), Call("mix_edges", r, (r,), status))


def _operator(zoom, r, op, status, block, second, lm):
    if op in "xyz":
        return _advection(zoom, r, op, status, block, second, lm)
    if op == "v":
        return (Call("convec_region", r, (r, CONV, NDYN, INVERSE), status),)
    if op == "s":
        return (Call("sources", r, (), status),)
    if op == "c":
        return (Call("chemistry", r, (), status),)
    raise ValueError(f"operator order of region {r}: unknown operator {op!r}")


# ------------------------------------------------------------------ the step
def _block_at(order, pos, n_ops, tref):
    """The block of operators that decides the scopes at position pos (the first of the tref
    copies the child runs per parent block), and whether pos is past the block's first copy."""
    span = n_ops * tref
    start = (pos // span) * span
    return order[start : start + n_ops], pos % span >= n_ops


def _handover(order, pos, end):
    """Where region's segment starting at pos stops for its children: after the first z that
    directly follows a y in the order, else at the block's end."""
    for k in range(pos, end):
        if order[k] == "z" and order[k - 1] == "y":
            return k + 1
    return end


def _cached(zoom, key, make):
    """A plan kept on the tree it was made for (the tree is frozen once built)."""
    plans = zoom.__dict__.setdefault("_plans", {})
    if key not in plans:
        plans[key] = make()
    return plans[key]


def _make_step_plan(zoom):
    lm, order = zoom.lm, zoom.splitorderzoom
    pos = [0] * (zoom.nregions + 1)
    calls = []

    def segment(r, stop):
        """Region r's operators from its position to stop, then the edge refill at a block's end."""
        tref = zoom.ref(r, "t")
        while pos[r] < stop:
            block, second = _block_at(order[r], pos[r], N_OPERATORS, tref)
            calls.extend(_operator(zoom, r, order[r][pos[r]], pos[r], block, second, lm))
            pos[r] += 1
        if pos[r] % N_OPERATORS == 0 and order[r][pos[r] - 1] != "x":
            # the children's halos refilled from the parent's state at the block's end
            calls.append(Call("put_xedges", r, (r,), pos[r]))
            calls.append(Call("put_yedges", r, (r,), pos[r]))

    def region_pass(r):
        """Region r over one of its parent's passes: its tref blocks, each with the children's
        passes after its x, y, z; then its block sums into the parent and its pressure."""
        for _ in range(zoom.ref(r, "t")):
            segment(r, _handover(order[r], pos[r], _block_end(pos[r])))
            for c in zoom.children[r]:
                region_pass(c)
            if pos[r] % N_OPERATORS != 0:  # the block's operators after the hand-over
                segment(r, _handover(order[r], pos[r], _block_end(pos[r])))
        if r != 1:
            calls.append(Call("update_parent", r, (r,), pos[r]))
            calls.append(Call("m2phlb", r, (r,), pos[r]))
        else:
            calls.append(Call("m2phlb1", 1, (1,), pos[1]))

    region_pass(1)  # the first half step
    region_pass(1)  # the second
    return tuple(calls)


def _block_end(pos, n_ops=N_OPERATORS):
    return (pos // n_ops + 1) * n_ops


def operator_calls(zoom, r, status):
    """The calls of the operator at position `status` of region r's order, on its own: what
    pydyn's zoom.OPERATORS[op](zoom, st, r) (or the v / s / c body) does at that position, as a
    replay of one dumped operator issues it."""
    order = zoom.splitorderzoom[r]
    block, second = _block_at(order, status, N_OPERATORS, zoom.ref(r, "t"))
    return _operator(zoom, r, order[status], status, block, second, zoom.lm)


def step_plan(zoom):
    """The calls of one step (tm5.F90's two half steps over the tree), fluxes already set."""
    return _cached(zoom, "step", lambda: _make_step_plan(zoom))


# ------------------------------------------------------------------ Setup_MassFlow
def massflow_plan(zoom):
    """Setup_MassFlow's calls: per region dynam0, then its fluxes and mass coarsened into every
    ancestor's footprint with the ancestor's pressure redone; then coarsen_ambm per region."""
    return _cached(zoom, "massflow", lambda: _make_massflow(zoom))


def _make_massflow(zoom):
    calls = []
    for r in zoom.regions():
        calls.append(Call("dynam0", r, (r, NDYN), 0))
        c = r
        while zoom.g(c).parent > 0:
            p = zoom.g(c).parent
            calls.append(Call("_coarsen_block", c, (c,), 0))
            calls.append(Call("m2phlb1", 1, (1,), 0) if p == 1 else Call("m2phlb", p, (p,), 0))
            c = p
    calls.extend(Call("coarsen_ambm", r, (r,), 0) for r in zoom.regions())
    return tuple(calls)


# ------------------------------------------------------------------ Check_CFL's rehearsal
def _mass_operator(zoom, r, op, status, block, second, lm, caps):
    sc = scopes(zoom, r, block)[op]
    quiet = (("report", False),)  # the planned rehearsal reads the device flag once per step
    cap = caps["xyz".index(op)]
    if op == "x":
        body = (Call("_dynamum_region1", 1, (*sc, cap), status, kw=quiet) if r == 1 else
                Call("_dynamum_child", r, (r, *sc, 1, lm, cap), status, kw=quiet))  # fmt: skip
        return (Call("put_xedges", r, (r,), status, kw=(("tracers", False),)),
                Call("outer_x_faces_zeroed", r, (r, second), status, (body,)))  # fmt: skip
    if op == "y":
        body = (Call("_dynamvm_region1", 1, (cap,), status, kw=quiet) if r == 1 else
                Call("_dynamvm_child", r, (r, *sc, 1, lm, cap), status, kw=quiet))  # fmt: skip
        return (Call("put_yedges", r, (r,), status, kw=(("tracers", False),)),
                Call("outer_y_faces_zeroed", r, (r, second), status, (body,)))  # fmt: skip
    calls = (Call("_dynamwm", r, (r, *sc, cap), status, kw=quiet),)
    if r != 1:
        calls += (Call("mix_edges", r, (r,), status, kw=(("tracers", False),)),)
    return calls


def _make_rehearsal(zoom, caps):
    lm = zoom.lm
    order = zoom.split_orders(CFL_SPLITORDER, CFL_N_OPERATORS)
    pos = [0] * (zoom.nregions + 1)
    calls = []

    def region_pass(r):
        tref = zoom.ref(r, "t")
        for _ in range(tref):
            end = _block_end(pos[r], CFL_N_OPERATORS)
            while pos[r] < end:  # the rehearsal hands over at block ends only
                block, second = _block_at(order[r], pos[r], CFL_N_OPERATORS, tref)
                calls.extend(_mass_operator(zoom, r, order[r][pos[r]], pos[r], block, second, lm, caps))
                pos[r] += 1
            for c in zoom.children[r]:
                region_pass(c)
        if r != 1:
            calls.append(Call("update_parent", r, (r,), pos[r], kw=(("tracers", False),)))

    region_pass(1)
    region_pass(1)
    return tuple(calls)


def rehearsal_plan(zoom, caps=CFL_CAPS):
    """The calls of one rehearsed step: Setup_MassFlow, then the mass-only operators of both
    half steps (`xyz`, `zyx`, blocks of three) over the tree."""
    caps = tuple(caps)
    return _cached(zoom, ("rehearsal", caps), lambda: massflow_plan(zoom) + _make_rehearsal(zoom, caps))


# ------------------------------------------------------------------ replay
def replay(calls, zoom, st, conv=None, ndyn=None, limits=True, inverse="crout", sources=None, chemistry=None):
    """Issue the calls on st.lib.  `conv[r]` is region r's convection input (None: no
    convection), `sources` / `chemistry` the step's hooks f(zoom, st, region) (None: no-ops).
    zoom.status[r] is set to each call's position first, as pydyn's hooks may read it."""
    lib = st.lib
    fill = {LIMITS: limits, NDYN: ndyn, INVERSE: inverse}
    hooks = {"sources": sources, "chemistry": chemistry}
    for c in calls:
        zoom.status[c.region] = c.status
        if c.body in hooks:
            if hooks[c.body] is not None:
                hooks[c.body](zoom, st, c.region)
            continue
        if c.body == "convec_region":
            if conv is None or conv.get(c.region) is None:
                continue
            args = (c.region, conv[c.region], ndyn, inverse)
        else:
            args = tuple(fill.get(a, a) if isinstance(a, str) else a for a in c.args)
        fn = getattr(lib, c.body)
        if c.inner:
            with fn(zoom, st, *args, **dict(c.kw)):
                replay(c.inner, zoom, st, conv, ndyn, limits, inverse, sources, chemistry)
        else:
            fn(zoom, st, *args, **dict(c.kw))


def step(zoom, st, conv, ndyn, limits=True, inverse="crout", sources=None, chemistry=None):
    """One step of the tree (fluxes already set); every region's position ends where a step
    leaves it."""
    zoom.status = [0] * (zoom.nregions + 1)
    replay(step_plan(zoom), zoom, st, conv, ndyn, limits, inverse, sources, chemistry)
    _finish_status(zoom)


def _finish_status(zoom):
    zoom.status = [0] + [len(zoom.splitorderzoom[r]) for r in zoom.regions()]


def setup_massflow(zoom, st, ndyn):
    replay(massflow_plan(zoom), zoom, st, ndyn=ndyn)


def rehearse_step(zoom, st, ndyn, caps=CFL_CAPS):
    """Enqueue one rehearsed step (Setup_MassFlow and the mass-only operators) on st."""
    replay(rehearsal_plan(zoom, caps), zoom, st, ndyn=ndyn)


# ------------------------------------------------------------------ Check_CFL
def shorter_step(ndyn, nread, tref_max):
    """The next time step Check_CFL tries after ndyn fails: the largest step below ndyn that
    divides the read interval and is a multiple of 2 tref_max (pydyn cfl.py:208-213)."""
    for dt in range(ndyn - 1, 0, -1):
        if nread % dt == 0 and dt % (2 * tref_max) == 0:
            return dt
    raise ValueError(f"Check_CFL: no time step below {ndyn} s divides {nread} s in multiples of {2 * tref_max}")


def check_cfl(zoom, st, ndyn, n, nread, interpolate=None, max_tries=100, caps=CFL_CAPS, rehearse=None):
    """Check_CFL on a region tree: rehearse the n steps of the read interval on st (a copy of the
    air mass); when one fails, restore m and the fluxes, take a shorter step and scale the
    fluxes to it, and rehearse again.  Returns (ndyn, n, tries).  `interpolate(zoom, st, i,
    ndyn)` sets step i's meteo first; `rehearse(st, i, n, ndyn)` replaces the planned rehearsal
    (a captured graph of it, for instance).  The state is left with m, am, bm, cm restored (and
    scaled), as TM5's advectm_cfl leaves it (pydyn zoom/check_cfl.py:258-290)."""
    lib = st.lib
    tref_max = max(zoom.g(r).tref for r in zoom.regions())
    for tries in range(1, max_tries + 1):
        lib.save(st, "check_cfl", ("m", "am", "bm", "cm"))  # also clears the rehearsal flag
        passed = True
        for i in range(1, n + 1):
            if rehearse is not None:
                rehearse(st, i, n, ndyn)
            else:
                if interpolate is not None:
                    interpolate(zoom, st, i, ndyn)
                rehearse_step(zoom, st, ndyn, caps)
            if not lib.cfl_all_ok(st):
                passed = False
                break
        lib.restore(st, "check_cfl")
        if passed:
            return ndyn, n, tries
        shorter = shorter_step(ndyn, nread, tref_max)
        n = nint(float(n * ndyn) / float(shorter))
        lib.scale(st, ("am", "bm", "cm"), float(shorter) / float(ndyn))
        ndyn = shorter
    raise RuntimeError(f"Check_CFL: no stable time step after {max_tries} tries")
