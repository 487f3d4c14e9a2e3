"""The state dumps of the Fortran module pydyn_dump (rc key `pydyn.dump`), read for a replay on
the device.

An event is a header `<dir>/e<seq:05d>_<tag>_r<region>_p<rank:03d>.meta` -- `key = value`
lines, an array declared as `array NAME = lb1 ub1 lb2 ub2 ...` (8-byte reals) or
`iarray NAME = ...` (4-byte integers) -- and one raw stream `<prefix>_<NAME>.bin` per array in
Fortran order.  `Event[name]` is the array on the host with its Fortran bounds (`FArray`);
`Event.device(name, dev)` puts the file's bytes on the device as they are and returns them
as a DevArray with the same bounds and Fortran strides, so that a section of it is copied into
the state (C order, level fastest) by a device kernel and no host transposes tens of GB.

A parallel run of TM5 splits the tracers over its ranks and replicates everything else:
`merge_ranks` puts the ranks' events back together as the serial run's.

The interface is pydyn's reader's (pydyn dump.py:23-370: Event, FArray, load_events,
merge_ranks, their names and errors), since the replay's callers address events by it."""

import re
from pathlib import Path

import numpy as np

__all__ = ["DumpError", "Event", "EventRef", "FArray", "MergedEvent", "RankMismatch", "load_events", "merge_ranks"]

META_NAME = re.compile(r"^e(\d{5})_(.+)_r(\d+)_p(\d{3})\.meta$")
REQUIRED = ("tag", "seq", "region", "im", "jm", "lm")


class DumpError(ValueError):
    """A header that pydyn_dump did not write: unreadable, truncated, or a malformed array line."""


class RankMismatch(ValueError):
    """The ranks of one event disagree where a tracer-split run replicates."""


# ------------------------------------------------------------------ Fortran-bounded host arrays
def _fortran_index(lower, shape, item):
    """NumPy index of an inclusive Fortran section `item` of an array with bounds `lower`."""
    if not isinstance(item, tuple):
        item = (item,)
    if len(item) > len(lower):
        raise IndexError(f"{len(item)} indices for {len(lower)} axes")
    out = []
    for lo, n, ix in zip(lower, shape, item, strict=False):
        if isinstance(ix, slice):
            if ix.step not in (None, 1):
                raise IndexError("strided Fortran sections are not supported")
            a = lo if ix.start is None else ix.start
            b = lo + n - 1 if ix.stop is None else ix.stop
            out.append(slice(a - lo, b - lo + 1))
        else:
            out.append(ix - lo)
    return tuple(out)


class FArray:
    """A host array and the Fortran lower bound of each axis: `a[1:60, 1:45, 1:34]` is the
    section (1:60, 1:45, 1:34), inclusive; an integer drops its axis; axes not indexed are
    taken whole."""

    def __init__(self, data, lower):
        self.data = data
        self.lower = tuple(int(x) for x in lower)

    @property
    def upper(self):
        return tuple(lo + n - 1 for lo, n in zip(self.lower, self.data.shape, strict=True))

    def __getitem__(self, item):
        return np.ascontiguousarray(self.data[_fortran_index(self.lower, self.data.shape, item)])

    def window(self, other):
        """The NumPy index of the cells of self that `other` (anything with lower / upper)
        spans."""
        return tuple(slice(lo - s, hi - s + 1) for lo, hi, s in zip(other.lower, other.upper, self.lower, strict=True))

    def covers(self, other):
        return all(s <= lo and hi <= t for lo, hi, s, t in zip(other.lower, other.upper, self.lower, self.upper,
                                                               strict=True))  # fmt: skip

    def __repr__(self):
        return f"FArray({', '.join(f'{lo}:{hi}' for lo, hi in zip(self.lower, self.upper, strict=True))})"


# ------------------------------------------------------------------ the header
def parse_value(text):
    """A header value: T / F, an integer, a real, a tuple of integers, else the text."""
    words = text.split()
    if len(words) == 1:
        w = words[0]
        if w in ("T", "F"):
            return w == "T"
        for kind in (int, float):
            try:
                return kind(w)
            except ValueError:
                pass
        return w
    try:
        return tuple(int(w) for w in words)
    except ValueError:
        return text.strip()


def _parse_header(path):
    """(meta, {name: (bounds, dtype)}) of a .meta file."""
    try:
        text = Path(path).read_text()
    except (OSError, UnicodeDecodeError) as e:
        raise DumpError(f"{path}: not readable as a dump header ({e})") from e
    meta, arrays = {}, {}
    for n, line in enumerate(text.splitlines(), 1):
        key, eq, value = line.partition("=")
        if not eq:
            continue
        key = key.strip()
        kind, _, name = key.partition(" ")
        if kind in ("array", "iarray") and name:
            name = name.strip()
            try:
                nums = [int(w) for w in value.split()]
            except ValueError as e:
                raise DumpError(f"{path}:{n}: not an array line: {line.strip()[:80]}") from e
            if not nums or len(nums) % 2 or not name.isidentifier():
                raise DumpError(f"{path}:{n}: bad array bounds or name: {line.strip()[:80]}")
            bounds = list(zip(nums[::2], nums[1::2], strict=True))
            if any(hi < lo - 1 for lo, hi in bounds):
                raise DumpError(f"{path}:{n}: bad array bounds or name: {line.strip()[:80]}")
            arrays[name] = (bounds, np.dtype("<i4" if kind == "iarray" else "<f8"))
        else:
            meta[key] = parse_value(value)
    missing = [k for k in REQUIRED if k not in meta]
    if missing:
        raise DumpError(f"{path}: no {', '.join(missing)} in the header (a truncated dump?)")
    return meta, arrays


class Event:
    """One dump event: `meta`, `tag`, `seq`, `region`, and its arrays by name, read when first
    asked for."""

    def __init__(self, meta_path):
        self.path = Path(meta_path)
        self.prefix = self.path.with_suffix("")
        self.meta, self._decl = _parse_header(self.path)
        self.tag, self.seq, self.region = self.meta["tag"], self.meta["seq"], self.meta["region"]
        self._cache = {}

    @property
    def arrays(self):
        return tuple(self._decl)

    def __contains__(self, name):
        return name in self._decl

    def bounds(self, name):
        return self._decl[name][0]

    def _raw(self, name):
        """The file's values, flat, in its (Fortran) order."""
        bounds, dtype = self._decl[name]
        shape = tuple(hi - lo + 1 for lo, hi in bounds)
        raw = np.fromfile(f"{self.prefix}_{name}.bin", dtype=dtype)
        if raw.size != int(np.prod(shape)):
            raise ValueError(f"{self.prefix}_{name}.bin: {raw.size} values for bounds {bounds}")
        return raw, shape, [lo for lo, _ in bounds]

    def __getitem__(self, name):
        if name not in self._cache:
            raw, shape, lower = self._raw(name)
            self._cache[name] = FArray(raw.reshape(shape, order="F"), lower)
        return self._cache[name]

    def interior(self, name):
        """The pydyn-layout interior of a state, flux or meteo array: the section of it that
        pydyn's NumPy arrays hold (halo cells dropped, boundary faces kept)."""
        return self[name][interior_section(name, self.meta["im"], self.meta["jm"], self.meta["lm"])]

    def device(self, name, dev):
        """The array on the device as the file holds it: a DevArray with its Fortran bounds and
        Fortran strides (the first index fastest).  Read from the host copy if there is one."""
        from .device import DevArray

        if name in self._cache:
            a = self._cache[name]
            flat, shape, lower = a.data.ravel(order="F"), a.data.shape, a.lower
        else:
            flat, shape, lower = self._raw(name)
        buf = DevArray.from_host(dev, flat)
        strides = [1]
        for n in shape[:-1]:
            strides.append(strides[-1] * n)
        return buf.reshape_axes(tuple(shape), tuple(strides), tuple(lower))

    def release(self):
        self._cache.clear()

    def cached(self):
        return list(self._cache)

    def ref(self):
        return EventRef(self.seq, self.tag, self.region, dict(self.meta), repr(self))

    def __repr__(self):
        return f"Event(seq={self.seq}, tag={self.tag!r}, region={self.region})"


class EventRef:
    """An event's identity and header without its arrays."""

    def __init__(self, seq, tag, region, meta, text):
        self.seq, self.tag, self.region, self.meta, self._text = seq, tag, region, meta, text

    def __repr__(self):
        return self._text


# the section of each array that pydyn's NumPy layout holds (pydyn layout.py:38-48)
_CELLS = "1:{im}, 1:{jm}, 1:{lm}"
INTERIOR = {
    **dict.fromkeys(("m", "rm", "rxm", "rym", "rzm", "temper"), _CELLS),
    "am": "0:{im}, 1:{jm}, 1:{lm}",
    "bm": "1:{im}, 1:{jm1}, 1:{lm}",
    **dict.fromkeys(("cm", "mfw1", "mfw2", "pw1", "pw2"), "1:{im}, 1:{jm}, 0:{lm}"),
    **dict.fromkeys(("pu", "pu1", "pu2", "mfu1", "mfu2"), "0:{im}, 1:{jm}, 1:{lm}"),
    **dict.fromkeys(("pv", "pv1", "pv2", "mfv1", "mfv2"), "1:{im}, 1:{jm1}, 1:{lm}"),
    **dict.fromkeys(("sp", "sp1", "sp2"), "1:{im}, 1:{jm}, 1"),
    "phlb": "1:{im}, 1:{jm}, 1:{lm1}",
}


def interior_section(name, im, jm, lm):
    """`INTERIOR[name]` as a tuple of inclusive slices and integers."""
    text = INTERIOR[name].format(im=im, jm=jm, lm=lm, jm1=jm + 1, lm1=lm + 1)
    out = []
    for part in text.split(","):
        lo, colon, hi = part.partition(":")
        out.append(slice(int(lo), int(hi)) if colon else int(lo))
    return tuple(out)


def load_events(dump_dir, tags=None, region=None, rank=None, merge=False):
    """The events of a dump directory in sequence order (then rank), optionally of some tags,
    one region or one rank; merge=True puts a parallel run's ranks back together."""
    events = []
    for p in sorted(Path(dump_dir).iterdir()):
        mo = META_NAME.match(p.name)
        if mo is None:
            continue
        tag, reg, rk = mo.group(2), int(mo.group(3)), int(mo.group(4))
        if (tags is not None and tag not in tags) or (region is not None and reg != region):
            continue
        if rank is not None and rk != rank:
            continue
        events.append(Event(p))
    events.sort(key=lambda e: (e.seq, e.meta.get("rank", 0)))
    if merge and len({e.meta.get("rank", 0) for e in events}) > 1:
        return merge_ranks(events)
    return events


# ------------------------------------------------------------------ a tracer-split run
# TM5's MPI decomposition is by tracer: rank r holds the tracers after those of ranks 0..r-1;
# only the tracer arrays are split, one header list holds the rank's local tracer numbers, and
# `emis` events come one per tracer a rank holds, numbered globally (pydyn dump.py:228-232).
TRACER_ARRAYS = ("rm", "rxm", "rym", "rzm")
RANK_LOCAL_TRACER_KEYS = ("ch4_tracers",)
PER_TRACER_TAGS = ("emis",)


class MergedEvent:
    """One event of a tracer-split run as the serial run would have written it: the tracer
    arrays are the ranks' slabs side by side in rank order, every other array must be the same
    bytes on every rank, and the header is the ranks' common one (a local tracer list made
    global)."""

    def __init__(self, parts, offsets):
        parts = sorted(parts, key=lambda e: e.meta["rank"])
        head = parts[0]
        for e in parts[1:]:
            if (e.tag, e.region) != (head.tag, head.region):
                raise RankMismatch(f"e{head.seq:05d}: ranks disagree on the event: {head!r} vs {e!r}")
            if e.arrays != head.arrays:
                raise RankMismatch(f"e{head.seq:05d} {head.tag}: ranks dump different arrays")
        self.parts, self.ranks = parts, [e.meta["rank"] for e in parts]
        self.tag, self.seq, self.region, self.path = head.tag, head.seq, head.region, head.path
        self.meta = {}
        for key in sorted(set().union(*(e.meta for e in parts)) - {"rank", "seq"}):
            values = [e.meta.get(key) for e in parts]
            if key in RANK_LOCAL_TRACER_KEYS:
                glob = []
                for rk, v in zip(self.ranks, values, strict=True):
                    glob += [offsets[rk] + int(x) for x in (v if isinstance(v, tuple) else (v,))]
                self.meta[key] = tuple(glob)
            elif all(v == values[0] for v in values):
                self.meta[key] = values[0]
            else:
                raise RankMismatch(f"e{head.seq:05d} {head.tag}: header `{key}` differs by rank: {values}")
        self._cache = {}

    @property
    def arrays(self):
        return self.parts[0].arrays

    def __contains__(self, name):
        return name in self.parts[0]

    def decomposed(self, name):
        return name in TRACER_ARRAYS

    def __getitem__(self, name):
        if name not in self._cache:
            arrays = [e[name] for e in self.parts]
            if self.decomposed(name):
                data = np.concatenate([a.data for a in arrays], axis=-1)
                if data.shape[-1] != self.meta["ntracet"]:
                    raise RankMismatch(f"e{self.seq:05d} {self.tag}: `{name}` slabs hold {data.shape[-1]} tracers, "
                                       f"the run has {self.meta['ntracet']}")  # fmt: skip
                self._cache[name] = FArray(np.asfortranarray(data), arrays[0].lower)
            else:
                first = arrays[0]
                for rk, a in zip(self.ranks[1:], arrays[1:], strict=True):
                    if a.lower != first.lower or a.data.shape != first.data.shape or \
                            a.data.tobytes() != first.data.tobytes():  # fmt: skip
                        raise RankMismatch(f"e{self.seq:05d} {self.tag}: `{name}` is not replicated -- rank {rk} "
                                           f"differs from rank {self.ranks[0]}")  # fmt: skip
                self._cache[name] = first
        return self._cache[name]

    def interior(self, name):
        return self[name][interior_section(name, self.meta["im"], self.meta["jm"], self.meta["lm"])]

    def device(self, name, dev):
        from .device import DevArray

        a = self[name]
        buf = DevArray.from_host(dev, a.data.ravel(order="F"))
        strides = [1]
        for n in a.data.shape[:-1]:
            strides.append(strides[-1] * n)
        return buf.reshape_axes(a.data.shape, tuple(strides), a.lower)

    def release(self):
        self._cache.clear()
        for e in self.parts:
            e.release()

    def cached(self):
        return list(self._cache)

    def ref(self):
        return EventRef(self.seq, self.tag, self.region, dict(self.meta), repr(self))

    def __repr__(self):
        return f"MergedEvent(seq={self.seq}, tag={self.tag!r}, region={self.region}, ranks={self.ranks})"


def _tracer_offsets(per_rank, ranks):
    """Each rank's first tracer (0-based): the tracer counts of the ranks before it, read from
    the last axis of the first event that has `rm`."""
    for ev in per_rank[ranks[0]]:
        if "rm" not in ev:
            continue
        counts = []
        for r in ranks:
            twin = next(x for x in per_rank[r] if x.seq == ev.seq)
            lo, hi = twin.bounds("rm")[-1]
            counts.append(hi - lo + 1)
        starts = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(int).tolist()
        return dict(zip(ranks, starts, strict=True))
    return dict.fromkeys(ranks, 0)


def merge_ranks(events):
    """A tracer-split run's events as the serial run's sequence: an event every rank wrote is
    merged (MergedEvent); a block of per-tracer events is taken from every rank and ordered by
    its global tracer number."""
    per_rank = {}
    for e in events:
        per_rank.setdefault(e.meta.get("rank", 0), []).append(e)
    ranks = sorted(per_rank)
    for r in ranks:
        per_rank[r].sort(key=lambda e: e.seq)
    offsets = _tracer_offsets(per_rank, ranks)
    pos = dict.fromkeys(ranks, 0)
    out = []
    while any(pos[r] < len(per_rank[r]) for r in ranks):
        heads = {r: per_rank[r][pos[r]] for r in ranks if pos[r] < len(per_rank[r])}
        if any(e.tag in PER_TRACER_TAGS for e in heads.values()):
            block = []
            for r in ranks:
                while pos[r] < len(per_rank[r]) and per_rank[r][pos[r]].tag in PER_TRACER_TAGS:
                    block.append(per_rank[r][pos[r]])
                    pos[r] += 1
            out += sorted(block, key=lambda e: e.meta["i_tracer"])
            continue
        if len(heads) != len(ranks):
            raise RankMismatch(f"ranks {sorted(set(ranks) - set(heads))} ran out of events before the others")
        out.append(MergedEvent(list(heads.values()), offsets))
        for r in ranks:
            pos[r] += 1
    return out
