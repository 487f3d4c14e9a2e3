"""The autotuner: launch shapes per member class, and the ensemble's width.

Shapes (pydyn_gb300.device.Device.tune: threads per block of the thread-per-column and
thread-per-cell kernels, warps per block and lanes per column of the convection LU, the
convection apply's block)
are chosen by coordinate descent from the library's defaults: for each shape in turn, every
candidate is set, the class's interval graph is captured again, replayed a few times and timed
with CUDA events on the run's stream; the fastest candidate stays.  The width of an ensemble is
chosen the same way over whole batched steps.  A shape only decides how work is laid onto
threads and blocks, never what an element computes, so tuning changes no member's bits.

Results are kept in a JSON cache keyed by the GPU and the class (tree, levels, physics,
convection levels); a later run with the same key reuses them."""

import json
import os
import statistics
import time
from pathlib import Path

SPACE = {
    "column_threads": (32, 64, 128, 256),
    "cell_threads": (64, 128, 256, 512),
    "lu_warps": (1, 2, 4),
    "apply_threads": (0, 64, 128, 256, 512),  # 0: the block that evens out the FP64 work over the SMs
    "lu_lanes": (8, 16, 32),
}
WIDTHS = (4, 8, 16, 32, 64, 128, 256)
CACHE = Path(os.environ.get("PYDYN_GB300_TUNE_CACHE", Path(__file__).resolve().parent / "_build" / "tune.json"))


def _key(gpu, spec):
    return f"{gpu}|{spec.tree}|lm{spec.lm}|phys{int(spec.physics)}|lmax{spec.lmax}"


def load_cache(path=CACHE):
    try:
        return json.loads(Path(path).read_text())
    except (OSError, ValueError):
        return {}


def save_cache(cache, path=CACHE):
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    tmp = path.with_suffix(".tmp")
    tmp.write_text(json.dumps(cache, indent=1, sort_keys=True))
    tmp.replace(path)


def time_interval(fw, replays=5):
    """Median device time (ms) of the run's captured interval over `replays` replays."""
    dev = fw.dev
    ms = []
    for _ in range(replays):
        a, b = dev.event(), dev.event()
        a.record()
        fw.enqueue_interval_async(fw.t)
        b.record()
        if fw.settle_interval(fw.t) != (fw.nread, 1):
            continue  # a redone interval is not the graph's time
        ms.append(a.elapsed_ms(b))
    return statistics.median(ms) if ms else float("inf")


def tune_run(fw, space=None, replays=5, log=None):
    """Coordinate descent over `space` (default SPACE) on one run (a scratch member: its state
    advances).  Returns ({shape: value}, best ms per interval)."""
    space = SPACE if space is None else space
    dev = fw.dev
    if "interval" not in fw.graphs:
        fw.interval(graph=True)
    best = dict(dev.tuning())
    best_ms = time_interval(fw, replays)
    for name, values in space.items():
        for v in values:
            if v == best[name]:
                continue
            dev.tune(**{name: v})
            fw.capture_interval()
            ms = time_interval(fw, replays)
            if log:
                log(f"  {name}={v}: {ms:.3f} ms (best {best_ms:.3f})")
            if ms < best_ms:
                best_ms, best[name] = ms, v
        dev.tune(**best)
    fw.capture_interval()
    return best, best_ms


def tune_classes(specs, device=0, cache_path=CACHE, retune=False, replays=5, log=None, space=None):
    """{class: (shapes, ms per interval)} for the classes of `specs`, tuned on a scratch run of
    each class's first member (or read from the cache)."""
    from .device import Device

    cache = load_cache(cache_path)
    out = {}
    for spec in specs:
        if spec.cls in out:
            continue
        dev = Device(device)
        key = _key(dev.name(), spec)
        if not retune and key in cache:
            out[spec.cls] = (cache[key]["shapes"], cache[key]["ms"])
            dev.close()
            continue
        fw = spec.forward(dev)
        t = time.perf_counter()
        shapes, ms = tune_run(fw, space=space, replays=replays, log=log)
        if log:
            log(f"{spec.cls}: {shapes} {ms:.3f} ms/interval (tuned in {time.perf_counter() - t:.1f} s)")
        cache[key] = {"shapes": shapes, "ms": ms}
        out[spec.cls] = (shapes, ms)
        fw.close()
        dev.close()
    save_cache(cache, cache_path)
    return out


def tune_width(ens, widths=WIDTHS, steps=2, log=None):
    """The width of the fastest batched step of `ens` (captured) over `widths`; sets it."""
    best_w, best_s = ens.width, float("inf")
    for w in widths:
        if w > len(ens.specs):
            w = len(ens.specs)
        ens.set_width(w)
        ens.step()  # settle the lanes
        t = time.perf_counter()
        for _ in range(steps):
            ens.step()
        sec = (time.perf_counter() - t) / steps
        if log:
            log(f"  width {w}: {sec * 1e3:.1f} ms/step")
        if sec < best_s:
            best_w, best_s = w, sec
        if w == len(ens.specs):
            break
    ens.set_width(best_w)
    return best_w, best_s
