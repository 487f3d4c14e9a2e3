"""Benchmark: simulated years per wall-clock hour of the dynamic step on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--config NAME] [--impl gbdyn|reference]

A step is one read interval of one simulated hour (ndyn = nread = 3600 s): Check_CFL's mass-only
rehearsal on a copy of the air mass, then the step itself -- Setup_MassFlow and the operator
sequence xyzvsc | csvzyx on every region of the tree (with physics: Calc_Kzz, convection, CH4
emission and chemistry) -- replayed as one captured CUDA graph.  The metric is pydyn's own
(pydyn gpu/bench.py:262, forward.py:518): 3600 * 3600 / (365 * 86400 * wall seconds per step).

value: device time (CUDA events on the context's stream) of K replays, inputs resident in HBM,
L2 flushed between replays (a 256 MiB write).  e2e: the same steps through the public API with
the step's meteo copied in from pinned host memory and the step's tracer mass copied out, timed
on the host clock.  roofline: the body that takes the most device time in an eagerly enqueued
interval, its algorithmic bytes (per cell per application: x, y 2(2+4nt), z (2+4nt)+(1+4nt),
v 6+8nt, c 3+8nt, m2phlb 2, dynam0 5 values of 8 bytes) over its measured time, against the
measured HBM copy bandwidth; and, since the float64 step is bound by FP64 issue and not by HBM,
its FP64 warp instructions per call (an ncu capture of the same kernels) x 32 lanes over the same
time, against the DMUL/DADD issue rate measured in the run (`roofline.fp64`).  cpu_baseline:
the oracle (a scalar C restatement of pydyn) on this host's cores on a bounded sample of the
same workload.  published_case (the default workload at N = 1): pydyn's own GPU benchmark case,
timed after the headline by the same rules, with its value over the A100's published 60.1.

--impl reference runs the CPU reference arm: the oracle port of pydyn (the Python reference
itself cannot be installed where this runs) on the same workload, with the same metric.
With N > 1 (torchrun), every rank runs an independent replica of the workload (the step has no
data-parallel split; the runs are independent members) and rank 0 reports the whole-job rate."""

import argparse
import hashlib
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

SECONDS_A_YEAR = 365.0 * 86400.0
WORKLOADS = {
    # name: (tree, levels, physics (False, True: full, "convection"), seed, convection levels)
    "glb6x4": ("glb6x4", 25, False, 11, None),
    "glb3x2-adv": ("glb3x2", 34, False, 21, None),
    "glb3x2+nam1x1-adv": ("glb3x2+nam1x1", 34, False, 31, None),
    "glb3x2": ("glb3x2", 34, True, 41, 34),
    "glb3x2+nam1x1": ("glb3x2+nam1x1", 34, True, 42, 34),
    # pydyn's own GPU benchmark case (pydyn gpu/bench.py:34-41): glb3x2 + a 72 x 44 child, convection
    # over 26 levels on a given dkg, no Calc_Kzz, emission or chemistry
    "a100-case": ("glb3x2+nam72x44", 34, "convection", 51, 26),
}
# published numbers of the same metric on the same workload: the A100's interval replayed as a
# CUDA graph, 6.8 ms (pydyn docs/gpu_port.md:196-202)
PUBLISHED = {"a100-case": 60.1}
DEFAULT = "glb3x2+nam1x1"
BYTES_PER_CELL = {"_dynamu_region1": 12, "_dynamv_region1": 12, "_dynamw_region1": 11, "_dynamu_child": 12,
                  "_dynamv_child": 12, "_dynamw_child": 11, "convec_region": 14, "chemistry_region": 11,
                  "sources_region": 4, "calc_kzz": 5, "m2phlb1": 2, "m2phlb": 2,
                  "dynam0": 5}  # fmt: skip  (values of 8 bytes per cell and application at nt = 1)


# Per call of a body, from one ncu capture of an eager interval of each workload on the current
# kernels -- a convection body's seven k_convec launches, averaged over its calls in the interval
# (fresh and reusing its inverses; the parent's per v, both segments), and the step's Calc_Kzz of
# every region with the rate constants (the k_kzz and k_chem_krates launches): DRAM bytes
# (dram__bytes_read.sum + dram__bytes_write.sum), the roofline's traffic, and FP64 warp
# instructions (smsp__inst_executed_pipe_fp64.sum), whose issue bounds the step
# (profiles/interval_dram_fp64_glb3x2+nam1x1.md, profiles/interval_dram_fp64_a100-case.md);
# Calc_Kzz's FP64 count with its levels and interfaces kernels re-captured after log's tails
# were given their common products (the same file's single-kernel capture)
TRAFFIC_PER_CALL = {"glb3x2+nam1x1": {"convec_region@2": 131.5e6, "convec_region@1": 240.9e6, "calc_kzz": 131.8e6},
                    "a100-case": {"convec_region@2": 49.66e6, "convec_region@1": 182.7e6}}
FP64_PER_CALL = {"glb3x2+nam1x1": {"convec_region@2": 2.623e6, "convec_region@1": 3.319e6, "calc_kzz": 13.603e6},
                 "a100-case": {"convec_region@2": 1.394e6, "convec_region@1": 3.827e6}}


def workload_config(workload, n_gpus):
    """The `config` of a workload's line, the same in both arms."""
    tree, lm, physics, seed, lmax = WORKLOADS[workload]
    return {"workload": workload, "tree": tree, "levels": lm, "nt": 1, "physics": physics, "lmax": lmax,
            "seed": seed, "step": "Check_CFL rehearsal + Setup_MassFlow + xyzvsc|csvzyx (one read interval)",
            "l2": "flushed between timed steps (256 MiB write)", "parallelism": f"replicas x{n_gpus}"}  # fmt: skip


def metric_name(workload):
    """The headline metric's name for the full-physics glb3x2 + nam1x1 tree, else the workload's."""
    if workload == "glb3x2+nam1x1":
        return "sim-years/hour glb3×2+nam1×1 FP64-bitwise"
    if workload == "a100-case":
        return "sim-years/hour glb3×2+nam1×1 (72×44) lmax 26 convection-only interval FP64-bitwise"
    return f"sim-years/hour {workload} FP64-bitwise"


def step_bytes_per_cell(physics, tref):
    """Algorithmic bytes a cell of a region with time refinement tref moves per step at nt = 1:
    2 tref half steps of x, y, z (296 B), plus v (112 B) with any physics and c (88 B) with full
    physics; then dynam0 (40 B), Calc_Kzz (40 B, full physics) and Check_CFL (248 B) once."""
    b_half = 296 + (112 if physics else 0) + (88 if physics is True else 0)
    return 2 * tref * b_half + 40 + (40 if physics is True else 0) + 248


def sim_years_per_hour(seconds_per_step, step_seconds=3600.0):
    return 3600.0 * step_seconds / (SECONDS_A_YEAR * seconds_per_step)


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi samples (200 ms) of SM clock and throttle reasons during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")  # fmt: skip

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.path = Path(tempfile.mkstemp(suffix=".csv")[1])

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)  # fmt: skip
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            self.proc.wait(timeout=10)
        return False

    def summary(self):
        rows = []
        for line in self.path.read_text().splitlines() if self.path.exists() else []:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no nvidia-smi samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9], strict=False) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}  # fmt: skip


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    return ws, int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0"))


def max_over_ranks(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist

    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def oracle_threads():
    """Host threads the oracle's column loops run on (OpenMP: OMP_NUM_THREADS, else every core)."""
    return int(os.environ.get("OMP_NUM_THREADS") or os.cpu_count() or 1)


def cpu_baseline(workload, seconds=15.0):
    """The oracle on this host: whole intervals of the same workload until ~`seconds` pass."""
    from oracle.forward import OracleRun

    tree, lm, physics, seed, lmax = WORKLOADS[workload]
    orc = OracleRun(tree, lm, seed, physics=physics, lmax=lmax)
    t0 = time.perf_counter()
    n = 0
    while n < 1 or (time.perf_counter() - t0 < seconds and n < 50):
        orc.interval()
        n += 1
    per = (time.perf_counter() - t0) / n
    cores = oracle_threads()
    return {"value": sim_years_per_hour(per), "unit": "sim-years/hour", "cores": cores, "kind": "port",
            "sample": f"{n} whole intervals of {workload} ({per:.3f} s each; the oracle's column loops on "
                      f"{cores} host threads, its driver and NumPy glue on one)"}  # fmt: skip


def run_reference_ensemble(args):
    """The reference arm of the ensemble: the oracle port looped over the members, timed on a
    bounded sample -- one interval of one member of each class -- and scaled by the mix."""
    from oracle.forward import OracleRun
    from pydyn_gb300.synth import ENSEMBLE_CLASSES as CLASSES
    from pydyn_gb300.synth import ENSEMBLE_MIX as MIX

    mix = MIX if not args.mix else tuple((c, int(n)) for c, n in (x.split(":") for x in args.mix.split(",")))
    per_step, sample = 0.0, []
    for cls, count in mix:
        tree, lm, lmax, seed = CLASSES[cls]
        orc = OracleRun(tree, lm, seed, physics=True, lmax=lmax)
        t0 = time.perf_counter()
        orc.interval()
        sec = time.perf_counter() - t0
        per_step += count * sec
        sample.append(f"{cls} {sec:.2f} s")
    n = sum(c for _, c in mix)
    v = n * sim_years_per_hour(per_step)
    line = {
        "impl": "reference", "metric": "member-years/hour, 256-member ensemble (128 glb6×4, 96 glb3×2, "
        "32 glb3×2+nam1×1) FP64-bitwise", "value": v, "unit": "member-years/hour", "n_gpus": args.gpus,
        "steps": 1, "warmup": 0, "ms_per_step": per_step * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "ensemble", "members": n, "mix": [list(m) for m in mix]},
        "cpu_baseline": {"value": v, "unit": "member-years/hour", "cores": oracle_threads(), "kind": "port",
                         "sample": "one interval of one member per class (the oracle's column loops on "
                                   f"{oracle_threads()} host threads): " + ", ".join(sample)
                                   + "; scaled by the member counts"},
        "e2e": {"value": v, "unit": "member-years/hour", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }  # fmt: skip
    print(json.dumps(line), flush=True)


def run_reference(args, ws, rank):
    """--impl reference: the CPU reference arm on rank 0 -- the oracle port of pydyn (its C
    restatement and its restatement of pydyn's driver; nothing of the package runs but the
    synthetic-input generator)."""
    if rank != 0:
        return
    from oracle.build import build as build_oracle

    build_oracle()
    from oracle.forward import OracleRun

    if args.config == "ensemble":
        run_reference_ensemble(args)
        return
    tree, lm, physics, seed, lmax = WORKLOADS[args.config]
    orc = OracleRun(tree, lm, seed, physics=physics, lmax=lmax)
    for _ in range(args.warmup):
        orc.interval()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        orc.interval()
    per = (time.perf_counter() - t0) / args.steps
    v = sim_years_per_hour(per)
    line = {
        "impl": "reference", "metric": metric_name(args.config), "value": v,
        "unit": "sim-years/hour", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": per * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": workload_config(args.config, args.gpus),
        "cpu_baseline": {"value": v, "unit": "sim-years/hour", "cores": oracle_threads(), "kind": "port",
                         "sample": f"{args.steps} whole intervals of {args.config} (the oracle's column loops on "
                                   f"{oracle_threads()} host threads, its driver and NumPy glue on one)"},
        "e2e": {"value": v, "unit": "sim-years/hour", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }  # fmt: skip
    print(json.dumps(line), flush=True)


def _ensemble_timed(ens, steps, fn):
    """Device time (s per step) of `steps` calls of fn(ens): an event on the first member's
    stream that every member's stream waits on opens the region, each member's own event after
    the last step closes it; the slowest member's span counts."""
    d0 = ens.devs[0]
    start = d0.event()
    start.record()
    for d in ens.devs[1:]:
        d.wait(start)
    for _ in range(steps):
        fn(ens)
    ends = []
    for d in ens.devs:
        e = d.event()
        e.record()
        ends.append(e)
    ens.sync()
    return max(start.elapsed_ms(e) for e in ends) / 1e3 / steps


def run_ensemble(args, ws, rank):
    """--config ensemble: the batched ensemble (pydyn_gb300.ensemble) against the plain step
    looped over the same members, member-years per hour; every rank runs its own ensemble."""
    from __graft_entry__ import build

    build()
    from pydyn_gb300.ensemble import MIX, Ensemble, member_specs
    from pydyn_gb300.hostbuf import PinnedArray
    from pydyn_gb300.tune import tune_classes, tune_width

    def log(msg):
        if rank == 0:
            print(msg, file=sys.stderr, flush=True)

    mix = MIX if not args.mix else tuple((c, int(n)) for c, n in (x.split(":") for x in args.mix.split(",")))
    specs = member_specs(mix, seed=2024 + rank)
    t_setup = time.perf_counter()
    tuned = tune_classes(specs, log=log)
    shapes = {c: s for c, (s, _) in tuned.items()}
    costs = {c: ms for c, (_, ms) in tuned.items()}
    ens = Ensemble(specs, shapes=shapes, costs=costs)
    ens.step()  # every member's first interval, uncaptured, and its capture
    width, _ = tune_width(ens, log=log)
    setup_s = time.perf_counter() - t_setup
    for _ in range(args.warmup):
        ens.step()
    barrier(ws)
    n0 = sum(fw.launches() for fw in ens.runs)
    with Clocks(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        batched = max_over_ranks(_ensemble_timed(ens, args.steps, lambda e: e.step()), ws)
    launches = sum(fw.launches() for fw in ens.runs) - n0
    looped = max_over_ranks(_ensemble_timed(ens, args.steps, lambda e: e.step_looped()), ws)

    # end to end: every member's new meteo instant in from pinned host memory, its tracer mass
    # out, on its own stream around its graph
    pin_in, pin_out, h2d, d2h = {}, {}, 0, 0
    for k, fw in enumerate(ens.runs):
        pin_in[k] = {r: [PinnedArray.copy_of(x) for x in fw.met.fluxes(r, 1)] for r in fw.zoom.regions()}
        pin_out[k] = {r: PinnedArray.empty((fw.zoom.g(r).im, fw.zoom.g(r).jm, fw.zoom.lm, 1)) for r in fw.zoom.regions()}
        h2d += sum(p.nbytes for v in pin_in[k].values() for p in v)
        d2h += sum(p.nbytes for p in pin_out[k].values())

    def before(k):
        fw = ens.runs[k]
        for r in fw.zoom.regions():
            pu1, pv1 = fw.meteo[r][1]
            pin_in[k][r][0].to_device(ens.devs[k], pu1)
            pin_in[k][r][1].to_device(ens.devs[k], pv1)

    def after(k):
        fw = ens.runs[k]
        for r in fw.zoom.regions():
            g = fw.zoom.g(r)
            pin_out[k][r].from_device(ens.devs[k], fw.st[r]["rm"][1 : g.im, 1 : g.jm, 1 : fw.zoom.lm])

    ens.step(before, after)  # the staging arrays of the strided reads are made outside the timing
    barrier(ws)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ens.step(before, after)
    e2e = max_over_ranks((time.perf_counter() - t0) / args.steps, ws)

    # every class's first member against its solo run over the same intervals
    from pydyn_gb300.device import Device

    def digest(fw):
        h = hashlib.sha1()
        for r in fw.zoom.regions():
            for name in sorted(fw.st[r]):
                h.update(np.ascontiguousarray(fw.st[r][name].host()).tobytes())
        return h.hexdigest()

    checked = []
    for cls, _ in mix:
        k = next(i for i, s in enumerate(specs) if s.cls == cls)
        fw = ens.runs[k]
        got = digest(fw)
        intervals = round(fw.t / fw.nread)
        solo_dev = Device(0)
        solo = specs[k].forward(solo_dev)
        for _ in range(intervals):
            solo.interval(graph=True)
        want = digest(solo)
        solo.close()
        solo_dev.close()
        checked.append({"member": k, "class": cls, "intervals": intervals, "bitwise": got == want})
    n = len(specs)
    step_bytes = 0
    hbm, how = peaks()
    for fw in ens.runs:
        for r in fw.zoom.regions():
            g = fw.zoom.g(r)
            step_bytes += g.im * g.jm * fw.zoom.lm * step_bytes_per_cell(True, g.tref)
    line = {
        "metric": "member-years/hour, 256-member ensemble (128 glb6×4, 96 glb3×2, 32 glb3×2+nam1×1) FP64-bitwise",
        "value": n * sim_years_per_hour(batched) * ws,
        "unit": "member-years/hour",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": batched * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded meteo per class, per-member wind scale and physics inputs; pydyn_gb300.synth)",
        "config": {"workload": "ensemble", "members": n, "mix": [list(m) for m in mix], "width": width,
                   "shapes": shapes, "physics": True,
                   "step": "every member's captured interval (Check_CFL rehearsal + step), members in flight together",
                   "l2": f"inputs larger than L2 (the members' state: {step_bytes / 1e9:.1f} GB of step traffic)",
                   "parallelism": f"ensemble x{ws}"},
        "plain_looped": {"value": n * sim_years_per_hour(looped) * ws, "unit": "member-years/hour",
                         "ms_per_step": looped * 1e3},
        "batched_vs_plain": looped / batched,
        "roofline": {"bound": "hbm", "achieved": step_bytes / batched / 1e9, "peak": hbm, "unit": "GB/s",
                     "frac": step_bytes / batched / 1e9 / hbm, "traffic": None, "peak_source": how,
                     "note": "algorithmic step bytes of all members over the batched step; the float64 "
                             "kernels are bound by the FP64 pipe, not HBM"},
        "e2e": {"value": n * sim_years_per_hour(e2e) * ws, "unit": "member-years/hour", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "bitwise_vs_solo": checked,
        "redone_intervals": ens.redone,
        "setup_s": setup_s,
        "cpu_baseline": None,
    }  # fmt: skip
    if rank == 0:
        print(json.dumps(line), flush=True)
    ens.close()


def run_adjoint(args, ws, rank):
    """--config adjoint: the CH4 surface-flux gradient on glb3x2 (34 levels, physics, unlimited
    slopes) through `--hours` one-hour intervals (default 168: 7 days), 500 seeded samples,
    checkpoints every 6 intervals: the forward J, the checkpointed adjoint, their ratio; the
    dot-product test on one interval; central differences on `--fd` flux elements."""
    from __graft_entry__ import build

    build()
    from pydyn_gb300.adjoint import FluxGradient, make_samples
    from pydyn_gb300.device import Device
    from pydyn_gb300.forward import Forward

    dev = Device(int(os.environ.get("LOCAL_RANK", "0")))
    hours = args.hours
    fw = Forward(dev, "glb3x2", 34, seed=41, physics=True, lmax=34, limits=False)
    im, jm = fw.zoom.g(1).im, fw.zoom.g(1).jm
    samples = make_samples(fw.zoom, hours, 500, seed=7)

    # the dot-product test on the first interval: tracers x, adjoints y (the state put back after)
    prob = FluxGradient(fw, hours, samples, np.zeros(len(samples)), every=6)
    flux = fw.physics.r[1]["flux"].host()
    rng = np.random.default_rng(9)
    shape = (4, im, jm, 34)
    scale = np.array([1.0, 0.3, 0.3, 0.3])[:, None, None, None]
    x, y = rng.random(shape) * scale, (rng.random(shape) + 0.5) * scale
    ax, (aty,) = prob.interval_pair(x, [y])
    lhs, rhs = float(np.dot(ax.ravel(), y.ravel())), float(np.dot(x.ravel(), aty.ravel()))
    dot_rel = abs(lhs - rhs) / abs(lhs)
    prob._restore(prob.start)
    prob.set_flux(flux)

    # observations: the first guess's sampled values perturbed by 2 %
    prob.cost(flux)
    rows = np.concatenate([prob.rm_at[h][0] for h in range(1, hours + 1)])
    vals = np.concatenate([prob.rm_at[h][1] for h in range(1, hours + 1)])
    obs = np.empty(len(samples))
    obs[rows] = vals * (1.0 + 0.02 * np.random.default_rng(4).standard_normal(len(vals)))
    prob.obs = obs
    prob.cost(flux)  # warm: every lazily made array exists
    prob.gradient().free()
    dev.sync()
    t0 = time.perf_counter()
    J = prob.cost(flux)
    t_fwd = time.perf_counter() - t0
    t0 = time.perf_counter()
    grad = prob.gradient().host()
    t_adj = time.perf_counter() - t0

    # central differences (step 1e-6 relative) on seeded flux elements
    fd_err, picks = [], np.random.default_rng(11).choice(im * jm, args.fd, replace=False)
    for k in picks:
        i, j = np.unravel_index(int(k), (im, jm))
        h = 1e-6 * abs(flux[i, j])
        fp, fm = flux.copy(), flux.copy()
        fp[i, j] += h
        fm[i, j] -= h
        fd = (prob.cost(fp) - prob.cost(fm)) / (2.0 * h)
        fd_err.append(abs(fd - grad[i, j]) / np.abs(grad).max())
    line = {
        "metric": "adjoint cost / forward cost, CH4 surface-flux gradient, glb3×2 7 days",
        "value": t_adj / t_fwd, "unit": "x forward", "higher_is_better": False,
        "n_gpus": ws, "steps": hours, "warmup": 1, "ms_per_step": t_adj / hours * 1e3,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (glb3x2 case of pydyn_gb300.synth, 500 seeded samples, 2 % perturbed observations)",
        "config": {"workload": "adjoint", "tree": "glb3x2", "levels": 34, "lmax": 34, "hours": hours,
                   "checkpoint_every": 6, "samples": len(samples), "limits": False},
        "forward_s": t_fwd, "adjoint_s": t_adj, "J": J,
        "dot_product_rel_err": dot_rel,
        "fd": {"elements": int(args.fd), "step": "1e-6 relative", "max_err_rel_to_max_grad": max(fd_err) if fd_err else None},
        "gpu_launches": None, "e2e": None, "cpu_baseline": None,
    }  # fmt: skip
    if rank == 0:
        print(json.dumps(line), flush=True)
    prob.close()
    fw.close()
    dev.close()


def published_case(dev, flush, steps, warmup, gpu):
    """The a100-case workload (pydyn gpu/bench.py:34-41) on the same device, timed as the
    headline is: graph replays after `warmup` of them, the L2 flushed between replays, CUDA
    events on the run's stream, clocks sampled during the timed region."""
    from pydyn_gb300.forward import Forward

    tree, lm, physics, seed, lmax = WORKLOADS["a100-case"]
    fw = Forward(dev, tree, lm, seed=seed, physics=physics, lmax=lmax)
    fw.interval(graph=False)
    for _ in range(warmup):
        fw.interval(graph=True)
    evs = [(dev.event(), dev.event()) for _ in range(steps)]
    dev.sync()
    with Clocks(gpu) as clk:
        t = fw.t
        for k in range(steps):
            flush.fill(float(k))
            a, b = evs[k]
            a.record()
            fw.enqueue_interval_async(t)
            b.record()
            t += fw.nread
        dev.sync()
    if fw.rehearsal_failed():
        raise RuntimeError("bench: Check_CFL rejected ndyn = nread in the published case")
    fw.t = t
    sec = sum(a.elapsed_ms(b) for a, b in evs) / steps / 1e3
    fw.close()
    value = sim_years_per_hour(sec)
    return {"workload": "a100-case", "metric": metric_name("a100-case"), "value": value,
            "unit": "sim-years/hour", "ms_per_step": sec * 1e3, "published": PUBLISHED["a100-case"],
            "vs_published": value / PUBLISHED["a100-case"], "steps": steps, "warmup": warmup,
            "config": workload_config("a100-case", 1), "clocks": clk.summary()}  # fmt: skip


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)  # ~1 s timed: several clock samples
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--config", default=DEFAULT, choices=sorted(WORKLOADS) + ["ensemble", "adjoint"])
    ap.add_argument("--hours", type=int, default=168, help="adjoint: one-hour intervals")
    ap.add_argument("--fd", type=int, default=50, help="adjoint: flux elements checked by central differences")
    ap.add_argument("--mix", default=None, help="ensemble members, e.g. glb6x4:128,glb3x2:96,glb3x2+nam1x1:32")
    ap.add_argument("--impl", default="gbdyn", choices=("gbdyn", "reference"))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    ws, rank, local = dist_env()
    if args.config == "ensemble":  # before the first CUDA call: one hardware queue per lane
        os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
    if ws > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    args.warmup = max(args.warmup, 3)
    if args.config == "adjoint":
        run_adjoint(args, ws, rank)
        return
    if args.config == "ensemble":
        if args.steps == 100:  # the plain step's default; an ensemble step is ~0.5 s
            args.steps = 5
        run_ensemble(args, ws, rank)
        return

    from __graft_entry__ import build

    build()
    from pydyn_gb300.device import DevArray, Device
    from pydyn_gb300.forward import Forward
    from pydyn_gb300.profile import BodyProfiler

    tree, lm, physics, seed, lmax = WORKLOADS[args.config]
    dev = Device(local)
    fw = Forward(dev, tree, lm, seed=seed, physics=physics, lmax=lmax)  # every replica runs the same case

    # per-body device time of one eager interval (after a first one has made every lazily
    # allocated array and grown the work space): the roofline's dominant body
    fw.interval(graph=False)
    with BodyProfiler(dev, fw.physics) as prof:
        fw.interval(graph=False)
    bodies = prof.report()

    for _ in range(args.warmup):
        fw.interval(graph=True)
    flush = DevArray.zeros(dev, (0, 32 * 1024 * 1024 - 1))  # 256 MiB > the 129 MB L2
    evs = [(dev.event(), dev.event()) for _ in range(args.steps)]
    n0 = fw.launches()
    barrier(ws)
    dev.sync()
    t_wall = time.perf_counter()
    with Clocks(local) as clk:
        t = fw.t
        for k in range(args.steps):
            flush.fill(float(k))
            a, b = evs[k]
            a.record()
            fw.enqueue_interval_async(t)
            b.record()
            t += fw.nread
        dev.sync()
    wall = time.perf_counter() - t_wall
    launches = fw.launches() - n0 - args.steps  # the flushes are not the step's
    if fw.rehearsal_failed():
        raise RuntimeError("bench: Check_CFL rejected ndyn = nread inside the timed region")
    fw.t = t
    ms = [a.elapsed_ms(b) for a, b in evs]
    sec_per_step = max_over_ranks(sum(ms) / len(ms) / 1e3, ws)

    # e2e: host buffers through the public API, the step's meteo in and tracer mass out
    host_in = {r: [np.ascontiguousarray(x) for x in fw.met.fluxes(r, 1)] for r in fw.zoom.regions()}
    pinned_in, pinned_out = {}, {}
    from pydyn_gb300.hostbuf import PinnedArray

    for r in fw.zoom.regions():
        pinned_in[r] = [PinnedArray.copy_of(x) for x in host_in[r]]
        g = fw.zoom.g(r)
        pinned_out[r] = [PinnedArray.empty((g.im, g.jm, lm, 1)) for _ in range(2)]  # alternate steps'
    h2d = sum(p.nbytes for v in pinned_in.values() for p in v)
    d2h = sum(p[0].nbytes for p in pinned_out.values())
    barrier(ws)
    dev.sync()
    # a host pipeline of one step in flight: step k's meteo in, its interval and its tracer mass
    # out are enqueued in stream order (so no copy races a kernel), then the host waits for step
    # k-1's tracer mass to be in host memory while step k runs; the last step's is waited for
    # inside the timed region too
    t0 = time.perf_counter()
    done = None
    for k in range(args.steps):
        for r in fw.zoom.regions():
            pu1, pv1 = fw.meteo[r][1]
            pinned_in[r][0].to_device(dev, pu1)
            pinned_in[r][1].to_device(dev, pv1)
        fw.enqueue_interval_async(fw.t)
        fw.t += fw.nread
        for r in fw.zoom.regions():
            g = fw.zoom.g(r)
            pinned_out[r][k % 2].from_device(dev, fw.st[r]["rm"][1 : g.im, 1 : g.jm, 1:lm])
        ev = dev.event()
        ev.record()
        if done is not None:
            done.synchronize()
        done = ev
    done.synchronize()
    e2e_sec = max_over_ranks((time.perf_counter() - t0) / args.steps, ws)
    if fw.rehearsal_failed():
        raise RuntimeError("bench: Check_CFL rejected ndyn = nread in the e2e loop")

    # roofline of the dominant body
    hbm, how = peaks()
    fp64 = dev.fp64_rates()  # measured here, after the timed region: the FP64 pipe's issue rates
    name, (calls, total_ms, nlaunch) = max(bodies.items(), key=lambda kv: kv[1][1])
    cells = {r: fw.zoom.g(r).im * fw.zoom.g(r).jm * lm for r in fw.zoom.regions()}
    body, _, region = name.partition("@")
    # a body named without a region (calc_kzz: the step's Calc_Kzz of every region) covers them all
    ncell = cells[int(region)] if region else sum(cells.values())
    per_call_bytes = 8 * BYTES_PER_CELL.get(body, 0) * ncell
    achieved = per_call_bytes / (total_ms / calls / 1e3) / 1e9 if per_call_bytes else None
    roof = {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": achieved / hbm if achieved else None,
            "traffic": TRAFFIC_PER_CALL.get(args.config, {}).get(name), "peak_source": how,
            "bytes_per_launch": per_call_bytes, "ms_per_launch": total_ms / calls,
            "fp64_rates_g_per_s": fp64,
            "note": "float64 with no contraction: the FP64 pipe (fp64_rates, measured in this run) bounds the step"}  # fmt: skip
    inst = FP64_PER_CALL.get(args.config, {}).get(name)
    if inst is not None:
        # the FP64 pipe holds a warp instruction for the same time whatever its active lanes: the
        # body's issue rate is its warp instructions x 32 lanes over its time per call, against
        # the DMUL/DADD issue rate measured in this run
        issued = inst * 32 / (total_ms / calls / 1e3) / 1e9
        roof["fp64"] = {"bound": "fp64", "achieved": issued, "peak": fp64["dmul_dadd"], "unit": "G FP64 lane-op/s",
                        "frac": issued / fp64["dmul_dadd"], "warp_inst_per_launch": inst,
                        "note": "FP64 warp instructions per call from an ncu capture of the same kernels "
                                "(smsp__inst_executed_pipe_fp64.sum) x 32 / the live time per call"}  # fmt: skip

    step_bytes = sum(n * step_bytes_per_cell(physics, fw.zoom.g(r).tref) for r, n in cells.items())
    total_time = sum(v[1] for v in bodies.values())
    line = {
        "metric": metric_name(args.config),
        "value": sim_years_per_hour(sec_per_step) * ws,
        "unit": "sim-years/hour",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": sec_per_step * 1e3,
        "higher_is_better": True, "scaling": "weak", "dtype": "f64",
        "vs_baseline": (sim_years_per_hour(sec_per_step) * ws / PUBLISHED[args.config]
                        if args.config in PUBLISHED else None),
        "data": "synthetic (seeded meteo of the configuration's shape; pydyn_gb300.synth)",
        "config": workload_config(args.config, ws),
        "roofline": roof,
        "step_bytes": step_bytes,
        "step_hbm_frac": step_bytes / sec_per_step / 1e9 / hbm,
        "e2e": {"value": sim_years_per_hour(e2e_sec) * ws, "unit": "sim-years/hour", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "wall_s": wall,
        "bodies_ms": {k: round(v[1], 4) for k, v in sorted(bodies.items(), key=lambda kv: -kv[1][1])},
        "eager_interval_ms": total_time,
    }  # fmt: skip
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args.config)
    fw.close()
    if ws == 1 and args.config == DEFAULT:
        # pydyn's own GPU benchmark case beside the headline, the only workload with a
        # published number: timed after the headline's timed region, by the same rules
        line["published_case"] = published_case(dev, flush, args.steps, args.warmup, local)
    if rank == 0:
        print(json.dumps(line), flush=True)
    dev.close()
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
