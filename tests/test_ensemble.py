"""The batched ensemble (pydyn_gb300.ensemble) and the autotuner (pydyn_gb300.tune).

CPU: the member mix and its seeds, the lane assignment, the tuning cache.  GPU: every member of
a small mixed ensemble, run batched over two lanes, is bitwise its solo run after every
interval, and a member made with a reference run's settings matches the reference's digests;
runs under non-default launch shapes match the reference too (the shapes decide the layout of
work onto threads, never an element's value)."""

import json
from pathlib import Path

import pytest

from pydyn_gb300.ensemble import MIX, MemberSpec, lanes_for, member_specs
from pydyn_gb300.tune import SPACE, load_cache, save_cache

GOLDEN = json.loads((Path(__file__).parent / "golden" / "steps.json").read_text())


def test_member_mix():
    specs = member_specs()
    assert len(specs) == 256
    counts = {c: sum(s.cls == c for s in specs) for c, _ in MIX}
    assert counts == {"glb6x4": 128, "glb3x2": 96, "glb3x2+nam1x1": 32}
    assert [s.index for s in specs] == list(range(256))
    assert all(0.9 <= s.wind_scale <= 1.1 for s in specs)
    assert len({s.member_seed for s in specs}) == 256
    assert all(s.physics for s in specs)
    assert specs == member_specs()  # seeded
    assert member_specs(seed=7) != specs


def test_lanes_longest_first():
    costs = [5.0] * 3 + [1.0] * 10 + [0.2] * 30
    for width in (1, 3, 7, 64):
        lanes = lanes_for(costs, width)
        assert sorted(k for lane in lanes for k in lane) == list(range(len(costs)))
        assert len(lanes) == min(width, len(costs))
        load = [sum(costs[k] for k in lane) for lane in lanes]
        assert max(load) - min(load) <= max(costs) + 1e-12
        for lane in lanes:  # each lane launches its members longest first
            assert [costs[k] for k in lane] == sorted((costs[k] for k in lane), reverse=True)


def test_tune_cache_round_trip(tmp_path):
    path = tmp_path / "t.json"
    assert load_cache(path) == {}
    cache = {"GPU sm_103 x152|glb6x4|lm25|phys1|lmax25": {"shapes": {"lu_warps": 2}, "ms": 1.5}}
    save_cache(cache, path)
    assert load_cache(path) == cache
    assert all(len(v) >= 3 for v in SPACE.values())


# ------------------------------------------------------------------ device
def _digest(fw):
    from make_golden import STATE_FIELDS, digest

    return digest({r: {n: fw.st[r][n].host() for n in STATE_FIELDS} for r in fw.zoom.regions()})


def _golden_spec(index, name):
    tree, lm, seed = GOLDEN[name]["config"], GOLDEN[name]["lm"], GOLDEN[name]["seed"]
    lmax = GOLDEN[name].get("lmax")
    return MemberSpec(index, name, tree, lm, lmax, lmax is not None, seed, seed, 1.0)


@pytest.mark.gpu
def test_batched_members_are_their_solo_runs(built):
    from pydyn_gb300.device import Device
    from pydyn_gb300.ensemble import Ensemble

    classes = {"g6": ("glb6x4", 10, 10, 11), "two": ("two", 8, 8, 21), "three": ("three", 6, 6, 22)}
    specs = member_specs((("g6", 2), ("two", 2), ("three", 1)), seed=5, classes=classes)
    specs.append(_golden_spec(len(specs), "two-phys"))
    nint = 3
    ens = Ensemble(specs, width=2)
    got = [[] for _ in specs]
    for _ in range(nint):
        ens.step()
        for k, fw in enumerate(ens.runs):
            got[k].append(_digest(fw))
    assert len(ens.lanes) == 2
    ens.close()
    for k, s in enumerate(specs):
        dev = Device(0)
        fw = s.forward(dev)
        for i in range(nint):
            fw.interval(graph=True)
            assert _digest(fw) == got[k][i], f"member {k} ({s.cls}): interval {i} differs from its solo run"
        fw.close()
        dev.close()
    want = [d for _, _, d in GOLDEN["two-phys"]["steps"][:nint]]
    assert got[-1] == want, "the member made as the reference run differs from the reference"


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["two-phys", "three-phys"])
def test_launch_shapes_keep_the_bits(built, name):
    from pydyn_gb300.device import Device

    spec = _golden_spec(0, name)
    run = GOLDEN[name]
    for shapes in ({"column_threads": 32, "cell_threads": 512, "lu_warps": 1, "apply_threads": 512, "lu_lanes": 8},
                   {"column_threads": 256, "cell_threads": 64, "lu_warps": 4, "apply_threads": 64, "lu_lanes": 32}):  # fmt: skip
        dev = Device(0)
        dev.tune(**shapes)
        assert dev.tuning() == shapes
        fw = spec.forward(dev)
        for k, (ndyn, n, want) in enumerate(run["steps"][:3]):
            assert fw.interval(graph=k > 0) == (ndyn, n)
            assert _digest(fw) == want, f"{name} under {shapes}: interval {k} differs from the reference"
        fw.close()
        dev.close()


@pytest.mark.gpu
def test_tune_set_rejects_bad_shapes(dev):
    from pydyn_gb300._native import DeviceError

    before = dev.tuning()
    for bad in ({"column_threads": 48}, {"cell_threads": 1024}, {"lu_warps": 8}, {"apply_threads": 2048},
                {"lu_lanes": 12}):
        with pytest.raises((DeviceError, ValueError)):
            dev.tune(**bad)
    assert dev.tuning() == before


@pytest.mark.gpu
def test_tuner_picks_shapes_from_the_space(built, tmp_path):
    from pydyn_gb300.tune import tune_classes

    specs = member_specs((("two", 1),), seed=3, classes={"two": ("two", 8, 8, 21)})
    space = {"lu_warps": (1, 2), "cell_threads": (64, 128)}  # each holding the library's default
    out = tune_classes(specs, cache_path=tmp_path / "t.json", replays=2, space=space)
    shapes, ms = out["two"]
    assert shapes["lu_warps"] in (1, 2) and shapes["cell_threads"] in (64, 128)
    assert ms > 0
    assert load_cache(tmp_path / "t.json")
