"""The region tree against the reference's known answers (pydyn tests/test_zoom.py:83-110:
the production glb3x2 + nam1x1 footprint and scope, the eur grandchild's split order) and, where
the reference is importable, attribute by attribute against pydyn's own Zoom."""

import os
import sys
from pathlib import Path

import numpy as np
import pytest

from pydyn_gb300 import tree as T


def _levels(lm):
    return np.linspace(2000.0, 0.0, lm + 1), np.linspace(1.0, 0.0, lm + 1)


def production(lm=4):
    glb = T.Region("glb3x2", 120, 90, xcyc=1, touch_sp=1, touch_np=1)
    nam = T.Region("nam1x1", 72, 44, xbeg=-132, xend=-60, ybeg=20, yend=64, xref=3, yref=2, tref=2, parent=1)
    return T.Zoom([glb, nam], lm, *_levels(lm))


def eur(lm=3):
    glb = T.Region("glb600x400", 60, 45, xcyc=1, touch_sp=1, touch_np=1)
    e3 = T.Region("eur300x200", 30, 36, xbeg=-36, xend=54, ybeg=2, yend=74, xref=2, yref=2, tref=2, parent=1)
    e1 = T.Region("eur100x100", 60, 54, xbeg=-21, xend=39, ybeg=12, yend=66, xref=6, yref=4, tref=4, parent=2)
    return T.Zoom([glb, e3, e1], lm, *_levels(lm))


def test_production_tree_known_answers():
    zm = production()
    assert (zm.ibeg[2], zm.iend[2], zm.jbeg[2], zm.jend[2]) == (17, 40, 56, 77)
    assert (zm.isr[2], zm.ier[2], zm.jsr[2], zm.jer[2]) == (4, 69, 3, 42)
    assert zm.children == {0: [], 1: [2], 2: []}
    assert zm.splitorderzoom[2] == "xyzvsc" + "csvzyx" + "csvzyx" + "xyzvsc"
    assert (zm.zoomed[1] == 2).sum() == (40 - 17 - 1) * (77 - 56 - 1)
    assert (zm.edge[2] == -1).sum() == 72 * 44 - (72 - 6) * (44 - 4)


def test_eur_grandchild_split_order():
    zm = eur()
    assert (zm.ibeg[2], zm.iend[2], zm.jbeg[2], zm.jend[2]) == (25, 39, 24, 41)
    assert (zm.ibeg[3], zm.iend[3], zm.jbeg[3], zm.jend[3]) == (6, 25, 6, 32)
    fwd, rev = "xyzvsc", "csvzyx"
    assert zm.splitorderzoom[3] == fwd + rev + rev + fwd + rev + fwd + fwd + rev


def test_config2_child_footprint():
    """nam1x1 at 140W-50W, 10N-80N on glb3x2: the corners are not on the 3-degree lines, and
    Fortran nint places the footprint at i 14..43, j 51..85."""
    glb = T.Region("glb3x2", 120, 90, xcyc=1, touch_sp=1, touch_np=1)
    nam = T.Region("nam1x1", 90, 70, xbeg=-140, xend=-50, ybeg=10, yend=80, xref=3, yref=2, tref=2, parent=1)
    zm = T.Zoom([glb, nam], 34, *_levels(34))
    assert (zm.ibeg[2], zm.iend[2], zm.jbeg[2], zm.jend[2]) == (14, 43, 51, 85)
    assert (zm.isr[2], zm.ier[2], zm.jsr[2], zm.jer[2]) == (4, 87, 3, 68)


@pytest.mark.parametrize(("child", "why"), [({"touch_np": 1}, "pole-touching"),
                                            ({"xbeg": -180, "xend": -60, "im": 120}, "halo")])  # fmt: skip
def test_unsupported_trees_refuse(child, why):
    kw = {"im": 72, "jm": 44, "xbeg": -132, "xend": -60, "ybeg": 20, "yend": 64, "xref": 3, "yref": 2, "tref": 2,
          "parent": 1}  # fmt: skip
    kw.update(child)
    glb = T.Region("glb3x2", 120, 90, xcyc=1, touch_sp=1, touch_np=1)
    with pytest.raises(NotImplementedError, match=why):
        T.Zoom([glb, T.Region("c", **kw)], 3)


# the pydyn reference checkout, where one is available (PYDYN_REFERENCE); these tests skip without it
REF = Path(os.environ.get("PYDYN_REFERENCE", "")) if os.environ.get("PYDYN_REFERENCE") else None


@pytest.mark.skipif(REF is None or not (REF / "pydyn").is_dir(), reason="PYDYN_REFERENCE is not set")
@pytest.mark.parametrize("make", [production, eur])
def test_tree_equals_the_reference(make):
    sys.path.insert(0, str(REF))
    from pydyn import zoom as Z

    ours = make()
    regions = [Z.Region(**{k: getattr(g, k) for k in g._fields if k != "redgrid"})
               for g in ours.region[1:]]  # fmt: skip
    theirs = Z.Zoom(regions, ours.lm, ours.at, ours.bt)
    for name in ("children", "ibeg", "iend", "jbeg", "jend", "lbeg", "lend", "isr", "ier", "jsr", "jer",
                 "splitorderzoom"):  # fmt: skip
        assert getattr(ours, name) == getattr(theirs, name), name
    for r in ours.regions():
        assert (ours.zoomed[r] == theirs.zoomed[r]).all()
        assert (ours.edge[r] == theirs.edge[r]).all()


def test_the_device_module_has_every_body_the_driver_runs():
    """The driver runs st.lib's bodies: pydyn_gb300.zoom has each name of pydyn's zoom.host.BODIES
    (the list pydyn's tests/test_gpu.py:64-70 checks its own device module against)."""
    from pydyn_gb300 import zoom as gz

    assert [n for n in gz.BODIES if not callable(getattr(gz, n, None))] == []


@pytest.mark.skipif(REF is None or not (REF / "pydyn").is_dir(), reason="PYDYN_REFERENCE is not set")
def test_the_body_names_are_the_reference_s():
    sys.path.insert(0, str(REF))
    from pydyn.zoom import host

    from pydyn_gb300 import zoom as gz

    assert sorted(gz.BODIES) == sorted(host.BODIES)
