"""ORACLE -- test infrastructure.  The replay's bitwise comparison report restated on the host
(pydyn harness.py:140-179: _ulp_distance, bits, compare): the checker of the device's gb_compare."""

import numpy as np


def ulp_distance(a, b):
    """|o(a) - o(b)| elementwise with o the sign-magnitude image of the bit patterns (int64,
    wrapping as NumPy's integer arithmetic does)."""

    def ordered(x):
        i = np.ascontiguousarray(x, dtype="<f8").view(np.int64)
        return np.where(i < 0, np.iinfo(np.int64).min - i, i)

    with np.errstate(over="ignore"):
        return np.abs(ordered(a) - ordered(b))


def compare(model, ours, name=""):
    """The report: equal, n_diff, max_ulp, max_abs, max_rel, and for a difference the first
    differing index in row-major order with both values there."""
    model = np.asarray(model, dtype=float)
    ours = np.asarray(ours, dtype=float)
    if model.shape != ours.shape:
        raise ValueError(f"{name}: shape {model.shape} vs {ours.shape}")
    differ = np.ascontiguousarray(model).view(np.int64) != np.ascontiguousarray(ours).view(np.int64)
    if not differ.any():
        return {"name": name, "equal": True, "n_diff": 0, "max_ulp": 0, "max_abs": 0.0, "max_rel": 0.0}
    with np.errstate(invalid="ignore", divide="ignore", over="ignore"):
        diff = np.abs(model - ours)
        rel = np.where(differ, diff / np.maximum(np.abs(model), np.abs(ours)), 0.0)
    first = tuple(int(i) for i in np.argwhere(differ)[0])
    return {"name": name, "equal": False, "n_diff": int(differ.sum()), "max_ulp": int(ulp_distance(model, ours).max()),
            "max_abs": float(diff.max()), "max_rel": float(rel.max()), "first": first,
            "first_values": (float(model[first]), float(ours[first]))}  # fmt: skip
