"""Comparison helpers shared by the parity tests."""
import numpy as np

from fvmic2d_gb300.mic_types import MARKER_DTYPE

F64_FIELDS = [n for n in MARKER_DTYPE.names if MARKER_DTYPE.fields[n][0] == np.dtype("<f8")]
I32_FIELDS = [n for n in MARKER_DTYPE.names if MARKER_DTYPE.fields[n][0] == np.dtype("<i4")]

# the floating-point parity bar: relative 1e-12, with an absolute floor of 1e-12 times the
# field's largest magnitude for values that cancel towards zero (stresses, stress changes)
RTOL = 1e-12


def close(a, b, rtol=RTOL):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    assert a.shape == b.shape
    nan_a, nan_b = np.isnan(a), np.isnan(b)
    if not np.array_equal(nan_a, nan_b):
        return False, "NaN pattern differs at %d entries" % int(np.sum(nan_a != nan_b))
    fa, fb = a[~nan_a], b[~nan_b]
    if fa.size == 0:
        return True, ""
    scale = np.max(np.abs(fb)) if np.all(np.isfinite(fb)) else 0.0
    tol = rtol * np.abs(fb) + rtol * scale
    err = np.abs(fa - fb)
    bad = ~(err <= tol) & ~(fa == fb)
    if np.any(bad):
        k = np.argmax(np.where(bad, err / np.maximum(tol, 1e-300), 0))
        return False, "max violation at %d: %r vs %r (tol %r), %d entries" % (k, fa[k], fb[k], tol[k], int(bad.sum()))
    return True, ""


def exact(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    if a.dtype.kind == "f":
        ok = np.array_equal(a, b, equal_nan=True)
        if not ok:
            d = np.nanmax(np.abs(a.astype(float) - b.astype(float)))
            return False, "max abs diff %r" % d
        return True, ""
    ok = np.array_equal(a, b)
    return ok, "" if ok else "%d entries differ" % int(np.sum(a != b))


def compare_markers(got, want, fields=None, rtol=None, skip=()):
    """Field-by-field comparison; exact when rtol is None.  Returns list of failures."""
    fails = []
    for f in fields or MARKER_DTYPE.names:
        if f in skip:
            continue
        if rtol is None or f in I32_FIELDS:
            ok, msg = exact(got[f], want[f])
        else:
            ok, msg = close(got[f], want[f], rtol)
        if not ok:
            fails.append("%s: %s" % (f, msg))
    return fails


def same_fields(a, b):
    """Every field of two marker arrays bit-identical (padding ignored, NaN compared by bits)."""
    if len(a) != len(b):
        return False, "lengths %d vs %d" % (len(a), len(b))
    for f in a.dtype.names:
        x, y = np.ascontiguousarray(a[f]), np.ascontiguousarray(b[f])
        if not np.array_equal(x.view(np.uint8), y.view(np.uint8)):
            rows = np.flatnonzero(x != y)
            return False, "field %s differs at %s" % (f, rows[:8])
    return True, ""
