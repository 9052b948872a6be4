"""Accuracy of a radargram against a reference radargram.

The accuracy bar of the fast (FP32 split-precision) form against an FP64
result has three parts, each computed here over traces (rows) of complex
radargrams shaped (ns, nr):

* the relative L2 error of the complex radargram, ``|got - ref| / |ref|``;
* the largest phase error, ``|angle(got / ref)|`` in radians, over the bins
  whose reference magnitude is above ``floor_db`` (default -40 dB) of that
  trace's peak;
* an exact match of every trace's peak range-bin index.

``compare`` returns all three (overall and worst trace) as plain floats, so a
benchmark line or a test can carry them.
"""
import numpy as np

REL_L2_BAR = 1e-3
PHASE_BAR = 0.01


def rel_l2(got, ref):
    got = np.asarray(got)
    ref = np.asarray(ref)
    den = np.linalg.norm(ref)
    return float(np.linalg.norm(got - ref) / den) if den > 0 else float(np.linalg.norm(got))


def phase_err_max(got, ref, floor_db=-40.0):
    """Largest |angle(got / ref)| over bins above floor_db of the row's peak."""
    got = np.atleast_2d(np.asarray(got))
    ref = np.atleast_2d(np.asarray(ref))
    worst = 0.0
    for a, b in zip(got, ref):
        mag = np.abs(b)
        if mag.max() <= 0:
            continue
        m = mag > mag.max() * 10 ** (floor_db / 20.0)
        worst = max(worst, float(np.max(np.abs(np.angle(a[m] / b[m])))))
    return worst


def peak_bins(x):
    return np.argmax(np.abs(np.asarray(x)), axis=-1)


def compare(got, ref, floor_db=-40.0):
    """Relative L2 (whole radargram and worst trace), max phase error above
    floor_db of each trace's peak, and whether every trace's peak bin
    matches.  Traces whose reference is all zero are compared by L2 only."""
    got = np.atleast_2d(np.asarray(got))
    ref = np.atleast_2d(np.asarray(ref))
    if got.shape != ref.shape:
        raise ValueError(f"shape mismatch {got.shape} vs {ref.shape}")
    live = np.abs(ref).max(axis=1) > 0
    per = [rel_l2(a, b) for a, b in zip(got[live], ref[live])]
    pk = bool(np.array_equal(peak_bins(got[live]), peak_bins(ref[live])))
    return {"rel_l2": rel_l2(got, ref),
            "rel_l2_worst_trace": max(per) if per else 0.0,
            "phase_max_rad": phase_err_max(got, ref, floor_db),
            "peak_bins_match": pk,
            "traces": int(got.shape[0]),
            "floor_db": floor_db}


def within_bar(res, rel=REL_L2_BAR, phase=PHASE_BAR):
    """Whether a ``compare`` result meets the fast form's accuracy bar."""
    return res["rel_l2_worst_trace"] <= rel and res["phase_max_rad"] <= phase and res["peak_bins_match"]
