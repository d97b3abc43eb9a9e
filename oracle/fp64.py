"""The FP64 run of the oracle (test infrastructure only, like the rest of oracle/): the same restatement of the
reference's transport, projection, composition and observer boxes (sos_oracle) evaluated in float64, so that the
double-single coordinate splits carry no low part and nothing is flushed to zero. The reference has no FP64 run of
this path (its arithmetic is float32 by construction, src/sosfuse2/backends/arithmetic.py:11); this one serves the
per-pixel error report of FP32 results (the reference's and the CUDA path's) against float64 arithmetic on the same
float32 inputs.

Usage: `with float64(): ...` around calls into oracle.sos_oracle (not thread-safe: it switches the module's working
precision for the duration)."""

import contextlib

import numpy as np

from . import sos_oracle as so


@contextlib.contextmanager
def float64():
    previous = so.F
    so.F = np.float64
    try:
        yield so
    finally:
        so.F = previous


def relative_error(values, exact, floor=1e-6):
    """Per-pixel relative error |values - exact| / |exact| over the entries above `floor` of the largest: (max,
    median, RMS)."""
    v = np.asarray(values, np.float64)
    e = np.asarray(exact, np.float64)
    big = np.abs(e) > floor * np.abs(e).max()
    rel = np.abs(v[big] - e[big]) / np.abs(e[big])
    return float(rel.max()), float(np.median(rel)), float(np.sqrt(np.mean(rel ** 2)))
