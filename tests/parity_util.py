"""Shared parity criteria of the GPU tests."""
import numpy as np


def per_cell_agreement(got, ref, cfg, nsp):
    """Per-cell adaptive integrations of a stiff problem agree to roundoff in cells that take
    the same accept/reject sequence; a cell whose sequence flips (an error estimate within
    roundoff of 1) ends at a different but equally valid point of the same tolerance.  So:
    every entry within 10 x (rtol |u| + atol), at most 1 % of cells with any entry beyond
    1 x that bound, and a median relative difference at roundoff level."""
    bound = cfg.rtol_C * np.abs(ref) + cfg.atol_C
    d = np.abs(got - ref) / bound
    assert d.max() <= 10.0, d.max()
    flipped = np.any(d.reshape(-1, nsp) > 1.0, axis=1)
    assert flipped.mean() <= 0.01, flipped.mean()
    rel = np.abs(got - ref) / np.maximum(np.abs(ref), cfg.atol_C)
    assert np.median(rel) < 1e-12, np.median(rel)
