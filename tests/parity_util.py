"""Shared parity criteria of the GPU tests."""
import numpy as np


def per_cell_agreement(got, ref, cfg, nsp, flip_frac=1e-3):
    """Per-cell adaptive integrations on the step-size lattice (4 fraction bits, 16 sizes per
    octave) agree to roundoff: a cell's step sequence changes only where a step proposal lies
    within roundoff of a lattice point or an error estimate within roundoff of 1.  So: every
    cell within 1e-6 relative (the absolute tolerance as the floor) except at most `flip_frac`
    of the cells, those within 10 x (rtol |u| + atol), and a median at roundoff level."""
    rel = np.abs(got - ref) / np.maximum(np.abs(ref), cfg.atol_C)
    cellmax = rel.reshape(-1, nsp).max(axis=1)
    assert np.mean(cellmax > 1e-6) <= flip_frac, (np.mean(cellmax > 1e-6), cellmax.max())
    bound = cfg.rtol_C * np.abs(ref) + cfg.atol_C
    d = np.abs(got - ref) / bound
    assert d.max() <= 10.0, d.max()
    assert np.median(rel) < 1e-12, np.median(rel)
