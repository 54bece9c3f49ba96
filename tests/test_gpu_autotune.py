"""The project-written autotuner picks launch shapes only: results after tuning are
bit-identical to the default shapes (transport pencils and the per-cell chemistry kernel)."""
import numpy as np
import pytest

from reseact.esm_gb300 import Solver, abi, workloads

pytestmark = pytest.mark.gpu


def _run(w, tune, steps=2, **kw):
    s = Solver.for_workload(w, **kw)
    s.set_state(w.u0_cellmajor())
    rep = s.autotune() if tune else None
    t, a, b = 0.0, w.dt0_T, w.dt0_C
    for _ in range(steps):
        _, a, b, _ = s.macro_step(t, t + w.dt_macro, a, b)
        t += w.dt_macro
    out = s.get_state()
    s.close()
    return out, rep


def test_autotune_transport_is_bitwise_neutral():
    w = workloads.c2(nlon=48, nlat=31, nlev=16)
    ref, _ = _run(w, False)
    got, rep = _run(w, True)
    assert "transport_choice" in rep and len(rep["pencils"]) == 6
    assert np.array_equal(ref, got)


def test_autotune_per_cell_is_bitwise_neutral():
    w = workloads.c3(ncells=8192)
    ref, _ = _run(w, False, steps=1)
    got, rep = _run(w, True, steps=1)
    assert "per_cell_choice" in rep and len(rep["per_cell"]) == 12
    assert np.array_equal(ref, got)
