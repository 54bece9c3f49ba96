"""Determinism hammer: the same macro step from the same state, run many times, gives the same
bits every time (the reference's nondeterminism hunt issued one call repeatedly and counted
differing results, tools/diag/README-nondet.md).  Reductions here are fixed trees and the
per-cell work queue only changes which thread integrates a cell, so every repetition must be
bit-identical: the FP64 method, the compensated FP32 transport form, and per-cell chemistry
(whose queue order differs from run to run)."""
import numpy as np
import pytest

from reseact.esm_gb300 import Solver, abi, workloads

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("form,reps", [("fp64", 100), ("mixed", 100), ("batched_mixed", 25)])
def test_same_step_same_bits(form, reps):
    """Per-cell chemistry carries each cell's step size from one macro step to the next inside
    the handle, so its repetitions start from fresh handles."""
    w = workloads.c2(nlon=48, nlat=31, nlev=16)
    kw = {"fp64": {}, "mixed": dict(precision=abi.RS_PREC_MIXED),
          "batched_mixed": dict(precision=abi.RS_PREC_MIXED, chem_mode=abi.RS_CHEM_PER_CELL)}[form]
    s = Solver.for_workload(w, **kw)
    u0 = w.u0_cellmajor()
    first = None
    for _ in range(reps):
        if form == "batched_mixed":
            s.close()
            s = Solver.for_workload(w, **kw)
        s.set_state(u0)
        rc, dT, dC, st = s.macro_step(0.0, 600.0, 15.0, 0.5)
        assert rc == 0
        out = (s.get_state(), dT, dC, st.naT, st.nrT, st.naC, st.nrC, st.chem_cell_steps)
        if first is None:
            first = out
            continue
        assert np.array_equal(out[0], first[0])
        assert out[1:] == first[1:]
