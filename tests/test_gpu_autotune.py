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
    # pencil widths 8 / 16 / 32 x rows 4..32 with 64..512 threads per block
    assert "transport_choice" in rep and len(rep["pencils"]) == 10
    assert np.array_equal(ref, got)


@pytest.mark.parametrize("shape", [dict(pencil=8, rows=8), dict(pencil=8, rows=32),
                                   dict(pencil=16, rows=32), dict(xthreads=96),
                                   dict(xthreads=160), dict(xthreads=192),
                                   dict(x_tracer_groups=3, yz_tracer_groups=4),
                                   dict(x_tracer_groups=5, yz_tracer_groups=2, pencil=8)])
def test_transport_launch_shapes_are_bitwise_neutral(shape):
    """Every FP64 pencil shape (lat/vertical pencil width x rows, threads per lon row, tracer
    groups per launch, including uneven groups) gives the same state bit for bit after
    adaptive macro steps."""
    w = workloads.c2(nlon=48, nlat=31, nlev=16)
    ref, _ = _run(w, False)
    s = Solver.for_workload(w)
    s.set_launch_shape(**shape)
    s.set_state(w.u0_cellmajor())
    t, a, b = 0.0, w.dt0_T, w.dt0_C
    for _ in range(2):
        _, a, b, _ = s.macro_step(t, t + w.dt_macro, a, b)
        t += w.dt_macro
    got = s.get_state()
    s.close()
    assert np.array_equal(ref, got)


def test_autotune_per_cell_is_bitwise_neutral():
    w = workloads.c3(ncells=8192)
    ref, _ = _run(w, False, steps=1)
    got, rep = _run(w, True, steps=1)
    # 3 x 4 thread-per-cell shapes, 2 capped at 32 registers, then 4 / 8 / 16 lanes per cell
    # (shared-memory work arrays)
    assert "per_cell_choice" in rep and len(rep["per_cell"]) == 17
    assert sorted(c["group"] for c in rep["per_cell"] if "group" in c) == [4, 8, 16]
    assert np.array_equal(ref, got)
