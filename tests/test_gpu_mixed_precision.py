"""Compensated FP32 transport (RS_PREC_MIXED) against the FP64 scheme on the full C2 grid.

The mixed form carries the transport reconstruction in double-float pairs on the FP32 pipe and
keeps the state, the air mass, the error norm and chemistry in FP64.  Its gate is the north
star's: every output within 1e-6 relative of the FP64 result (relative to max(|u|, 1e-9), the
chemistry's absolute tolerance as the floor) over a window as long as the bench's (20 macro
steps of 600 s after 5 warm-up steps, i.e. t = 3,000 .. 15,000 s), with the same accept /
reject decisions.  An FP32 reconstruction of deviations misses this gate by 3.7x in NO / NO2
cells far smaller than their neighbours; the compensated form stays at FP64-class error.
"""
import numpy as np
import pytest

from reseact.esm_gb300 import Solver, abi, workloads

pytestmark = pytest.mark.gpu

WARMUP, STEPS, DTM = 5, 20, 600.0


def _run(solver, u, t, dtT, dtC, n):
    solver.set_state(u)
    counts = []
    for _ in range(n):
        _, dtT, dtC, st = solver.macro_step(t, t + DTM, dtT, dtC)
        counts.append((st.naT, st.nrT, st.naC, st.nrC))
        t += DTM
    return solver.get_state(), t, dtT, dtC, counts


def _rel(a, b, floor=1e-9):
    return np.abs(a - b) / np.maximum(np.abs(b), floor)


@pytest.fixture(scope="module")
def c2_start():
    """The FP64 state after the bench's warm-up (t = 3,000 s)."""
    w = workloads.c2()
    s = Solver.for_workload(w)
    u, t, dtT, dtC, _ = _run(s, w.u0_cellmajor(), 0.0, w.dt0_T, w.dt0_C, WARMUP)
    s.close()
    return w, u, t, dtT, dtC


def test_mixed_within_1e6_of_fp64_over_bench_window(c2_start):
    w, u, t, dtT, dtC = c2_start
    A, _, _, _, cA = _run(Solver.for_workload(w), u, t, dtT, dtC, STEPS)
    B, _, _, _, cB = _run(Solver.for_workload(w, precision=abi.RS_PREC_MIXED), u, t, dtT, dtC,
                          STEPS)
    assert cA == cB  # the same accept / reject decisions in both halves
    rel = _rel(B, A)
    assert rel.max() <= 1e-6, (rel.max(), np.unravel_index(rel.argmax(), (w.ncells, w.nsp)))
    # the precision change is far below the gate: FP64-class arithmetic
    assert rel.max() < 1e-10, rel.max()
    assert np.median(rel) < 1e-13, np.median(rel)


def test_mixed_transport_only_fp64_class(c2_start):
    """Transport alone (no chemistry to amplify differences): the compensated pencils track the
    FP64 pencils to ~1e-12 relative after 20 macro steps, including cells far smaller than
    their neighbours.  The air mass is FP64 in both; it differs only through step sizes that
    the error norm (which sees the tracers) sets a few ulps apart."""
    w, u, t, dtT, dtC = c2_start
    A, _, _, _, cA = _run(Solver.for_workload(w, do_chemistry=False), u, t, dtT, dtC, STEPS)
    B, _, _, _, cB = _run(Solver.for_workload(w, do_chemistry=False,
                                              precision=abi.RS_PREC_MIXED), u, t, dtT, dtC, STEPS)
    assert cA == cB
    nsp = w.nsp
    a, b = A.reshape(-1, nsp), B.reshape(-1, nsp)
    assert np.max(np.abs(a[:, -1] - b[:, -1]) / a[:, -1]) < 1e-13  # air mass
    rel = _rel(b[:, :-1], a[:, :-1])
    assert rel.max() < 1e-10, rel.max()


def _masses(w, u_cm):
    """Tracer masses sum_c area_c m_c q_c per species (area on the unit sphere)."""
    g, nsp = w.grid, w.nsp
    phie = workloads.lat_edges(g)
    area = np.sin(np.radians(phie[1:])) - np.sin(np.radians(phie[:-1]))
    u = u_cm.reshape(g["nlon"], g["nlat"], g["nlev"], nsp)
    wm = u[..., -1] * area[None, :, None]
    return np.einsum("ijk,ijks->s", wm, u[..., :-1])


def test_mixed_conserves_tracer_mass_like_fp64(c2_start):
    """Total tracer mass of every species: the mixed form's change over 20 transport steps
    equals the FP64 form's to roundoff (the CWC stage updates of both schemes move the total by
    the same small amount; what the precision change adds is roundoff)."""
    w, u, t, dtT, dtC = c2_start
    A, _, _, _, _ = _run(Solver.for_workload(w, do_chemistry=False), u, t, dtT, dtC, STEPS)
    B, _, _, _, _ = _run(Solver.for_workload(w, do_chemistry=False,
                                             precision=abi.RS_PREC_MIXED), u, t, dtT, dtC, STEPS)
    m0, ma, mb = _masses(w, u), _masses(w, A), _masses(w, B)
    assert np.all(np.abs(mb - ma) <= 1e-12 * np.abs(m0)), np.abs(mb - ma) / np.abs(m0)
    assert np.all(np.abs(mb - m0) <= np.abs(ma - m0) + 1e-12 * np.abs(m0))


def test_mixed_freestream_exact():
    """q == 1 stays exactly 1 through adaptive transport steps in the mixed form."""
    w = workloads.c2(nlon=48, nlat=31, nlev=16)
    w.u0[:-1] = 1.0
    s = Solver.for_workload(w, do_chemistry=False, precision=abi.RS_PREC_MIXED)
    u, *_ = _run(s, w.u0_cellmajor(), 0.0, 15.0, 0.5, 3)
    q = u.reshape(-1, w.nsp)[:, :-1]
    assert np.all(q == 1.0)
