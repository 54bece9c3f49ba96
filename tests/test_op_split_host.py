"""Host logic of the Lie-Trotter drivers (op_split.jl:100-164, 219-241) with a fake solver:
stop grid (macro-dt lattice + forcing boundaries in the half-open (t0, tf] + tf), refresh at
cadence boundaries, carried dts, bisection on failure down to min_macro_dt."""
import numpy as np
import pytest

from reseact.esm_gb300 import abi, op_split


class FakeSolver:
    def __init__(self, fail_if=lambda t0, t1: False, n=4):
        self.cfg = type("cfg", (), {"clamp_nonneg": 1})()
        self.calls, self.fail_if, self.u = [], fail_if, np.zeros(n)

    def set_state(self, u):
        self.u = np.array(u, dtype=float)

    def get_state(self):
        return self.u.copy()

    def macro_step(self, t0, t1, dtT, dtC, check=True):
        self.calls.append((t0, t1, dtT, dtC))
        st = abi.rs_stats()
        if self.fail_if(t0, t1):
            st.naC = 1
            return abi.RS_ERR_MAXITERS, dtT, dtC, st
        self.u = self.u + (t1 - t0)
        st.naT, st.naC, st.nrC = 2, 3, 1
        return abi.RS_OK, dtT * 1.5, dtC * 2.0, st


def test_stop_grid_half_open_forcing_boundaries():
    stops, fstops = op_split._stop_grid(0.0, 3600.0, 600.0, [1800.0, 3600.0, 0.0, 5400.0])
    assert stops == [600.0, 1200.0, 1800.0, 2400.0, 3000.0, 3600.0]
    assert fstops == {1800.0, 3600.0}  # t0 excluded, tf included, outside excluded
    stops, _ = op_split._stop_grid(0.0, 1000.0, 300.0, [450.0])
    assert stops == [300.0, 450.0, 600.0, 900.0, 1000.0]


def test_solve_refresh_counts_and_carried_dt():
    s = FakeSolver()
    seen = []
    r = op_split.lie_trotter_solve(s, np.zeros(4), (0.0, 1800.0), macro_dt=600.0,
                                   refresh=seen.append, forcing_tstops=[1800.0])
    assert r.retcode == "Success" and r.nmacro == 3
    assert seen == [1800.0]  # refresh at tf (half-open on the right)
    assert (r.naT, r.naC, r.nrC) == (6, 9, 3)
    assert s.calls[1][2] == pytest.approx(15.0 * 1.5) and s.calls[2][3] == pytest.approx(0.5 * 4)
    assert np.allclose(r.u, 1800.0)


def test_bisect_retries_failed_window():
    # fail any window longer than 300 s
    s = FakeSolver(fail_if=lambda t0, t1: (t1 - t0) > 300.0)
    notes = []
    r = op_split.lie_trotter_solve_bisect(s, np.zeros(4), (0.0, 600.0), macro_dt=600.0,
                                          min_macro_dt=9.0, on_bisect=lambda a, b: notes.append((a, b)))
    assert r.retcode == "Success"
    assert notes == [(0.0, 600.0)]
    assert r.nmacro == 2 and np.allclose(r.u, 600.0)


def test_bisect_gives_up_below_min_macro_dt():
    s = FakeSolver(fail_if=lambda t0, t1: True)
    r = op_split.lie_trotter_solve_bisect(s, np.zeros(4), (0.0, 40.0), macro_dt=40.0,
                                          min_macro_dt=9.0)
    assert r.retcode.startswith("Failure")
    # 40 -> 20 -> 10 -> stop (10 > 9 still splits to 5 < 9)
    assert min(t1 - t0 for t0, t1, _, _ in s.calls) >= 5.0
