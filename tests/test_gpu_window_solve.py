"""rs_lie_trotter_solve (the library's own stop grid, forcing refresh and bisection on the
device-resident state, op_split.jl:100-164 / 219-241) against the host mirror of the same
drivers (reseact.esm_gb300.op_split): same stops, refresh times, bisections and counts, and
the same bits, since both run the same device macro steps."""
import numpy as np
import pytest

from reseact.esm_gb300 import Solver, abi, lie_trotter_solve_bisect, workloads

pytestmark = pytest.mark.gpu


def _run_both(w, maxiters=2e4, **kw):
    f = w.forcing_abi()
    out = []
    for native in (False, True):
        s = Solver.for_workload(w, maxiters=maxiters)
        refreshed, bisected = [], []
        refresh = lambda t: (refreshed.append(t), s.set_forcing(f))
        on_bisect = lambda a, b: bisected.append((a, b))
        if native:
            s.set_state(w.u0_cellmajor())
            rc, dtT, dtC, r = s.lie_trotter_solve(0.0, 3600.0, 15.0, 0.5, refresh=refresh,
                                                  on_bisect=on_bisect, **kw)
            counts = (r.naT, r.nrT, r.naC, r.nrC, r.nmacro)
            res = (rc, s.get_state(), counts, dtT, dtC)
        else:
            r = lie_trotter_solve_bisect(s, w.u0_cellmajor(), (0.0, 3600.0), refresh=refresh,
                                         on_bisect=on_bisect, **kw)
            counts = (r.naT, r.nrT, r.naC, r.nrC, r.nmacro)
            res = (0 if r.retcode == "Success" else 1, r.u, counts, r.dtT, r.dtC)
        out.append((res, refreshed, bisected))
        s.close()
    return out


def test_stop_grid_and_refresh_match_the_host_mirror():
    w = workloads.c1()
    (a, ra, ba), (b, rb, bb) = _run_both(w, macro_dt=600.0, forcing_tstops=[1000.0, 1800.0, 3600.0])
    assert a[0] == 0 and b[0] == abi.RS_OK
    assert ra == rb == [1000.0, 1800.0, 3600.0]
    assert ba == bb == []
    assert a[2] == b[2] and a[2][4] == 7  # 6 lattice stops + the cadence stop at 1000 s
    assert np.array_equal(a[1], b[1]) and a[3] == b[3] and a[4] == b[4]


def test_bisection_matches_the_host_mirror():
    # 130 attempts per adaptive solve: too few for the first 600 s window from dtC = 0.5 s
    # (the start-up transient needs 87 attempts for the first 9.4 s alone), enough once the
    # window is halved -- the oracle's controller, which the GPU's follows attempt for attempt,
    # bisects 5 times and then succeeds with 9 macro steps
    w = workloads.c1()
    (a, ra, ba), (b, rb, bb) = _run_both(w, maxiters=130, macro_dt=600.0, min_macro_dt=9.0)
    assert ba == bb and len(ba) >= 1
    assert a[0] == 0 and b[0] == abi.RS_OK
    assert a[2] == b[2]
    assert np.array_equal(a[1], b[1])
