"""Host mirror of the reference's Lie-Trotter drivers over the GPU macro step.

``lie_trotter_solve`` and ``lie_trotter_solve_bisect`` keep the keyword signature and the
behaviour of ``OpSplit.lie_trotter_solve{,_bisect}`` (tools/reactant_handoff/op_split.jl:
100-164, 219-241): the stop grid is the macro-dt lattice joined with the forcing cadence
boundaries in the half-open interval (t0, tf] and tf itself; each stop interval is one
``rs_macro_step`` (transport SSPRK43 then chemistry ROS23, both clamped to >= 0); ``refresh``
fires when a stop lands on a cadence boundary; a failed macro step is retried over two
half-intervals down to ``min_macro_dt``.  What the reference passes as RHS closures
(f_trans!, fc) is the .esm mechanism and the transport forcing held by the Solver.

Returns the same fields as the reference: u, retcode, naT, nrT, naC, nrC, nmacro (plus the
carried dtT/dtC, as the device-resident adv() returns them).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import abi
from ._lib import RsError


@dataclass
class SplitResult:
    u: np.ndarray
    retcode: str
    naT: int
    nrT: int
    naC: int
    nrC: int
    nmacro: int
    dtT: float
    dtC: float


def _stop_grid(t0, tf, macro_dt, forcing_tstops):
    fstops = {round(t, 6) for t in forcing_tstops if t0 + 1e-6 < t <= tf + 1e-6}
    grid = []
    x = t0 + macro_dt
    while x <= tf - 1e-9:
        grid.append(x)
        x = t0 + macro_dt * (len(grid) + 1)
    return sorted(set(grid) | fstops | {tf}), fstops


def lie_trotter_solve(solver, u0, tspan, *, macro_dt, dtT=15.0, dtC=0.5,
                      refresh=lambda t: None, forcing_tstops=(), clamp_nonneg=True):
    """Advance u0 (cell-major host array) over tspan with the GPU split step."""
    if not clamp_nonneg and solver.cfg.clamp_nonneg:
        raise ValueError("clamp_nonneg is fixed at Solver creation (rs_config.clamp_nonneg)")
    t0, tf = float(tspan[0]), float(tspan[1])
    solver.set_state(u0)
    stops, fstops = _stop_grid(t0, tf, float(macro_dt), forcing_tstops)
    tcur, nmacro = t0, 0
    tot = dict(naT=0, nrT=0, naC=0, nrC=0)
    retcode = "Success"
    for tnext in stops:
        if tnext <= tcur + 1e-9:
            continue
        rc, dtT, dtC, st = solver.macro_step(tcur, tnext, dtT, dtC, check=False)
        tot["naT"] += int(st.naT); tot["nrT"] += int(st.nrT)
        tot["naC"] += int(st.naC); tot["nrC"] += int(st.nrC)
        if rc != abi.RS_OK:
            retcode = "Failure:" + abi.STATUS_NAMES.get(rc, str(rc))
            break
        tcur = tnext
        nmacro += 1
        if round(tcur, 6) in fstops:
            refresh(tcur)
    return SplitResult(solver.get_state(), retcode, tot["naT"], tot["nrT"], tot["naC"],
                       tot["nrC"], nmacro, dtT, dtC)


def _ok(r):
    return r.retcode == "Success"


def lie_trotter_solve_bisect(solver, u0, tspan, *, macro_dt, min_macro_dt=9.0,
                             on_bisect=lambda t0, tf: None, **kw):
    """lie_trotter_solve, retrying a failed window over two halves down to min_macro_dt."""
    t0, tf = float(tspan[0]), float(tspan[1])
    r = lie_trotter_solve(solver, u0, (t0, tf), macro_dt=macro_dt, **kw)
    if _ok(r) or (tf - t0) <= min_macro_dt + 1e-9:
        return r
    tm = 0.5 * (t0 + tf)
    on_bisect(t0, tf)
    half = min(float(macro_dt), tm - t0)
    r1 = lie_trotter_solve_bisect(solver, u0, (t0, tm), macro_dt=half,
                                  min_macro_dt=min_macro_dt, on_bisect=on_bisect, **kw)
    if not _ok(r1):
        return r1
    kw2 = dict(kw)
    kw2["dtT"], kw2["dtC"] = r1.dtT, r1.dtC
    r2 = lie_trotter_solve_bisect(solver, r1.u, (tm, tf), macro_dt=min(float(macro_dt), tf - tm),
                                  min_macro_dt=min_macro_dt, on_bisect=on_bisect, **kw2)
    if not _ok(r2):
        return r2
    return SplitResult(r2.u, r2.retcode, r1.naT + r2.naT, r1.nrT + r2.nrT, r1.naC + r2.naC,
                       r1.nrC + r2.nrC, r1.nmacro + r2.nmacro, r2.dtT, r2.dtC)


__all__ = ["lie_trotter_solve", "lie_trotter_solve_bisect", "SplitResult", "RsError"]
