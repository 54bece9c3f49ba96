"""The reference's macro-step loop (run_reseact.jl:337-400) over the GPU split step.

Each window is one macro step (t, min(t + macro_dt, t_end)) solved by the library's own
stop-grid / refresh / bisection driver (rs_lie_trotter_solve); every out_every steps the state
goes to a streaming species-major Zarr store; each step reports the continuity drift when the
hybrid coefficients are known; a failed window stops the run and, if asked, dumps the
pre-step and post-failure states in the reference's STATEDUMP format:
  <statedump>        Int64 NS, Int64 NC, Float64 t, Float64[NS*NC] pre-step u (cell-major,
                     restartable), Float64[NS*NC] the state where the step gave up
  <statedump>.names  "# NS=.. NC=.. t=..  layout: cell-major, u[(c-1)*NS+s]" and one line
                     "<1-based position>\\t<name>" per species
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import abi, workloads


@dataclass
class RunResult:
    ok: bool
    t: float
    nstep: int
    nT: int
    nC: int
    nbisect: int
    rows: list = field(default_factory=list)


def write_statedump(path, species_names, t, u_pre, u_post):
    ns = len(species_names)
    nc = len(u_pre) // ns
    with open(path, "wb") as fh:
        np.array([ns, nc], dtype="<i8").tofile(fh)
        np.array([t], dtype="<f8").tofile(fh)
        np.asarray(u_pre, dtype="<f8").tofile(fh)
        np.asarray(u_post, dtype="<f8").tofile(fh)
    with open(str(path) + ".names", "w") as fh:
        fh.write("# NS=%d NC=%d t=%r  layout: cell-major, u[(c-1)*NS+s]\n" % (ns, nc, t))
        for b, name in enumerate(species_names, start=1):
            fh.write("%d\t%s\n" % (b, name))


def read_statedump(path):
    with open(path, "rb") as fh:
        ns, nc = np.fromfile(fh, dtype="<i8", count=2)
        t = float(np.fromfile(fh, dtype="<f8", count=1)[0])
        pre = np.fromfile(fh, dtype="<f8", count=ns * nc)
        post = np.fromfile(fh, dtype="<f8", count=ns * nc)
    return int(ns), int(nc), t, pre, post


def run_split(solver, w, t0, t_end, *, macro_dt, min_macro_dt=9.0, out_every=1, sink=None,
              statedump=None, forcing_tstops=(), refresh=None, report=None, dtT=None,
              dtC=None):
    """Advance the solver's resident state from t0 to t_end; returns RunResult."""
    g = w.grid
    names = list(w.mech.species) + (["m"] if w.has_air_mass else [])
    hyb = "hyb_a" in w.forcing and "hyb_b" in w.forcing and w.has_air_mass
    dtT = w.dt0_T if dtT is None else dtT
    dtC = w.dt0_C if dtC is None else dtC

    def soa():
        return workloads.cellmajor_to_soa(solver.get_state(), w.nsp, g["nlon"], g["nlat"],
                                          g["nlev"])

    def drift(t):
        if not hyb:
            return None
        ps = np.asarray(w.forcing.get("ps", np.full((g["nlat"], g["nlon"]),
                                                   w.forcing["hyb_a"][0])))
        if "dps_dt" in w.forcing:
            ps = ps + np.asarray(w.forcing["dps_dt"]) * (t - t0)
        return solver.continuity_drift(ps)

    res = RunResult(True, t0, 0, 0, 0, 0)
    if sink is not None:
        sink.write(t0, soa())
    if report:
        report(t0, drift(t0))
    t = t0
    while t < t_end - 1e-9:
        res.nstep += 1
        tnext = min(t + macro_dt, t_end)
        pre = solver.get_state() if statedump else None
        rc, dtT, dtC, r = solver.lie_trotter_solve(t, tnext, dtT, dtC, macro_dt=tnext - t,
                                                   min_macro_dt=min_macro_dt,
                                                   forcing_tstops=forcing_tstops,
                                                   refresh=refresh)
        res.nbisect += int(r.nbisect)
        if rc != abi.RS_OK:
            res.ok = False
            if statedump:
                write_statedump(statedump, names, t, pre, solver.get_state())
            break
        res.nT += int(r.naT)
        res.nC += int(r.naC)
        t = tnext
        res.t = t
        d = drift(t)
        res.rows.append((t, d))
        if report:
            report(t, d)
        if sink is not None and res.nstep % out_every == 0:
            sink.write(t, soa())
    return res
