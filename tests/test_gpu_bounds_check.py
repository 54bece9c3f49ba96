"""The bounds-check build (libreseact_gb300_check.so, -DRS_BOUNDS_CHECK=1): every shared-memory
row index, halo / ghost load and bulk-copy box start of the transport pencils is checked
against its array, and a failed check is reported as a status (RS_ERR_INVALID), never a trap.
Small grids at the stencil's limits (the minimum 3 x 3 x 3, regional open walls, odd sizes)
and the full C2 grid run through adaptive macro steps in the FP64 and compensated-FP32 forms,
with bulk-copy and plain-load staging: no check fires, and the results equal the production
build's bit for bit (the checks change no arithmetic)."""
import numpy as np
import pytest

from reseact.esm_gb300 import Solver, abi, mechanism, workloads
from reseact.esm_gb300._lib import STAGING_BULK, STAGING_PLAIN

pytestmark = pytest.mark.gpu


def _regional(n=7):
    g, mx, my, mz, dp = workloads.regional_freestream(n)
    mech = mechanism.superfast()
    dp3 = np.broadcast_to(dp[:, None, None], (n, n, n)).copy()
    rng = np.random.default_rng(5)
    qb_lon = 1.0 + 0.1 * rng.random((mech.ns, n, n))
    qb_lat = 1.0 + 0.1 * rng.random((mech.ns, n, n))
    forcing = dict(mx=mx, my=my, mz=mz, dp=dp3, qbc_w=qb_lon, qbc_e=qb_lon[::-1].copy(),
                   qbc_s=qb_lat, qbc_n=qb_lat[::-1].copy(), temperature=np.full((n, n, n), 280.0),
                   pressure=np.full((n, n, n), 8e4), flux_omega=0.0)
    u0 = np.concatenate([1.0 + rng.random((mech.ns, n, n, n)), dp3[None]])
    # transport only (the checks guard the pencils; these tracer values are not a chemical
    # state), over 0.5 s windows: the divergent freestream fluxes of this slice move a cell's
    # whole air mass within about a minute
    return workloads.Workload("regional %d^3" % n, g, mech, forcing, np.ascontiguousarray(u0),
                              0.5, 1, do_chemistry=False, dt0_T=0.05)


CASES = {
    "min3": lambda: workloads.c2(nlon=3, nlat=3, nlev=3),
    "odd": lambda: workloads.c2(nlon=17, nlat=9, nlev=7),
    "regional": lambda: _regional(7),
    "c2small": lambda: workloads.c2(nlon=48, nlat=31, nlev=16),
}


def _steps(w, check, n, staging=None, stream=None, **kw):
    s = Solver.for_workload(w, check=check, do_transport=w.do_transport,
                            do_chemistry=w.do_chemistry, **kw)
    if staging is not None:
        s.set_transport_staging(staging)
    if stream is not None:
        s.set_launch_shape(mixed_x_stream=stream, mixed_yz_stream=stream)
    s.set_state(w.u0_cellmajor())
    t, a, b = 0.0, w.dt0_T, w.dt0_C
    for _ in range(n):
        rc, a, b, _ = s.macro_step(t, t + w.dt_macro, a, b)  # raises on a failed index check
        assert rc == 0
        t += w.dt_macro
    out = s.get_state()
    s.close()
    return out


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("form", ["fp64", "mixed_bulk", "mixed_plain", "mixed_stream"])
def test_no_index_check_fires_and_bits_unchanged(case, form):
    w = CASES[case]()
    kw = {"fp64": {}, "mixed_bulk": dict(precision=abi.RS_PREC_MIXED, staging=STAGING_BULK),
          "mixed_plain": dict(precision=abi.RS_PREC_MIXED, staging=STAGING_PLAIN),
          "mixed_stream": dict(precision=abi.RS_PREC_MIXED, stream=1)}[form]
    if form == "mixed_bulk" and w.grid["nlon"] % 4:
        kw["staging"] = None  # the copy engine's alignment rule: the library picks plain loads
    got = _steps(w, True, 2, **dict(kw))
    ref = _steps(w, False, 2, **dict(kw))
    assert np.array_equal(got, ref)


def test_full_c2_no_index_check_fires():
    w = workloads.c2()
    for kw in ({}, dict(precision=abi.RS_PREC_MIXED, stream=0),
               dict(precision=abi.RS_PREC_MIXED, stream=1)):
        got = _steps(w, True, 1, **dict(kw))
        ref = _steps(w, False, 1, **dict(kw))
        assert np.array_equal(got, ref)
