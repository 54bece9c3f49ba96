"""Bulk-copy (TMA) staging of the mixed-precision transport pencils against plain loads, and
the streaming forms (no shared memory) against the pencils.

The two stagings load the same values into the same shared-memory rows, so the fluxes and
every state after them are bit-identical.  The cases cover every tracer grouping (one tracer
per block, pairs, and groups of three and more, where each of the two copy buffers is reused
and its mbarrier phase flips), both pencil widths, open boundaries (ghost cells from the
boundary values), grids where only some directions meet the copy engine's rules, grids where
none does, and the exact freestream of the open-wall case.
"""
import numpy as np
import pytest

from reseact.esm_gb300 import Solver, abi, mechanism, workloads
from reseact.esm_gb300._lib import STAGING_AUTO, STAGING_BULK, STAGING_PLAIN, RsError

pytestmark = pytest.mark.gpu


def _run(w, staging, shapes, steps=2):
    s = Solver.for_workload(w, do_chemistry=False, precision=abi.RS_PREC_MIXED)
    s.set_transport_staging(staging)
    s.set_launch_shape(**shapes)
    s.set_state(w.u0_cellmajor())
    t, a = 0.0, 15.0
    for _ in range(steps):
        rc, a, _, _ = s.macro_step(t, t + 600.0, a, 1.0)
        assert rc == 0
        t += 600.0
    out, info = s.get_state(), s.transport_staging()
    s.close()
    return out, info


@pytest.mark.parametrize("shapes", [
    dict(mixed_x_tracers=1, mixed_yz_tracers=1),
    dict(mixed_x_tracers=2, mixed_yz_tracers=2, mixed_pencil=32, mixed_rows=4),
    dict(mixed_x_tracers=5, mixed_yz_tracers=3, mixed_xthreads=256),
    dict(mixed_x_tracers=12, mixed_yz_tracers=12, mixed_pencil=16, mixed_rows=16),
])
def test_bulk_staging_is_bit_identical_to_plain_loads(shapes):
    w = workloads.c2(nlon=36, nlat=19, nlev=10)
    a, ia = _run(w, STAGING_BULK, shapes)
    b, ib = _run(w, STAGING_PLAIN, shapes)
    assert ia[0] == STAGING_BULK
    assert (ia[1]["lon_rows"], ia[1]["lat_pencils"], ia[1]["vertical_pencils"]) == ("bulk",) * 3
    assert ib[0] == STAGING_PLAIN
    assert np.all(np.isfinite(a))
    assert np.array_equal(a, b)


def test_bulk_staging_where_only_the_vertical_pencils_qualify():
    # nlon = 38 (rows of 152 bytes): no lon-row or lat-pencil copies; 38 x 18 columns do qualify
    w = workloads.c2(nlon=38, nlat=18, nlev=10)
    a, ia = _run(w, STAGING_BULK, dict(mixed_yz_tracers=4))
    b, _ = _run(w, STAGING_PLAIN, dict(mixed_yz_tracers=4))
    assert (ia[1]["lon_rows"], ia[1]["lat_pencils"], ia[1]["vertical_pencils"]) == (
        "unavailable", "unavailable", "bulk")
    assert np.array_equal(a, b)


def test_grid_without_bulk_copies_reports_and_falls_back():
    w = workloads.c2(nlon=30, nlat=19, nlev=10)  # 30 x 19 = 570 columns: no 16-byte rows
    s = Solver.for_workload(w, do_chemistry=False, precision=abi.RS_PREC_MIXED)
    with pytest.raises(RsError) as e:
        s.set_transport_staging(STAGING_BULK)
    assert e.value.status == abi.RS_ERR_UNSUPPORTED
    s.set_transport_staging(STAGING_AUTO)
    mode, info = s.transport_staging()
    assert mode == STAGING_PLAIN and "why" in info
    s.set_state(w.u0_cellmajor())
    rc, _, _, _ = s.macro_step(0.0, 600.0, 15.0, 1.0)
    assert rc == 0
    s.close()


def _regional(n, q, qb):
    g, mx, my, mz, dp = workloads.regional_freestream(n)
    mech = mechanism.superfast()
    dp3 = np.broadcast_to(dp[:, None, None], (n, n, n)).copy()
    f = abi.ForcingABI(mx=mx, my=my, mz=mz, dp=dp3, qbc_w=qb, qbc_e=qb, qbc_s=qb, qbc_n=qb)
    mabi = abi.MechanismABI(mech)
    cfg = abi.make_config(g, mabi, do_chemistry=False, precision=abi.RS_PREC_MIXED)
    u = np.concatenate([q, dp3[None] * (1 + 0.1 * np.random.default_rng(0).random((1, n, n, n)))])
    return g, mech, cfg, mabi, f, workloads.soa_to_cellmajor(u, n, n, n)


def _regional_steps(staging, n, q, qb, stream=0):
    g, mech, cfg, mabi, f, u0 = _regional(n, q, qb)
    s = Solver(cfg, mabi)
    s.set_forcing(f)
    s.set_transport_staging(staging)
    s.set_launch_shape(mixed_x_tracers=3, mixed_yz_tracers=3, mixed_x_stream=stream,
                       mixed_yz_stream=stream)
    s.set_state(u0)
    dtT = 0.05
    for k in range(4):
        rc, dtT, _, _ = s.macro_step(0.1 * k, 0.1 * (k + 1), dtT, 1.0)
        assert rc == 0
    out = s.get_state().reshape(-1, mech.ns + 1)
    s.close()
    return out


def test_open_boundaries_bulk_equals_plain_and_freestream_is_exact():
    n = 8  # 8 x 8 x 8 open-wall slice: every direction qualifies for bulk copies
    ns = mechanism.superfast().ns
    ones, qb1 = np.ones((ns, n, n, n)), np.ones((ns, n, n))
    out = _regional_steps(STAGING_BULK, n, ones, qb1)
    assert np.all(out[:, :-1] == 1.0)
    rng = np.random.default_rng(5)
    q = 1e-9 * (1 + rng.random((ns, n, n, n)))
    qb = 1e-9 * (1 + rng.random((ns, n, n)))
    a = _regional_steps(STAGING_BULK, n, q, qb)
    b = _regional_steps(STAGING_PLAIN, n, q, qb)
    assert np.all(np.isfinite(a))
    assert np.array_equal(a, b)


@pytest.mark.parametrize("sper", [1, 2, 3, 4, 5, 12])
def test_streaming_forms_are_bit_identical_to_the_pencils(sper):
    """The streaming kernels (a warp of shuffles per lon-row segment, one thread per lat /
    vertical line) form the same pairs in the same order as the pencils: the same bits, on a
    global grid (periodic rows, mirrored poles and levels) and on open walls, for tracer
    groupings that divide the 12 tracers evenly and that leave a shorter last group."""
    w = workloads.c2(nlon=36, nlat=19, nlev=10)
    a, _ = _run(w, STAGING_AUTO, dict(mixed_x_stream=1, mixed_yz_stream=1, mixed_x_tracers=sper,
                                      mixed_yz_tracers=sper))
    b, _ = _run(w, STAGING_PLAIN, dict(mixed_x_tracers=sper, mixed_yz_tracers=sper))
    assert np.all(np.isfinite(a))
    assert np.array_equal(a, b)


def test_streaming_forms_open_boundaries_and_freestream():
    n = 8
    ns = mechanism.superfast().ns
    out = _regional_steps(STAGING_AUTO, n, np.ones((ns, n, n, n)), np.ones((ns, n, n)), stream=1)
    assert np.all(out[:, :-1] == 1.0)
    rng = np.random.default_rng(6)
    q = 1e-9 * (1 + rng.random((ns, n, n, n)))
    qb = 1e-9 * (1 + rng.random((ns, n, n)))
    a = _regional_steps(STAGING_AUTO, n, q, qb, stream=1)
    b = _regional_steps(STAGING_PLAIN, n, q, qb)
    assert np.array_equal(a, b)
