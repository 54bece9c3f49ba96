"""The allocation-free chemistry attempt, rs_ros23_attempt_noalloc.

It exists for callers that cannot allocate device memory when they step the chemistry (their
own memory pool owns the device, or an allocation would stall a latency-critical loop): its
scratch is a fixed array inside the library.  Here it is called through the C ABI on device
buffers the test owns, twice in a row (the second call must not see the first call's
scratch), and compared with the existing single-step entry point, rs_single_step, to the
tolerance the parity tests use for one attempt.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from reseact.esm_gb300 import Solver, abi, mechanism, workloads

pytestmark = pytest.mark.gpu


def _dptr(t):
    return C.c_void_p(t.data_ptr())


def test_noalloc_attempt_matches_single_step_twice():
    torch = pytest.importorskip("torch")
    w = workloads.c2(nlon=16, nlat=9, nlev=6)
    s = Solver.for_workload(w)
    g = w.grid
    for call, dt in enumerate((2.0, 7.5)):
        u_cm = w.u0_cellmajor() * (1.0 + 0.01 * call)
        ref, e_ref = s.single_step(abi.RS_OP_CHEMISTRY, u_cm, 0.0, dt)
        u_soa = workloads.cellmajor_to_soa(u_cm, w.nsp, g["nlon"], g["nlat"], g["nlev"])
        d_in = torch.tensor(u_soa, dtype=torch.float64, device="cuda")
        d_out = torch.full_like(d_in, float("nan"))
        torch.cuda.synchronize()
        e = C.c_double(-1.0)
        rc = s.L.rs_ros23_attempt_noalloc(s.h, dt, _dptr(d_in), _dptr(d_out), C.byref(e))
        assert rc == abi.RS_OK, s.L.rs_last_error(s.h)
        got = workloads.soa_to_cellmajor(d_out.cpu().numpy(), g["nlon"], g["nlat"], g["nlev"])
        err = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-9)
        assert err.max() <= 1e-12, (call, err.max())
        assert e.value == pytest.approx(e_ref, rel=1e-12)


def test_noalloc_second_call_allocates_no_device_memory():
    """The property the entry point exists for: once the handle exists (rs_create resolved the
    scratch array's address), a call changes the device's free memory by nothing."""
    torch = pytest.importorskip("torch")
    w = workloads.c2(nlon=16, nlat=9, nlev=6)
    s = Solver.for_workload(w)
    g = w.grid
    u_soa = workloads.cellmajor_to_soa(w.u0_cellmajor(), w.nsp, g["nlon"], g["nlat"], g["nlev"])
    d_in = torch.tensor(u_soa, dtype=torch.float64, device="cuda")
    d_out = torch.empty_like(d_in)
    e = C.c_double()
    torch.cuda.synchronize()
    rc = s.L.rs_ros23_attempt_noalloc(s.h, 3.0, _dptr(d_in), _dptr(d_out), C.byref(e))
    assert rc == abi.RS_OK, s.L.rs_last_error(s.h)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        rc = s.L.rs_ros23_attempt_noalloc(s.h, 3.0, _dptr(d_in), _dptr(d_out), C.byref(e))
        assert rc == abi.RS_OK
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


def test_noalloc_rejects_grids_beyond_its_limit():
    torch = pytest.importorskip("torch")
    # one species, one first-order loss: just enough to build a handle of 2^24 + 4096 cells
    m = mechanism.Mechanism("tiny", ["A"], {"A": 1.0}, [], [],
                            [mechanism.Reaction("R1", [(0, 1)], [], [mechanism.OP_CONST], [1e-3])])
    g = workloads.latlon_grid(4096, 4097, 1, pole_centred=False)
    mabi = abi.MechanismABI(m)
    cfg = abi.make_config(g, mabi, has_air_mass=False, do_transport=False)
    s = Solver(cfg, mabi)
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda")
    e = C.c_double()
    rc = s.L.rs_ros23_attempt_noalloc(s.h, 1.0, _dptr(dummy), _dptr(dummy), C.byref(e))
    assert rc == abi.RS_ERR_INVALID
    assert b"16,777,216" in s.L.rs_last_error(s.h)
