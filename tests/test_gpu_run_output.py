"""The reference's macro-step loop over the GPU split step (reseact.esm_gb300.run.run_split):
one library window per macro step, species-major Zarr records at the output cadence that
match the device state, continuity drift per step with the pressure fixer."""
import numpy as np
import pytest

from reseact.esm_gb300 import Solver, run, workloads, zarr_out

pytestmark = pytest.mark.gpu


def test_run_writes_zarr_records_and_reports_drift(tmp_path):
    w = workloads.with_pressure_fixer(workloads.c2(nlon=16, nlat=9, nlev=12, steps=1))
    s = Solver.for_workload(w)
    s.set_state(w.u0_cellmajor())
    g = w.grid
    names = list(w.mech.species) + ["m"]
    sink = zarr_out.ZarrSink(tmp_path / "c2.zarr", names, g, [0.0, 1200.0, 2400.0]).open()
    res = run.run_split(s, w, 0.0, 2400.0, macro_dt=600.0, out_every=2, sink=sink)
    assert res.ok and res.nstep == 4 and res.t == 2400.0
    assert all(d[0] < 1e-13 for _, d in res.rows)   # rms interior drift per step
    u_end = workloads.cellmajor_to_soa(s.get_state(), w.nsp, g["nlon"], g["nlat"], g["nlev"])
    for q, name in enumerate(names):
        a = zarr_out.read_array(tmp_path / "c2.zarr", name)
        assert np.array_equal(a[0], w.u0[q])
        assert np.array_equal(a[2], u_end[q])
        assert not np.any(np.isnan(a[1]))
