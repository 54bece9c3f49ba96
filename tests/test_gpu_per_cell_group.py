"""Per-cell adaptive chemistry with G lanes per cell (work arrays in shared memory), and the
thread-per-cell kernel capped at 32 registers, against the thread-per-cell kernel: the same
operations in the same order, so the same bits -- states, accepted and attempted step counts --
for every G, with and without emissions and the clamp, on the large synthetic mechanism and on
SuperFast's table kernels."""
import numpy as np
import pytest

from reseact.esm_gb300 import RsError, Solver, abi, workloads

pytestmark = pytest.mark.gpu


def _window(w, group, t1=600.0, kind=None, **cfg):
    s = Solver.for_workload(w, **cfg)
    if kind is not None:
        s.set_chem_kernel(kind)
    s.set_launch_shape(per_cell_group=group)
    s.set_state(w.u0_cellmajor())
    rc, _, _, st = s.macro_step(0.0, t1, 1.0, w.dt0_C, check=False)
    out = s.get_state()
    s.close()
    return rc, out, (st.naC, st.nrC)


def _with_emission(w, seed=7):
    rng = np.random.default_rng(seed)
    g = w.grid
    emis = np.zeros((w.mech.ns, g["nlev"], g["nlat"], g["nlon"]))
    for s in rng.choice(w.mech.ns, size=5, replace=False):
        emis[s] = 1e-10 * rng.uniform(0.0, 1.0, size=emis.shape[1:])
    w.forcing["emission"] = emis
    return w


@pytest.mark.parametrize("group", [4, 8, 16])
@pytest.mark.parametrize("variant", ["plain", "emission", "no_clamp"])
def test_group_kernel_matches_thread_kernel(group, variant):
    w = workloads.c3(ncells=4096)
    cfg = {}
    if variant == "emission":
        w = _with_emission(w)
    if variant == "no_clamp":
        cfg["clamp_nonneg"] = False
    rc0, ref, n0 = _window(w, 0, **cfg)
    rc1, got, n1 = _window(w, group, **cfg)
    # without the clamp some cells of this random mechanism go negative and run into maxiters:
    # both kernels stop them at the same attempt
    assert rc0 == rc1 and (rc0 == 0 or variant == "no_clamp")
    assert n0 == n1
    assert np.array_equal(ref, got)


@pytest.mark.parametrize("group", [4, 16])
def test_group_kernel_superfast_tables(group):
    """SuperFast (12 chemistry species + air mass) on the table-walking kernels."""
    w = workloads.c2(nlon=24, nlat=16, nlev=8)
    kw = dict(do_transport=False, chem_mode=abi.RS_CHEM_PER_CELL)
    from reseact.esm_gb300._lib import CHEM_KERNEL_TABLE
    rc0, ref, n0 = _window(w, 0, kind=CHEM_KERNEL_TABLE, **kw)
    rc1, got, n1 = _window(w, group, kind=CHEM_KERNEL_TABLE, **kw)
    assert rc0 == rc1 == 0 and n0 == n1
    assert np.array_equal(ref, got)


@pytest.mark.parametrize("threads", [128, 256])
def test_register_capped_kernel_matches(threads):
    """The thread-per-cell kernel capped at 32 registers (2048 resident threads per SM)."""
    w = workloads.c3(ncells=4096)
    rc0, ref, n0 = _window(w, 0)
    s = Solver.for_workload(w)
    s.set_launch_shape(per_cell_threads=threads, per_cell_blocks_per_sm=2048 // threads,
                       per_cell_regcap=1)
    s.set_state(w.u0_cellmajor())
    rc1, _, _, st = s.macro_step(0.0, 600.0, 1.0, w.dt0_C, check=False)
    got = s.get_state()
    s.close()
    assert rc0 == rc1 == 0 and n0 == (st.naC, st.nrC)
    assert np.array_equal(ref, got)


def test_group_kernel_carries_per_cell_dt():
    """Two consecutive windows: the second starts from each cell's carried step size."""
    w = workloads.c3(ncells=2048)
    outs = []
    for group in (0, 8):
        s = Solver.for_workload(w)
        s.set_launch_shape(per_cell_group=group)
        s.set_state(w.u0_cellmajor())
        s.macro_step(0.0, 300.0, 1.0, w.dt0_C)
        _, _, _, st = s.macro_step(300.0, 600.0, 1.0, w.dt0_C)
        outs.append((s.get_state(), st.naC, st.nrC))
        s.close()
    assert np.array_equal(outs[0][0], outs[1][0]) and outs[0][1:] == outs[1][1:]


def test_strict_build_refuses_group_kernel():
    w = workloads.c3(ncells=256)
    s = Solver.for_workload(w, strict=True)
    with pytest.raises(RsError):
        s.set_launch_shape(per_cell_group=8)
    s.close()


def test_cell_steps_diagnostics():
    """rs_get_cell_steps: each cell's accepted substeps of the last window sum to the macro
    step's total, and the carried step sizes are on the step-size lattice."""
    w = workloads.c3(ncells=2048)
    s = Solver.for_workload(w)
    s.set_state(w.u0_cellmajor())
    _, _, _, st = s.macro_step(0.0, 600.0, 1.0, w.dt0_C)
    steps, dt = s.cell_steps()
    assert steps.shape == (1, w.grid["nlat"], w.grid["nlon"])
    assert steps.min() >= 1 and steps.sum() == st.chem_cell_steps
    bits = dt.reshape(-1).view(np.uint64)
    assert np.all(dt > 0) and np.all(bits & np.uint64((1 << 48) - 1) == 0)
    s.close()

