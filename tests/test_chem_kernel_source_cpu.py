"""The mechanism-specialised chemistry kernels are generated and compiled without a GPU:
the source for SuperFast holds the mechanism's arithmetic as straight-line code, NVRTC
compiles it for sm_103a (ptxas reports every entry point), and mechanisms beyond the
straight-line limits are refused with a reason."""
import pytest

from reseact.esm_gb300 import abi, mechanism
from reseact.esm_gb300._lib import RsError, chem_kernel_compile, chem_kernel_source


def test_superfast_source_is_straight_line():
    m = mechanism.superfast()
    src = chem_kernel_source(abi.MechanismABI(m))
    assert "#define NS %d" % m.ns in src and "#define NRA %d" % m.nr in src
    for name in ("rs_jit_attempt_r0", "rs_jit_attempt_r1", "rs_jit_attempt_s0",
                 "rs_jit_attempt_s1", "rs_jit_per_cell_0", "rs_jit_per_cell_1",
                 "rs_jit_step_0", "rs_jit_step_1", "rs_jit_vjp_0", "rs_jit_vjpk_1"):
        assert name in src
    # no table walk: every W slot is named by a constant
    assert "WV(0) =" in src and "elim_ptr" not in src
    strict = chem_kernel_source(abi.MechanismABI(m), strict=True)
    assert ") / WV(" in strict and ") * pv[" in src
    # production: the fused RHS (heads u_r, no rate array) and W from the scaled rate
    # constants kd_r = -dtg K_r; strict: the oracle's rate array and -dtg per Jacobian entry
    assert "const double u0_ = " in src and "const double kd0_ = -dtg * K(0);" in src
    assert "v[0] = " in strict and "-(dtg*(" in strict and "kd0_" not in strict
    # the stage tape: the attempt writes k1 and z2 to its slot, the VJP variant reads them
    assert "kzo[(u64)s * N + c] = k1[s];" in src and "kzi[(u64)s * N + c]" in src


@pytest.mark.parametrize("strict", [False, True])
def test_superfast_compiles_for_sm103a(strict):
    rep = chem_kernel_compile(abi.MechanismABI(mechanism.superfast()), strict=strict)
    for name in ("rs_jit_attempt_r0", "rs_jit_attempt_s1", "rs_jit_per_cell_1",
                 "rs_jit_step_0", "rs_jit_vjpk_0"):
        assert "Compiling entry function '%s' for 'sm_103a'" % name in rep


def test_large_mechanism_is_refused():
    with pytest.raises(RsError) as e:
        chem_kernel_source(abi.MechanismABI(mechanism.synthetic()))
    assert e.value.status == abi.RS_ERR_UNSUPPORTED
