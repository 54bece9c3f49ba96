"""C-ABI checks that need no GPU: the library builds and loads, exports every symbol the
public header declares, host-only entry points behave, and without a CUDA device the product
path fails loudly (there is no CPU fallback)."""
import ctypes as C
import os
import re

import pytest

from reseact.esm_gb300 import _lib, abi, mechanism, workloads

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "reseact_gb300.h")).read()
    decl = r"^(?:rs_status|void|const char\*|size_t|int32_t|void\*)\s+\*?(rs_[a-z0-9_]+)\s*\("
    return sorted(set(re.findall(decl, txt, flags=re.M)))


@pytest.mark.parametrize("strict", [False, True])
def test_library_exports_header_symbols(strict):
    L = _lib.load(strict)
    syms = header_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(L, s), s
    assert set(syms) == set(_lib.SYMBOLS)


def test_default_config_matches_reference_constants():
    L = _lib.load()
    cfg = abi.rs_config()
    L.rs_default_config(C.byref(cfg))
    assert cfg.api_version == abi.RS_API_VERSION
    assert (cfg.rtol_T, cfg.atol_T, cfg.rtol_C, cfg.atol_C) == (1e-4, 1e-6, 1e-4, 1e-9)
    assert cfg.ctrl_C.beta1 == 7 / 20 and cfg.ctrl_C.beta2 == 1 / 5 and cfg.ctrl_C.qsteady_max == 6 / 5
    assert cfg.ctrl_T.beta1 == 7 / 30 and cfg.ctrl_T.beta2 == 2 / 15 and cfg.ctrl_T.qsteady_max == 1.0
    assert cfg.maxiters == 2e4 and cfg.clamp_nonneg == 1
    ref = abi.pictrl_ros23()
    assert [getattr(ref, f) for f, _ in abi.rs_controller._fields_] == \
        [getattr(cfg.ctrl_C, f) for f, _ in abi.rs_controller._fields_]


def test_create_fails_loudly_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    w = workloads.c1()
    with pytest.raises(_lib.RsError) as ei:
        _lib.Solver.for_workload(w)
    assert ei.value.status in (abi.RS_ERR_CUDA, abi.RS_ERR_NOMEM)


def test_null_arguments_rejected():
    L = _lib.load()
    assert L.rs_create(None, None) == abi.RS_ERR_INVALID
    assert L.rs_macro_step(None, 0.0, 1.0, None, None, None) == abi.RS_ERR_INVALID
    assert L.rs_state_size(None) == 0


def test_ctypes_mirrors_match_the_header_layout(tmp_path):
    """Every ctypes mirror of a header struct has the header's size and field offsets
    (a small C program built with the host compiler prints them)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = {"rs_grid": abi.rs_grid, "rs_controller": abi.rs_controller,
               "rs_mechanism": abi.rs_mechanism, "rs_config": abi.rs_config,
               "rs_forcing": abi.rs_forcing, "rs_stats": abi.rs_stats,
               "rs_solve_opts": abi.rs_solve_opts, "rs_solve_result": abi.rs_solve_result}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "reseact_gb300.h"',
             'int main(void) {']
    for name, cls in structs.items():
        lines.append('  printf("%s %%zu\\n", sizeof(%s));' % (name, name))
        for f in cls._fields_:
            lines.append('  printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (name, f[0], name, f[0]))
    lines.append('  return 0; }')
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = dict(l.split() for l in subprocess.run([str(exe)], capture_output=True, text=True,
                                                  check=True).stdout.splitlines())
    for name, cls in structs.items():
        assert int(out[name]) == C.sizeof(cls), name
        for f in cls._fields_:
            assert int(out["%s.%s" % (name, f[0])]) == getattr(cls, f[0]).offset, (name, f[0])


@pytest.mark.parametrize("dims", [(2, 9, 6), (16, 2, 6), (16, 9, 2)])
def test_transport_grid_below_the_stencil_is_rejected(dims):
    """A transport grid with fewer than 3 cells along any direction cannot hold the PPM
    stencil (three cells each side, mirrored or wrapped): rs_create refuses it before any
    device call, so this holds without a GPU."""
    nlon, nlat, nlev = dims
    w = workloads.c2(nlon=nlon, nlat=nlat, nlev=nlev, steps=1)
    with pytest.raises(_lib.RsError) as ei:
        _lib.Solver.for_workload(w)
    assert ei.value.status == abi.RS_ERR_INVALID
    assert "nlon, nlat, nlev >= 3" in str(ei.value)


def test_adjoint_tape_budget_rejects_negative_values():
    L = _lib.load()
    assert L.rs_set_adjoint_tape(None, -1) == abi.RS_ERR_INVALID  # no handle
    assert L.rs_record_taped(None) == 0
