"""The three mirrors of the C ABI's structs agree byte for byte.

* include/reseact_gb300.h, through offsetof / sizeof in tests/abi_layout.c (built here with
  gcc); its output is committed as tests/golden/abi_layout.json, so a header change that the
  mirrors do not follow fails here;
* the Python ctypes mirrors in reseact/esm_gb300/abi.py;
* the Julia isbits mirrors in julia/src/ReseactGPU.jl, laid out by the C rules Julia applies
  to isbits structs (each field at its natural alignment, the size rounded up to the largest
  alignment); Julia is not installed here, so the layout is computed from the field types.
"""
import ctypes as C
import json
import os
import re
import shutil
import subprocess

import pytest

from reseact.esm_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "abi_layout.json")
JULIA_SRC = os.path.join(ROOT, "julia", "src", "ReseactGPU.jl")
JULIA_NAMES = {"RsMechanism": "rs_mechanism", "RsGrid": "rs_grid", "RsController": "rs_controller",
               "RsConfig": "rs_config", "RsForcing": "rs_forcing", "RsStats": "rs_stats",
               "RsSolveOpts": "rs_solve_opts", "RsSolveResult": "rs_solve_result"}


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    exe = str(tmp_path_factory.mktemp("abi") / "abi_layout")
    subprocess.run([cc, "-std=c99", "-Wall", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "abi_layout.c"), "-o", exe], check=True)
    return json.loads(subprocess.run([exe], check=True, capture_output=True, text=True).stdout)


def test_header_layout_matches_committed_table(c_layout):
    with open(GOLDEN) as fh:
        assert c_layout == json.load(fh)


def test_ctypes_mirrors_match_header(c_layout):
    for name, lay in c_layout.items():
        cls = getattr(abi, name)
        assert C.sizeof(cls) == lay["size"], name
        got = {f: getattr(cls, f).offset for f, _ in cls._fields_}
        assert got == lay["fields"], name


def _julia_structs():
    src = open(JULIA_SRC).read()
    out = {}
    for m in re.finditer(r"^(?:mutable )?struct (\w+)\n(.*?)^end", src, re.S | re.M):
        fields = []
        for part in re.split(r"[;\n]", m.group(2)):
            part = part.split("#")[0].strip()
            if "::" in part:
                n, t = part.split("::", 1)
                fields.append((n.strip(), t.strip()))
        out[m.group(1)] = fields
    return out


def _julia_layout(structs, name, memo):
    if name in memo:
        return memo[name]
    prim = {"Int32": 4, "Float64": 8, "Csize_t": 8, "Cint": 4, "Int64": 8, "UInt32": 4}
    off, align, fields = 0, 1, {}
    for f, t in structs[name]:
        if t in prim:
            sz = al = prim[t]
        elif t.startswith("Ptr{"):
            sz = al = 8
        else:
            sz, al = _julia_layout(structs, t, memo)[:2]
        off = (off + al - 1) // al * al
        fields[f] = off
        off += sz
        align = max(align, al)
    size = (off + align - 1) // align * align
    memo[name] = (size, align, fields)
    return memo[name]


def test_julia_mirrors_match_header(c_layout):
    structs = _julia_structs()
    memo = {}
    for jname, cname in JULIA_NAMES.items():
        assert jname in structs, jname
        size, _, fields = _julia_layout(structs, jname, memo)
        assert size == c_layout[cname]["size"], (jname, size)
        assert fields == c_layout[cname]["fields"], jname


def test_julia_package_declares_the_extension():
    """julia/Project.toml makes ReseactGPUChainRulesExt a package extension on ChainRulesCore,
    and the extension imports the parent package by name (an extension is a top-level module)."""
    toml = open(os.path.join(ROOT, "julia", "Project.toml")).read()
    assert re.search(r'^name = "ReseactGPU"$', toml, re.M)
    assert re.search(r"^\[weakdeps\]\nChainRulesCore = \"d360d2e6-b24c-11e9-a2a3-2a2ae2dbcce4\"",
                     toml, re.M)
    assert re.search(r'^\[extensions\]\nReseactGPUChainRulesExt = "ChainRulesCore"', toml, re.M)
    ext = open(os.path.join(ROOT, "julia", "ext", "ReseactGPUChainRulesExt.jl")).read()
    assert "module ReseactGPUChainRulesExt" in ext
    assert re.search(r"^using ReseactGPU: ", ext, re.M)
    assert os.path.exists(JULIA_SRC)
