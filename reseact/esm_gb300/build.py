"""Build libreseact_gb300.so (and its strict-arithmetic twin) in-tree with nvcc for sm_103a.

Two builds of the same sources:
  _build/libreseact_gb300.so         production: FMA contraction, reciprocal multiplies
  _build/libreseact_gb300_strict.so  --fmad=false and -DRS_STRICT=1: divides where the
                                     reference divides, no contraction; bit-compatible with
                                     the CPU restatement given identical rate constants.
and on demand a third, _build/libreseact_gb300_check.so (-DRS_BOUNDS_CHECK=1), the production
arithmetic with index checks in the transport pencils.
Host code is compiled with -ffp-contract=off so the geometry and PPM coefficient tables are
identical on x86_64 and aarch64.  Translation units compile in parallel.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
SOURCES = ["rs_api.cu", "rs_chem.cu", "rs_transport.cu", "rs_control.cu", "rs_adjoint.cu",
           "rs_jit.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
LIBS = {"libreseact_gb300.so": ["--fmad=true", "-DRS_STRICT=0"],
        "libreseact_gb300_strict.so": ["--fmad=false", "-DRS_STRICT=1"]}
# Bounds-check build of the production arithmetic: the transport pencils check every
# shared-memory row, halo load and bulk-copy box start and report a failed check as a status
# (no trap).  Built on demand by the tests that use it (build(only=[CHECK_LIB])).
CHECK_LIB = "libreseact_gb300_check.so"
CHECK_FLAGS = ["--fmad=true", "-DRS_STRICT=0", "-DRS_BOUNDS_CHECK=1"]


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _compile(args):
    src, obj, extra = args
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
           "-I", os.path.join(HERE, "..", "..", "include"), *extra, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return obj, r.stderr


def lib_path(strict=False, check=False):
    if check:
        return os.path.join(OUT, CHECK_LIB)
    return os.path.join(OUT, "libreseact_gb300_strict.so" if strict else "libreseact_gb300.so")


def up_to_date(lib):
    if not os.path.exists(lib):
        return False
    t = os.path.getmtime(lib)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f != "peak_probe.cu"]
    deps.append(os.path.join(HERE, "..", "..", "include", "reseact_gb300.h"))
    deps.append(os.path.abspath(__file__))
    return all(os.path.getmtime(d) <= t for d in deps)


def build(force=False, verbose=False, only=None):
    os.makedirs(OUT, exist_ok=True)
    jobs, links = [], []
    libs = dict(LIBS)
    if only and CHECK_LIB in only:
        libs[CHECK_LIB] = CHECK_FLAGS
    for lib, flags in libs.items():
        if only and lib not in only:
            continue
        path = os.path.join(OUT, lib)
        if not force and up_to_date(path):
            continue
        tag = lib.replace(".so", "")
        objs = []
        for s in SOURCES:
            obj = os.path.join(OUT, "%s_%s.o" % (tag, s.replace(".cu", "")))
            jobs.append((os.path.join(CSRC, s), obj, flags))
            objs.append(obj)
        links.append((path, objs))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            for obj, err in ex.map(_compile, jobs):
                if verbose and err.strip():
                    print(err, file=sys.stderr)
    for path, objs in links:
        tmp = path + ".tmp"
        cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s" % r.stderr)
        os.replace(tmp, path)
    probe = probe_path()
    src = os.path.join(CSRC, "peak_probe.cu")
    if force or not os.path.exists(probe) or os.path.getmtime(probe) < os.path.getmtime(src):
        r = subprocess.run([nvcc(), *ARCH, "-O3", "-o", probe, src], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("peak probe build failed:\n%s" % r.stderr)
    return [lib_path(False), lib_path(True)]


def probe_path():
    """FP64/FP32 FMA-rate probe (roofline denominator for the FP64-bound kernels)."""
    return os.path.join(OUT, "peak_probe")


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
