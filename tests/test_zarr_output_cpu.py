"""Streaming species-major Zarr v3 output and the STATEDUMP format, without a GPU: stores
written record by record read back exactly, with the v3 metadata the specification asks for,
unwritten records as the fill value, and the dump round trip."""
import json
import os

import numpy as np

from reseact.esm_gb300 import run, workloads, zarr_out


def test_zarr_store_streams_and_reads_back(tmp_path):
    g = workloads.latlon_grid(8, 5, 4)
    species = ["CO", "NO", "O3"]
    times = [0.0, 600.0, 1200.0, 1800.0]
    rng = np.random.default_rng(0)
    sink = zarr_out.ZarrSink(tmp_path / "out.zarr", species, g, times,
                             attrs={"model": "test"}).open()
    states = {}
    for t in (0.0, 1200.0, 1800.0):   # 600 s never written
        u = rng.standard_normal((4, 4, 5, 8))  # 3 species + air mass
        sink.write(t, u)
        states[t] = u
    sink.close()
    root = json.load(open(tmp_path / "out.zarr" / "zarr.json"))
    assert root["zarr_format"] == 3 and root["node_type"] == "group"
    assert root["attributes"]["species"] == species
    meta = json.load(open(tmp_path / "out.zarr" / "NO" / "zarr.json"))
    assert meta["node_type"] == "array" and meta["shape"] == [4, 4, 5, 8]
    assert meta["dimension_names"] == ["time", "lev", "lat", "lon"]
    assert [c["name"] for c in meta["codecs"]] == ["bytes", "gzip"]
    for q, s in enumerate(species):
        a = zarr_out.read_array(tmp_path / "out.zarr", s)
        for r, t in enumerate(times):
            if t in states:
                assert np.array_equal(a[r], states[t][q])
            else:
                assert np.all(np.isnan(a[r]))
    assert np.array_equal(zarr_out.read_array(tmp_path / "out.zarr", "time"), times)
    assert os.path.exists(tmp_path / "out.zarr" / "O3" / "c" / "2" / "0" / "0" / "0")


def test_statedump_round_trip(tmp_path):
    names = ["CO", "NO", "m"]
    pre = np.arange(12.0)
    post = -np.arange(12.0)
    p = tmp_path / "dump.bin"
    run.write_statedump(p, names, 1800.0, pre, post)
    ns, nc, t, a, b = run.read_statedump(p)
    assert (ns, nc, t) == (3, 4, 1800.0)
    assert np.array_equal(a, pre) and np.array_equal(b, post)
    lines = open(str(p) + ".names").read().splitlines()
    assert lines[0].startswith("# NS=3 NC=4 t=1800.0") and lines[1:] == ["1\tCO", "2\tNO", "3\tm"]
