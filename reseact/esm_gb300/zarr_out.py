"""Streaming Zarr v3 output of the split step, species-major (the gridded output of
run_reseact.jl:257-271, written there by EarthSciIO's Zarr v3 sink; EarthSciIO is not
vendored, so this writer follows the public Zarr v3 storage specification directly).

Layout of a store:
  <path>/zarr.json                group; attributes: model metadata, species list, grid
  <path>/<species>/zarr.json      array [time, lev, lat, lon] float64, one chunk per record
  <path>/<species>/c/<r>/0/0/0    chunk r: the species plane at output time r (C order,
                                  little-endian, gzip codec unless compression=None)
  <path>/time, lon, lat, lev      coordinate arrays (one chunk each)
Records are written as the run reaches each output time (streaming); unwritten records read
as the fill value NaN.  read_array() reads a store back (for checks without the zarr package).
"""
from __future__ import annotations

import gzip
import json
import os

import numpy as np

_FILL = "NaN"


def _array_meta(shape, chunks, dims, compression, attrs=None):
    codecs = [{"name": "bytes", "configuration": {"endian": "little"}}]
    if compression == "gzip":
        codecs.append({"name": "gzip", "configuration": {"level": 5}})
    return {"zarr_format": 3, "node_type": "array", "shape": list(shape),
            "data_type": "float64",
            "chunk_grid": {"name": "regular", "configuration": {"chunk_shape": list(chunks)}},
            "chunk_key_encoding": {"name": "default", "configuration": {"separator": "/"}},
            "fill_value": _FILL, "codecs": codecs, "attributes": attrs or {},
            "dimension_names": list(dims)}


def _write_json(path, obj):
    tmp = path + ".tmp"
    with open(tmp, "w") as fh:
        json.dump(obj, fh, indent=1)
    os.replace(tmp, path)


def _encode(a, compression):
    raw = np.ascontiguousarray(a, dtype="<f8").tobytes()
    return gzip.compress(raw, compresslevel=5) if compression == "gzip" else raw


class ZarrSink:
    """Species-major Zarr v3 store with one record per output time."""

    def __init__(self, path, species, grid, output_times, attrs=None, compression="gzip"):
        self.path = str(path)
        self.species = list(species)
        self.grid = dict(grid)
        self.times = np.asarray(output_times, dtype=np.float64)
        self.attrs = dict(attrs or {})
        self.compression = compression
        self.written = set()

    @property
    def shape(self):
        g = self.grid
        return (len(self.times), g["nlev"], g["nlat"], g["nlon"])

    def open(self):
        os.makedirs(self.path, exist_ok=True)
        g = self.grid
        root = {"zarr_format": 3, "node_type": "group",
                "attributes": dict(self.attrs, species=self.species,
                                   layout="species-major [time, lev, lat, lon]",
                                   grid={k: g[k] for k in ("nlon", "nlat", "nlev", "lon0_deg",
                                                            "dlon_deg", "lat0_deg", "dlat_deg")
                                         if k in g})}
        _write_json(os.path.join(self.path, "zarr.json"), root)
        nt, nlev, nlat, nlon = self.shape
        for s in self.species:
            os.makedirs(os.path.join(self.path, s), exist_ok=True)
            _write_json(os.path.join(self.path, s, "zarr.json"),
                        _array_meta(self.shape, (1, nlev, nlat, nlon),
                                    ("time", "lev", "lat", "lon"), self.compression))
        coords = {"time": self.times,
                  "lon": g.get("lon0_deg", 0.0) + np.arange(nlon) * g.get("dlon_deg", 1.0),
                  "lat": g.get("lat0_deg", 0.0) + np.arange(nlat) * g.get("dlat_deg", 1.0),
                  "lev": np.arange(nlev, dtype=np.float64)}
        for name, v in coords.items():
            d = os.path.join(self.path, name)
            os.makedirs(os.path.join(d, "c"), exist_ok=True)
            _write_json(os.path.join(d, "zarr.json"),
                        _array_meta(v.shape, v.shape, (name,), self.compression))
            with open(os.path.join(d, "c", "0"), "wb") as fh:
                fh.write(_encode(v, self.compression))
        return self

    def record_of(self, t):
        r = np.nonzero(np.abs(self.times - float(t)) <= 1e-6)[0]
        if r.size == 0:
            raise ValueError("t=%g is not an output time of this store" % t)
        return int(r[0])

    def write(self, t, u_soa):
        """Write the state at output time t; u_soa is [species(+m)][lev][lat][lon] (extra
        trailing planes, such as the air mass, are written only if named in species)."""
        r = self.record_of(t)
        u = np.asarray(u_soa)
        for q, s in enumerate(self.species):
            d = os.path.join(self.path, s, "c", str(r), "0", "0")
            os.makedirs(d, exist_ok=True)
            tmp = os.path.join(d, "0.tmp")
            with open(tmp, "wb") as fh:
                fh.write(_encode(u[q], self.compression))
            os.replace(tmp, os.path.join(d, "0"))
        self.written.add(r)

    def flush(self):
        pass  # every record is complete on disk when write() returns

    def close(self):
        self.flush()


def read_array(path, name):
    """Read one array of a store written by ZarrSink (regular chunks, bytes + optional gzip)."""
    with open(os.path.join(path, name, "zarr.json")) as fh:
        meta = json.load(fh)
    shape, chunks = meta["shape"], meta["chunk_grid"]["configuration"]["chunk_shape"]
    gz = any(c["name"] == "gzip" for c in meta["codecs"])
    out = np.full(shape, np.nan)
    grid = [range((n + c - 1) // c) for n, c in zip(shape, chunks)]
    for idx in np.ndindex(*[len(g) for g in grid]):
        f = os.path.join(path, name, "c", *[str(i) for i in idx])
        if not os.path.exists(f):
            continue
        with open(f, "rb") as fh:
            raw = fh.read()
        a = np.frombuffer(gzip.decompress(raw) if gz else raw, dtype="<f8").reshape(chunks)
        sl = tuple(slice(i * c, min((i + 1) * c, n)) for i, c, n in zip(idx, chunks, shape))
        out[sl] = a[tuple(slice(0, s.stop - s.start) for s in sl)]
    return out
