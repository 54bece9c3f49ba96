"""Synthetic workloads: grids, forcing and seeded initial states.

The reference runs on GEOS-FP 4x5 meteorology and NEI2016 emissions
(``prototypes/reseact_3d_chem/split_common.jl:256-339``), neither of which exists here; the
analytic winds and seeded lognormal fields below stand in for them with the shapes, sizes
and value ranges of the benchmark configurations:

* C1  36x18x10 global, 10 deg, levels 1000->100 hPa, solid-body u = 20 cos(lat) m/s,
      SuperFast, lognormal ICs (median = mechanism default, sigma 0.5), dt 600 s x 144.
* C2  144x91x47 global (2.5 x 2 deg, pole-centred), deformational
      u = 40 sin^2(lon) sin(2 lat) cos(pi t / 86400), w = +-0.05 Pa/s sin(pi p / p_s) (seeded
      sign per column), dt 600 s x 144 (24 h).
* C3  2^20 independent cells, synthetic 30-species / 60-reaction mechanism, T ~ U(200,310) K,
      concentrations log-uniform 1e-12..1e-6 mol/mol, chemistry only.
* C4  72x46x47 (5 x 4 deg), C2 winds, 24 h; surface NO emission field for the adjoint.
* C5  360x181x72 with the 72-level hybrid table, C2 winds, C3 mechanism, dt 300 s x 72.

Face fluxes follow the reference's metric on the unit sphere: Mx = dp_face*U_face/a,
My = dp_face*V_face/a (Pa/s), Mz at the lower edge of each level, +ve upward
(``reseact.esm`` metadata; ``prototypes/transport_3d/gen_t3d.py:68-80``).  All three scale
in time by cos(flux_omega*t).

Layouts: the device and the oracle hold grid SoA planes u[s][k][j][i] (lon fastest); the
C ABI's host state is the reference's cell-major u[c*NS+s] with c = (i*nlat+j)*nlev+k.
"""
from __future__ import annotations

import json
import math
import os

import numpy as np

from . import abi
from . import mechanism as mechmod

A_EARTH = 6.371e6
D2R = math.pi / 180.0
HERE = os.path.dirname(os.path.abspath(__file__))


# ------------------------------------------------------------------ layout helpers
def soa_to_cellmajor(u_soa, nlon, nlat, nlev):
    """[ns][nlev][nlat][nlon] -> cell-major [(i*nlat+j)*nlev+k][ns] flattened."""
    ns = u_soa.shape[0]
    a = np.asarray(u_soa).reshape(ns, nlev, nlat, nlon)
    return np.ascontiguousarray(a.transpose(3, 2, 1, 0)).reshape(-1)


def cellmajor_to_soa(u_cm, ns, nlon, nlat, nlev):
    a = np.asarray(u_cm).reshape(nlon, nlat, nlev, ns)
    return np.ascontiguousarray(a.transpose(3, 2, 1, 0))


# ------------------------------------------------------------------ grids and forcing
def latlon_grid(nlon, nlat, nlev, lon_bc=abi.RS_BC_PERIODIC, lat_bc=abi.RS_BC_CLOSED,
                lon0=None, lat0=None, dlon=None, dlat=None, pole_centred=None):
    if dlon is None:
        dlon = 360.0 / nlon
    if lon0 is None:
        lon0 = 0.5 * dlon if lon_bc == abi.RS_BC_PERIODIC else 0.0
    if pole_centred is None:
        pole_centred = nlat % 2 == 1 or nlat in (46,)
    if dlat is None:
        dlat = 180.0 / (nlat - 1) if pole_centred else 180.0 / nlat
    if lat0 is None:
        lat0 = -90.0 if pole_centred else -90.0 + 0.5 * dlat
    return dict(nlon=nlon, nlat=nlat, nlev=nlev, lon_bc=lon_bc, lat_bc=lat_bc,
                lon0_deg=lon0, dlon_deg=dlon, lat0_deg=lat0, dlat_deg=dlat)


def lat_edges(g):
    j = np.arange(g["nlat"] + 1)
    return np.clip(g["lat0_deg"] + (j - 0.5) * g["dlat_deg"], -90.0, 90.0)


def pressure_levels(nlev, p_bot=100000.0, p_top=10000.0):
    """Pure pressure levels (dB = 0): returns (dp[nlev], p_mid[nlev]) bottom-up."""
    pe = p_bot + (p_top - p_bot) * np.arange(nlev + 1) / nlev
    return pe[:-1] - pe[1:], 0.5 * (pe[:-1] + pe[1:])


def hybrid72(ps=101325.0):
    """GEOS-FP 72-level hybrid sigma-pressure table (bottom-up), dp and mid pressure."""
    with open(os.path.join(HERE, "mechanisms", "hybrid_coefs_L72.json")) as fh:
        h = json.load(fh)
    dA, dB = np.asarray(h["dA"]), np.asarray(h["dB"])
    dp = dA + dB * ps
    pe = ps - np.concatenate([[0.0], np.cumsum(dp)])
    return dp, 0.5 * (pe[:-1] + pe[1:])


def standard_temperature(p):
    """US standard atmosphere troposphere T(p), isothermal 216.65 K above the tropopause."""
    return np.maximum(288.15 * (np.asarray(p) / 101325.0) ** 0.1902632, 216.65)


def winds_solid_body(g, dp, u0=20.0):
    nlon, nlat, nlev = g["nlon"], g["nlat"], g["nlev"]
    latc = g["lat0_deg"] + np.arange(nlat) * g["dlat_deg"]
    u = u0 * np.cos(latc * D2R)
    mx = np.empty((nlev, nlat, nlon + 1))
    mx[:] = (dp[:, None, None] * u[None, :, None] / A_EARTH)
    my = np.zeros((nlev, nlat + 1, nlon))
    mz = np.zeros((nlev + 1, nlat, nlon))
    return mx, my, mz


def winds_deformational(g, dp, u0=40.0, w0=0.05, seed=7, w_shape="constant"):
    """u = U0 sin^2(lon_face) sin(2 lat), v = 0, Mz = +-w0 (seeded sign per column).

    w_shape "constant": Mz = +-w0 at every interior interface (zero at the surface and the
    model top).  "sine": Mz = +-w0 sin(pi p / p_s) at interface pressure p, which vanishes
    towards the model top and the surface, so that thin layers (the 1 Pa top layer of the
    72-level hybrid grid) are not emptied: with the constant shape that layer loses its
    whole mass in 20 s."""
    nlon, nlat, nlev = g["nlon"], g["nlat"], g["nlev"]
    latc = g["lat0_deg"] + np.arange(nlat) * g["dlat_deg"]
    lonf = g["lon0_deg"] + (np.arange(nlon + 1) - 0.5) * g["dlon_deg"]
    u = u0 * np.sin(lonf * D2R)[None, :] ** 2 * np.sin(2 * latc * D2R)[:, None]
    mx = dp[:, None, None] * u[None, :, :] / A_EARTH
    my = np.zeros((nlev, nlat + 1, nlon))
    rng = np.random.default_rng(seed)
    sign = rng.choice([-1.0, 1.0], size=(nlat, nlon))
    mz = np.zeros((nlev + 1, nlat, nlon))
    if nlev > 1:
        if w_shape == "sine":
            p_int = np.concatenate([[0.0], np.cumsum(dp[::-1])])[::-1]  # interface k, k=0 surface
            shape = np.sin(np.pi * p_int[1:nlev] / p_int[0])
            mz[1:nlev] = w0 * shape[:, None, None] * sign[None, :, :]
        else:
            mz[1:nlev] = w0 * sign[None, :, :]
    return np.ascontiguousarray(mx), my, mz


def lognormal_state(mech, g, dp3, seed, sigma=0.5, has_air_mass=True):
    rng = np.random.default_rng(seed)
    shape = (g["nlev"], g["nlat"], g["nlon"])
    planes = []
    for s in mech.species:
        med = mech.defaults[s]
        planes.append(med * np.exp(sigma * rng.standard_normal(shape)))
    if has_air_mass:
        planes.append(np.broadcast_to(dp3, shape).copy())
    return np.ascontiguousarray(np.stack(planes))


class Workload:
    """A configured problem: grid, mechanism, forcing, initial state (grid SoA), schedule."""

    def __init__(self, name, grid, mech, forcing, u0, dt_macro, n_steps, has_air_mass=True,
                 do_transport=True, do_chemistry=True, precision=abi.RS_PREC_FP64,
                 chem_mode=abi.RS_CHEM_GLOBAL_DT, dt0_T=15.0, dt0_C=0.5, t0=0.0, notes=""):
        self.name, self.grid, self.mech, self.forcing = name, grid, mech, forcing
        self.u0, self.dt_macro, self.n_steps = u0, dt_macro, n_steps
        self.has_air_mass, self.do_transport, self.do_chemistry = has_air_mass, do_transport, do_chemistry
        self.precision, self.chem_mode = precision, chem_mode
        self.dt0_T, self.dt0_C, self.t0, self.notes = dt0_T, dt0_C, t0, notes

    @property
    def ncells(self):
        g = self.grid
        return g["nlon"] * g["nlat"] * g["nlev"]

    @property
    def nsp(self):
        return self.mech.ns + (1 if self.has_air_mass else 0)

    def config(self, mech_abi, **kw):
        args = dict(has_air_mass=self.has_air_mass, do_transport=self.do_transport,
                    do_chemistry=self.do_chemistry, precision=self.precision,
                    chem_mode=self.chem_mode)
        args.update(kw)
        return abi.make_config(self.grid, mech_abi, **args)

    def forcing_abi(self):
        f = dict(self.forcing)
        om = f.pop("flux_omega", 0.0)
        tau = f.pop("tau_pblmix", 0.0)
        return abi.ForcingABI(flux_omega=om, tau_pblmix=tau, **f)

    def u0_cellmajor(self):
        g = self.grid
        return soa_to_cellmajor(self.u0, g["nlon"], g["nlat"], g["nlev"])


def _column_fields(g, dp, pmid):
    shape = (g["nlev"], g["nlat"], g["nlon"])
    dp3 = np.broadcast_to(dp[:, None, None], shape).copy()
    p3 = np.broadcast_to(pmid[:, None, None], shape).copy()
    return dp3, p3, standard_temperature(p3)


def with_pbl(w, tau=900.0, pblh_median=1000.0, sigma=0.5, seed=11):
    """Switch on the full PBL mixing term of the transport half: a seeded lognormal PBL height
    per column (median pblh_median m), the workload's own interface pressures as hybrid
    coefficients (A = p_interface, B = 0; surface pressure is uniform in these grids) and the
    relaxation time tau (the reference's default is 900 s)."""
    g = w.grid
    dp = np.asarray(w.forcing["dp"])[:, 0, 0]
    pmid = np.asarray(w.forcing["pressure"])[:, 0, 0]
    p_int = np.empty(g["nlev"] + 1)
    p_int[0] = pmid[0] + 0.5 * dp[0]
    for k in range(g["nlev"]):
        p_int[k + 1] = p_int[k] - dp[k]
    rng = np.random.default_rng(seed)
    w.forcing["pblh"] = pblh_median * np.exp(sigma * rng.standard_normal((g["nlat"], g["nlon"])))
    w.forcing["ps"] = np.full((g["nlat"], g["nlon"]), p_int[0])
    w.forcing["hyb_a"] = p_int
    w.forcing["hyb_b"] = np.zeros(g["nlev"] + 1)
    w.forcing["tau_pblmix"] = float(tau)
    w.name += " + PBL mixing"
    return w


def with_pressure_fixer(w, dps_amp=2e-3, seed=12):
    """Switch on the pressure fixer with diagnosed vertical mass flux: steady fluxes, hybrid
    coefficients of the workload's own levels that reach B = 0 at the lid (B_k = (p_k - p_top)
    / (PS - p_top), A_k = p_top (1 - B_k), so that dm_k/dt = dB_k dPS/dt is exercised and the
    diagnosed Mz closes at the top) and a seeded surface-pressure tendency field of amplitude
    dps_amp (Pa/s).  The given mz is ignored once the fixer is on."""
    g = w.grid
    dp = np.asarray(w.forcing["dp"])[:, 0, 0]
    pmid = np.asarray(w.forcing["pressure"])[:, 0, 0]
    p_int = np.empty(g["nlev"] + 1)
    p_int[0] = pmid[0] + 0.5 * dp[0]
    for k in range(g["nlev"]):
        p_int[k + 1] = p_int[k] - dp[k]
    rng = np.random.default_rng(seed)
    w.forcing["flux_omega"] = 0.0
    b = (p_int - p_int[-1]) / (p_int[0] - p_int[-1])
    w.forcing["hyb_a"] = p_int[-1] * (1.0 - b)
    w.forcing["hyb_b"] = b
    w.forcing["ps"] = np.full((g["nlat"], g["nlon"]), p_int[0])
    w.forcing["dps_dt"] = dps_amp * rng.standard_normal((g["nlat"], g["nlon"]))
    w.name += " + pressure fixer"
    return w


def c1(seed=1, mech=None):
    mech = mech or mechmod.superfast()
    g = latlon_grid(36, 18, 10)
    dp, pm = pressure_levels(10)
    dp3, p3, t3 = _column_fields(g, dp, pm)
    mx, my, mz = winds_solid_body(g, dp)
    u0 = lognormal_state(mech, g, dp3, seed)
    forcing = dict(mx=mx, my=my, mz=mz, dp=dp3, temperature=t3, pressure=p3, flux_omega=0.0)
    return Workload("C1 36x18x10 SuperFast FP64", g, mech, forcing, u0, 600.0, 144)


def c2(seed=2, mech=None, nlon=144, nlat=91, nlev=47, steps=144):
    mech = mech or mechmod.superfast()
    g = latlon_grid(nlon, nlat, nlev, lon0=0.0, dlon=360.0 / nlon)
    dp, pm = pressure_levels(nlev)
    dp3, p3, t3 = _column_fields(g, dp, pm)
    # w = +-0.05 Pa/s shaped as sin(pi p / p_s): a constant +-0.05 Pa/s takes ~1,300 of the
    # 1,915 Pa out of the surface layer of every upward column by t = 9.3 h and the transport
    # step then collapses (the oracle stalls there in a 24 h C4 run); the sine keeps the
    # amplitude in the mid troposphere and bounds each layer's mass change to a few per cent
    mx, my, mz = winds_deformational(g, dp, seed=seed + 100, w_shape="sine")
    u0 = lognormal_state(mech, g, dp3, seed)
    forcing = dict(mx=mx, my=my, mz=mz, dp=dp3, temperature=t3, pressure=p3,
                   flux_omega=math.pi / 86400.0)
    return Workload("C2 %dx%dx%d SuperFast FP64" % (nlon, nlat, nlev), g, mech, forcing, u0,
                    600.0, steps)


def c3(seed=3, ncells=1 << 20, mech=None):
    mech = mech or mechmod.synthetic()
    nlon = 1024 if ncells >= 1024 else ncells
    nlat = max(1, ncells // nlon)
    g = latlon_grid(nlon, nlat, 1, pole_centred=False)
    rng = np.random.default_rng(seed)
    shape = (1, nlat, nlon)
    t3 = rng.uniform(200.0, 310.0, size=shape)
    p3 = np.full(shape, 101325.0)
    u0 = np.ascontiguousarray(10.0 ** rng.uniform(-12.0, -6.0, size=(mech.ns,) + shape))
    forcing = dict(temperature=t3, pressure=p3, dp=np.ones(shape))
    return Workload("C3 %d cells synthetic %dx%d" % (ncells, mech.ns, mech.nr), g, mech,
                    forcing, u0, 600.0, 1, has_air_mass=False, do_transport=False,
                    chem_mode=abi.RS_CHEM_PER_CELL, dt0_C=1e-3)


def c4(seed=4, mech=None):
    mech = mech or mechmod.superfast()
    w = c2(seed=seed, mech=mech, nlon=72, nlat=46, nlev=47)
    w.name = "C4 72x46x47 SuperFast FP64 (adjoint)"
    rng = np.random.default_rng(seed + 10)
    g = w.grid
    emis = np.zeros((mech.ns, g["nlev"], g["nlat"], g["nlon"]))
    emis[mech.species.index("NO"), 0] = 1e-4 * np.exp(0.5 * rng.standard_normal((g["nlat"], g["nlon"])))
    w.forcing["emission"] = emis
    return w


def c5(seed=5, mech=None, precision=abi.RS_PREC_MIXED):
    mech = mech or mechmod.synthetic()
    g = latlon_grid(360, 181, 72, lon0=0.0, dlon=1.0)
    dp, pm = hybrid72()
    dp3, p3, t3 = _column_fields(g, dp, pm)
    mx, my, mz = winds_deformational(g, dp, seed=seed + 100, w_shape="sine")
    rng = np.random.default_rng(seed)
    shape = (g["nlev"], g["nlat"], g["nlon"])
    planes = [10.0 ** rng.uniform(-12.0, -6.0, size=shape) for _ in mech.species]
    planes.append(dp3)
    u0 = np.ascontiguousarray(np.stack(planes))
    forcing = dict(mx=mx, my=my, mz=mz, dp=dp3, temperature=t3, pressure=p3,
                   flux_omega=math.pi / 86400.0)
    return Workload("C5 360x181x72 synthetic mixed", g, mech, forcing, u0, 300.0, 72,
                    precision=precision)


def regional_freestream(n=7):
    """The transport_3d.esm freestream case: 7x7x7 CONUS slice, open walls, q = qbc = 1,
    divergent analytic fluxes (prototypes/transport_3d/gen_t3d.py, transport_3d.esm)."""
    g = latlon_grid(n, n, n, lon_bc=abi.RS_BC_OPEN, lat_bc=abi.RS_BC_OPEN, lon0=-110.0,
                    dlon=5.0, lat0=26.0, dlat=4.0, pole_centred=False)
    phie = lat_edges(g)
    lonf = -112.5 + np.arange(n + 1) * 5.0
    lonc = -112.5 + (np.arange(n) + 0.5) * 5.0
    kk = np.arange(n)
    latmid = 0.5 * (phie[:-1] + phie[1:])
    mx = (0.7 * np.cos(D2R * lonf)[None, None, :] * (1 + 0.3 * np.sin(D2R * latmid))[None, :, None]
          * (1 + 0.05 * kk)[:, None, None])
    my = (0.5 * np.sin(2 * D2R * lonc)[None, None, :] * np.cos(D2R * phie)[None, :, None]
          * (1 + 0.05 * kk)[:, None, None])
    s = np.arange(n + 1) / n
    mz = np.broadcast_to((0.05 * (4 * s * (1 - s) * (1 - 2 * s)))[:, None, None], (n + 1, n, n)).copy()
    Ap = [0.0, 4.804826, 659.3752, 1313.48, 1961.311, 2609.201, 3257.081, 3898.201]
    Bp = [1.0, 0.984952, 0.963406, 0.941865, 0.920387, 0.898908, 0.877429, 0.856018]
    dA = np.array([Ap[k] - Ap[k + 1] for k in range(7)])
    dB = np.array([Bp[k] - Bp[k + 1] for k in range(7)])
    dp = dA + dB * 101325.0
    if n != 7:  # other sizes: the 7 layer thicknesses interpolated onto n layers
        dp = np.interp(np.linspace(0.0, 6.0, n), np.arange(7.0), dp)
    return g, np.ascontiguousarray(mx), np.ascontiguousarray(my), mz, dp
