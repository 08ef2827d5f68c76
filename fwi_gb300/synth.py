"""Seeded synthetic models and acquisition geometries of the benchmark workloads.

The reference ships no data (its sample datasets are not published), so the
workloads are synthetic with the shapes, sizes and value ranges of each
workload; receiver and source grid indices are computed with the reference's
own FP32 rules (fwi_mcs_geometry).  Observed data are synthesised from the
true model by the same solver.
"""
from __future__ import annotations

import numpy as np

from .survey import ShotSpec, SurveySpec


def _F(a):
    return np.asfortranarray(np.asarray(a, dtype=np.float32))


# The FP32 index rules, wavelet and time rules the generators use: the
# library's (fwi_mcs_geometry, fwi_ricker, fwi_time_rules) unless a caller
# supplies host functions with the same signatures and results -- a CPU
# baseline that must not load the library does.
_HOST = {}


def use_host_functions(mcs_geometry=None, ricker=None, time_rules=None, was_geometry=None):
    """Generate workloads with these functions instead of the library's
    (None: the library's)."""
    _HOST.clear()
    for k, f in (("mcs_geometry", mcs_geometry), ("ricker", ricker), ("time_rules", time_rules),
                 ("was_geometry", was_geometry)):
        if f is not None:
            _HOST[k] = f


def _fn(name):
    if name in _HOST:
        return _HOST[name]
    from . import api
    return {"mcs_geometry": api.mcs_geometry, "ricker": api.Ricker_mcs, "time_rules": api.time_rules,
            "was_geometry": api.was_geometry}[name]


def ricker_shifted(freq, dt, nt, shift):
    """Ricker_mcs wavelet (get_mcs_data.f90:346-362) delayed by `shift` s."""
    w = _fn("ricker")(freq, dt, nt)
    if shift:
        t = np.arange(nt) * dt
        w = np.interp(t - shift, t, w, left=0.0, right=0.0).astype(np.float32)
    return w


def model_single_shot(seed=1, anomaly=True):
    """200 x 400 at 25 m: 500 m of water at 1500 m/s over a linear gradient
    1800 -> 4500 m/s, plus a +200 m/s Gaussian anomaly (sigma 300 m) at
    (x=5 km, z=2.5 km) with a seeded position jitter (+-100 m)."""
    rng = np.random.default_rng(seed)
    ny, nx, d = 200, 400, 25.0
    z = (np.arange(ny) + 0.5) * d
    x = (np.arange(nx) + 0.5) * d
    vp = np.empty((ny, nx), np.float64)
    water = z < 500.0
    below = ~water
    zb = z[below] - 500.0
    grad = 1800.0 + (4500.0 - 1800.0) * zb / (ny * d - 500.0)
    vp[water, :] = 1500.0
    vp[below, :] = grad[:, None]
    if anomaly:
        jx, jz = rng.uniform(-100.0, 100.0, size=2)
        X, Z = np.meshgrid(x, z)
        vp += 200.0 * np.exp(-((X - 5000.0 - jx) ** 2 + (Z - 2500.0 - jz) ** 2) / (2 * 300.0 ** 2)) * below[:, None]
    return _F(vp), int(round(500.0 / d))


def model_layered(ny, nx, d, seed, nlayers=8, water_depth=None, vmin=1800.0, vmax=5000.0, lateral=0.10,
                  lenses=()):
    """Water at 1500 m/s over `nlayers` layers of random thickness 200-600 m
    with monotone random velocities in [vmin, vmax] and a +-lateral
    sinusoidal lateral perturbation; optional Gaussian low-velocity lenses
    (x, z, sigma, dv)."""
    rng = np.random.default_rng(seed)
    wd = water_depth if water_depth is not None else 500.0
    z = (np.arange(ny) + 0.5) * d
    x = (np.arange(nx) + 0.5) * d
    thick = rng.uniform(200.0, 600.0, size=nlayers)
    tops = wd + np.concatenate([[0.0], np.cumsum(thick)[:-1]])
    vels = np.sort(rng.uniform(vmin, vmax, size=nlayers))
    phase = rng.uniform(0, 2 * np.pi, size=nlayers)
    wavelength = rng.uniform(3000.0, 9000.0, size=nlayers)
    vp = np.full((ny, nx), 1500.0)
    for k in range(nlayers):
        mask = z >= tops[k]
        pert = 1.0 + lateral * np.sin(2 * np.pi * x / wavelength[k] + phase[k])
        vp[mask, :] = vels[k] * pert[None, :]
    X, Z = np.meshgrid(x, z)
    for (lx, lz, sig, dv) in lenses:
        vp += dv * np.exp(-((X - lx) ** 2 + (Z - lz) ** 2) / (2 * sig ** 2)) * (Z >= wd)
    return _F(vp), int(np.ceil(wd / d))


def lam_from_vp(vp):
    """lambda = rho*Vp**2 with rho = 1000 (auxiliar.f90:205-209), in FP32."""
    v = np.asarray(vp, np.float32)
    return _F(np.float32(1000.0) * (v * v))


def mcs_survey(vp, d, dt, nt, xs_list, nrec, drec, near=150.0, sdepth=10.0, rdepth=10.0, freq=10.0, acc=3,
               dpml=20, store_snap=10, seed=0, water_rows=None, windows=None, shift_max=0.0):
    """MCS survey on model vp: one Ricker source per shot (seeded time shift
    in [0, shift_max]) and a trailing streamer of nrec channels.  `windows`
    optionally gives (x0, nx) per shot; geometry indices are window
    relative."""
    mcs_geometry = _fn("mcs_geometry")
    rng = np.random.default_rng(seed)
    ny, nxm = vp.shape
    shots = []
    for i, xs in enumerate(xs_list):
        nxs, nys, nxr, nyr = mcs_geometry(xs, sdepth, rdepth, near, drec, d, nrec)
        x0, nxw = (0, nxm) if windows is None else windows[i]
        sh = float(rng.uniform(0.0, shift_max)) if shift_max else 0.0
        src = ricker_shifted(freq, dt, nt, sh).reshape(nt, 1, order="F")
        shots.append(ShotSpec(x0=x0, nx=nxw, nxSou=np.array([nxs - x0], np.int32), nySou=np.array([nys], np.int32),
                              nxRec=(nxr - x0).astype(np.int32), nyRec=nyr.astype(np.int32), src=_F(src)))
    wr = None
    if water_rows is not None:
        wr = np.full(nxm, water_rows, np.int32) if np.isscalar(water_rows) else np.asarray(water_rows, np.int32)
    return SurveySpec(ny=ny, nx_model=nxm, d=d, dt=dt, nt=nt, shots=shots, store_snap=store_snap, acc=acc,
                      dpml=dpml, water_rows=wr)


def single_shot(seed=1):
    """Plain single shot (200 x 400 cells, 8th order, 3000 steps): returns
    (spec, vp_true, vp_start).  The shot sits at a seeded x in [6000, 7000) m,
    so that its 200-channel streamer (150 m near offset, trailing towards
    x = 0) lies inside the model and over the anomaly at x = 5 km; a shot near
    x = 2.6 km would record almost nothing of the anomaly (a residual at the
    FP32 rounding level)."""
    vp_true, wrows = model_single_shot(seed, anomaly=True)
    vp0, _ = model_single_shot(seed, anomaly=False)
    rng = np.random.default_rng(seed + 100)
    spec = mcs_survey(vp_true, 25.0, 0.002, 3000, [6000.0 + 25.0 * int(rng.integers(0, 40))], 200, 12.5, near=150.0,
                      sdepth=10.0, rdepth=10.0, freq=8.0, acc=4, dpml=20, seed=seed, water_rows=wrows,
                      shift_max=0.02)
    return spec, vp_true, vp0


def mcs_batch(seed=2, nshots=64, nt=6000, store_snap=10):
    """Batched MCS survey: 400 x 2000 at 12.5 m, 64 shots
    at 250 m spacing, 480 channels at 12.5 m, 6 s at dt = 1 ms, 10 Hz.
    Returns (spec, vp_true, vp_start) where the start model is the true
    model smoothed laterally and vertically."""
    vp_true, wrows = model_layered(400, 2000, 12.5, seed)
    xs = [6250.0 + 250.0 * i for i in range(nshots)]
    spec = mcs_survey(vp_true, 12.5, 0.001, nt, xs, 480, 12.5, near=150.0, freq=10.0, acc=3, dpml=20,
                      store_snap=store_snap, seed=seed, water_rows=wrows, shift_max=0.01)
    return spec, vp_true, smooth(vp_true, 8)


def inversion_workload(seed=5, nshots=128, nt=8000, store_snap=10, window_margin=2000.0):
    """Full-inversion workload: 600 x 3000 at 12.5 m, a
    layered model with two Gaussian low-velocity lenses, 128 MCS shots of 480
    channels at 12.5 m, 8 s records at dt = 1 ms, 10 Hz Ricker.  Each shot
    propagates on its own window: from window_margin metres behind the last
    channel to window_margin metres ahead of the source.  Returns (spec,
    vp_true, vp_start) with the start model = the smoothed model without the
    lenses."""
    rng = np.random.default_rng(seed)
    ny, nx, d = 600, 3000, 12.5
    lenses = [(float(rng.uniform(9000, 16000)), float(rng.uniform(2200, 3500)), 700.0, -450.0),
              (float(rng.uniform(22000, 30000)), float(rng.uniform(3000, 4800)), 900.0, -400.0)]
    vp_true, wrows = model_layered(ny, nx, d, seed, lenses=lenses)
    vp_bg, _ = model_layered(ny, nx, d, seed)
    nrec, drec, near = 480, 12.5, 150.0
    x_first = near + nrec * drec + window_margin + 500.0
    x_last = nx * d - window_margin - 500.0
    xs = [x_first + (x_last - x_first) * i / max(nshots - 1, 1) for i in range(nshots)]
    windows = []
    for x in xs:
        lo = max(0, int((x - near - nrec * drec - window_margin) / d))
        hi = min(nx, int(np.ceil((x + window_margin) / d)))
        windows.append((lo, hi - lo))
    spec = mcs_survey(vp_true, d, 0.001, nt, xs, nrec, drec, near=near, freq=10.0, acc=3, dpml=20,
                      store_snap=store_snap, seed=seed, water_rows=wrows, windows=windows)
    return spec, vp_true, smooth(vp_bg, 8)


def smooth(vp, r):
    """Box-smoothed copy of vp (r cells each way) for starting models."""
    v = np.asarray(vp, np.float64)
    k = 2 * r + 1
    pad = np.pad(v, r, mode="edge")
    c = np.cumsum(np.cumsum(pad, 0), 1)
    c = np.pad(c, ((1, 0), (1, 0)))
    out = (c[k:, k:] - c[:-k, k:] - c[k:, :-k] + c[:-k, :-k]) / (k * k)
    return _F(out)


def small_survey(seed=0, ny=40, nxm=90, nshots=3, nt=200, acc=3, dpml=8, d=10.0, dt=1e-3, nrec=20, windows=None,
                 store_snap=10):
    """A small survey for parity tests (CPML, windows, duplicates...)."""
    rng = np.random.default_rng(seed)
    vp = 1500.0 + 1000.0 * (np.arange(ny)[:, None] / ny) + rng.uniform(-50, 50, size=(ny, nxm))
    vp = _F(vp)
    shots = []
    for i in range(nshots):
        x0, nx = (0, nxm) if windows is None else windows[i]
        nsou = 1 + (i % 2)
        nxs = rng.integers(1, nx + 1, size=nsou).astype(np.int32)
        nys = rng.integers(1, min(ny, 6) + 1, size=nsou).astype(np.int32)
        nxr = rng.integers(-dpml, nx + dpml, size=nrec).astype(np.int32)
        nyr = rng.integers(1, ny + dpml, size=nrec).astype(np.int32)
        nxr[:3] = nxr[0]
        nyr[:3] = nyr[0]  # three receivers in one cell
        src = _F(rng.standard_normal((nt, nsou)))
        shots.append(ShotSpec(x0=x0, nx=nx, nxSou=nxs, nySou=nys, nxRec=nxr, nyRec=nyr, src=src))
    spec = SurveySpec(ny=ny, nx_model=nxm, d=d, dt=dt, nt=nt, shots=shots, store_snap=store_snap, acc=acc,
                      dpml=dpml, water_rows=rng.integers(0, 4, size=nxm).astype(np.int32))
    return spec, vp


def model_crustal(seed=3, ny=600, nx=6000, d=25.0):
    """Crustal model of the uneven-size WAS batch (150 x 15 km at 25 m):
    water from the surface to a seeded seafloor near 3 km, sediments
    1.8 -> 3 km/s (2 km thick), crust 5.5 -> 7 km/s, mantle 8 km/s below a
    Moho at 12 km with seeded +-1 km topography.  Returns (vp, seafloor
    depth per column in m)."""
    rng = np.random.default_rng(seed)
    x = (np.arange(nx) + 0.5) * d
    z = (np.arange(ny) + 0.5) * d

    def smooth_noise(amp, nmodes=6):
        s = np.zeros(nx)
        for _ in range(nmodes):
            s += rng.uniform(-1, 1) * np.sin(2 * np.pi * x / rng.uniform(15e3, 80e3) + rng.uniform(0, 2 * np.pi))
        return amp * s / max(np.abs(s).max(), 1e-9)

    sea = 2800.0 + smooth_noise(200.0)
    sed_base = sea + 2000.0
    moho = 12000.0 + smooth_noise(1000.0)
    Z = z[:, None]
    vp = np.full((ny, nx), 1500.0)
    sed = (Z >= sea) & (Z < sed_base)
    vp = np.where(sed, 1800.0 + 1200.0 * (Z - sea) / 2000.0, vp)
    crust = (Z >= sed_base) & (Z < moho)
    vp = np.where(crust, 5500.0 + 1500.0 * (Z - sed_base) / np.maximum(moho - sed_base, 1.0), vp)
    vp = np.where(Z >= moho, 8000.0, vp)
    return _F(vp), sea


def was_batch(seed=3, nt=None, nshots=30, freq=5.0, tfin=20.0):
    """Uneven-size WAS batch with OBS as reciprocal
    sources: 30 OBS at 5 km on the seafloor, 1200 surface receivers at 125 m
    (10 m deep), each shot on its own window of 30-100 km (seeded).  The
    stated dt = 2.5 ms violates the CFL limit at 8 km/s and 25 m, so the
    reference's own rule dt = d/(2 vmax) (calculate_misfit_gradient.f90:198)
    is used: 1.5625 ms, nt = 12800 for 20 s.  Returns (spec, vp_true, vp_start)."""
    time_rules = _fn("time_rules")
    rng = np.random.default_rng(seed + 1)
    d = 25.0
    vp, sea = model_crustal(seed)
    ny, nxm = vp.shape
    lam = lam_from_vp(vp)
    dt, nt_full, _ = time_rules(lam, d, tfin, 10)
    nt = nt_full if nt is None else nt
    f32 = np.float32
    # the reference's WAS geometry (get_was_data.f90): shots (the receivers) at
    # 125 m with the model's water depth under each, OBS (the sources) at 5 km
    # relocated to the bathymetry model that INTRPL draws through the shots'
    # water depths
    rec_x = np.array([62.5 + 125.0 * j for j in range(1200)], np.float32)
    cols = np.minimum((rec_x / f32(d)).astype(np.int64), nxm - 1)
    xo_all = np.array([2500.0 + 5000.0 * i for i in range(nshots)], np.float32)
    geo = _fn("was_geometry")(xo_all, np.zeros(nshots, np.float32), rec_x, np.asarray(sea, np.float32)[cols], 10.0,
                              d, nxm, True)
    rec_grid = np.asarray(geo["nxRec"], np.int32)
    rec_row = int(geo["nyRec"])
    shots = []
    for i in range(nshots):
        xo = float(xo_all[i])
        xg, zg = int(geo["nxSou"][i]), int(geo["nySou"][i])
        width = rng.uniform(30e3, 100e3)
        c0 = max(0, int((xo - width / 2) / d))
        c1 = min(nxm, int((xo + width / 2) / d))
        inside = (rec_grid - 1 >= c0) & (rec_grid - 1 < c1)
        nxr = (rec_grid[inside] - c0).astype(np.int32)
        src = ricker_shifted(freq, float(dt), nt, 0.0).reshape(nt, 1, order="F")
        shots.append(ShotSpec(x0=c0, nx=c1 - c0, nxSou=np.array([xg - c0], np.int32), nySou=np.array([zg], np.int32),
                              nxRec=nxr, nyRec=np.full(nxr.size, rec_row, np.int32), src=_F(src)))
    water = (1 + np.ceil(np.asarray(sea, np.float32) / f32(d))).astype(np.int32)
    spec = SurveySpec(ny=ny, nx_model=nxm, d=d, dt=float(dt), nt=nt, shots=shots, store_snap=10, acc=3, dpml=20,
                      water_rows=water)
    return spec, vp, smooth(vp, 6)
