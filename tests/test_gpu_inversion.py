"""A small frequency-continuation inversion (two low-pass bands, two NLCG
iterations each) through the device path -- filter and resampling on the
device, fwi_survey_set_time per trial model, batched gradient -- against
the same driver on the CPU oracle backend (oracle/prep.py filter and
resampling, oracle gradient): same line-search decisions, misfits and steps
within 1e-3, and the misfit and the model error fall."""
import dataclasses

import numpy as np
import pytest

from oracle import oracle as O
from oracle import prep as OP

pytestmark = pytest.mark.gpu
F32 = np.float32


def _problem():
    import fwi_gb300 as F
    from fwi_gb300.survey import ShotSpec, SurveySpec
    ny, nx, d = 40, 140, F32(10.0)
    z = np.arange(ny)[:, None] * np.ones((1, nx))
    x = np.ones((ny, 1)) * np.arange(nx)[None, :]
    vp0 = np.where(z < 6, 1500.0, 1800.0 + 800.0 * (z - 6) / (ny - 6))
    lens = -250.0 * np.exp(-(((z - 24) / 5.0) ** 2 + ((x - 70) / 12.0) ** 2))
    vp_true = np.where(z < 6, 1500.0, vp0 + lens)
    lam_t = np.asfortranarray((F32(1000.0) * vp_true.astype(F32) ** 2).astype(F32))
    lam0 = np.asfortranarray((F32(1000.0) * vp0.astype(F32) ** 2).astype(F32))
    shots = []
    for sx in (30, 70, 110):
        nxr = np.arange(4, nx - 3, 3, dtype=np.int32)
        shots.append(ShotSpec(0, nx, np.array([sx], np.int32), np.array([2], np.int32), nxr,
                              np.full(len(nxr), 2, np.int32), None))
    tfin = F32(0.9)
    dt, nt, _ = F.time_rules(lam_t, d, tfin, 10)
    w = F.Ricker_mcs(10.0, dt, nt)
    for sh in shots:
        sh.src = w.reshape(nt, 1)
    spec = SurveySpec(ny, nx, float(d), float(dt), nt, shots, water_rows=np.full(nx, 6, np.int32))
    sv = F.Survey(spec)
    sv.set_lambda(lam_t)
    sv.run(2)
    obs = np.concatenate([sv.synthetic(i) for i in range(len(shots))], axis=1)
    sv.close()
    return spec, lam_t, lam0, vp_true, obs, w, float(dt)


class OracleGradient:
    """calculate_misfit_gradient over all shots with the CPU oracle."""

    def __init__(self, spec, raw, store_snap=10, typef=1):
        self.spec, self.raw, self.store_snap, self.typef = spec, raw, store_snap, typef
        self.obs_band, self.src_band = raw.obs, raw.src[:, None]

    def set_band(self, f1, f2):
        self.obs_band = OP.time_filter(self.raw.obs, self.raw.dt_data, self.typef, f1, f2).astype(F32)
        self.src_band = OP.time_filter(self.raw.src[:, None], self.raw.dt_data, self.typef, f1, f2).astype(F32)

    def __call__(self, lam, step, grad=None):
        import fwi_gb300 as F
        dt, nt, _ = F.time_rules(lam, self.spec.d, self.raw.tfin, self.store_snap)
        obs = OP.akima(self.obs_band, self.raw.dt_data, dt, nt)
        src = OP.akima(self.src_band, self.raw.dt_data, dt, nt)
        shots, o = [], 0
        for sh in self.spec.shots:
            n = len(sh.nxRec)
            shots.append(dataclasses.replace(sh, src=src, obs=np.asfortranarray(obs[:, o:o + n])))
            o += n
        sv = dataclasses.replace(self.spec, dt=float(dt), nt=nt, shots=shots)
        vp = np.sqrt(lam / F32(1000.0)).astype(F32)
        kern, _, m64, _ = O.gradient_batch(sv, vp, step=step, nthreads=3)
        if step == 1:
            G = np.zeros(lam.shape)
            for sh, k in zip(self.spec.shots, kern):
                G[:, sh.x0:sh.x0 + sh.nx] += k
            G[:6, :] = 0.0
            grad += G.astype(F32)
        return float(m64.sum()), grad


def _rel(a, b):
    return abs(a - b) / max(abs(b), 1e-30)


def test_inversion_two_bands_vs_oracle_backend():
    from fwi_gb300.inversion import DeviceGradient, RawData, invert
    spec, lam_t, lam0, vp_true, obs, w, dt = _problem()
    raw = RawData(obs, w, dt)
    bands = [(0.0, 6.0), (0.0, 10.0)]
    dev = DeviceGradient(spec, raw)
    try:
        lam_g, log_g = invert(lam0, dev, bands, 2, vp_true=vp_true)
    finally:
        dev.close()
    def beta64(g, o):  # Beta_calculous with FP64 dot products, on the host
        g64, o64 = g.astype(np.float64), o.astype(np.float64)
        return float(F32(np.sum(g64 * (g64 - o64)) / np.sum(o64 * o64)))

    from oracle.nlcg import HostModelOps
    lam_o, log_o = invert(lam0, OracleGradient(spec, raw), bands, 2, vp_true=vp_true, beta_fn=beta64,
                          ops=HostModelOps)
    for lg, lo in zip(log_g, log_o):
        print(f"iter {lg.iter} band {lg.band}: misfit {lg.misfit:.6e} / {lo.misfit:.6e}, step {lg.step:.4e} / "
              f"{lo.step:.4e}, trials {len(lg.trials)} / {len(lo.trials)}, model error {lg.model_error:.5f}")
    assert [l.iter for l in log_g] == [1, 2, 3, 4] == [l.iter for l in log_o]
    # The two runs make the same line-search decisions.  Values agree to 1e-3:
    # the observed traces are filtered with an FP32 FFT on the device and a
    # float64 FFT here, and the misfit of max-normalised traces magnifies
    # those differences by the inverse of the residual's relative size.
    for lg, lo in zip(log_g, log_o):
        assert len(lg.trials) == len(lo.trials)
        assert _rel(lg.misfit, lo.misfit) <= 1e-3
        assert _rel(lg.step, lo.step) <= 1e-3
        for (n1, m1), (n2, m2) in zip(lg.trials, lo.trials):
            assert _rel(n1, n2) <= 1e-3 and _rel(m1, m2) <= 1e-3
    for band in bands:   # misfit falls within a band
        ms = [l.misfit for l in log_g if l.band == band]
        assert ms[1] < ms[0]
    err0 = float(np.linalg.norm(np.sqrt(lam0 / 1000.0) - vp_true) / np.linalg.norm(vp_true))
    assert log_g[-1].model_error < err0
    assert np.abs(lam_g.astype(np.float64) / lam_o - 1.0).max() <= 1e-3


def test_nlcg_model_ops_on_device():
    """fwi_first_step and fwi_model_update (FWI.f90:175, :227, :315): exp and
    log rounded once from FP64 give the bits of the float64-rounded
    restatement, and stay within one unit in the last place of numpy's
    float32 functions; host and device pointers give the same result."""
    import fwi_gb300 as F
    from oracle import nlcg as ON
    rng = np.random.default_rng(17)
    ny, nx = 300, 700
    var = np.asfortranarray((1000.0 * rng.uniform(1450.0, 5200.0, (ny, nx)) ** 2).astype(F32))
    search = np.asfortranarray((rng.standard_normal((ny, nx)) * 10.0 ** rng.uniform(-12, -6, (ny, nx))).astype(F32))
    search[:5, :5] = 0.0
    nut = F.first_step(search, var)
    assert nut == ON.first_step_rounded(search, var)
    assert abs(float(nut) / float(ON.HostModelOps.first_step(search, var)) - 1.0) <= 4 * 2.0 ** -23
    ones = np.ones_like(var)
    for step in (nut, F32(0.0), F32(nut * F32(37.5))):
        lam = F.model_update(search, var, step)
        np.testing.assert_array_equal(lam, ON.update_rounded(search, var, step))
        # the exp factor alone (var = 1) is within a few units of numpy's float32
        # exp, which is not correctly rounded itself (up to two units here)
        e_dev = F.model_update(search, ones, step)
        e_np = ON.HostModelOps.update(search, ones, step)
        ulp = np.abs(e_dev.view(np.int32).astype(np.int64) - e_np.view(np.int32).astype(np.int64))
        assert ulp.max() <= 4
    np.testing.assert_array_equal(F.model_update(search[:5, :5], var[:5, :5], nut), var[:5, :5])
    # device pointers (the call detects them)
    import torch
    s_d = torch.from_numpy(np.ascontiguousarray(search.reshape(-1, order="F"))).cuda()
    v_d = torch.from_numpy(np.ascontiguousarray(var.reshape(-1, order="F"))).cuda()
    out = torch.empty_like(v_d)
    import ctypes as C
    st = C.c_float(nut)
    F.load().fwi_model_update(C.c_void_p(s_d.data_ptr()), C.c_void_p(v_d.data_ptr()), C.byref(st),
                              C.byref(C.c_int(nx)), C.byref(C.c_int(ny)), C.c_void_p(out.data_ptr()))
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy().reshape((ny, nx), order="F"), F.model_update(search, var, nut))
