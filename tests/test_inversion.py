"""NLCG driver (fwi_gb300/inversion.py) on the CPU: polyfit against the golden
vectors executed from polyfit.f90, and the FWI.f90 iteration on an analytic
misfit (the gradient callback is a quadratic in lambda)."""
import os

import numpy as np

from fwi_gb300.inversion import fwi_band, polyfit
from oracle.nlcg import HostModelOps

HERE = os.path.dirname(os.path.abspath(__file__))


def test_polyfit_golden():
    z = np.load(os.path.join(HERE, "golden", "polyfit.npz"))
    got = np.array([polyfit(*row[:4], int(row[4])) for row in z["cases"]], np.float32)
    assert np.array_equal(got, z["endstep"])


def _beta_fp64(g, o):
    # Polak-Ribiere as Beta_calculous (Beta_calculous.f90:1-25), dot products in FP64
    g64, o64 = g.astype(np.float64), o.astype(np.float64)
    return float(np.float32(np.sum(g64 * (g64 - o64)) / np.sum(o64 * o64)))


class Quadratic:
    """misfit = 0.5*sum(w*(lam-lam_t)^2) (scaled), gradient w*(lam-lam_t)."""

    def __init__(self, lam_t, w):
        self.lam_t, self.w, self.calls = lam_t, w, []

    def __call__(self, lam, step, grad=None):
        r = (lam.astype(np.float64) - self.lam_t) * self.w
        m = 0.5 * float(np.sum(r * (lam - self.lam_t))) * 1e-18
        self.calls.append((step, m))
        if step == 1:
            grad += (r * 1e-18).astype(np.float32)
        return m, grad


def test_fwi_band_line_search_rules():
    rng = np.random.default_rng(2)
    ny, nx = 12, 20
    lam_t = (1000.0 * rng.uniform(1800, 3000, (ny, nx)) ** 2)
    lam0 = np.asfortranarray((lam_t * rng.uniform(0.8, 1.2, (ny, nx))).astype(np.float32))
    w = rng.uniform(0.5, 2.0, (ny, nx))
    q = Quadratic(lam_t, w)
    log = []
    lam, it = fwi_band(lam0, q, 0.0, 5.0, 4, iter0=3, beta_fn=_beta_fp64, log=log, ops=HostModelOps)
    assert it == 7 and [l.iter for l in log] == [3, 4, 5, 6]
    mis = [l.misfit for l in log]
    assert all(b < a for a, b in zip(mis, mis[1:]))               # misfit falls every iteration
    first = log[0]
    # first trial: 1 % of the largest relative change of lambda (FWI.f90:186-190)
    g = np.zeros((ny, nx), np.float32)
    q2 = Quadratic(lam_t, w)
    q2(lam0, 1, g)
    s = -g
    nut0 = np.float32(np.float32(np.float32(1.0) / np.float32(100.0)) / np.abs(s / np.log(lam0)).max())
    assert np.float32(first.trials[0][0]) == nut0
    # the trials double the step while the misfit falls; the last one rose
    t = first.trials
    for (n1, m1), (n2, m2) in zip(t, t[1:]):
        assert np.float32(n2) == np.float32(np.float32(n1) * np.float32(2.0))
    assert t[-1][1] > t[-2][1] or len(t) == 1
    assert 0.0 < first.step <= t[-1][0]
