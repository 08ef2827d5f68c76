"""Source estimation (fwi_gb300/source.py): the device Green's functions with
the reference's dPML = 50 CPML are bit-identical to the oracle's, and the
Wiener estimate recovers the band-limited wavelet that made the data."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu
F32 = np.float32


def _case():
    import fwi_gb300 as F
    from fwi_gb300.synth import ricker_shifted
    # 500 m of water: the estimate uses the direct arrivals, which the mute
    # keeps up to half a period before the water-bottom reflection
    ny, nx, d, dt, nt = 80, 160, F32(10.0), F32(0.001), 1200
    z = np.arange(ny)[:, None] * np.ones((1, nx))
    vp = np.asfortranarray(np.where(z < 50, 1500.0, 2000.0 + 800.0 * (z - 50) / (ny - 50)).astype(F32))
    nxs, nys = 40, 2
    nxr = np.arange(50, 151, 2, dtype=np.int32)
    nyr = np.full(len(nxr), 2, np.int32)
    w = ricker_shifted(12.0, float(dt), nt, 0.03)
    obs = np.zeros((nt, len(nxr)), np.float32, order="F")
    F.set_solver_options(3, 20)
    F.solver_acoustic_SS(0, 0, 1, len(nxr), [nxs], [nys], nxr, nyr, w.reshape(nt, 1), None, d, dt, ny, nx, vp,
                         nt + 1, 0, nt, None, None, obs)
    return vp, d, dt, nt, nxs, nys, nxr, nyr, w, obs


def test_green_functions_dpml50_bit_exact():
    from fwi_gb300.source import green_functions
    vp, d, dt, nt, nxs, nys, nxr, nyr, w, obs = _case()
    g = green_functions(vp, d, dt, nt, nxs, nys, nxr, nyr)
    s0 = np.zeros((nt, 1), np.float32, order="F")
    s0[0, 0] = F32(1.0) / dt
    ny, nx = vp.shape
    ref = O.solver_acoustic_ss(0, [nxs], [nys], nxr, nyr, s0, None, d, dt, vp, nt + 1, 0, nt,
                               np.zeros((ny, nx), np.float32, order="F"), np.zeros((ny, nx), np.float32, order="F"),
                               acc=3, dpml=50)
    assert np.array_equal(g, ref)


def test_wiener_estimate_recovers_wavelet():
    from fwi_gb300.source import source_estimation
    vp, d, dt, nt, nxs, nys, nxr, nyr, w, obs = _case()
    f1, f2 = 0.0, 30.0
    sst = source_estimation(f1, f2, vp, d, dt, nt, nxs, nys, nxr, nyr, obs)
    assert sst.shape == (nt,) and np.all(np.isfinite(sst))
    # the estimate is the wavelet's spectrum on the spectral indices
    # 1..1+floor(f2/df), df = 1/(nt dt), of the 2 nt padded transform (one-sided,
    # real part taken): project the true wavelet on the same indices
    n_pad = 2 * nt
    df = F32(1.0) / (F32(nt) * dt)
    b1 = 1 + int(np.floor(F32(f2) / df))
    W = np.fft.fft(w.astype(np.float64), n=n_pad)
    Wb = np.zeros(n_pad, np.complex128)
    Wb[:b1] = W[:b1]
    ref = np.real(np.fft.ifft(Wb))[:nt]
    c = float(np.dot(sst, ref) / (np.linalg.norm(sst) * np.linalg.norm(ref)))
    assert c > 0.95, c
    assert abs(int(np.argmax(np.abs(sst))) - int(np.argmax(np.abs(ref)))) <= 3
