"""Source wavelet estimation by Wiener deconvolution (source_estimation.f90).

The Green's functions of one shot come from the device forward solver with
the reference's wider CPML (dPML = 50, solver_forward_simple.f90:82, the same
stencil as solver_acoustic_SS); the rest is small per-band host work done as
the reference does it:

1. Gs = the shot's traces for an impulse source of amplitude 1/dt at the
   first sample (source_estimation.f90:57-61, :114-115);
2. below the water-bottom reflection (two-way time at the midpoint depth
   where Vp first exceeds 1500 m/s, minus half a period of the centre
   frequency) both Gs and the observed traces Go are muted (:96-131);
3. both are normalised by their largest magnitude (:136-137);
4. each trace is zero-padded to 2*nt and transformed (forward transform
   normalised by 1/(2 nt), as FFTPACK5's cfft1f); for the spectral indices
   if1..if2 = 1+floor(f/df), df = 1/(nt*dt) -- the reference's spacing for
   the unpadded length -- the receiver sums kk = sum |Gs|^2 and
   bb = sum conj(Gs) Go give ss = bb / (kk + 0.001 max kk) (:152-174);
5. the inverse transform's real part over the first nt samples, divided by
   2 nt, is the wavelet (:176-177).
"""
from __future__ import annotations

from typing import Optional

import numpy as np

from . import api

F32 = np.float32


def green_functions(model_vp, d, dt, nt, nxs, nys, nxr, nyr, dpml=50, acc=3, restore=(3, 20)) -> np.ndarray:
    """Traces (nt, nr) of one shot for the impulse source 1/dt at sample 1,
    computed on the device with a dPML-wide CPML (solver_forward_simple)."""
    vp = np.asfortranarray(model_vp, dtype=np.float32)
    ny, nx = vp.shape
    nr = len(nxr)
    s0 = np.zeros((nt, 1), np.float32, order="F")
    s0[0, 0] = F32(F32(1.0) / F32(dt))
    rec = np.zeros((nt, nr), np.float32, order="F")
    api.set_solver_options(acc, dpml)
    try:
        api.solver_acoustic_SS(0, 0, 1, nr, [nxs], [nys], nxr, nyr, s0, None, d, dt, ny, nx, vp, nt + 1, 0, nt,
                               None, None, rec)
    finally:
        api.set_solver_options(*restore)
    return rec


def wiener_estimate(Gs, Go, model_vp, d, dt, f1, f2, nxs, nxr) -> np.ndarray:
    """Steps 2-5 above for Green's functions Gs and observed traces Go (nt, nr)."""
    Gs = np.array(Gs, dtype=np.float32, order="F")
    Go = np.array(Go, dtype=np.float32, order="F")
    vp = np.asarray(model_vp, np.float32)
    ny, nx = vp.shape
    nt, nr = Gs.shape
    d, dt, f1, f2 = F32(d), F32(dt), F32(f1), F32(f2)
    df = F32(F32(1.0) / F32(F32(nt) * dt))
    if1 = 1 + int(np.floor(f1 / df))
    if2 = 1 + int(np.floor(f2 / df))
    fc = F32(F32(f1 + f2) / F32(2.0))
    # water-bottom depth per model column: first cell faster than 1500 m/s
    z_wb = np.full(nx, F32(F32(ny - 1) * d), np.float32)
    for i in range(nx):
        hit = np.nonzero(vp[:, i] > F32(1500.0))[0]
        if hit.size:
            z_wb[i] = F32(F32(hit[0]) * d)
    # mute below the water-bottom reflection
    for ir in range(nr):
        xmid = F32(F32(F32(0.5) * F32(int(nxr[ir]) + int(nxs))) * d)
        ixm = int(xmid / d) + 1
        zwb = z_wb[ixm - 1]
        off = F32(F32(F32(abs(int(nxr[ir]) - int(nxs))) * d) * F32(0.5))
        t_wb = F32(F32(F32(2.0) * np.sqrt(F32(off * off + zwb * zwb), dtype=np.float32)) / F32(1500.0))
        t2 = F32(t_wb - F32(F32(0.5) / fc))
        it2 = min(nt, 1 + int(t2 / dt))
        Gs[it2:, ir] = 0.0
        Go[it2:, ir] = 0.0
    Gs = Gs / np.abs(Gs).max()
    Go = Go / np.abs(Go).max()
    n_pad = 2 * nt
    Gws = np.fft.fft(Gs.astype(np.float64), n=n_pad, axis=0) / n_pad
    Gwo = np.fft.fft(Go.astype(np.float64), n=n_pad, axis=0) / n_pad
    b0, b1 = if1 - 1, if2            # 0-based half-open range of if1..if2
    kk = np.sum(np.conj(Gws[b0:b1]) * Gws[b0:b1], axis=1)
    bb = np.sum(np.conj(Gws[b0:b1]) * Gwo[b0:b1], axis=1)
    eps = 0.001 * np.max(kk.real)
    ss = np.zeros(n_pad, np.complex128)
    ss[b0:b1] = bb / (kk + eps)
    # the unnormalised inverse (cfft1b) is n_pad * numpy's ifft; /n_pad after it
    return np.real(np.fft.ifft(ss) * n_pad)[:nt].astype(np.float32) / F32(n_pad)


def source_estimation(f1, f2, model_vp, d, dt, nt, nxs, nys, nxr, nyr, obs, iteration=1,
                      dpml=50) -> np.ndarray:
    """source_estimation(iter,f1,f2,nx,ny,nt,nr,dmodel,dt,nxs,nys,nxr,nyr,model,sst)
    for the observed traces obs (nt, nr) of one shot; returns sst (nt,)."""
    if iteration != 1:
        # only the first iteration uses the impulse; the reference's later
        # calls would divide by a zero Green's function
        raise ValueError("source_estimation is defined for the first iteration of a band")
    Gs = green_functions(model_vp, d, dt, nt, nxs, nys, nxr, nyr, dpml=dpml)
    return wiener_estimate(Gs, obs, model_vp, d, dt, f1, f2, nxs, nxr)
