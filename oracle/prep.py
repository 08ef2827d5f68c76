"""CPU restatement of the reference's trace pre-processing.

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker of the device
filter and resampler; the product package never imports it.

* time_filter  -- time_filter.f90:1-40 with filters_function1D / butterworth
  (filters.f90:39-186): the trace sits at the end of a 24x zero-padded
  buffer, the buffer is transformed (forward transform normalised by 1/n, as
  FFTPACK5's cfft1f), multiplied by the Butterworth response H(f) and
  transformed back; the output is the real part of the last nt samples.
  FFT in float64 (numpy), H from the reference's product formula with the
  frequency advanced by an FP32 accumulation of fe/ts (filters.f90:94-98).
* was_geometry -- the WAS geometry of get_was_data.f90 (:112-115, :155-159,
  :201-205, :223-231, :584-613), with INTRPL for the bathymetry model.
* akima        -- interpolation_akima.f90:1-31 with INTRPL (akima433.f90:6-170,
  ACM Algorithm 433, Comm. ACM 15(10):914): per output abscissa, the interval
  by bisection, slopes of the neighbouring intervals (end slopes extrapolated),
  Akima's weighted end-point slopes and the local cubic; outside [x(1), x(L)]
  the end interval's cubic is shifted outward.  float32 arithmetic in the
  Fortran evaluation order (numpy float32 operations round like the
  reference's REAL operations), vectorised over the output samples.
"""
from __future__ import annotations

import numpy as np

F32 = np.float32


def butterworth_response(n: int, typef: int, fc: float, f1: float, fe: float, ts: int) -> np.ndarray:
    """H(j*fe/ts), j = 0..ts/2 (complex128); filters.f90:88-181, parity 0."""
    fs, f2 = F32(40.0), F32(fc)
    f1 = F32(f1)
    f0 = np.sqrt(F32(f1 * f2), dtype=F32)
    Q = F32(f0 / F32(f2 - f1)) if f2 != f1 else F32(np.inf)
    df = F32(F32(fe) / F32(ts))
    nf = ts // 2 + 1
    # FP32 accumulation of the frequency, as the reference's f = f + fe/ts
    f = np.empty(nf, np.float32)
    acc = F32(0.0)
    for j in range(nf):
        f[j] = acc
        acc = F32(acc + df)
    f = f.astype(np.float64)
    B = np.ones(nf, np.complex128)
    pi = 3.14159265
    with np.errstate(divide="ignore", invalid="ignore"):
        for k in range(1, n // 2 + 1):
            c = np.cos((2 * k + n - 1) * pi / (2.0 * n))
            if typef == 1:
                s = 1j * f / float(fc)
            elif typef == 2:
                s = float(fs) / (1j * f)
            else:
                s = float(Q) * ((1j * f) / float(f0) + float(f0) / (1j * f))
            B = B * (s * s - 2.0 * s * c + 1.0)
        H = 1.0 / B
    H[0] = 1.0 if typef == 1 else 0.0
    return H


def time_filter(data: np.ndarray, dt: float, typef: int, f1: float, fc: float, order: int = 6) -> np.ndarray:
    """data (nt, num) -> filtered copy (float64)."""
    data = np.asarray(data, dtype=np.float64)
    nt, num = data.shape
    ts = 24 * nt
    fe = F32(1.0) / F32(dt)
    H = butterworth_response(order, typef, fc, f1, fe, ts)
    # full Hermitian response (filters.f90:177-179); the real part of the
    # inverse only sees its Hermitian part, so the Nyquist bin enters as Re(H)
    Hn = H.copy()
    Hn[-1] = Hn[-1].real
    out = np.zeros_like(data)
    for i in range(num):
        if not np.any(data[:, i] != 0):  # is_not_cero: all-zero traces are left as they are
            continue
        buf = np.zeros(ts)
        buf[ts - nt:] = data[:, i]
        Z = np.fft.rfft(buf) / ts
        y = np.fft.irfft(Z * Hn, n=ts) * ts
        out[:, i] = y[ts - nt:]
    return out


def akima(data: np.ndarray, dt_in: float, dt_out: float, nt_out: int) -> np.ndarray:
    """data (L, ntr) float32 sampled at (i-1)*dt_in -> (nt_out, ntr) at (i-1)*dt_out."""
    y = np.asarray(data, dtype=np.float32)
    L = y.shape[0]
    dt_in, dt_out = F32(dt_in), F32(dt_out)
    X = (np.arange(L, dtype=np.float32) * dt_in).astype(np.float32)       # x(i) = real(i-1)*dt
    U = (np.arange(nt_out, dtype=np.float32) * dt_out).astype(np.float32)
    return akima_x(X, y, U)


def akima_x(X: np.ndarray, data: np.ndarray, U: np.ndarray) -> np.ndarray:
    """INTRPL: data (L, ntr) at the increasing abscissae X (L) -> (len(U), ntr)
    at the abscissae U."""
    y = np.asarray(data, dtype=np.float32)
    if y.ndim == 1:
        return akima_x(X, y[:, None], U)[:, 0]
    X = np.asarray(X, np.float32)
    U = np.asarray(U, np.float32)
    L, ntr = y.shape
    nt_out = U.size
    # interval index I (1-based): 1 before x(1), L+1 at or after x(L), else the
    # smallest i >= 2 with x(i) > u (the bisection's result)
    if L == 2:
        I = np.full(nt_out, 2, np.int64)
    else:
        I = np.searchsorted(X, U, side="right") + 1
        I = np.where(U >= X[L - 1], L + 1, I)
        I = np.where(U < X[0], 1, I)
    J = np.clip(I, 2, L)

    def xs(j):  # x(j), 1-based, float32
        return X[j - 1]

    def ys(j):  # y(j, :) for each output sample -> (nt_out, ntr)
        return y[j - 1, :]

    def col(v):
        return v[:, None]

    x3, y3 = col(xs(J - 1)), ys(J - 1)
    x4, y4 = col(xs(J)), ys(J)
    a3 = (x4 - x3).astype(np.float32)
    m3 = ((y4 - y3) / a3).astype(np.float32)
    zero = np.zeros_like(m3)
    a2 = np.zeros_like(a3)
    a4 = np.zeros_like(a3)
    if L == 2:
        m2, m4 = m3.copy(), m3.copy()
        m1 = m2 + m2 - m3
        m5 = m4 + m4 - m3
    else:
        jm2 = np.maximum(J - 2, 1)
        x2, y2 = col(xs(jm2)), ys(jm2)
        has2 = col(J != 2)
        a2 = np.where(has2, x3 - x2, a2).astype(np.float32)
        m2 = np.where(has2, (y3 - y2) / np.where(has2, a2, F32(1.0)), zero).astype(np.float32)
        jp1 = np.minimum(J + 1, L)
        x5, y5 = col(xs(jp1)), ys(jp1)
        last = col(J == L)
        a4 = np.where(last, a4, x5 - x4).astype(np.float32)
        m4n = ((y5 - y4) / np.where(last, F32(1.0), a4)).astype(np.float32)
        m4 = np.where(last, m3 + m3 - m2, m4n).astype(np.float32)
        m2 = np.where(col(J == 2), m3 + m3 - m4, m2).astype(np.float32)
        jm3 = np.maximum(J - 3, 1)
        a1 = (x2 - col(xs(jm3))).astype(np.float32)
        m1n = ((y2 - ys(jm3)) / np.where(col(J <= 3), F32(1.0), a1)).astype(np.float32)
        m1 = np.where(col(J <= 3), m2 + m2 - m3, m1n).astype(np.float32)
        jp2 = np.minimum(J + 2, L)
        a5 = (col(xs(jp2)) - x5).astype(np.float32)
        m5n = ((ys(jp2) - y5) / np.where(col(J >= L - 1), F32(1.0), a5)).astype(np.float32)
        m5 = np.where(col(J >= L - 1), m4 + m4 - m3, m5n).astype(np.float32)
    first, past = col(I == 1), col(I == L + 1)
    with np.errstate(divide="ignore", invalid="ignore"):
        # slope at the interval's left end
        w2, w3 = np.abs(m4 - m3), np.abs(m2 - m1)
        sw = (w2 + w3).astype(np.float32)
        z = sw == 0
        w2, w3, sw = np.where(z, F32(0.5), w2), np.where(z, F32(0.5), w3), np.where(z, F32(1.0), sw)
        t3 = ((w2 * m2 + w3 * m3) / sw).astype(np.float32)
        # slope at the right end
        w3b, w4 = np.abs(m5 - m4), np.abs(m3 - m2)
        sw = (w3b + w4).astype(np.float32)
        z = sw == 0
        w3b, w4, sw = np.where(z, F32(0.5), w3b), np.where(z, F32(0.5), w4), np.where(z, F32(1.0), sw)
        t4 = ((w3b * m3 + w4 * m4) / sw).astype(np.float32)
        # before x(1): shift the first interval's cubic outward
        sa = (a3 + a4).astype(np.float32)
        t3f = (F32(0.5) * (m1 + m2 - a4 * (a3 - a4) * (m3 - m4) / (sa * sa))).astype(np.float32)
        # at or after x(L): shift the last interval's cubic outward
        sa2 = (a2 + a3).astype(np.float32)
        t4p = (F32(0.5) * (m4 + m5 - a2 * (a2 - a3) * (m2 - m3) / (sa2 * sa2))).astype(np.float32)
    T3 = np.where(first, t3f, np.where(past, t4, t3))
    T4 = np.where(first, t3, np.where(past, t4p, t4))
    X3 = np.where(first, x3 - a4, np.where(past, x4, x3))
    Y3 = np.where(first, y3 - m2 * a4, np.where(past, y4, y3))
    A3 = np.where(first, a4, np.where(past, a2, a3))
    M3 = np.where(first, m2, np.where(past, m4, m3))
    with np.errstate(divide="ignore", invalid="ignore"):
        q2 = ((F32(2.0) * (M3 - T3) + M3 - T4) / A3).astype(np.float32)
        q3 = ((-M3 - M3 + T3 + T4) / (A3 * A3)).astype(np.float32)
    d = (col(U) - X3).astype(np.float32)
    return (Y3 + d * (T3 + d * (q2 + d * q3))).astype(np.float32)


def was_geometry(xobs, zobs, xshot, bat, shot_depth, dmodel, nxmodel, relocate=True):
    """WAS geometry (OBS as sources, shots as receivers; added_space_model = 0):
    shot columns 1+ceiling(|xs|/d) (get_was_data.f90:155-156); the bathymetry
    model by INTRPL through (0, shot positions, (nxmodel-1)*d) and the shots'
    water depths, ends repeated, at (i-1)*d (:584-613); OBS columns
    1+ceiling(|x|/d) and rows 1+ceiling(z/d) with z the model bathymetry at
    the OBS column when relocated (:112-115, :201-205); the receiver row
    1+ceiling(shot_depth/d) (:223-231).  FP32 as the reference's REALs."""
    d = F32(dmodel)
    grid = lambda v: (1 + np.ceil(np.asarray(v, np.float32) / d)).astype(np.int32)  # noqa: E731
    pos_shot = (F32(0.0) + np.abs(np.asarray(xshot, np.float32))).astype(np.float32)
    pos_bat = np.abs(np.asarray(bat, np.float32)).astype(np.float32)
    L = pos_shot.size + 2
    xm = np.zeros(L, np.float32)
    yb = np.zeros(L, np.float32)
    xm[1:-1], yb[1:-1] = pos_shot, pos_bat
    xm[-1] = F32(F32(nxmodel - 1) * d)
    yb[0], yb[-1] = yb[1], yb[-2]
    U = (np.arange(nxmodel, dtype=np.float32) * d).astype(np.float32)
    model = akima_x(xm, yb, U)
    gx = grid(F32(0.0) + np.abs(np.asarray(xobs, np.float32)))
    z = model[gx - 1] if relocate else np.abs(np.asarray(zobs, np.float32))
    return dict(nxSou=gx, nySou=grid(z), nxRec=grid(pos_shot), nyRec=int(grid([shot_depth])[0]), bat_model=model,
                bat_model_grid=grid(model))
