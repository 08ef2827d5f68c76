"""CPU checks of the pre-processing restatement (oracle/prep.py)."""
import numpy as np

from oracle import prep as P


def test_akima_reproduces_lines_and_nodes():
    t = np.arange(400, dtype=np.float32) * np.float32(0.004)
    y = np.stack([np.float32(1.5) + np.float32(2.0) * t, np.cos(7 * t)], 1).astype(np.float32)
    out = P.akima(y, 0.004, 0.004, 400)          # same axis: the nodes themselves
    assert np.array_equal(out, y)
    u = np.arange(1100, dtype=np.float32) * np.float32(0.0013)
    lin = P.akima(y, 0.004, 0.0013, 1100)[:, 0]
    assert np.abs(lin - (1.5 + 2.0 * u.astype(np.float64))).max() < 2e-5


def test_butterworth_lowpass_gain():
    dt, n = 0.002, 3000
    t = np.arange(n) * dt
    slow = P.time_filter(np.sin(2 * np.pi * 1.0 * t)[:, None], dt, 1, 0.0, 10.0)[:, 0]
    fast = P.time_filter(np.sin(2 * np.pi * 60.0 * t)[:, None], dt, 1, 0.0, 10.0)[:, 0]
    assert abs(np.abs(slow[1500:]).max() - 1.0) < 1e-3     # passband gain 1
    assert np.abs(fast[1500:]).max() < 1e-4                 # 60 Hz through a 6th-order 10 Hz low-pass
    H = P.butterworth_response(6, 1, 10.0, 0.0, 500.0, 1000)
    f10 = int(round(10.0 / (500.0 / 1000)))
    assert abs(abs(H[f10]) - 2 ** -0.5) < 1e-3              # -3 dB at the cut-off
    assert not np.any(P.time_filter(np.zeros((50, 2)), dt, 1, 0.0, 10.0))


def test_akima_oracle_vs_reference_golden():
    """oracle/prep.akima against INTRPL executed from akima433.f90."""
    import os
    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "akima.npz"))
    for k in range(int(z["ncases"])):
        d, out = z[f"c{k}_data"], z[f"c{k}_out"]
        got = P.akima(d, z[f"c{k}_dt_in"], z[f"c{k}_dt_out"], out.shape[0])
        assert np.array_equal(got, out), k
