"""Trace pre-processing on the device against the CPU restatement
(oracle/prep.py): Akima resampling bit-exact, Butterworth filtering within
FP32 FFT rounding (relative L2 <= 2e-5 against a float64 FFT)."""
import numpy as np
import pytest

from oracle import prep as O

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("L,dt_in,nt_out,dt_out", [
    (1000, 0.004, 3100, 0.0013),    # finer step, past the last input sample (extrapolation)
    (1000, 0.001, 400, 0.0025),     # coarser step
    (2, 0.01, 7, 0.004),            # two points: straight line
    (3, 0.01, 9, 0.003),
    (4, 0.01, 11, 0.004),
    (5, 0.002, 1, 0.001),
    (600, 0.0025, 1200, 0.00125),
])
def test_akima_bit_exact(L, dt_in, nt_out, dt_out):
    import fwi_gb300 as F
    rng = np.random.default_rng(L * 7 + nt_out)
    ntr = 5
    data = np.asfortranarray(rng.standard_normal((L, ntr)).astype(np.float32))
    data[:, 1] = np.float32(0.25) * np.arange(L, dtype=np.float32)   # linear trace
    data[:, 2] = 0.0                                                 # flat trace: zero slopes (sw = 0 branch)
    if L > 6:
        data[L // 2:L // 2 + 3, 3] = 1.0                             # plateau: equal neighbouring slopes
    got = F.interpolation_akima(data, dt_in, L, ntr, dt_out, nt_out)
    ref = O.akima(data, dt_in, dt_out, nt_out)
    assert np.array_equal(got, ref), np.abs(got - ref).max()


def test_akima_device_pointers():
    import torch
    import fwi_gb300 as F
    rng = np.random.default_rng(3)
    data = np.asfortranarray(rng.standard_normal((800, 6)).astype(np.float32))
    host = F.interpolation_akima(data, 0.004, 800, 6, 0.0015, 2000)
    src = torch.from_numpy(np.ascontiguousarray(data.T)).cuda()      # column-major (800, 6) = row-major (6, 800)
    dst = torch.zeros((6, 2000), dtype=torch.float32, device="cuda")
    F.interpolation_akima(src.data_ptr(), 0.004, 800, 6, 0.0015, 2000, out=dst.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(dst.cpu().numpy().T, host)


@pytest.mark.parametrize("typef,f1,fc,order", [(1, 0.0, 10.0, 6), (1, 0.0, 3.0, 4), (3, 2.0, 12.0, 6), (2, 0.0, 10.0, 6)])
def test_time_filter_vs_oracle(typef, f1, fc, order):
    import fwi_gb300 as F
    from fwi_gb300.synth import ricker_shifted
    rng = np.random.default_rng(typef * 10 + order)
    nt, dt = 1500, 0.002
    data = np.zeros((nt, 4), np.float32, order="F")
    data[:, 0] = rng.standard_normal(nt)
    data[:, 1] = ricker_shifted(10.0, dt, nt, 0.1)
    data[:, 3] = np.sin(2 * np.pi * 5.0 * np.arange(nt) * dt)
    F.set_filter_order(order)
    try:
        got = F.time_filter(data.copy(order="F"), nt, dt, 4, typef, f1, fc)
    finally:
        F.set_filter_order(6)
    ref = O.time_filter(data, dt, typef, f1, fc, order=order)
    assert not np.any(got[:, 2])                          # an all-zero trace stays zero
    for i in (0, 1, 3):
        # relative to the output, or to 1 % of the input where the filter
        # removes (nearly) all of the trace (FP32 FFT rounding is relative to
        # the input's spectrum)
        scale = max(np.linalg.norm(ref[:, i]), 1e-2 * np.linalg.norm(data[:, i]))
        err = np.linalg.norm(got[:, i].astype(np.float64) - ref[:, i]) / scale
        assert err <= 2e-5, (i, err)


def test_time_filter_vs_reference_golden():
    """The device filter (cuFFT, FP32) against time_filter executed from the
    reference (FFTPACK5, FP32): low-, high- and band-pass at order 6, low-pass
    at order 4; the two FP32 transforms round differently, within 1e-5."""
    import os

    import fwi_gb300 as F
    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "filter.npz"))
    data = z["data"]
    nt, num = data.shape
    for k in range(int(z["ncases"])):
        F.set_filter_order(int(z[f"c{k}_order"]))
        try:
            got = F.time_filter(np.asfortranarray(data.copy()), nt, float(z["dt"]), num, int(z[f"c{k}_typef"]),
                                float(z[f"c{k}_f1"]), float(z[f"c{k}_fc"]))
        finally:
            F.set_filter_order(6)
        out = z[f"c{k}_out"]
        assert np.array_equal(got[:, 2], out[:, 2])
        assert _rel(got[:, :2], out[:, :2].astype(np.float64)) <= 1e-5, k


def test_time_filter_device_pointer_and_batches():
    import torch
    import fwi_gb300 as F
    rng = np.random.default_rng(11)
    nt, dt, ntr = 3000, 0.001, 64
    data = np.asfortranarray(rng.standard_normal((nt, ntr)).astype(np.float32))
    host = F.time_filter(data.copy(order="F"), nt, dt, ntr, 1, 0.0, 7.0)
    dev = torch.from_numpy(np.ascontiguousarray(data.T)).cuda()
    F.time_filter(dev.data_ptr(), nt, dt, ntr, 1, 0.0, 7.0)
    torch.cuda.synchronize()
    assert np.array_equal(dev.cpu().numpy().T, host)
    ref = O.time_filter(data, dt, 1, 0.0, 7.0)
    assert _rel(host, ref) <= 2e-5


def test_akima_device_vs_reference_golden():
    """The device resampler against INTRPL executed from akima433.f90."""
    import os
    import fwi_gb300 as F
    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "akima.npz"))
    for k in range(int(z["ncases"])):
        d, out = z[f"c{k}_data"], z[f"c{k}_out"]
        got = F.interpolation_akima(np.asfortranarray(d), float(z[f"c{k}_dt_in"]), d.shape[0], d.shape[1],
                                    float(z[f"c{k}_dt_out"]), out.shape[0])
        assert np.array_equal(got, out), k
