"""Precision form (snapshots every 4 steps stored in BF16 or FP16 with a
power-of-two scale per 128 values, FP64 gradient stack) against an FP64
end-to-end oracle run of the same solver, on the model and geometry of the
batched MCS workload (12.5 m grid, 10 Hz, 480 channels): two shots, each
propagated on a 540-column window that holds its streamer, 1.2 s records so
that the water-bottom and first layer reflections are in the data.  Prints
the errors it measures (run with -s to see them).
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_precision_form_vs_fp64_oracle():
    import fwi_gb300 as F
    from fwi_gb300 import synth
    from fwi_gb300.synth import lam_from_vp
    spec, vp_true, vp0 = synth.mcs_batch(nshots=2, nt=1200, store_snap=4)
    for i, sh in enumerate(spec.shots):  # windows holding each streamer
        x0 = 20 * i
        sh.nxSou = sh.nxSou - x0
        sh.nxRec = sh.nxRec - x0
        sh.x0, sh.nx = x0, 540
    lam_t, lam0 = lam_from_vp(vp_true), lam_from_vp(vp0)
    sv = F.Survey(spec)
    sv.set_lambda(lam_t)
    sv.run(2)
    for i, sh in enumerate(spec.shots):
        sh.obs = sv.synthetic(i)
    sv.close()
    vp_ref = np.sqrt(lam0 / np.float32(1000.0))
    kern, _, m64, _ = O.gradient_batch(spec, vp_ref.astype(np.float64), step=1, fp64=True, nthreads=2)
    G = np.zeros((spec.ny, spec.nx_model))
    for sh, k in zip(spec.shots, kern):
        G[:, sh.x0:sh.x0 + sh.nx] += k
    for i, kk in enumerate(spec.water_rows):
        G[:kk, i] = 0.0
    mis_ref = float(m64.sum())
    out = {}
    for name, form in (("fp32", F.SNAP_F32), ("bf16", F.SNAP_BF16), ("fp16", F.SNAP_F16)):
        s = F.Survey(spec, snap_form=form)
        s.set_lambda(lam0)
        g = np.zeros((spec.ny, spec.nx_model), np.float32, order="F")
        m, _ = s.run(1, g)
        s.close()
        out[name] = (_rel(g.astype(np.float64), G), abs(m - mis_ref) / mis_ref)
    for name, (eg, em) in out.items():
        print(f"precision form {name:5s}: gradient rel L2 vs FP64 oracle {eg:.3e}, misfit rel {em:.3e}")
    # measured on GB300: fp32 2.5e-5, fp16 6.4e-5, bf16 4.7e-4 (gradient);
    # the misfit (1.7e-3 for every form: snapshots do not enter it) is the
    # FP32 forward against the FP64 one, amplified by the normalised residual
    # being a few % of the traces
    assert out["fp32"][0] <= 1e-4 and out["fp16"][0] <= 1e-4 and out["bf16"][0] <= 2e-3
    assert all(em <= 5e-3 for _, em in out.values())
