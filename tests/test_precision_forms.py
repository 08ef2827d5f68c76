"""Stored-snapshot precision forms on the CPU: the gradient error of 16-bit
snapshots against an FP64 run of the same solver, for two scalings -- one
max-abs scale per snapshot, and the power-of-two scale per 128-column row
segment that the device kernels use -- in FP16 and in BF16 (the oracle's
quantize_snapshots; the solver itself is the reference's FP32 arithmetic).

By default a reduced MCS case runs in seconds.  FWI_FORMS_FULL=1 runs shots
0 and 32 of the precision-form workload at full size (400 x 2000 cells,
6000 steps, snapshots every 4 steps; minutes on the host cores) and prints
the errors as one JSON line."""
import json
import os

import numpy as np
import pytest

from fwi_gb300 import synth
from fwi_gb300.synth import lam_from_vp
from oracle import oracle as O

FULL = os.environ.get("FWI_FORMS_FULL") == "1"


def _case():
    if FULL:
        spec, vp_true, vp0 = synth.mcs_batch(seed=2, nshots=64, nt=6000, store_snap=4)
        spec.shots = [spec.shots[0], spec.shots[32]]
        return spec, vp_true, vp0
    vp_true, wrows = synth.model_layered(80, 320, 12.5, seed=4, nlayers=4, water_depth=200.0)
    spec = synth.mcs_survey(vp_true, 12.5, 0.001, 800, [3200.0, 3600.0], 120, 12.5, near=150.0, freq=10.0,
                            acc=3, dpml=20, store_snap=4, seed=4, water_rows=wrows, shift_max=0.0)
    return spec, vp_true, synth.smooth(vp_true, 4)


def _grad(spec, kern):
    G = np.zeros((spec.ny, spec.nx_model))
    for sh, k in zip(spec.shots, kern):
        G[:, sh.x0:sh.x0 + sh.nx] += sh.grad_weight * np.asarray(k, np.float64)
    return G


@pytest.fixture(scope="module")
def forms():
    synth.use_host_functions(O.mcs_geometry, O.ricker, O.time_rules)
    try:
        spec, vp_true, vp0 = _case()
    finally:
        synth.use_host_functions()
    nth = max(1, min(len(spec.shots), os.cpu_count() or 1))
    vt = np.sqrt(lam_from_vp(vp_true) / np.float32(1000.0)).astype(np.float32)
    vs = np.sqrt(lam_from_vp(vp0) / np.float32(1000.0)).astype(np.float32)
    # observed data: the FP32 solver's traces on the true model
    _, _, _, syn = O.gradient_batch(spec, vt, step=2, nthreads=nth, want_synth=True)
    for sh, s in zip(spec.shots, syn):
        sh.obs = np.asarray(s, np.float32)
    k64, _, _, _ = O.gradient_batch(spec, vs.astype(np.float64), step=1, fp64=True, nthreads=nth)
    G64 = _grad(spec, k64)
    keep = np.ones_like(G64)
    keep[np.arange(spec.ny)[:, None] < np.asarray(spec.water_rows)[None, :]] = 0.0
    out, grads = {}, {}
    for name, code in O.SNAP_FORMS.items():
        k, _, _, _ = O.gradient_batch(spec, vs, step=1, nthreads=nth, snap_form=code)
        G = _grad(spec, k)
        grads[name] = G
        out[name] = {"grad_rel_l2": float(np.linalg.norm(G - G64) / np.linalg.norm(G64)),
                     "grad_rel_l2_water_masked": float(np.linalg.norm((G - G64) * keep)
                                                       / np.linalg.norm(G64 * keep))}
    if FULL or os.environ.get("FWI_FORMS_PRINT") == "1":
        name = ("precision-form MCS survey, shots 0 and 32, 400x2000, nt=6000, store_snap=4" if FULL else
                "reduced MCS case, 2 shots, 80x320, nt=800, store_snap=4")
        print(json.dumps({"workload": name, "errors_vs_fp64_oracle": out}), flush=True)
    return spec, vs, out, grads


def test_fp32_form_is_the_plain_solver(forms):
    spec, vs, _, grads = forms
    k, _, _, _ = O.gradient_batch(spec, vs, step=1, nthreads=len(spec.shots))
    np.testing.assert_array_equal(_grad(spec, k), grads["f32"])


def test_sixteen_bit_forms_error(forms):
    _, _, out, _ = forms
    e = {k: v["grad_rel_l2"] for k, v in out.items()}
    for k, v in e.items():
        assert np.isfinite(v), k
    # every 16-bit form adds error to the FP32 solver's own; BF16 (8-bit
    # significand) adds more than FP16 (11-bit) under either scaling
    for k in ("f16_snapshot_scale", "bf16_snapshot_scale", "f16_segment_pow2", "bf16_segment_pow2"):
        assert e[k] >= e["f32"], k
    assert e["bf16_segment_pow2"] > 2 * e["f16_segment_pow2"]
    assert e["bf16_snapshot_scale"] > 2 * e["f16_snapshot_scale"]
    # FP16's significand, not its scale, sets the error: the two scalings
    # agree within a factor 1.5 in either direction
    for p in ("f16", "bf16"):
        r = e[p + "_segment_pow2"] / e[p + "_snapshot_scale"]
        assert 1 / 1.5 < r < 1.5, (p, r)


def _bf16(x):
    """Round float32 to the nearest bfloat16 (ties to even), as float32."""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def _f16(x):
    return np.asarray(x, np.float32).astype(np.float16).astype(np.float32)


def _forms_numpy(A, form):
    """The snapshot forms restated in numpy: one max-abs scale per snapshot
    (forms 1, 2) or a power-of-two scale per 128-column segment of a row
    (forms 3, 4); FP16 (1, 3) or BF16 (2, 4)."""
    rnd = _f16 if form in (1, 3) else _bf16
    out = A.copy()
    f32 = np.float32
    for k in range(A.shape[2]):
        S = out[:, :, k]
        if form in (1, 2):
            m = f32(np.abs(S).max())
            if m == 0:
                continue
            up, down = f32(16384.0) / m, m / f32(16384.0)
            out[:, :, k] = rnd(S * up) * down
        else:
            for j in range(S.shape[0]):
                for i0 in range(0, S.shape[1], 128):
                    seg = S[j, i0:i0 + 128]
                    m = f32(np.abs(seg).max())
                    ex = int(np.frexp(m)[1]) if m > 0 else 0
                    sh = 14 - ex
                    S[j, i0:i0 + 128] = np.ldexp(rnd(np.ldexp(seg, sh)), -sh)
    return out


def test_quantize_snapshots_matches_numpy():
    """The oracle's snapshot forms (quantize_snapshots) against their numpy
    restatement, bit for bit, on values spanning nine decades, zeros, an
    all-zero snapshot and a ragged last segment."""
    rng = np.random.default_rng(3)
    ny, nx, ns = 7, 300, 4
    A = (rng.standard_normal((ny, nx, ns)) * 10.0 ** rng.uniform(-6, 3, size=(ny, nx, ns))).astype(np.float32)
    A[:, :5, 1] = 0.0
    A[:, :, 3] = 0.0
    A = np.asfortranarray(A)
    for form in (1, 2, 3, 4):
        got = O.quantize_snapshots(np.asfortranarray(A.copy()), form)
        np.testing.assert_array_equal(got, _forms_numpy(A, form), err_msg=f"form {form}")
        assert not np.array_equal(got, A)  # the form rounds
    np.testing.assert_array_equal(O.quantize_snapshots(np.asfortranarray(A.copy()), 0), A)
