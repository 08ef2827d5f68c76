"""Shots split over ranks on the GPU: one rank reproduces the survey's
gradient bit for bit through the host stack and finalisation; two shards run
one after the other on one GPU sum to the whole survey's gradient."""
import os
import socket

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _survey(seed=21):
    from fwi_gb300 import synth
    from oracle import oracle as O
    spec, vp = synth.small_survey(seed=seed, nshots=4, nxm=200, windows=[(0, 120), (30, 170), (60, 140), (0, 200)])
    vp_obs = np.asfortranarray(vp * np.float32(1.03))
    _, _, _, obs = O.gradient_batch(spec, vp_obs, step=2, nthreads=4, want_synth=True)
    for sh, o in zip(spec.shots, obs):
        sh.obs = np.asfortranarray(o)
    spec.numtasks = 2
    return spec, synth.lam_from_vp(vp)


def test_one_rank_is_the_survey_and_two_shards_sum_to_it():
    import torch.distributed as dist
    import fwi_gb300 as F
    from fwi_gb300 import multi
    spec, lam = _survey()
    sv = F.Survey(spec)
    sv.set_lambda(lam)
    g0 = np.zeros((spec.ny, spec.nx_model), np.float32, order="F")
    m0, _ = sv.run(1, g0)
    stack0 = sv.stack()
    sv.close()
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    dist.init_process_group("gloo", rank=0, world_size=1, init_method=f"tcp://127.0.0.1:{port}")
    try:
        local, (a, b) = multi.shard_spec(spec, 0, 1)
        assert (a, b) == (0, len(spec.shots))
        s1 = F.Survey(local)
        s1.set_lambda(lam)
        g1 = np.zeros_like(g0)
        m1, _ = multi.misfit_gradient(s1, spec, 1, g1)
        np.testing.assert_array_equal(g1, g0)
        assert m1 == m0
        m2, _ = multi.misfit_gradient(s1, spec, 2)
        assert m2 == pytest.approx(m0, rel=1e-12)
        s1.close()
    finally:
        dist.destroy_process_group()
    # two shards of the same survey, run one after the other
    total = np.zeros((spec.ny, spec.nx_model), np.float64, order="F")
    mis = 0.0
    for r in range(2):
        part, _ = multi.shard_spec(spec, r, 2)
        sp = F.Survey(part)
        sp.set_lambda(lam)
        m, _ = sp.run(1, None)
        total += sp.stack()
        mis += m
        sp.close()
    np.testing.assert_allclose(total, stack0, rtol=1e-12, atol=1e-12 * np.abs(stack0).max())
    assert mis == pytest.approx(m0, rel=1e-12)
    g2 = multi.finalize(np.zeros_like(g0), total, spec.numtasks, spec.water_rows)
    np.testing.assert_allclose(g2, g0, rtol=1e-6, atol=1e-6 * np.abs(g0).max())
