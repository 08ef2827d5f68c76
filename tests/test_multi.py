"""Shots split over ranks (fwi_gb300.multi): the shard partition, the host
finalisation, and the sum-allreduce of the gradient stack and misfit over two
gloo ranks on the CPU (the reference's MPI_REDUCE + MPI_BCAST of Grad and
Misfit, calculate_misfit_gradient.f90:299-300, :339-340)."""
import itertools
import os
import socket

import numpy as np
import pytest

from fwi_gb300 import multi


def _best_max(w, world):
    """Brute force: the smallest largest-part weight over all contiguous
    partitions of w into at most `world` parts."""
    n = len(w)
    best = float("inf")
    for k in range(1, min(world, n) + 1):
        for cuts in itertools.combinations(range(1, n), k - 1):
            b = (0,) + cuts + (n,)
            best = min(best, max(sum(w[b[i]:b[i + 1]]) for i in range(k)))
    return best


def test_shard_ranges_contiguous_and_balanced():
    rng = np.random.default_rng(0)
    for _ in range(300):
        n = int(rng.integers(0, 9))
        world = int(rng.integers(1, 6))
        w = [float(x) for x in rng.integers(1, 20, size=n)]
        r = multi.shard_ranges(w, world)
        assert len(r) == world
        assert r[0][0] == 0 and r[-1][1] == n
        for (a, b), (c, d) in zip(r, r[1:]):
            assert b == c and a <= b and c <= d
        if n:
            got = max(sum(w[a:b]) for a, b in r)
            assert got <= _best_max(w, world) * (1 + 1e-9)


def test_shard_spec_and_weights():
    from fwi_gb300 import synth
    spec, _ = synth.small_survey(seed=1, nshots=5, nxm=300,
                                 windows=[(0, 100), (20, 200), (50, 250), (100, 120), (150, 150)])
    w = multi.shot_weights(spec)
    assert w[1] > w[0] and w[2] > w[1]
    parts = [multi.shard_spec(spec, r, 3) for r in range(3)]
    assert sum(len(p.shots) for p, _ in parts) == 5
    assert [s for p, _ in parts for s in p.shots] == spec.shots


def test_finalize_matches_device_arithmetic():
    rng = np.random.default_rng(3)
    ny, nx = 7, 9
    g0 = np.asfortranarray(rng.standard_normal((ny, nx)).astype(np.float32))
    G = np.asfortranarray(rng.standard_normal((ny, nx)))
    water = rng.integers(0, 4, size=nx).astype(np.int32)
    got = multi.finalize(g0.copy(order="F"), G, 3, water)
    for j in range(ny):
        for i in range(nx):
            v = np.float32(g0[j, i]) + np.float32(G[j, i] / 3.0)
            assert got[j, i] == (0.0 if j < water[i] else v)


def _stack(shots, ny, nxm, kernels):
    G = np.zeros((ny, nxm), np.float64, order="F")
    for sh, k in zip(shots, kernels):
        G[:, sh.x0:sh.x0 + sh.nx] += sh.grad_weight * k
    return G


def _rank(rank, world, port, spec, kernels, misfits, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local, (a, b) = multi.shard_spec(spec, rank, world)
        G = _stack(local.shots, spec.ny, spec.nx_model, kernels[a:b])
        total, m = multi.allreduce_stack(G, float(sum(misfits[a:b])), None)
        grad = np.zeros((spec.ny, spec.nx_model), np.float32, order="F")
        multi.finalize(grad, total, spec.numtasks, spec.water_rows)
        m2 = multi.allreduce_misfit(float(sum(misfits[a:b])))
        np.savez(os.path.join(out, f"rank{rank}.npz"), total=total, m=m, m2=m2, grad=grad, a=a, b=b)
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("world", [2, 3])
def test_gloo_ranks_sum_gradient_and_misfit(tmp_path, world):
    import torch.multiprocessing as mp
    from fwi_gb300 import synth
    spec, _ = synth.small_survey(seed=2, nshots=5, nxm=300,
                                 windows=[(0, 150), (70, 230), (140, 160), (10, 60), (0, 300)])
    spec.numtasks = 2
    rng = np.random.default_rng(5)
    kernels = [rng.standard_normal((spec.ny, sh.nx)) for sh in spec.shots]
    for i, sh in enumerate(spec.shots):
        sh.grad_weight = 1.0 + 0.25 * i
    misfits = [float(x) for x in rng.random(len(spec.shots))]
    mp.start_processes(_rank, args=(world, _free_port(), spec, kernels, misfits, str(tmp_path)), nprocs=world,
                       join=True, start_method="spawn")
    full = _stack(spec.shots, spec.ny, spec.nx_model, kernels)
    ref = multi.finalize(np.zeros((spec.ny, spec.nx_model), np.float32, order="F"), full, spec.numtasks,
                         spec.water_rows)
    res = [np.load(os.path.join(tmp_path, f"rank{r}.npz")) for r in range(world)]
    assert sorted((int(r["a"]), int(r["b"])) for r in res)[0][0] == 0
    assert sum(int(r["b"]) - int(r["a"]) for r in res) == len(spec.shots)
    for r in res:
        np.testing.assert_allclose(r["total"], full, rtol=1e-13, atol=1e-12)
        assert r["m"] == pytest.approx(sum(misfits), rel=1e-14) and r["m2"] == r["m"]
        np.testing.assert_allclose(r["grad"], ref, rtol=2e-7, atol=1e-6)
        np.testing.assert_array_equal(r["grad"], res[0]["grad"])   # every rank holds the same gradient
