"""Batched survey (all shots of calculate_misfit_gradient in one graph) on
the GPU against the oracle run shot by shot."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def stacked_oracle(spec, vp, fp64=False, step=1):
    kern, mr, m64, synth = O.gradient_batch(spec, vp, step=step, fp64=fp64, nthreads=8, want_synth=True)
    G = np.zeros((spec.ny, spec.nx_model), np.float64)
    for sh, k in zip(spec.shots, kern):
        G[:, sh.x0:sh.x0 + sh.nx] += sh.grad_weight * k.astype(np.float64)
    return G, mr, m64, synth


def make(seed, **kw):
    from fwi_gb300 import synth
    spec, vp = synth.small_survey(seed=seed, **kw)
    # observed data: the same survey on a perturbed model (oracle, FP32)
    vp_obs = np.asfortranarray(vp * np.float32(1.03))
    _, _, _, obs = O.gradient_batch(spec, vp_obs, step=2, nthreads=8, want_synth=True)
    for sh, o in zip(spec.shots, obs):
        sh.obs = np.asfortranarray(o)
    return spec, vp


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("kw", [dict(), dict(acc=4, dpml=20, ny=33, nxm=170, nshots=4),
                                dict(nshots=3, nxm=300, windows=[(0, 150), (70, 230), (140, 160)]),
                                dict(store_snap=4, nt=160)])
def test_survey_gradient_vs_oracle(kw):
    import fwi_gb300 as F
    from fwi_gb300.synth import lam_from_vp
    spec, vp = make(5, **kw)
    lam = lam_from_vp(vp)
    vp_ref = np.sqrt(lam / np.float32(1000.0))  # Vpmodel = sqrt(lambda/1000.)
    G, mr, m64, synth = stacked_oracle(spec, vp_ref)
    sv = F.Survey(spec)
    sv.set_lambda(lam)
    grad = np.zeros((spec.ny, spec.nx_model), np.float32, order="F")
    mis, _ = sv.run(1, grad)
    for i in range(len(spec.shots)):
        np.testing.assert_array_equal(sv.synthetic(i), synth[i])        # traces bit-exact
    assert abs(mis - m64.sum()) <= 1e-12 * abs(m64.sum())
    assert abs(mis - mr.sum()) <= 1e-4 * abs(mis)                       # vs FP32 sequential sums
    Gm = G.copy()
    for i, k in enumerate(spec.water_rows):
        Gm[:k, i] = 0.0
    assert rel(grad.astype(np.float64), Gm) <= 1e-6
    # a second run reuses the captured graph and gives identical results
    grad2 = np.zeros_like(grad)
    mis2, _ = sv.run(1, grad2)
    assert mis2 == mis and np.array_equal(grad2, grad)


@pytest.mark.parametrize("kw,rc,form", [
    (dict(), False, 0), (dict(acc=4, dpml=20, ny=33, nxm=170, nshots=4), False, 0),
    (dict(nshots=3, nxm=300, windows=[(0, 150), (70, 230), (140, 160)]), False, 0),
    (dict(store_snap=3, nt=151), False, 0), (dict(acc=4, store_snap=7, nt=97, ny=12), False, 0),
    (dict(store_snap=3, nt=151), False, 2), (dict(store_snap=4, nt=120), False, 1),
    (dict(nt=301, store_snap=5), True, 0), (dict(acc=4, nt=160, store_snap=4), True, 2)])
def test_two_step_passes_bit_identical(kw, rc, form):
    """Pairs of steps advanced by either two-step interior kernel (register
    queues, or the p_{n+1} rows in shared memory), in one band or in bands of
    13 rows, with the edge tiles in the same bands or in bands of their own,
    with the single-step lists beside them, give the same bits as
    single steps: traces, misfit and gradient, forward and adjoint, with
    snapshot stores and imaging inside passes (FP32 snapshots; 16-bit ones are
    stored by single steps), and with checkpointed recomputation.  Single
    steps as one fused launch each give the same bits too."""
    import fwi_gb300 as F
    from fwi_gb300.synth import lam_from_vp
    spec, vp = make(9, **kw)
    lam = lam_from_vp(vp)
    res = []
    for two, kern, rows, edge in ((False, 0, 0, 0), (True, 1, 64, 10 ** 6), (True, 2, 64, 10 ** 6), (True, 2, 13, 10 ** 6),
                                  (True, 2, 64, 8), (True, 1, 16, 7), ("fused", 0, 0, 0)):
        sv = F.Survey(spec, snap_form=form, two_step=two is True, recompute=rc, tile_kernel=kern, tile_rows=rows,
                      tile_edge_rows=edge, fused_step=two == "fused")
        if two is True:
            assert sv.tiles()[:2] == (kern, rows) and sv.edge_tiles()[0] == edge
        else:
            assert sv.stepping()[0] == ("single-fused" if two == "fused" else "single")
        sv.set_lambda(lam)
        g = np.zeros((spec.ny, spec.nx_model), np.float32, order="F")
        m, _ = sv.run(1, g)
        res.append((m, g, [sv.synthetic(i).copy() for i in range(len(spec.shots))]))
        sv.close()
    m1, g1, s1 = res[0]
    for m2, g2, s2 in res[1:]:
        for a, b in zip(s2, s1):
            np.testing.assert_array_equal(a, b)
        assert m2 == m1
        np.testing.assert_array_equal(g2, g1)
    assert np.abs(g1).max() > 0


def test_tuner_picks_a_measured_tile(monkeypatch):
    """The tuner times both two-step kernels at each tile height on the first
    wave and keeps the fastest, then the bottom edge band, then single steps
    against the chosen two-step passes; every choice is the fastest
    measured one."""
    monkeypatch.setenv("FWI_TUNE_CACHE", "")  # no cross-process cache file
    import fwi_gb300 as F
    from fwi_gb300.synth import lam_from_vp
    spec, vp = make(11, ny=70, nxm=400, nshots=4)
    sv = F.Survey(spec)
    stepping, st = sv.stepping()
    kern, rows, meas = sv.tiles()
    assert meas  # nothing cached: every candidate was timed
    best = min(meas, key=meas.get)
    assert set(st) == {"two-step", "single", "single-fused"} and min(st.values()) > 0
    fastest_single = min(st["single"], st["single-fused"])
    if stepping != "two-step":
        assert kern == 0 and rows == 0 and fastest_single < 0.98 * st["two-step"]
        assert st[stepping] == fastest_single
    else:
        assert fastest_single >= 0.98 * st["two-step"]
        assert kern in (1, 2) and rows in (16, 32, 48, 64, 96) and (kern, rows) == best
        edge, emeas = sv.edge_tiles()
        assert edge in (0, 8, 16, 32)
        assert edge in emeas and emeas[edge] == min(emeas.values())
    sv.set_lambda(lam_from_vp(vp))
    g = np.zeros((spec.ny, spec.nx_model), np.float32, order="F")
    sv.run(1, g)
    assert np.isfinite(g).all()
    sv.close()


def test_wave_split_is_bit_identical_and_fp32_form():
    import fwi_gb300 as F
    from fwi_gb300.synth import lam_from_vp
    spec, vp = make(6, nshots=5)
    lam = lam_from_vp(vp)
    outs = []
    for wave in (0, 1, 2):
        sv = F.Survey(spec, wave_shots=wave)
        sv.set_lambda(lam)
        g = np.zeros((spec.ny, spec.nx_model), np.float32, order="F")
        m, _ = sv.run(1, g)
        outs.append((m, g))
    for m, g in outs[1:]:
        assert m == outs[0][0] and np.array_equal(g, outs[0][1])
    # FP32 per-shot accumulation (the reference's) agrees to FP32 rounding
    sv = F.Survey(spec, grad_form=F.GRAD_F32)
    sv.set_lambda(lam)
    g32 = np.zeros_like(outs[0][1])
    sv.run(1, g32)
    assert rel(g32.astype(np.float64), outs[0][1].astype(np.float64)) <= 1e-5


def test_step2_numtasks_and_accumulation():
    import fwi_gb300 as F
    from fwi_gb300.synth import lam_from_vp
    spec, vp = make(7, nshots=2)
    lam = lam_from_vp(vp)
    sv1 = F.Survey(spec)                # numtasks = 1
    sv1.set_lambda(lam)
    g1 = np.zeros((spec.ny, spec.nx_model), np.float32, order="F")
    m0, _ = sv1.run(1, g1)
    spec.numtasks = 2
    sv = F.Survey(spec)
    sv.set_lambda(lam)
    g0 = np.full((spec.ny, spec.nx_model), 0.25, np.float32, order="F")
    g = g0.copy(order="F")
    m1, _ = sv.run(1, g, misfit=1.5)    # Misfit and Grad accumulate
    m2, _ = sv.run(2, None)             # forward + misfit only
    assert m1 - 1.5 == pytest.approx(m0, rel=1e-12) and m2 == pytest.approx(m0, rel=1e-12)
    # Grad = Grad + stack/numtasks, then the water rows are zeroed
    expect = (g0.astype(np.float64) + g1.astype(np.float64) / 2).astype(np.float32)
    for i, k in enumerate(spec.water_rows):
        expect[:k, i] = 0
    assert rel(g.astype(np.float64), expect.astype(np.float64)) <= 1e-6


@pytest.mark.parametrize("form,tol", [(1, 2e-2), (2, 2e-3)])
def test_16bit_snapshots_error_vs_fp64_oracle(form, tol):
    import fwi_gb300 as F
    from fwi_gb300.synth import lam_from_vp
    spec, vp = make(8, nshots=2, nt=300)
    lam = lam_from_vp(vp)
    vp_ref = np.sqrt(lam / np.float32(1000.0))
    G64, _, m64, _ = stacked_oracle(spec, vp_ref.astype(np.float64), fp64=True)
    for i, k in enumerate(spec.water_rows):
        G64[:k, i] = 0
    res = {}
    for f in (0, form):
        sv = F.Survey(spec, snap_form=f)
        sv.set_lambda(lam)
        g = np.zeros((spec.ny, spec.nx_model), np.float32, order="F")
        m, _ = sv.run(1, g)
        res[f] = (m, g.astype(np.float64))
    e32 = rel(res[0][1], G64)
    e16 = rel(res[form][1], G64)
    assert e32 <= 1e-4
    assert e16 <= tol
    assert res[form][0] == res[0][0]  # the misfit does not depend on snapshots


def test_batch_entry_point_matches_survey():
    import fwi_gb300 as F
    from fwi_gb300.synth import lam_from_vp
    spec, vp = make(9, nshots=3)
    lam = lam_from_vp(vp)
    g = np.zeros((spec.ny, spec.nx_model), np.float32, order="F")
    m = F.calculate_misfit_gradient(spec, lam, 1, np.float32(0.0), g)
    sv = F.Survey(spec)
    sv.set_lambda(lam)
    g2 = np.zeros_like(g)
    m2, _ = sv.run(1, g2)
    assert np.array_equal(g, g2) and m == np.float32(m2)
    # second call with the same geometry reuses the cached plan
    g3 = np.zeros_like(g)
    m3 = F.calculate_misfit_gradient(spec, lam, 1, np.float32(0.0), g3)
    assert np.array_equal(g3, g) and m3 == m


@pytest.mark.parametrize("kw,form", [(dict(nt=300), 0), (dict(nt=200, store_snap=4), 1), (dict(nt=600, nshots=4), 2)])
def test_checkpointed_recompute_is_bit_identical(kw, form):
    import fwi_gb300 as F
    from fwi_gb300.synth import lam_from_vp
    spec, vp = make(11, **kw)
    lam = lam_from_vp(vp)
    res = []
    for rc in (False, True):
        sv = F.Survey(spec, snap_form=form, recompute=rc)
        c, j = sv.recompute_plan()
        assert (j > 1) == rc
        sv.set_lambda(lam)
        g = np.zeros((spec.ny, spec.nx_model), np.float32, order="F")
        m, _ = sv.run(1, g)
        res.append((m, g, [sv.synthetic(i) for i in range(len(spec.shots))]))
        m2, _ = sv.run(2)  # forward-only runs keep no snapshots
        assert m2 == m
    assert res[0][0] == res[1][0]
    np.testing.assert_array_equal(res[0][1], res[1][1])
    for a, b in zip(res[0][2], res[1][2]):
        np.testing.assert_array_equal(a, b)


def test_small_budget_selects_recompute():
    import fwi_gb300 as F
    from fwi_gb300.synth import lam_from_vp
    spec, vp = make(12, nshots=2, nt=3000)
    lam = lam_from_vp(vp)
    full = F.Survey(spec)
    full.set_lambda(lam)
    g0 = np.zeros((spec.ny, spec.nx_model), np.float32, order="F")
    m0, _ = full.run(1, g0)
    full.close()
    # resident data ~ traces; give room for far less than one shot's snapshots
    resident = 4 * spec.nt * sum(len(s.nxRec) for s in spec.shots) * 3 + 8 * spec.ny * spec.nx_model * 2
    sv = F.Survey(spec, hbm_budget=resident + 6_000_000)
    assert sv.recompute_plan()[1] > 1
    sv.set_lambda(lam)
    g = np.zeros_like(g0)
    m, _ = sv.run(1, g)
    assert m == m0 and np.array_equal(g, g0)


def test_batch_entry_line_search_trials_one_plan():
    """Three line-search trials through the drop-in batch call, each with the
    dt and nt that FWI.f90:225-227 derives from its trial model
    (calculate_misfit_gradient.f90:198-203), build one plan: the later trials
    move it to their time axis, with results bit-identical to a survey moved
    by fwi_survey_set_time."""
    import copy

    import fwi_gb300 as F
    from fwi_gb300 import _native as N
    from fwi_gb300.synth import lam_from_vp
    spec, vp = make(12, nshots=2, nt=200)
    lam = lam_from_vp(vp)
    rng = np.random.default_rng(3)
    tfin = 0.4
    trials = []
    for scale in (1.0, 1.3, 0.75):  # trial models: lambda scaled, dt from the CFL rule (nt 200, 230, 170)
        lam_k = np.asfortranarray(lam * np.float32(scale))
        dt, nt, _ = F.time_rules(lam_k, spec.d, tfin, spec.store_snap)
        sp = copy.deepcopy(spec)
        sp.dt, sp.nt = float(dt), int(nt)
        for sh in sp.shots:
            sh.src = np.asfortranarray(rng.standard_normal((nt, len(sh.nxSou))).astype(np.float32))
            sh.obs = np.asfortranarray(rng.standard_normal((nt, len(sh.nxRec))).astype(np.float32))
        trials.append((lam_k, sp))
    assert len({sp.nt for _, sp in trials}) == 3
    p0 = N.load().fwi_batch_plans()
    sv = F.Survey(trials[0][1])
    for k, (lam_k, sp) in enumerate(trials):
        g = np.zeros((sp.ny, sp.nx_model), np.float32, order="F")
        m = F.calculate_misfit_gradient(sp, lam_k, 1, np.float32(0.0), g)
        if k:
            src = np.concatenate([np.asarray(sh.src).reshape(-1, order="F") for sh in sp.shots])
            sv.set_time(sp.dt, sp.nt, src, sp.obs_packed())
        else:
            sv.set_observed(sp.obs_packed())
        sv.set_lambda(lam_k)
        g2 = np.zeros_like(g)
        m2, _ = sv.run(1, g2)
        np.testing.assert_array_equal(g, g2)
        assert m == np.float32(m2) and np.abs(g).max() > 0
    assert N.load().fwi_batch_plans() - p0 == 1
    sv.close()
    F.load().fwi_batch_release()


def test_launch_form_chosen_by_timing_bit_identical():
    """The first run of a time axis launches directly, the second replays a
    captured graph; both are timed and the slower form is dropped (a graph
    that looks faster is checked against one more direct run).  Every run
    gives the same bits, whichever form it took."""
    import fwi_gb300 as F
    from fwi_gb300.synth import lam_from_vp
    spec, vp = make(9, nshots=3)
    sv = F.Survey(spec)
    sv.set_lambda(lam_from_vp(vp))
    assert sv.launch_form(1)[0] == "undecided"
    outs = []
    for k in range(4):
        g = np.zeros((spec.ny, spec.nx_model), np.float32, order="F")
        m, _ = sv.run(1, g)
        outs.append((m, g))
        form, t_direct, t_graph = sv.launch_form(1)
        if k == 0:
            assert form == "undecided" and t_direct > 0 and t_graph == 0
        else:
            assert form in ("graph", "direct") and t_direct > 0 and t_graph > 0
            assert (form == "direct") == (t_graph > 1.002 * t_direct)
    for m, g in outs[1:]:
        assert m == outs[0][0] and np.array_equal(g, outs[0][1])
    # the forward-only runs decide on their own
    assert sv.launch_form(2)[0] == "undecided"
    plain = F.Survey(spec, graph=False)
    plain.set_lambda(lam_from_vp(vp))
    g = np.zeros_like(outs[0][1])
    m, _ = plain.run(1, g)
    assert plain.launch_form(1)[0] == "direct"
    assert m == outs[0][0] and np.array_equal(g, outs[0][1])


@pytest.mark.parametrize("graph", [False, True])
def test_batch_entry_packed_data_and_new_observations(graph):
    """The batch call with all shots' sources and observed traces as slices of
    one array each (the copies merged, the traces uploaded on a copy stream
    beside the forward pass) gives the bits of separate per-shot arrays, and
    observed traces changed between calls reach that call's misfit -- also
    when every call replays the captured graph (the graph waits for the
    upload inside, before the misfit)."""
    import fwi_gb300 as F
    from fwi_gb300.synth import lam_from_vp
    spec, vp = make(13, nshots=4)
    lam = lam_from_vp(vp)
    nt = spec.nt
    flags = F.SURVEY_GRAPH if graph else 0
    F.batch_release()

    def batch():
        g = np.zeros((spec.ny, spec.nx_model), np.float32, order="F")
        m = F.calculate_misfit_gradient(spec, lam, 1, np.float32(0.0), g, flags=flags)
        return m, g

    ref = batch()  # separate arrays per shot
    nrec = [len(sh.nxRec) for sh in spec.shots]
    nsou = [np.asarray(sh.src).reshape(nt, -1, order="F").shape[1] for sh in spec.shots]
    obs_all = np.asfortranarray(np.concatenate([np.asarray(sh.obs, np.float32) for sh in spec.shots], axis=1))
    src_all = np.asfortranarray(np.concatenate(
        [np.asarray(sh.src, np.float32).reshape(nt, -1, order="F") for sh in spec.shots], axis=1))
    ro = np.concatenate([[0], np.cumsum(nrec)])
    so = np.concatenate([[0], np.cumsum(nsou)])
    for i, sh in enumerate(spec.shots):
        sh.obs = obs_all[:, ro[i]:ro[i + 1]]
        sh.src = src_all[:, so[i]:so[i + 1]]
        assert sh.obs.flags.f_contiguous and sh.src.flags.f_contiguous
    packed = batch()
    assert packed[0] == ref[0] and np.array_equal(packed[1], ref[1])
    # new observations in place (a time-shifted mix: the misfit normalises
    # every trace by its maximum, so a plain scale would not change it): the
    # next call's misfit and gradient follow them
    for r in range(2):
        obs_all += np.float32(0.3) * np.roll(obs_all, 7 + r, axis=0)
        m_half, g_half = batch()
        sv = F.Survey(spec)
        sv.set_lambda(lam)
        g2 = np.zeros_like(g_half)
        m2, _ = sv.run(1, g2)
        sv.close()
        assert m_half == np.float32(m2) and np.array_equal(g_half, g2)
        assert m_half != ref[0]
    if graph:
        assert F.batch_survey().launch_form(1)[0] == "graph"


def test_tuning_cache_file_across_processes(tmp_path):
    """The tuner's choices persist in $FWI_TUNE_CACHE: a second process with
    the same grid reads them from the file (no candidate timed) and makes the
    same choices; a line of the older five-value form is still read."""
    import json
    import os
    import subprocess
    import sys
    cache = tmp_path / "tuning.txt"
    code = r'''
import json, sys
sys.path.insert(0, {root!r})
sys.path.insert(0, {tests!r})
import fwi_gb300 as F
from test_gpu_survey import make
spec, vp = make(17, ny=70, nxm=400, nshots=3)
sv = F.Survey(spec)
k, r, meas = sv.tiles()
form, st = sv.stepping()
print(json.dumps({{"tiles": [k, r], "band": sv.tuning()[1], "form": form, "measured": len(meas) + len(st)}}))
'''.format(root=os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
           tests=os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, FWI_TUNE_CACHE=str(cache))

    def run():
        out = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
        assert out.returncode == 0, out.stderr[-2000:]
        return json.loads([l for l in out.stdout.splitlines() if l.startswith("{")][-1])

    first = run()
    assert first["measured"] > 0
    lines = cache.read_text().split("\n")
    assert any(len(l.split()) == 6 for l in lines)
    second = run()
    assert second["measured"] == 0  # every choice came from the file
    assert {k: second[k] for k in ("tiles", "band", "form")} == {k: first[k] for k in ("tiles", "band", "form")}
    # the older five-value form: two-step passes, as the file says
    key, band, var, rows, eb, _ = [l for l in lines if len(l.split()) == 6][-1].split()
    cache.write_text(f"{key} {band} {var} {rows} {eb}\n")
    third = run()
    assert third["measured"] == 0 and third["form"] == "two-step" and third["tiles"] == [int(var) + 1, int(rows)]
