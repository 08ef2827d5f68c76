"""The CPU oracle against golden vectors produced by executing the
reference's own Fortran routines (tests/golden/make_golden.py): bit-exact."""
import numpy as np
import pytest

from oracle import oracle as O

SOLVER_CASES = ["solver_acc3", "solver_acc4", "solver_acc3_dpml8"]


def test_fd_coefficients(golden):
    g = golden("coeffs")
    for acc in (3, 4):
        for num in (1, 2):
            assert np.array_equal(O.fd_coef(num, acc), g[f"fd_num{num}_acc{acc}"])


@pytest.mark.parametrize("tag", ["a", "b", "c"])
def test_pml_coefficients(golden, tag):
    g = golden("coeffs")
    acc, dpml = (int(v) for v in g[f"pml_{tag}_cfg"])
    dt, d = (float(v) for v in g[f"pml_{tag}_dtd"])
    fA, fB, cA, cB = O.pml_coeffs(acc, dpml, dt, d)
    assert np.array_equal(fA, g[f"pml_{tag}_fA"]) and np.array_equal(fB, g[f"pml_{tag}_fB"])
    assert np.array_equal(cA, g[f"pml_{tag}_cornA"]) and np.array_equal(cB, g[f"pml_{tag}_cornB"])


def _run(z, iprop, kernel, fields):
    return O.solver_acoustic_ss(iprop, z["nxSou"], z["nySou"], z["nxRec"], z["nyRec"], z["S"], z["Sadj"],
                                float(z["d"]), float(z["dt"]), z["ctmp"], int(z["store_snap"]), int(z["nt_store"]),
                                int(z["nt"]), kernel, fields, acc=int(z["acc"]), dpml=int(z["dpml"]))


@pytest.mark.parametrize("case", SOLVER_CASES)
def test_solver_forward_adjoint(golden, case):
    z = golden(case)
    ny, nx, nts = int(z["ny"]), int(z["nx"]), int(z["nt_store"])
    F = np.zeros((ny, nx * (nts + 1)), np.float32, order="F")
    K = np.asfortranarray(z["kernel_in"].copy())
    rec = _run(z, 1, K, F)
    assert np.array_equal(rec, z["rec_fwd"])
    assert np.array_equal(F, z["fields_fwd"])
    assert np.array_equal(K, z["kernel_in"])          # forward leaves kernel alone
    assert np.abs(rec).max() > 0
    K = np.asfortranarray(z["kernel_in"].copy())
    rec2 = _run(z, 2, K, F)
    assert np.array_equal(K, z["kernel_adj"])
    assert np.array_equal(rec2, z["rec_adj"])         # adjoint zeroes Rec_point
    assert not np.array_equal(K, z["kernel_in"])


@pytest.mark.parametrize("tag", ["a", "b"])
def test_misfit_and_beta(golden, tag):
    g = golden("misfit_beta")
    m, m64, adj = O.misfit_function(g[f"{tag}_synth"], g[f"{tag}_trace"], float(g[f"{tag}_dt"]))
    assert m == g[f"{tag}_misfit"]
    assert np.array_equal(adj, g[f"{tag}_adj"])
    assert abs(m64 - float(g[f"{tag}_misfit"])) <= 1e-5 * abs(m64)
    b, n64, d64 = O.beta_calculous(g[f"beta_{tag}_g"], g[f"beta_{tag}_o"])
    assert b == g[f"beta_{tag}"]
    assert abs(n64 / d64 - float(b)) <= 1e-5 * abs(n64 / d64)


def test_ricker_geometry_time_rules(golden):
    g = golden("geometry")
    for t in "abc":
        f0, dtm, ntm = g[f"ricker_{t}_par"]
        assert np.array_equal(O.ricker(float(f0), float(dtm), int(ntm)), g[f"ricker_{t}"])
    for t in "abcd":
        xs, sd, rd, near, drec, dm = (float(v) for v in g[f"geom_{t}_par"])
        a, b, c, d = O.mcs_geometry(xs, sd, rd, near, drec, dm, int(g[f"geom_{t}_nrec"]))
        assert a == g[f"geom_{t}_nxSou"] and b == g[f"geom_{t}_nySou"]
        assert np.array_equal(c, g[f"geom_{t}_nxRec"]) and np.array_equal(d, g[f"geom_{t}_nyRec"])
        dm, tf = (float(v) for v in g[f"time_{t}_par"])
        dt, nt, nts = O.time_rules(g[f"time_{t}_lambda"], dm, tf)
        assert dt == g[f"time_{t}_dt"] and nt == g[f"time_{t}_nt"] and nts == g[f"time_{t}_ntstore"]


def test_filter_oracle_vs_reference_golden(golden):
    """oracle/prep.time_filter (float64 FFT) against time_filter ->
    filters_function1D/butterworth -> FFTPACK5 executed from the reference in
    FP32 (the FFTPACK5 rounding is the difference): low-, high- and
    band-pass at order 6 and a low-pass at order 4; the all-zero trace is left
    untouched."""
    from oracle import prep as P
    z = golden("filter")
    data = z["data"]
    for k in range(int(z["ncases"])):
        out = z[f"c{k}_out"]
        got = P.time_filter(data, float(z["dt"]), int(z[f"c{k}_typef"]), float(z[f"c{k}_f1"]), float(z[f"c{k}_fc"]),
                            order=int(z[f"c{k}_order"]))
        assert np.array_equal(out[:, 2], data[:, 2]) and not np.any(got[:, 2])
        e = np.linalg.norm(got[:, :2] - out[:, :2]) / np.linalg.norm(out[:, :2].astype(np.float64))
        assert e <= 1e-6, (k, e)


def test_was_geometry_oracle_vs_reference_golden(golden):
    """oracle/prep.was_geometry against the statements of get_was_data.f90
    executed from the reference: bit-exact indices and bathymetry model."""
    from oracle import prep as P
    z = golden("was_geometry")
    args = (z["xobs"], z["zobs"], z["xs"], z["bat"], float(z["shot_depth"]), float(z["dmodel"]), int(z["nxmodel"]))
    g = P.was_geometry(*args)
    assert np.array_equal(g["bat_model"], z["bat_model_was"])
    assert np.array_equal(g["bat_model_grid"], z["bat_model_grid_was"])
    assert np.array_equal(g["nxSou"], z["nxsou_was"]) and np.array_equal(g["nySou"], z["nysou_was"])
    assert np.array_equal(g["nxRec"], z["nxrec_was"][:, 0]) and g["nyRec"] == z["nyrec_was"][0, 0]
    assert np.array_equal(P.was_geometry(*args, relocate=False)["nySou"], z["zobs_grid_nav"])


def test_wiener_estimate_vs_reference_golden(golden):
    """The Wiener step of source estimation (fwi_gb300/source.py:
    wiener_estimate, float64 FFT) against source_estimation.f90 executed
    from the reference after its forward solve (mute, normalisation,
    FFTPACK5, kk/bb sums, eps, inverse transform) on the same Green's
    functions and observed traces."""
    from fwi_gb300.source import wiener_estimate
    z = golden("source_estimation")
    got = wiener_estimate(z["Gs"], z["Go"], z["model"], float(z["d"]), float(z["dt"]), float(z["f1"]),
                          float(z["f2"]), int(z["nxs"]), z["nxr"])
    sst = z["sst"].astype(np.float64)
    assert np.linalg.norm(got - sst) / np.linalg.norm(sst) <= 1e-6
