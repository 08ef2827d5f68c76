"""Drop-in solver_acoustic_SS on the GPU against the golden vectors of the
reference's own Fortran and against the oracle: bit-exact (FP32, same
operation order, no fused multiply-add)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

SOLVER_CASES = ["solver_acc3", "solver_acc4", "solver_acc3_dpml8"]


def gpu_solver(z, iprop, kernel, fields, acc=None, dpml=None, **over):
    import fwi_gb300 as F
    F.set_solver_options(int(z["acc"]) if acc is None else acc, int(z["dpml"]) if dpml is None else dpml)
    nt = int(over.get("nt", z["nt"]))
    nrec = len(z["nxRec"])
    rec = np.full((nt, nrec), 7.0, np.float32, order="F")
    F.solver_acoustic_SS(0, iprop, len(z["nxSou"]), nrec, z["nxSou"], z["nySou"], z["nxRec"], z["nyRec"], z["S"],
                         z["Sadj"], float(z["d"]), float(z["dt"]), int(z["ny"]), int(z["nx"]), z["ctmp"],
                         int(z["store_snap"]), int(z["nt_store"]), nt, kernel, fields, rec)
    return rec


@pytest.mark.parametrize("case", SOLVER_CASES)
def test_forward_adjoint_bit_exact_vs_reference_golden(golden, case):
    z = golden(case)
    ny, nx, nts = int(z["ny"]), int(z["nx"]), int(z["nt_store"])
    F_ = np.zeros((ny, nx * (nts + 1)), np.float32, order="F")
    K = np.asfortranarray(z["kernel_in"].copy())
    rec = gpu_solver(z, 1, K, F_)
    np.testing.assert_array_equal(rec, z["rec_fwd"])
    np.testing.assert_array_equal(F_, z["fields_fwd"])
    np.testing.assert_array_equal(K, z["kernel_in"])
    K = np.asfortranarray(z["kernel_in"].copy())
    rec2 = gpu_solver(z, 2, K, F_)
    np.testing.assert_array_equal(K, z["kernel_adj"])
    np.testing.assert_array_equal(rec2, z["rec_adj"])


def test_fields_block0_left_untouched(golden):
    z = golden("solver_acc3")
    ny, nx, nts = int(z["ny"]), int(z["nx"]), int(z["nt_store"])
    F_ = np.full((ny, nx * (nts + 1)), 3.5, np.float32, order="F")
    K = np.zeros((ny, nx), np.float32, order="F")
    gpu_solver(z, 1, K, F_)
    assert np.all(F_[:, :nx] == 3.5)
    np.testing.assert_array_equal(F_[:, nx:], z["fields_fwd"][:, nx:])


def random_case(seed, ny, nx, nt, acc, dpml, store_snap, nsou, nrec):
    rng = np.random.default_rng(seed)
    vp = np.asfortranarray((1500 + 1500 * rng.random((ny, nx))).astype(np.float32))
    dn = dpml + 2 * acc
    z = dict(acc=acc, dpml=dpml, ny=ny, nx=nx, nt=nt, store_snap=store_snap, nt_store=nt // store_snap,
             d=np.float32(12.5), dt=np.float32(0.001), ctmp=vp,
             nxSou=rng.integers(-dn + 1, nx + dn, size=nsou).astype(np.int32),
             nySou=rng.integers(1, ny + dn, size=nsou).astype(np.int32),
             nxRec=rng.integers(-dn + 1, nx + dn, size=nrec).astype(np.int32),
             nyRec=rng.integers(-dn + 1, ny + dn, size=nrec).astype(np.int32),
             S=np.asfortranarray(rng.standard_normal((nt, nsou)).astype(np.float32)),
             Sadj=np.asfortranarray(rng.standard_normal((nt, nrec)).astype(np.float32)))
    z["nxSou"][0], z["nySou"][0] = nx // 2, 3
    return z


@pytest.mark.parametrize("acc,dpml,ny,nx,store", [(3, 20, 37, 301, 10), (4, 20, 50, 130, 4), (3, 5, 23, 77, 7),
                                                   (4, 11, 64, 250, 10), (3, 20, 40, 1, 10),
                                                   (3, 20, 20, 2000, 10), (4, 20, 16, 1100, 10),
                                                   # dn > 32: side strips of two columns per lane
                                                   (3, 30, 30, 200, 10), (4, 40, 24, 90, 7), (3, 50, 20, 60, 10),
                                                   (3, 30, 12, 5, 10)])
def test_random_geometry_bit_exact_vs_oracle(acc, dpml, ny, nx, store):
    """Random sources and receivers anywhere in the padded grid (pads, top
    pad, corners, duplicates), odd widths that exercise the tile edges."""
    z = random_case(acc * 100 + nx, ny, nx, 120, acc, dpml, store, 4, 40)
    nts = z["nt_store"]
    Fg = np.zeros((ny, nx * (nts + 1)), np.float32, order="F")
    Fo = np.zeros_like(Fg)
    Kg = np.zeros((ny, nx), np.float32, order="F")
    Ko = Kg.copy(order="F")
    rec_g = gpu_solver(z, 1, Kg, Fg)
    rec_o = O.solver_acoustic_ss(1, z["nxSou"], z["nySou"], z["nxRec"], z["nyRec"], z["S"], z["Sadj"], z["d"], z["dt"],
                                 z["ctmp"], store, nts, 120, Ko, Fo, acc=acc, dpml=dpml)
    np.testing.assert_array_equal(rec_g, rec_o)
    np.testing.assert_array_equal(Fg, Fo)
    gpu_solver(z, 2, Kg, Fg)
    O.solver_acoustic_ss(2, z["nxSou"], z["nySou"], z["nxRec"], z["nyRec"], z["S"], z["Sadj"], z["d"], z["dt"],
                         z["ctmp"], store, nts, 120, Ko, Fo, acc=acc, dpml=dpml)
    np.testing.assert_array_equal(Kg, Ko)


def test_out_of_grid_receiver_is_rejected():
    import fwi_gb300 as F
    z = random_case(1, 20, 30, 20, 3, 20, 10, 1, 2)
    z["nxRec"][1] = -40  # dn + nxRec < 1: the reference would index out of bounds
    with pytest.raises(F.FwiError, match="outside the padded grid"):
        gpu_solver(z, 1, np.zeros((20, 30), np.float32, order="F"), np.zeros((20, 90), np.float32, order="F"))


def test_cfl_violation_reports_nonfinite():
    import fwi_gb300 as F
    z = random_case(2, 30, 60, 400, 3, 10, 10, 1, 4)
    z["dt"] = np.float32(0.02)  # c*dt/d ~ 4.8 >> stability limit
    with pytest.raises(F.FwiError) as e:
        gpu_solver(z, 1, np.zeros((30, 60), np.float32, order="F"), np.zeros((30, 60 * 41), np.float32, order="F"))
    assert e.value.code == -4


def test_misfit_function_vs_golden(golden):
    import fwi_gb300 as F
    g = golden("misfit_beta")
    for tag in "ab":
        s, t = g[f"{tag}_synth"], g[f"{tag}_trace"]
        adj = np.zeros_like(s, order="F")
        m, m64 = F.Misfit_function(0, 5.0, s, t, s.shape[1], s.shape[0], float(g[f"{tag}_dt"]), adj)
        np.testing.assert_array_equal(adj, g[f"{tag}_adj"])
        _, o64, _ = O.misfit_function(s, t, float(g[f"{tag}_dt"]))
        assert abs(m64 - o64) <= 1e-12 * abs(o64)
        # the reference sums in FP32; the FP64 sum agrees to FP32 rounding
        assert abs(m - g[f"{tag}_misfit"]) <= 1e-5 * abs(g[f"{tag}_misfit"])


def test_beta_calculous_vs_golden(golden):
    import fwi_gb300 as F
    g = golden("misfit_beta")
    for tag in "ab":
        gg, oo = g[f"beta_{tag}_g"], g[f"beta_{tag}_o"]
        b, n64, d64 = F.Beta_calculous(gg, oo, gg.shape[1], gg.shape[0])
        _, on, od = O.beta_calculous(gg, oo)
        assert abs(n64 - on) <= 1e-12 * abs(on) and abs(d64 - od) <= 1e-12 * abs(od)
        assert abs(b - g[f"beta_{tag}"]) <= 1e-5 * abs(g[f"beta_{tag}"])
