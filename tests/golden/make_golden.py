"""Generate the golden vectors in tests/golden/*.npz from the reference source.

Run where a checkout of the reference exists: its path is the first
argument, or the environment variable FWI_REFERENCE.  Each case executes the
reference's own Fortran routines -- solver_acoustic_SS and the files it
calls, Misfit_function/Misfit_L2, Beta_calculous, Ricker_mcs, polyfit,
interpolation_akima/INTRPL, time_filter with filters_function1D/butterworth
and the FFTPACK5 transforms, the post-solver part of source_estimation, and
the geometry and time-step statements of get_mcs_data.f90, get_was_data.f90
and calculate_misfit_gradient.f90 -- through fortran_exec.py in IEEE single
precision, on small seeded inputs, and stores inputs and outputs.

The fixtures are committed; tests read them and never need the reference.

    python tests/golden/make_golden.py /path/to/reference [case ...]
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import fortran_exec as fe  # noqa: E402

V = fe.Var
F32 = np.float32


def farr(a, dtype=np.float32):
    return np.asfortranarray(np.asarray(a, dtype=dtype))


def solver_program(src, acc=None, dpml=None):
    files = [os.path.join(src, f) for f in (
        "solver_acoustic_SS.f90", "solver_space_derivs.f90", "solver_FD_coeffs.f90",
        "solver_PML_coeffs.f90", "solver_PML_matrices.f90")]
    ov = {}
    if acc is not None:
        ov[("solver_acoustic_ss", "acc")] = acc
    if dpml is not None:
        ov[("solver_acoustic_ss", "dpml")] = dpml
    return fe.Program(files, overrides=ov)


def run_solver(prog, iprop, geom, S, Sadj, d, dt, ctmp, store_snap, nt_store, nt, kernel, fields):
    nxSou, nySou, nxRec, nyRec = geom
    ny, nx = ctmp.shape
    rec = farr(np.zeros((nt, len(nxRec))))
    args = [V(0, "integer"), V(iprop, "integer"), V(len(nxSou), "integer"), V(len(nxRec), "integer"),
            V(farr(nxSou, np.int64), "integer"), V(farr(nySou, np.int64), "integer"),
            V(farr(nxRec, np.int64), "integer"), V(farr(nyRec, np.int64), "integer"),
            V(S, "real"), V(Sadj, "real"), V(F32(d)), V(F32(dt)), V(ny, "integer"), V(nx, "integer"),
            V(ctmp), V(store_snap, "integer"), V(nt_store, "integer"), V(nt, "integer"),
            V(kernel), V(fields), V(rec)]
    prog.call("solver_acoustic_ss", *args)
    return rec


def case_solver(src, name, acc, dpml, ny, nx, nt, store_snap, d, dt, geom, seed):
    rng = np.random.default_rng(seed)
    prog = solver_program(src, acc=acc, dpml=dpml)
    nt_store = nt // store_snap
    yy, xx = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    vp = 1500.0 + 60.0 * yy + 15.0 * np.sin(xx / 2.0) + rng.uniform(-40, 40, size=(ny, nx))
    ctmp = farr(vp)
    S = farr(rng.standard_normal((nt, len(geom[0]))))
    Sadj = farr(rng.standard_normal((nt, len(geom[2]))))
    fields = farr(np.zeros((ny, nx * (nt_store + 1))))
    kernel0 = farr(rng.standard_normal((ny, nx)) * 1e-3)
    kernel_f = kernel0.copy(order="F")
    t0 = time.time()
    rec = run_solver(prog, 1, geom, S, Sadj, d, dt, ctmp, store_snap, nt_store, nt, kernel_f, fields)
    fields_fwd = fields.copy(order="F")
    kernel_a = kernel0.copy(order="F")
    rec_adj = run_solver(prog, 2, geom, S, Sadj, d, dt, ctmp, store_snap, nt_store, nt, kernel_a, fields)
    print(f"{name}: solver fwd+adj {time.time() - t0:.1f}s, |rec|max={np.abs(rec).max():.3e} "
          f"|kernel-k0|max={np.abs(kernel_a - kernel0).max():.3e}")
    np.savez_compressed(
        os.path.join(HERE, f"{name}.npz"), acc=acc, dpml=20 if dpml is None else dpml, ny=ny, nx=nx, nt=nt, store_snap=store_snap,
        nt_store=nt_store, d=F32(d), dt=F32(dt), nxSou=np.array(geom[0], np.int32), nySou=np.array(geom[1], np.int32),
        nxRec=np.array(geom[2], np.int32), nyRec=np.array(geom[3], np.int32), ctmp=ctmp, S=S, Sadj=Sadj,
        kernel_in=kernel0, rec_fwd=rec, fields_fwd=fields_fwd, kernel_fwd=kernel_f, kernel_adj=kernel_a,
        rec_adj=rec_adj, fields_after_adj=fields)


def case_coeffs(src):
    prog = fe.Program([os.path.join(src, "solver_FD_coeffs.f90"), os.path.join(src, "solver_PML_coeffs.f90")])
    out = {}
    for acc in (3, 4):
        for num in (1, 2):
            c = farr(np.zeros(acc + 1))
            prog.call("finite_difference_coef", V(num, "integer"), V(acc, "integer"), V(c))
            out[f"fd_num{num}_acc{acc}"] = c
    for tag, acc, dpml, dt, d in (("a", 3, 20, 1e-3, 10.0), ("b", 4, 20, 2e-3, 25.0), ("c", 3, 20, 1e-3, 12.5)):
        dn = dpml + 2 * acc
        fA, fB = farr(np.zeros(dn)), farr(np.zeros(dn))
        mats = [farr(np.zeros((dn, dn))) for _ in range(8)]
        prog.call("pml_coeffs", V(acc, "integer"), V(dpml, "integer"), V(F32(dt)), V(F32(d)), V(dn, "integer"),
                  V(fA), V(fB), *[V(m) for m in mats])
        out[f"pml_{tag}_cfg"] = np.array([acc, dpml], np.int32)
        out[f"pml_{tag}_dtd"] = np.array([dt, d], np.float32)
        out[f"pml_{tag}_fA"], out[f"pml_{tag}_fB"] = fA, fB
        # argument order in the reference: ld_A, rd_A, lu_A, ru_A, ld_B, rd_B, lu_B, ru_B
        out[f"pml_{tag}_cornA"] = np.stack(mats[0:4])
        out[f"pml_{tag}_cornB"] = np.stack(mats[4:8])
    np.savez_compressed(os.path.join(HERE, "coeffs.npz"), **out)
    print("coeffs: done")


def case_misfit(src):
    rng = np.random.default_rng(7)
    prog = fe.Program([os.path.join(src, "Misfit.f90"), os.path.join(src, "Misfit_L2.f90"),
                       os.path.join(src, "auxiliar.f90")],
                      globals_={"misfit_type": V(1, "integer")})
    out = {}
    for tag, nrec, nt, dt in (("a", 6, 50, 1e-3), ("b", 3, 120, 2.5e-3)):
        synth = farr(rng.standard_normal((nt, nrec)) * 3e-2)
        trace = farr(rng.standard_normal((nt, nrec)) * 7.0)
        trace[:, 1] = 0.0                      # observed trace all zero: skipped
        if nrec > 3:
            synth[:, 3] = 0.0                  # synthetic trace all zero: no normalisation
            trace[:10, 4] = 0.0
        mis = V(F32(123.0))
        adj = farr(np.zeros((nt, nrec)))
        prog.call("misfit_function", V(0, "integer"), V(F32(5.0)), V(synth), V(trace), V(nrec, "integer"),
                  V(nt, "integer"), V(F32(dt)), mis, V(adj))
        out.update({f"{tag}_synth": synth, f"{tag}_trace": trace, f"{tag}_dt": F32(dt),
                    f"{tag}_misfit": F32(mis.value), f"{tag}_adj": adj})
    prog2 = fe.Program([os.path.join(src, "Beta_calculous.f90")])
    for tag, ny, nx in (("a", 7, 9), ("b", 31, 17)):
        g = farr(rng.standard_normal((ny, nx)))
        o = farr(rng.standard_normal((ny, nx)))
        beta = V(F32(0))
        prog2.call("beta_calculous", V(g), V(o), V(nx, "integer"), V(ny, "integer"), beta)
        out.update({f"beta_{tag}_g": g, f"beta_{tag}_o": o, f"beta_{tag}": F32(beta.value)})
    np.savez_compressed(os.path.join(HERE, "misfit_beta.npz"), **out)
    print("misfit/beta: done")


def case_geometry(src):
    mcs = os.path.join(src, "get_mcs_data.f90")
    cmg = os.path.join(src, "calculate_misfit_gradient.f90")
    out = {}
    # Ricker_mcs (get_mcs_data.f90:331-369)
    for tag, f0, dtm, ntm in (("a", 10.0, 0.004, 500), ("b", 8.0, 0.002, 1000), ("c", 5.0, 0.0025, 2000)):
        g = {"freq_ricker": V(F32(f0)), "dt_mcs": V(F32(dtm)), "nt_mcs": V(ntm, "integer")}
        prog = fe.Program([mcs], globals_=g)
        raw = farr(np.zeros(ntm))
        prog.call("ricker_mcs", V(0, "integer"), V(1, "integer"), V(raw))
        out[f"ricker_{tag}"] = raw
        out[f"ricker_{tag}_par"] = np.array([f0, dtm, ntm], np.float64)
    # receiver/shot grid indices (get_mcs_data.f90:113-114, 150, 154, 508-510)
    shots = []
    for tag, xs, sd, rd, near, drec, dmodel, nrec in (
            ("a", 2637.5, 10.0, 10.0, 150.0, 12.5, 25.0, 200),
            ("b", 9875.0, 7.5, 10.0, 150.0, 12.5, 12.5, 480),
            ("c", 31337.3, 12.0, 8.0, 100.0, 25.0, 25.0, 240),
            ("d", 1000.1, 5.0, 5.0, 62.5, 12.5, 12.5, 64)):
        env = {
            "i": V(1, "integer"), "ishot": V(1, "integer"), "irec": V(0, "integer"),
            "added_space_model": V(F32(0)), "xs": V(F32(xs)), "dmodel": V(F32(dmodel)),
            "pos_shot_mcs": V(farr(np.zeros(1))), "pos_shot_grid_mcs": V(farr(np.zeros(1, np.int64), np.int64), "integer"),
            "nxsou_mcs": V(farr(np.zeros(1, np.int64), np.int64), "integer"),
            "nysou_mcs": V(farr(np.zeros(1, np.int64), np.int64), "integer"),
            "nxrec_mcs": V(farr(np.zeros((nrec, 1), np.int64), np.int64), "integer"),
            "nyrec_mcs": V(farr(np.zeros((nrec, 1), np.int64), np.int64), "integer"),
            "shot_depth_mcs": V(F32(sd)), "streamer_depth": V(F32(rd)),
            "offset_header": V(0, "integer"), "numrec_mcs": V(nrec, "integer"),
            "pos_rec": V(farr(np.zeros((nrec, 1)))), "pos_rec_grid": V(farr(np.zeros((nrec, 1), np.int64), np.int64), "integer"),
            "near_offset": V(F32(near)), "drec": V(F32(drec)),
        }
        fe.run_snippet(mcs, 113, 114, env)
        fe.run_snippet(mcs, 503, 514, env)
        fe.run_snippet(mcs, 149, 155, env)
        out[f"geom_{tag}_par"] = np.array([xs, sd, rd, near, drec, dmodel], np.float32)
        out[f"geom_{tag}_nrec"] = np.int32(nrec)
        out[f"geom_{tag}_nxSou"] = np.int32(env["nxsou_mcs"].value[0])
        out[f"geom_{tag}_nySou"] = np.int32(env["nysou_mcs"].value[0])
        out[f"geom_{tag}_nxRec"] = env["nxrec_mcs"].value[:, 0].astype(np.int32)
        out[f"geom_{tag}_nyRec"] = env["nyrec_mcs"].value[:, 0].astype(np.int32)
        shots.append(tag)
    # CFL time step and snapshot rules (calculate_misfit_gradient.f90:198-203)
    rng = np.random.default_rng(11)
    for tag, vmax, dmodel, tfin in (("a", 4500.0, 25.0, 6.0), ("b", 5000.0, 12.5, 6.0), ("c", 8000.0, 25.0, 20.0),
                                    ("d", 1733.3, 10.0, 0.731)):
        vp = rng.uniform(1500.0, vmax, size=(9, 11)).astype(np.float32)
        vp[3, 4] = F32(vmax)
        rho = farr(np.full((9, 11), 1000.0))
        lam = farr(rho * vp * vp)
        env = {"dmodel": V(F32(dmodel)), "lambda": V(lam), "rho": V(rho), "tfin": V(F32(tfin)),
               "dt": V(F32(0)), "nt": V(0, "integer"), "temp": V(F32(0)), "store_snap": V(10, "integer"),
               "nt_store": V(0, "integer")}
        fe.run_snippet(cmg, 198, 203, env)
        out[f"time_{tag}_lambda"] = lam
        out[f"time_{tag}_par"] = np.array([dmodel, tfin], np.float32)
        out[f"time_{tag}_dt"] = F32(env["dt"].value)
        out[f"time_{tag}_nt"] = np.int32(env["nt"].value)
        out[f"time_{tag}_ntstore"] = np.int32(env["nt_store"].value)
    np.savez_compressed(os.path.join(HERE, "geometry.npz"), **out)
    print("geometry/ricker/time rules: done")


def case_polyfit(src):
    """polyfit.f90 (line-search step from three trials), single process."""
    prog = fe.Program([os.path.join(src, "polyfit.f90")], mpi_stub=True,
                      globals_={"mpi_comm_world": V(0, "integer"), "mpi_status_size": V(1, "integer")})
    rng = np.random.default_rng(11)
    cases = [(0.3, 10.0, 8.0, 9.0, 2), (0.7, 7.0, 6.5, 6.9, 3), (1e-3, 5.0, 4.0, 4.5, 2),
             (2.5e-4, 1.0, 0.9, 0.95, 4), (0.01, 3.0, 3.0, 3.0, 2),      # flat: ties, the last sample wins
             (0.05, 3.0, 2.0, 1.0, 2), (0.05, 1.0, 2.0, 3.0, 3),        # monotone fits: an end of the range
             (0.2, 4.0, 5.0, 4.0, 2)]                                   # concave
    for _ in range(24):
        nut = float(F32(10.0 ** rng.uniform(-5, 1)))
        m = np.sort(rng.uniform(0.5, 2.0, 3))[::-1] if rng.random() < 0.5 else rng.uniform(0.5, 2.0, 3)
        cases.append((nut, float(m[0]), float(m[1]), float(m[2]), int(rng.integers(2, 6))))
    inp = np.array(cases, dtype=np.float64)
    out = np.zeros(len(cases), np.float32)
    for i, (nut, m0, m1, m2, li) in enumerate(cases):
        end = V(F32(0))
        prog.call("polyfit", V(F32(nut)), V(F32(m0)), V(F32(m1)), V(F32(m2)), V(int(li), "integer"), end)
        out[i] = F32(end.value)
    np.savez_compressed(os.path.join(HERE, "polyfit.npz"), cases=inp, endstep=out)
    print("polyfit: done")


def case_akima(src):
    """interpolation_akima.f90 + INTRPL (akima433.f90): resampling of traces
    between time axes, incl. two/three/four input samples, flat and linear
    traces and output times past the last input sample."""
    prog = fe.Program([os.path.join(src, "interpolation_akima.f90"), os.path.join(src, "akima433.f90")])
    rng = np.random.default_rng(13)
    out = {}
    cases = [(60, 0.004, 190, 0.0013), (2, 0.01, 7, 0.004), (3, 0.01, 9, 0.003), (4, 0.01, 11, 0.004),
             (5, 0.002, 1, 0.001), (90, 0.001, 40, 0.0025), (48, 0.0025, 96, 0.00125)]
    for k, (L, dti, nto, dto) in enumerate(cases):
        ntr = 5
        data = farr(rng.standard_normal((L, ntr)))
        data[:, 1] = F32(0.25) * np.arange(L, dtype=np.float32)
        data[:, 2] = 0.0
        if L > 6:
            data[L // 2:L // 2 + 3, 3] = 1.0
        res = farr(np.zeros((nto, ntr)))
        prog.call("interpolation_akima", V(data), V(F32(dti)), V(L, "integer"), V(res), V(ntr, "integer"),
                  V(F32(dto)), V(nto, "integer"))
        out.update({f"c{k}_data": data, f"c{k}_dt_in": F32(dti), f"c{k}_dt_out": F32(dto), f"c{k}_out": res})
    out["ncases"] = len(cases)
    np.savez_compressed(os.path.join(HERE, "akima.npz"), **out)
    print("akima: done")


def case_filter(src):
    """time_filter (time_filter.f90) -> filters_function1D/butterworth
    (filters.f90) -> cfft1i/cfft1f/cfft1b (fftpack.f90) on a 20-sample record
    (480-point transforms: radix 4, 4, 2, 3, 5), three traces of which one is
    zero (left untouched), for the low-pass, high-pass and band-pass types and
    the reference's order 6, plus the low-pass at order 4 (the order set
    through the interpreter's override of n = 6)."""
    t0 = time.time()
    paths = [os.path.join(src, f) for f in ("time_filter.f90", "filters.f90", "fftpack.f90", "auxiliar.f90")]
    rng = np.random.default_rng(21)
    nt, num, dt = 20, 3, F32(0.004)
    base = farr(np.zeros((nt, num)))
    base[:, 0] = rng.standard_normal(nt).astype(F32)
    tt = np.arange(nt, dtype=np.float32) * dt
    base[:, 1] = (np.sin(F32(2 * np.pi * 12.0) * tt) + F32(0.5) * np.sin(F32(2 * np.pi * 70.0) * tt)).astype(F32)
    cases = [(1, 0.0, 30.0, 6), (2, 0.0, 30.0, 6), (3, 10.0, 60.0, 6), (1, 0.0, 25.0, 4)]
    out = {"data": base, "dt": dt, "nt": nt}
    for k, (typef, f1, fc, order) in enumerate(cases):
        prog = fe.Program(paths, overrides={("filters_function1d", "n"): order})
        d = farr(base.copy())
        prog.call("time_filter", V(d), V(nt, "integer"), V(dt), V(num, "integer"), V(typef, "integer"),
                  V(F32(f1)), V(F32(fc)))
        out.update({f"c{k}_typef": typef, f"c{k}_f1": F32(f1), f"c{k}_fc": F32(fc), f"c{k}_order": order,
                    f"c{k}_out": d})
        print(f"filter case {k}: {time.time() - t0:.0f} s", flush=True)
    out["ncases"] = len(cases)
    np.savez_compressed(os.path.join(HERE, "filter.npz"), **out)
    print("filter: done")


def case_was(src):
    """The WAS geometry (get_was_data.f90): shot navigation (receivers of the
    reciprocal inversion, :153-159), OBS navigation (:201-205), the
    bathymetry model by INTRPL over the shots' water depths (:584-613), the
    relocation of the OBS to it (:112-115) and the source/receiver indices
    (:223-231), executed statement by statement from the source with the
    module variables they use; added_space_model = 0 as no parfile key sets
    it (modules.f90:153)."""
    path = os.path.join(src, "get_was_data.f90")
    prog = fe.Program([os.path.join(src, "akima433.f90")])
    rng = np.random.default_rng(31)
    ns, nobs, d, nxm = 9, 4, F32(25.0), 120
    xs = (F32(100.0) + F32(337.5) * np.arange(ns, dtype=np.float32) + rng.uniform(-40, 40, ns).astype(F32)).astype(F32)
    bat = (F32(1800.0) + rng.uniform(-300, 300, ns).astype(F32)).astype(F32)
    xobs = np.array([212.0, 1010.0, 1999.9, 2600.3], np.float32)
    zobs = np.array([1700.0, 1900.0, 2100.0, 1750.0], np.float32)
    g = {}

    def gv(name, value, ftype):
        g[name] = V(value, ftype)

    gv("numshots_was", ns, "integer")
    gv("numrec_was", ns, "integer")
    gv("numobs", nobs, "integer")
    gv("dmodel", d, "real")
    gv("added_space_model", F32(0.0), "real")
    gv("shot_depth_was", F32(10.0), "real")
    gv("nxmodel", nxm, "integer")
    gv("length_model", F32(F32(nxm - 1) * d), "real")  # modules.f90:431
    for nm, n, ft in (("shotid_nav_was", ns, "integer"), ("pos_shot_was", ns, "real"), ("pos_shot_grid_was", ns, "integer"),
                      ("pos_bat_was", ns, "real"), ("pos_bat_grid_was", ns, "integer"), ("pos_xobs", nobs, "real"),
                      ("pos_xobs_grid", nobs, "integer"), ("pos_zobs", nobs, "real"), ("pos_zobs_grid", nobs, "integer"),
                      ("bat_model_was", nxm, "real"), ("bat_model_grid_was", nxm, "integer"),
                      ("nxsou_was", nobs, "integer"), ("nysou_was", nobs, "integer")):
        gv(nm, np.zeros(n, np.int64 if ft == "integer" else np.float32), ft)
    gv("nxrec_was", np.zeros((ns, nobs), np.int64, order="F"), "integer")
    gv("nyrec_was", np.zeros((ns, nobs), np.int64, order="F"), "integer")
    for i in range(ns):
        env = {"i": V(i + 1, "integer"), "xs": V(xs[i]), "bat": V(bat[i]), "shotid": V(i + 1, "integer")}
        fe.run_snippet(path, 153, 159, env, g)
    for i in range(nobs):
        env = {"i": V(i + 1, "integer"), "xs": V(xobs[i]), "xz": V(zobs[i])}
        fe.run_snippet(path, 201, 205, env, g)
    obs_grid_nav = g["pos_zobs_grid"].value.copy()
    env = {"i": V(0, "integer"), "err": V(0, "integer"), "xmodel": V(None, "real", alloc=True),
           "xmodel_": V(None, "real", alloc=True), "xbat_": V(None, "real", alloc=True)}
    fe.run_snippet(path, 584, 613, env, g, program=prog)
    fe.run_snippet(path, 112, 115, {"i": V(0, "integer")}, g)
    fe.run_snippet(path, 223, 231, {"iobs": V(0, "integer"), "irec": V(0, "integer")}, g)
    out = {"xs": xs, "bat": bat, "xobs": xobs, "zobs": zobs, "dmodel": d, "nxmodel": nxm,
           "shot_depth": F32(10.0), "zobs_grid_nav": obs_grid_nav}
    for nm in ("pos_shot_grid_was", "pos_bat_grid_was", "pos_xobs_grid", "pos_zobs", "pos_zobs_grid", "bat_model_was",
               "bat_model_grid_was", "nxsou_was", "nysou_was", "nxrec_was", "nyrec_was"):
        v = g[nm].value
        out[nm] = v.astype(np.int32) if v.dtype.kind in "iu" else v
    np.savez_compressed(os.path.join(HERE, "was_geometry.npz"), **out)
    print("was geometry: done")


def case_source(src):
    """source_estimation (source_estimation.f90) after its forward solve: the
    water-bottom mute (:76-107), normalisation (:109-110), FFTPACK5 transforms
    of Gs and Go (:124-134), the receiver sums kk and bb (:144-154), eps and
    the Wiener quotient (:156-159) and the inverse transform (:169-171).  The
    Green's functions Gs (solver_forward_simple) and the observed traces Go
    (get_shot_data) are supplied inputs: the two calls are replaced by Python
    stand-ins that copy them in."""
    paths = [os.path.join(src, f) for f in ("source_estimation.f90", "fftpack.f90")]
    rng = np.random.default_rng(41)
    ny, nx, nt, nr = 24, 40, 120, 6
    d, dt, f1, f2 = F32(10.0), F32(0.002), F32(0.0), F32(30.0)
    z = np.arange(ny)[:, None] * np.ones((1, nx))
    model = farr(np.where(z < 9, 1500.0, 1800.0 + 30.0 * (z - 9)))
    nxs, nys = 12, 2
    nxr = np.array([14, 17, 20, 23, 26, 29], np.int64)
    nyr = np.full(nr, 2, np.int64)
    tt = np.arange(nt, dtype=np.float64) * float(dt)
    Gs = np.zeros((nt, nr))
    Go = np.zeros((nt, nr))
    for r in range(nr):
        t0 = 0.02 + 0.003 * r
        a = (np.pi * 25.0 * (tt - t0)) ** 2
        Gs[:, r] = (1 - 2 * a) * np.exp(-a) * (1.0 + 0.1 * r)
        a2 = (np.pi * 18.0 * (tt - t0 - 0.01)) ** 2
        Go[:, r] = (1 - 2 * a2) * np.exp(-a2) * (0.8 + 0.05 * r) + 0.01 * rng.standard_normal(nt)
    Gs, Go = farr(Gs), farr(Go)

    def get_shot_data(k, arr):
        arr.value[...] = Go

    def solver_forward_simple(*a):
        a[-1].value[...] = Gs

    prog = fe.Program(paths, natives={"get_shot_data": get_shot_data, "solver_forward_simple": solver_forward_simple})
    sst = farr(np.zeros(nt))
    prog.call("source_estimation", V(1, "integer"), V(f1), V(f2), V(nx, "integer"), V(ny, "integer"),
              V(nt, "integer"), V(nr, "integer"), V(d), V(dt), V(nxs, "integer"), V(nys, "integer"),
              V(nxr.copy(), "integer"), V(nyr.copy(), "integer"), V(model), V(sst))
    np.savez_compressed(os.path.join(HERE, "source_estimation.npz"), Gs=Gs, Go=Go, model=model, nxs=nxs, nys=nys,
                        nxr=nxr.astype(np.int32), nyr=nyr.astype(np.int32), d=d, dt=dt, f1=f1, f2=f2, sst=sst)
    print("source estimation: done")


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("FWI_REFERENCE")
    if not ref:
        sys.exit("usage: make_golden.py /path/to/reference [case ...]  (or set FWI_REFERENCE)")
    src = os.path.join(ref, "src")
    only = set(sys.argv[2:])  # optional case names: coeffs misfit geometry polyfit akima filter was source solver
    names = ("coeffs", "misfit", "geometry", "polyfit", "akima", "filter", "was", "source")
    if only:
        for name in names:
            if name in only:
                globals()["case_" + name](src)
        if "solver" not in only:
            return
    else:
        for name in names:
            globals()["case_" + name](src)
    # acc=3 (the reference's hard-coded order), snapshots every 10 steps;
    # sources incl. one outside the interior; receivers with duplicates,
    # in the left pad, in the bottom strip and in a bottom corner.
    geom3 = ([5, 11, -3], [3, 7, 2], [1, 3, 3, 8, 16, 0, -10, 20], [2, 2, 2, 2, 2, 5, 14, 20])
    case_solver(src, "solver_acc3", 3, None, 12, 16, 60, 10, 10.0, 1e-3, geom3, seed=3)
    # acc=4 (8th order, the reference's own acc=4 tables), snapshots every 4
    geom4 = ([7], [4], [2, 2, 9, 15, 1, -2], [3, 3, 3, 3, 10, 11])
    case_solver(src, "solver_acc4", 4, None, 10, 14, 40, 4, 12.5, 1.5e-3, geom4, seed=4)
    # a thinner CPML to check that dPML is a true parameter of the restatement
    geom5 = ([4, 9], [2, 2], [1, 5, 9, 13], [2, 2, 2, 2])
    case_solver(src, "solver_acc3_dpml8", 3, 8, 9, 13, 70, 10, 10.0, 1e-3, geom5, seed=5)


if __name__ == "__main__":
    main()
