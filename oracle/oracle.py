"""ctypes bindings for the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline legs of bench.py as the checker.  The product package never
imports this module.

Arrays follow the reference's Fortran conventions: column-major (numpy
order='F'), 1-based grid indices in the geometry arrays.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_P = C.c_void_p
_lib = None


def build(force: bool = False) -> str:
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(
            os.path.join(HERE, "fwi_oracle.cpp")):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB_PATH)
        I, F, D, Z = C.c_int, C.c_float, C.c_double, C.c_size_t
        _lib.oracle_solver_acoustic_ss_f32.argtypes = [I, I, I, _P, _P, _P, _P, _P, _P, F, F, I, I, _P, I, I, I,
                                                      _P, _P, _P, I, I]
        _lib.oracle_solver_acoustic_ss_f64.argtypes = [I, I, I, _P, _P, _P, _P, _P, _P, D, D, I, I, _P, I, I, I,
                                                      _P, _P, _P, I, I]
        _lib.oracle_misfit_function_f32.argtypes = [I, I, F, _P, _P, _P, _P, _P]
        _lib.oracle_misfit_function_f64.argtypes = [I, I, D, _P, _P, _P, _P, _P]
        _lib.oracle_beta_calculous.argtypes = [_P, _P, I, I, _P, _P, _P]
        _lib.oracle_ricker.argtypes = [F, F, I, _P]
        _lib.oracle_mcs_geometry.argtypes = [F, F, F, F, F, F, I, _P, _P, _P, _P]
        _lib.oracle_time_rules.argtypes = [_P, Z, F, F, I, _P, _P, _P]
        _lib.oracle_fd_coef_f32.argtypes = [I, I, _P]
        _lib.oracle_pml_coeffs_f32.argtypes = [I, I, F, F, _P, _P, _P, _P]
        _lib.oracle_gradient_batch_f32.argtypes = [I, I, F, F, I, I, I, I, _P, I, _P, _P, _P, _P, _P, _P, _P, _P,
                                                  _P, _P, _P, _P, I, _P, _P, _P, _P, _P, I]
        _lib.oracle_gradient_batch_f64.argtypes = [I, I, D, D, I, I, I, I, _P, I, _P, _P, _P, _P, _P, _P, _P, _P,
                                                  _P, _P, _P, _P, I, _P, _P, _P, _P, _P, I]
        _lib.oracle_quantize_snapshots.argtypes = [_P, I, I, I, I]
        _lib.oracle_gradient_batch_f32_form.argtypes = [I, I, F, F, I, I, I, I, _P, I, _P, _P, _P, _P, _P, _P, _P,
                                                       _P, _P, _P, _P, _P, I, _P, _P, _P, _P, _P, I, I]
    return _lib


def _ptr(a):
    return a.ctypes.data_as(_P) if a is not None else None


def _f(a, dt=np.float32):
    return np.asfortranarray(np.asarray(a, dtype=dt))


def _i(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.int32).reshape(-1))


def solver_acoustic_ss(iprop, nxSou, nySou, nxRec, nyRec, S, Sadj, d, dt, ctmp, store_snap, nt_store, nt,
                       kernel, fields, acc=3, dpml=20, fp64=False):
    """Run the oracle solver; kernel and fields are updated in place
    (Fortran shapes (ny,nx) and (ny, nx*(nt_store+1))).  Returns Rec_point."""
    dtp = np.float64 if fp64 else np.float32
    ny, nx = ctmp.shape
    nsou, nrec = len(nxSou), len(nxRec)
    ctmp = _f(ctmp, dtp)
    S = _f(S, dtp) if S is not None else np.zeros((nt, max(nsou, 1)), dtp, order="F")
    Sadj = _f(Sadj, dtp) if Sadj is not None else np.zeros((nt, max(nrec, 1)), dtp, order="F")
    assert kernel.dtype == dtp and kernel.flags.f_contiguous and fields.dtype == dtp and fields.flags.f_contiguous
    rec = np.zeros((nt, nrec), dtp, order="F")
    fn = lib().oracle_solver_acoustic_ss_f64 if fp64 else lib().oracle_solver_acoustic_ss_f32
    xs, ys, xr, yr = _i(nxSou), _i(nySou), _i(nxRec), _i(nyRec)
    fn(iprop, nsou, nrec, _ptr(xs), _ptr(ys), _ptr(xr), _ptr(yr), _ptr(S), _ptr(Sadj), d, dt, ny, nx,
       _ptr(ctmp), store_snap, nt_store, nt, _ptr(kernel), _ptr(fields), _ptr(rec), acc, dpml)
    return rec


def misfit_function(synth, trace, dt, fp64=False):
    """Misfit_function + Misfit_L2 (misfit_type 1).  Returns
    (misfit accumulated like the reference, misfit accumulated in FP64,
    adjoint source)."""
    dtp = np.float64 if fp64 else np.float32
    synth, trace = _f(synth, dtp), _f(trace, dtp)
    nt, nrec = synth.shape
    adj = np.zeros((nt, nrec), dtp, order="F")
    m = np.zeros(1, dtp)
    m64 = np.zeros(1, np.float64)
    fn = lib().oracle_misfit_function_f64 if fp64 else lib().oracle_misfit_function_f32
    fn(nrec, nt, dt, _ptr(synth), _ptr(trace), _ptr(m), _ptr(m64), _ptr(adj))
    return m[0], float(m64[0]), adj


def beta_calculous(grad, old):
    grad, old = _f(grad), _f(old)
    ny, nx = grad.shape
    b = np.zeros(1, np.float32)
    n64 = np.zeros(1, np.float64)
    d64 = np.zeros(1, np.float64)
    lib().oracle_beta_calculous(_ptr(grad), _ptr(old), nx, ny, _ptr(b), _ptr(n64), _ptr(d64))
    return b[0], float(n64[0]), float(d64[0])


def ricker(freq, dt, nt):
    out = np.zeros(nt, np.float32)
    lib().oracle_ricker(freq, dt, nt, _ptr(out))
    return out


def mcs_geometry(xs, shot_depth, streamer_depth, near_offset, drec, dmodel, nrec):
    nxs, nys = np.zeros(1, np.int32), np.zeros(1, np.int32)
    nxr, nyr = np.zeros(nrec, np.int32), np.zeros(nrec, np.int32)
    lib().oracle_mcs_geometry(xs, shot_depth, streamer_depth, near_offset, drec, dmodel, nrec, _ptr(nxs), _ptr(nys),
                              _ptr(nxr), _ptr(nyr))
    return int(nxs[0]), int(nys[0]), nxr, nyr


def time_rules(lam, dmodel, tfin, store_snap=10):
    lam = _f(lam)
    dt = np.zeros(1, np.float32)
    nt, nts = np.zeros(1, np.int32), np.zeros(1, np.int32)
    lib().oracle_time_rules(_ptr(lam), lam.size, dmodel, tfin, store_snap, _ptr(dt), _ptr(nt), _ptr(nts))
    return dt[0], int(nt[0]), int(nts[0])


def fd_coef(num, acc):
    c = np.zeros(acc + 2, np.float32)
    lib().oracle_fd_coef_f32(num, acc, _ptr(c))
    return c[:acc + 1]


def pml_coeffs(acc, dpml, dt, d):
    dn = dpml + 2 * acc
    fA, fB = np.zeros(dn, np.float32), np.zeros(dn, np.float32)
    cA, cB = np.zeros((4, dn, dn), np.float32), np.zeros((4, dn, dn), np.float32)
    lib().oracle_pml_coeffs_f32(acc, dpml, dt, d, _ptr(fA), _ptr(fB), _ptr(cA), _ptr(cB))
    # each dn*dn block is column-major: transpose the C-order view
    return fA, fB, cA.transpose(0, 2, 1).copy(), cB.transpose(0, 2, 1).copy()


# stored-snapshot forms of gradient_batch(snap_form=...) (FP32 solver only)
SNAP_FORMS = {"f32": 0, "f16_snapshot_scale": 1, "bf16_snapshot_scale": 2, "f16_segment_pow2": 3,
              "bf16_segment_pow2": 4}


def quantize_snapshots(fields, form):
    """The stored-snapshot form `form` (SNAP_FORMS) applied to a float32
    array of snapshots (ny, nx, nsnap) in Fortran order, in place; returns it."""
    assert fields.dtype == np.float32 and fields.flags.f_contiguous and fields.ndim == 3
    ny, nx, ns = fields.shape
    lib().oracle_quantize_snapshots(_ptr(fields), ny, nx, ns, int(form))
    return fields


def gradient_batch(survey, vp_model, step=1, fp64=False, nthreads=1, want_synth=False, snap_form=0):
    """Per-shot forward + misfit + adjoint for a survey (see
    fwi_gb300.survey.Survey for the fields).  Returns (kernels list,
    misfit_ref array, misfit64 array, synth list or None).  snap_form (FP32
    only, SNAP_FORMS) stores the snapshots between the forward and the
    adjoint run in a 16-bit form: FP16 or BF16 with one max-abs scale per
    snapshot, or with a power-of-two scale per 128-column row segment."""
    dtp = np.float64 if fp64 else np.float32
    sv = survey
    ns = len(sv.shots)
    x0 = _i([s.x0 for s in sv.shots])
    nxw = _i([s.nx for s in sv.shots])
    nsou = _i([len(s.nxSou) for s in sv.shots])
    nrec = _i([len(s.nxRec) for s in sv.shots])
    sou_off = _i(np.concatenate([[0], np.cumsum(nsou)[:-1]]))
    rec_off = _i(np.concatenate([[0], np.cumsum(nrec)[:-1]]))
    nxS = _i(np.concatenate([s.nxSou for s in sv.shots]))
    nyS = _i(np.concatenate([s.nySou for s in sv.shots]))
    nxR = _i(np.concatenate([s.nxRec for s in sv.shots]))
    nyR = _i(np.concatenate([s.nyRec for s in sv.shots]))
    S = np.concatenate([np.asarray(s.src, dtp).reshape(sv.nt, -1, order="F") for s in sv.shots], axis=1)
    S = np.asfortranarray(S)
    obs = np.asfortranarray(np.concatenate([
        (np.asarray(s.obs, dtp).reshape(sv.nt, -1, order="F") if s.obs is not None
         else np.zeros((sv.nt, len(s.nxRec)), dtp)) for s in sv.shots], axis=1))
    sizes = [sv.ny * s.nx for s in sv.shots]
    koff = np.ascontiguousarray(np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.uint64))
    kern = np.zeros(int(sum(sizes)), dtp)
    synth = np.zeros((sv.nt, int(nrec.sum())), dtp, order="F") if want_synth else None
    mr = np.zeros(ns, dtp)
    m64 = np.zeros(ns, np.float64)
    vp = _f(vp_model, dtp)
    if snap_form and fp64:
        raise ValueError("the 16-bit snapshot forms run with the FP32 solver")
    fn = lib().oracle_gradient_batch_f64 if fp64 else lib().oracle_gradient_batch_f32
    extra = ()
    if snap_form:
        fn, extra = lib().oracle_gradient_batch_f32_form, (int(snap_form),)
    fn(ns, sv.ny, sv.d, sv.dt, sv.nt, sv.store_snap, sv.acc, sv.dpml, _ptr(vp), vp.shape[1], _ptr(x0), _ptr(nxw),
       _ptr(nsou), _ptr(sou_off), _ptr(nxS), _ptr(nyS), _ptr(S), _ptr(nrec), _ptr(rec_off), _ptr(nxR), _ptr(nyR),
       _ptr(obs), step, _ptr(koff), _ptr(kern), _ptr(synth), _ptr(mr), _ptr(m64), nthreads, *extra)
    kernels = [kern[int(koff[i]):int(koff[i]) + sizes[i]].reshape(sv.ny, sv.shots[i].nx, order="F")
               for i in range(ns)]
    synths = None
    if want_synth:
        synths = [synth[:, int(rec_off[i]):int(rec_off[i]) + int(nrec[i])] for i in range(ns)]
    return kernels, mr, m64, synths
