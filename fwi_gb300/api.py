"""Python mirror of the reference routines on the hot path.

Names, argument order and meaning follow the Fortran routines they replace;
arrays are numpy arrays in Fortran order (column-major) with 1-based grid
indices, so code written against the reference reads the same:

    solver_acoustic_SS   src/solver_acoustic_SS.f90:9-11
    Misfit_function      src/Misfit.f90:1 (misfit_type 1, Misfit_L2.f90)
    Beta_calculous       src/Beta_calculous.f90:1
    calculate_misfit_gradient  src/calculate_misfit_gradient.f90:1 (all shots)
    Ricker_mcs           src/get_mcs_data.f90:331
    mcs_geometry         src/get_mcs_data.f90:113-114,147-155,503-512
    time_rules           src/calculate_misfit_gradient.f90:198-203

Every call goes through libfwi_gb300.so; errors raise FwiError.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .survey import SurveySpec


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _ri(v):
    return C.byref(C.c_int(int(v)))


def _rf(v):
    return C.byref(C.c_float(float(v)))


def _f32(a):
    return np.asfortranarray(np.asarray(a, dtype=np.float32))


def _i32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.int32).reshape(-1))


def init(device: int = 0):
    N.check(N.load().fwi_init(device))


def set_solver_options(acc: int = 3, dpml: int = 20):
    """Spatial half-order and CPML width of solver_acoustic_SS (reference: 3, 20)."""
    N.check(N.load().fwi_set_solver_options(acc, dpml))


def set_stream(cuda_stream_handle):
    N.check(N.load().fwi_set_stream(C.c_void_p(cuda_stream_handle)))


def kernel_launch_count() -> int:
    return int(N.load().fwi_kernel_launch_count())


def solver_acoustic_SS(rank, iprop, NumSou, NumRec, nxSou, nySou, nxRec, nyRec, S, Sadj, d, dt, ny, nx, ctmp,
                       store_snap, nt_Store, nt, kernel, Fields, Rec_point):
    """Drop-in for solver_acoustic_SS.  kernel, Fields and Rec_point are
    float32 Fortran-ordered arrays updated in place (kernel accumulated for
    iprop=2, Fields written for iprop=1, Rec_point overwritten)."""
    for name, a in (("kernel", kernel), ("Fields", Fields), ("Rec_point", Rec_point)):
        if a is not None and (a.dtype != np.float32 or not a.flags.f_contiguous):
            raise TypeError(f"{name} must be a float32 Fortran-ordered array")
    xs, ys, xr, yr = _i32(nxSou), _i32(nySou), _i32(nxRec), _i32(nyRec)
    S_ = _f32(S) if S is not None else None
    Sa = _f32(Sadj) if Sadj is not None else None
    ct = _f32(ctmp)
    N.check(N.load().fwi_solver_acoustic_ss(
        _ri(rank), _ri(iprop), _ri(NumSou), _ri(NumRec), _p(xs), _p(ys), _p(xr), _p(yr), _p(S_), _p(Sa), _rf(d),
        _rf(dt), _ri(ny), _ri(nx), _p(ct), _ri(store_snap), _ri(nt_Store), _ri(nt), _p(kernel), _p(Fields),
        _p(Rec_point)))


def Misfit_function(rank, freq, Data_Synth, Data_trace, NumRec, nt, dt, AdjSource):
    """Returns (Misfit as float32, misfit accumulated in FP64); AdjSource is
    written in place."""
    if AdjSource.dtype != np.float32 or not AdjSource.flags.f_contiguous:
        raise TypeError("AdjSource must be a float32 Fortran-ordered array")
    s, t = _f32(Data_Synth), _f32(Data_trace)
    m = C.c_float(0.0)
    m64 = C.c_double(0.0)
    N.check(N.load().fwi_misfit_function(_ri(rank), _rf(freq), _p(s), _p(t), _ri(NumRec), _ri(nt), _rf(dt),
                                         C.byref(m), _p(AdjSource), C.byref(m64)))
    return np.float32(m.value), m64.value


def Beta_calculous(Grad, OldGrad, nx, ny):
    """Polak-Ribiere beta with FP64 dot products: (beta, num64, den64)."""
    g, o = _f32(Grad), _f32(OldGrad)
    b = C.c_float(0.0)
    n64, d64 = C.c_double(0.0), C.c_double(0.0)
    N.check(N.load().fwi_beta_calculous(_p(g), _p(o), _ri(nx), _ri(ny), C.byref(b), C.byref(n64), C.byref(d64)))
    return np.float32(b.value), n64.value, d64.value


def first_step(Search, var_orig):
    """nut = 1/100/maxval(abs(Search/log(var_orig))) on the device (FWI.f90:175)."""
    s, v = _f32(Search), _f32(var_orig)
    ny, nx = s.shape
    nut = C.c_float(0.0)
    N.check(N.load().fwi_first_step(_p(s), _p(v), _ri(nx), _ri(ny), C.byref(nut)))
    return np.float32(nut.value)


def model_update(Search, var_orig, step):
    """lambda = exp(Search*step)*var_orig on the device (FWI.f90:227, :315)."""
    s, v = _f32(Search), _f32(var_orig)
    ny, nx = s.shape
    out = np.zeros((ny, nx), np.float32, order="F")
    N.check(N.load().fwi_model_update(_p(s), _p(v), _rf(step), _ri(nx), _ri(ny), _p(out)))
    return out


def Ricker_mcs(freq, dt, nt):
    out = np.zeros(nt, np.float32)
    N.check(N.load().fwi_ricker(freq, dt, nt, _p(out)))
    return out


def mcs_geometry(xs, shot_depth, streamer_depth, near_offset, drec, dmodel, num_rec):
    """(nxSou, nySou, nxRec[num_rec], nyRec[num_rec]) 1-based grid indices."""
    a, b = C.c_int(0), C.c_int(0)
    xr, yr = np.zeros(num_rec, np.int32), np.zeros(num_rec, np.int32)
    N.check(N.load().fwi_mcs_geometry(xs, shot_depth, streamer_depth, near_offset, drec, dmodel, num_rec,
                                      C.byref(a), C.byref(b), _p(xr), _p(yr)))
    return a.value, b.value, xr, yr


def was_geometry(xobs, zobs, xshot, bat, shot_depth, dmodel, nxmodel, relocate=True):
    """WAS geometry of get_was_data.f90 (OBS as sources, shots as
    receivers): returns dict(nxSou, nySou, nxRec, nyRec, bat_model,
    bat_model_grid) with 1-based grid indices."""
    xo, zo = np.ascontiguousarray(xobs, np.float32), np.ascontiguousarray(zobs, np.float32)
    xs, bt = np.ascontiguousarray(xshot, np.float32), np.ascontiguousarray(bat, np.float32)
    no, ns = xo.size, xs.size
    nxS, nyS, nxR = np.zeros(no, np.int32), np.zeros(no, np.int32), np.zeros(ns, np.int32)
    nyR = C.c_int(0)
    bm, bg = np.zeros(nxmodel, np.float32), np.zeros(nxmodel, np.int32)
    N.check(N.load().fwi_was_geometry(no, _p(xo), _p(zo), ns, _p(xs), _p(bt), C.c_float(shot_depth),
                                      C.c_float(dmodel), int(nxmodel), int(bool(relocate)), _p(nxS), _p(nyS),
                                      _p(nxR), C.byref(nyR), _p(bm), _p(bg)))
    return dict(nxSou=nxS, nySou=nyS, nxRec=nxR, nyRec=nyR.value, bat_model=bm, bat_model_grid=bg)


def time_rules(lam, dmodel, tfin, store_snap=10):
    """(dt, nt, nt_Store) of calculate_misfit_gradient.f90:198-203."""
    lam = _f32(lam)
    dt, nt, nts = C.c_float(0), C.c_int(0), C.c_int(0)
    N.check(N.load().fwi_time_rules(_p(lam), lam.shape[0], lam.shape[1], dmodel, tfin, store_snap, C.byref(dt),
                                    C.byref(nt), C.byref(nts)))
    return np.float32(dt.value), nt.value, nts.value


def set_filter_order(order: int = 6):
    """Butterworth order of time_filter (the reference's filters.f90 uses 6)."""
    N.check(N.load().fwi_set_filter_order(int(order)))


def time_filter(Data_trace, nt, dt, Num, typef, f1, fc):
    """time_filter (time_filter.f90:1): filters Data_trace(nt, Num) in place on
    the device.  Data_trace: float32 Fortran array (host) or an integer device
    address."""
    if isinstance(Data_trace, int):
        ptr = C.c_void_p(Data_trace)
    else:
        if Data_trace.dtype != np.float32 or not Data_trace.flags.f_contiguous:
            raise TypeError("Data_trace must be a float32 Fortran-ordered array")
        ptr = _p(Data_trace)
    N.check(N.load().fwi_time_filter(ptr, _ri(nt), _rf(dt), _ri(Num), _ri(typef), _rf(f1), _rf(fc)))
    return Data_trace


def interpolation_akima(Data_tmp, dt_Data, nt_Data, NumRec, dt, nt, out=None):
    """interpolation_akima (interpolation_akima.f90:1): resamples Data_tmp
    (nt_Data, NumRec) to (nt, NumRec) at step dt.  Host arrays, or integer
    device addresses for Data_tmp and `out` (then `out` is required)."""
    src = C.c_void_p(Data_tmp) if isinstance(Data_tmp, int) else None
    if src is None:
        Data_tmp = _f32(Data_tmp)
        src = _p(Data_tmp)
    if out is None:
        out = np.zeros((nt, NumRec), np.float32, order="F")
    dst = C.c_void_p(out) if isinstance(out, int) else _p(out)
    N.check(N.load().fwi_interpolation_akima(src, _rf(dt_Data), _ri(nt_Data), dst, _ri(NumRec), _rf(dt), _ri(nt)))
    return out


def su_info(path, big_endian=False):
    """(ns, dt, ntraces) of an SU file."""
    ns, dt, n = C.c_int(0), C.c_float(0), C.c_int(0)
    N.check(N.load().fwi_su_info(str(path).encode(), int(bool(big_endian)), C.byref(ns), C.byref(dt), C.byref(n)))
    return ns.value, np.float32(dt.value), n.value


def su_read(path, nt, ntr, big_endian=False):
    """The first ntr traces (nt samples each) of an SU file: (nt, ntr) float32,
    Fortran order, as get_shot_data reads a shot gather."""
    out = np.zeros((nt, ntr), np.float32, order="F")
    N.check(N.load().fwi_su_read(str(path).encode(), int(nt), int(ntr), int(bool(big_endian)), _p(out)))
    return out


def su_write(path, data, dt, big_endian=False):
    """data (nt, ntr) as an SU file (tracl, ns, dt headers), as write_new_data."""
    d = _f32(data)
    nt, ntr = d.shape
    N.check(N.load().fwi_su_write(str(path).encode(), _p(d), nt, ntr, C.c_float(dt), int(bool(big_endian))))


def su_supershot(paths, coding, nt, ntr, big_endian=False):
    """get_obs_data: the first ntr traces of each OBS file in `paths` summed
    with their coding factors, raw_data (nt, ntr) float32 Fortran order."""
    arr = (C.c_char_p * len(paths))(*[str(p).encode() for p in paths])
    cod = np.ascontiguousarray(coding, np.float32)
    if cod.size != len(paths):
        raise ValueError("one coding factor per file")
    out = np.zeros((nt, ntr), np.float32, order="F")
    N.check(N.load().fwi_su_supershot(arr, len(paths), _p(cod), int(nt), int(ntr), int(bool(big_endian)), _p(out)))
    return out


def read_nav(path):
    """Navigation list of MCS shots: (shot numbers int32, x float32, water
    depth float32), as read_nav_shot_mcs reads it."""
    n = C.c_int(0)
    N.check(N.load().fwi_read_nav(str(path).encode(), 0, None, None, None, C.byref(n)))
    ids, xs, bat = np.zeros(n.value, np.int32), np.zeros(n.value, np.float32), np.zeros(n.value, np.float32)
    N.check(N.load().fwi_read_nav(str(path).encode(), n.value, _p(ids), _p(xs), _p(bat), C.byref(n)))
    return ids, xs, bat


class _DescHolder:
    """Keeps the numpy arrays behind a FwiSurveyDesc alive."""

    def __init__(self, spec: SurveySpec, snap_form=0, grad_form=1, hbm_budget=0, wave_shots=0, band_rows=0,
                 flags=0, tile_kernel=0, tile_rows=0, tile_edge_rows=0):
        self.keep = []
        shots = (N.FwiShot * len(spec.shots))()
        for i, sh in enumerate(spec.shots):
            arrs = [_i32(sh.nxSou), _i32(sh.nySou), _i32(sh.nxRec), _i32(sh.nyRec),
                    _f32(np.asarray(sh.src).reshape(spec.nt, -1, order="F")) if sh.src is not None else None,
                    _f32(np.asarray(sh.obs).reshape(spec.nt, -1, order="F")) if sh.obs is not None else None]
            self.keep.extend(a for a in arrs if a is not None)
            shots[i] = N.FwiShot(sh.x0, sh.nx, len(sh.nxSou), len(sh.nxRec), _p(arrs[0]), _p(arrs[1]), _p(arrs[2]),
                                 _p(arrs[3]), _p(arrs[4]), _p(arrs[5]), sh.grad_weight, sh.misfit_weight)
        self.shots = shots
        water = None
        if spec.water_rows is not None:
            water = _i32(spec.water_rows)
            self.keep.append(water)
        self.desc = N.FwiSurveyDesc(spec.ny, spec.nx_model, spec.d, spec.dt, spec.nt, spec.store_snap, spec.acc,
                                    spec.dpml, spec.numtasks, snap_form, grad_form, len(spec.shots), shots,
                                    _p(water), hbm_budget, wave_shots, band_rows, flags, tile_kernel, tile_rows,
                                    tile_edge_rows)


class Survey:
    """Device-resident batched survey (fwi_survey_create & co)."""

    def __init__(self, spec: SurveySpec, snap_form=N.SNAP_F32, grad_form=N.GRAD_F64, hbm_budget=0, wave_shots=0,
                 band_rows=0, graph=True, recompute=False, two_step=True, tile_kernel=0, tile_rows=0,
                 tile_edge_rows=0, fused_step=False):
        """tile_kernel: 0 = the tuner's choice, 1 = register-queue, 2 = shared-queue
        two-step kernel; tile_rows: rows per two-step tile; tile_edge_rows: rows
        of the bottom edge band, the last two-step rows (0 = the tuner's;
        above the model's rows: the last core-height band); two_step=False:
        single steps; fused_step: single steps, one launch each."""
        self.spec = spec
        flags = ((0 if graph else N.SURVEY_NO_GRAPH) | (N.SURVEY_RECOMPUTE if recompute else 0)
                 | (0 if two_step else N.SURVEY_SINGLE_STEP) | (N.SURVEY_FUSED_STEP if fused_step else 0))
        self._h = _DescHolder(spec, snap_form, grad_form, hbm_budget, wave_shots, band_rows, flags, tile_kernel,
                              tile_rows, tile_edge_rows)
        handle = C.c_void_p()
        N.check(N.load().fwi_survey_create(C.byref(self._h.desc), C.byref(handle)))
        self.handle = handle
        self.nt, self.dt = spec.nt, spec.dt

    def close(self):
        if getattr(self, "_borrowed", False):  # the library owns it (batch_survey)
            self.handle = C.c_void_p()
            return
        if getattr(self, "handle", None) and self.handle.value:
            N.load().fwi_survey_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_lambda(self, lam):
        """lambda (ny, nx_model): numpy (host) array or an integer device address."""
        if isinstance(lam, int):
            N.check(N.load().fwi_survey_set_lambda(self.handle, C.c_void_p(lam)))
        else:
            self._lam = _f32(lam)
            N.check(N.load().fwi_survey_set_lambda(self.handle, _p(self._lam)))

    def set_observed(self, obs_packed):
        if isinstance(obs_packed, int):
            N.check(N.load().fwi_survey_set_observed(self.handle, C.c_void_p(obs_packed)))
        else:
            self._obs = np.ascontiguousarray(obs_packed, dtype=np.float32)
            N.check(N.load().fwi_survey_set_observed(self.handle, _p(self._obs)))

    def set_time(self, dt, nt, src_packed=None, obs_packed=None):
        """New time axis (dt, nt) with the sources and observed traces resampled
        to it, packed in shot order ((nt, n) column-major blocks): numpy arrays
        or integer device addresses; None = zeros (fwi_survey_set_time)."""
        def arg(a, keep):
            if a is None:
                return None
            if isinstance(a, int):
                return C.c_void_p(a)
            arr = np.ascontiguousarray(a, dtype=np.float32)
            setattr(self, keep, arr)
            return _p(arr)
        N.check(N.load().fwi_survey_set_time(self.handle, C.c_float(dt), int(nt), arg(src_packed, "_src_t"),
                                             arg(obs_packed, "_obs_t")))
        self.nt, self.dt = int(nt), float(dt)

    def run(self, step=1, grad=None, misfit=0.0):
        """Returns (misfit + this run's misfit, grad) where grad (ny, nx_model)
        float32 Fortran array is updated in place if given."""
        m = C.c_double(misfit)
        if grad is not None and (grad.dtype != np.float32 or not grad.flags.f_contiguous):
            raise TypeError("grad must be a float32 Fortran-ordered array")
        N.check(N.load().fwi_survey_run(self.handle, step, C.byref(m), _p(grad)))
        return m.value, grad

    def run_device_grad(self, step=1, grad_dev_ptr=None):
        m = C.c_double(0.0)
        N.check(N.load().fwi_survey_run(self.handle, step, C.byref(m),
                                        None if grad_dev_ptr is None else C.c_void_p(grad_dev_ptr)))
        return m.value

    def synthetic(self, shot):
        nrec = len(self.spec.shots[shot].nxRec)
        out = np.zeros((self.nt, nrec), np.float32, order="F")
        N.check(N.load().fwi_survey_get_synthetic(self.handle, shot, _p(out)))
        return out

    def stack(self):
        """The FP64 gradient stack of the last step-1 run, (ny, nx_model) Fortran
        order, before the numtasks divisor and the water mask."""
        out = np.zeros((self.spec.ny, self.spec.nx_model), np.float64, order="F")
        N.check(N.load().fwi_survey_get_stack(self.handle, _p(out)))
        return out

    def grad_stack_device_ptr(self):
        p = C.c_void_p()
        N.check(N.load().fwi_survey_grad_device(self.handle, C.byref(p)))
        return p.value

    def step_bytes(self):
        b = C.c_double(0)
        N.check(N.load().fwi_survey_step_bytes(self.handle, C.byref(b)))
        return b.value

    def two_step_bytes(self):
        """(algorithmic bytes per time step with two-step passes, two-step tiles' bytes per pass)."""
        a, t = C.c_double(0), C.c_double(0)
        N.check(N.load().fwi_survey_two_step_bytes(self.handle, C.byref(a), C.byref(t)))
        return a.value, t.value

    def tuning(self):
        w, b = C.c_int(0), C.c_int(0)
        N.check(N.load().fwi_survey_tuning(self.handle, C.byref(w), C.byref(b)))
        return w.value, b.value

    def tiles(self):
        """(tile kernel 1|2 or 0 without two-step tiles, rows per tile, {(kernel, rows): ms per
        forward two-step pass of the first wave} as measured by the tuner)."""
        k, r, n = C.c_int(0), C.c_int(0), C.c_int(0)
        cand = (C.c_int * 8)()
        times = (C.c_float * 16)()
        N.check(N.load().fwi_survey_tiles(self.handle, C.byref(k), C.byref(r), cand, times, C.byref(n)))
        meas = {}
        for kk in range(2):
            for c in range(n.value):
                if times[kk * n.value + c] >= 0:
                    meas[(kk + 1, cand[c])] = float(times[kk * n.value + c])
        return k.value, r.value, meas

    def edge_tiles(self):
        """(rows of the bottom edge band, 0 = the last core-height band; {rows:
        ms per forward two-step pass of the first wave} as measured by the
        tuner)."""
        e, n = C.c_int(0), C.c_int(0)
        cand = (C.c_int * 8)()
        times = (C.c_float * 8)()
        N.check(N.load().fwi_survey_edge_tiles(self.handle, C.byref(e), cand, times, C.byref(n)))
        return e.value, {cand[c]: float(times[c]) for c in range(n.value) if times[c] >= 0}

    def stepping(self):
        """("two-step" | "single" | "single-fused", {form: ms}): the survey's
        time stepping ("single-fused": one launch per step) and the tuner's
        timings of the first wave per two time steps (empty where not
        measured: a forced or cached choice)."""
        t, a, b, c = C.c_int(0), C.c_float(0.0), C.c_float(0.0), C.c_float(0.0)
        N.check(N.load().fwi_survey_stepping(self.handle, C.byref(t), C.byref(a), C.byref(b), C.byref(c)))
        times = {k: float(v.value) for k, v in (("two-step", a), ("single", b), ("single-fused", c)) if v.value >= 0}
        return {0: "single", 1: "two-step", 2: "single-fused"}[t.value], times

    def launch_form(self, step=1):
        """("graph" | "direct" | "undecided", direct-launch ms, graph-replay ms)
        of the first wave's runs with this step: the first run of a time axis
        is timed as direct launches, the first replay of its graph as a
        replay, and the slower form is dropped."""
        f, d, g = C.c_int(0), C.c_float(0.0), C.c_float(0.0)
        N.check(N.load().fwi_survey_launch_form(self.handle, int(step), C.byref(f), C.byref(d), C.byref(g)))
        return {0: "undecided", 1: "graph", 2: "direct"}[f.value], float(d.value), float(g.value)

    def recompute_plan(self):
        """(forward steps per segment, segments); (0, 0) without recomputation."""
        c, j = C.c_int(0), C.c_int(0)
        N.check(N.load().fwi_survey_recompute(self.handle, C.byref(c), C.byref(j)))
        return c.value, j.value

    def time_steps(self, steps):
        N.check(N.load().fwi_survey_time_steps(self.handle, steps))


def calculate_misfit_gradient(spec: SurveySpec, lam, step, Misfit, Grad, snap_form=N.SNAP_F32,
                              grad_form=N.GRAD_F64, flags=0):
    """calculate_misfit_gradient over every shot of `spec` in one call with
    host buffers.  Returns the updated Misfit (float32); Grad (ny, nx_model)
    float32 Fortran array is updated in place (step=1).  flags: SURVEY_* bits
    of the plan (part of its key)."""
    h = _DescHolder(spec, snap_form, grad_form, flags=flags)
    lam = _f32(lam)
    m = C.c_float(Misfit)
    N.check(N.load().fwi_misfit_gradient_batch(C.byref(h.desc), _p(lam), step, C.byref(m), _p(Grad)))
    return np.float32(m.value)


def batch_survey():
    """The survey of fwi_misfit_gradient_batch's current plan (owned by the
    library) for the query methods -- tiles(), edge_tiles(), stepping(),
    launch_form(), tuning() -- or None before the first call.  Valid until the
    batch call changes geometry or the plan is released."""
    h = C.c_void_p()
    N.check(N.load().fwi_batch_survey(C.byref(h)))
    if not h.value:
        return None
    v = Survey.__new__(Survey)
    v.handle = h
    v.spec = None
    v._borrowed = True
    return v


def batch_release():
    """Release fwi_misfit_gradient_batch's plan (its survey and buffers)."""
    N.check(N.load().fwi_batch_release())
