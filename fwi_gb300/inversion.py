"""NLCG full-waveform inversion over the device gradient path.

The host driver mirrors the reference's Fortran driver:

* ``fwi_band``  -- FWI.f90 (one frequency band): the gradient of the current
  model, the Polak–Ribière search direction (Beta_calculous, with its two dot
  products in FP64 on the device), the line search that halves the trial step
  while the first trial raises the misfit and doubles it while the misfit
  falls (at most 6 trials, then the iteration is repeated once), the quadratic
  fit of ``polyfit`` for the final step, and the model update
  ``lambda = exp(Search*step)*var_orig`` (FWI.f90:118-317);
* ``invert``    -- the band loop of 00-main_Inversion.f90:83-98 (frequency
  continuation, one ``fwi_band`` per band, the global iteration count carried
  across bands);
* ``polyfit``   -- polyfit.f90:1-100 with the scaled-partial-pivoting Gaussian
  elimination it calls (LEGS/ELGS, T. Pang, *An Introduction to
  Computational Physics*), in FP64 with the reference's FP32 trial points.

The search direction is FP32 numpy, as the reference's REAL arrays; the first
trial step and the exponential model update run on the device
(``DeviceModelOps``).  ``DeviceGradient`` is calculate_misfit_gradient for
all shots on the device: the observed traces and the source are filtered once
per band (``time_filter``), every call takes dt and nt from the trial model
(``time_rules``), resamples the filtered traces to them
(``interpolation_akima``) and runs the batched survey (``fwi_survey_*``).
"""
from __future__ import annotations

import dataclasses
from typing import Callable, List, Optional, Tuple

import numpy as np

from . import _native as N
from . import api
from .survey import SurveySpec

F32 = np.float32


# ---------------------------------------------------------------------------
# polyfit (polyfit.f90)
# ---------------------------------------------------------------------------

def _solve_scaled_pivoting(A: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Solve A x = b (3x3, float64) by Gaussian elimination with scaled
    partial pivoting: row scale factors from the largest |a_ij| of each row,
    pivot = the row with the largest |a_ij|/scale in the column, the
    elimination ratios stored below the diagonal, then forward substitution
    of b in pivot order and back substitution (the LEGS/ELGS pair called by
    polyfit.f90:44, :79)."""
    A = np.array(A, dtype=np.float64)
    b = np.array(b, dtype=np.float64)
    n = A.shape[0]
    idx = list(range(n))
    c = [max(abs(A[i, j]) for j in range(n)) for i in range(n)]
    for j in range(n - 1):
        best, k = 0.0, j
        for i in range(j, n):
            r = abs(A[idx[i], j]) / c[idx[i]]
            if r > best:
                best, k = r, i
        idx[j], idx[k] = idx[k], idx[j]
        for i in range(j + 1, n):
            pj = A[idx[i], j] / A[idx[j], j]
            A[idx[i], j] = pj
            for kk in range(j + 1, n):
                A[idx[i], kk] = A[idx[i], kk] - pj * A[idx[j], kk]
    for i in range(n - 1):
        for j in range(i + 1, n):
            b[idx[j]] = b[idx[j]] - A[idx[j], i] * b[idx[i]]
    x = np.zeros(n)
    x[n - 1] = b[idx[n - 1]] / A[idx[n - 1], n - 1]
    for i in range(n - 2, -1, -1):
        x[i] = b[idx[i]]
        for j in range(i + 1, n):
            x[i] = x[i] - A[idx[i], j] * x[j]
        x[i] = x[i] / A[idx[i], i]
    return x


def polyfit(nut, misfit, misfit_test1, misfit_test, loopind) -> np.float32:
    """Step of the line search (polyfit.f90:1-100): the parabola through the
    three (step, misfit) trials is sampled at 2001 points of [0, nut]
    (loopind = 2: trials at 0, nut/2, nut) or [nut/4, nut] (loopind > 2: trials
    at nut/4, nut/2, nut) and the last sample attaining the minimum is
    returned as an FP32 step.  Steps are normalised by their mean and sample
    standard deviation before the fit.  loopind < 2 leaves the step at 0."""
    nut = F32(nut)
    length = 2001
    if loopind == 2:
        v = np.array([0.0, float(F32(F32(0.5) * nut)), float(nut)])
    elif loopind > 2:
        v = np.array([float(F32(F32(0.25) * nut)), float(F32(F32(0.5) * nut)), float(nut)])
    else:
        return F32(0.0)
    mean = (v[0] + v[1] + v[2]) / 3.0
    d = v - mean
    std = float(np.power(np.float64(0.5 * ((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2])), 0.5))
    vn = (v - mean) / std
    A = np.array([[vn[j] ** 0 if i == 0 else (vn[j] if i == 1 else vn[j] * vn[j]) for i in range(3)] for j in range(3)])
    y = np.array([float(F32(misfit)), float(F32(misfit_test1)), float(F32(misfit_test))])
    coef = _solve_scaled_pivoting(A, y)
    j = np.arange(length, dtype=np.float32)
    if loopind == 2:
        grid = ((j * nut).astype(np.float32) / F32(length - 1)).astype(np.float32)
    else:
        grid = (F32(F32(0.25) * nut) + ((j * F32(F32(0.75) * nut)).astype(np.float32) / F32(length - 1))
                .astype(np.float32)).astype(np.float32)
    g = grid.astype(np.float64)
    t = (g - mean) / std
    poly = t * t * coef[2] + t * coef[1] + coef[0]
    last = int(np.nonzero(poly == poly.min())[0][-1])
    return F32(g[last])


# ---------------------------------------------------------------------------
# gradient backend: calculate_misfit_gradient on the device
# ---------------------------------------------------------------------------

@dataclasses.dataclass
class RawData:
    """Recorded data of a survey at the acquisition sampling: observed traces
    of all shots packed in shot order, (nt_data, ntr) column-major, and the
    source wavelet S0(nt_data) shared by every shot (the MCS case of
    calculate_misfit_gradient.f90:173-174)."""
    obs: np.ndarray
    src: np.ndarray
    dt_data: float

    @property
    def nt_data(self) -> int:
        return int(self.obs.shape[0])

    @property
    def tfin(self) -> np.float32:
        # tfin_mcs = (nt_mcs-1)*dt_mcs  (modules.f90:445)
        return F32(F32(self.nt_data - 1) * F32(self.dt_data))


class DeviceGradient:
    """calculate_misfit_gradient(step, lambda) over every shot of ``spec`` on
    the device.  ``set_band`` filters the observed traces and the source once
    per band (time_filter, calculate_misfit_gradient.f90:193-194); every call
    derives dt and nt from the model (calculate_misfit_gradient.f90:198-203),
    resamples the filtered traces (interpolation_akima, :241-244) and runs the
    batched survey.  Returns (misfit, Grad) with Grad updated as the reference
    does (Grad + stack/numtasks, water rows zeroed) for step 1."""

    def __init__(self, spec: SurveySpec, raw: RawData, snap_form=N.SNAP_F32, grad_form=N.GRAD_F64,
                 hbm_budget=0, store_snap=10, typef=1, device=0):
        import torch
        self.torch = torch
        self.spec = spec
        self.raw = raw
        self.snap_form, self.grad_form, self.hbm_budget = snap_form, grad_form, hbm_budget
        self.store_snap = store_snap
        self.typef = typef
        self.dev = torch.device("cuda", device)
        self.ntr = sum(len(s.nxRec) for s in spec.shots)
        self.nsou = [len(s.nxSou) for s in spec.shots]
        if raw.obs.shape[1] != self.ntr:
            raise ValueError("raw observed traces do not match the survey's receivers")
        # column-major (nt, n) arrays live on the device as row-major (n, nt)
        self.obs_raw = torch.from_numpy(np.ascontiguousarray(np.asarray(raw.obs, np.float32).T)).to(self.dev)
        self.src_raw = torch.from_numpy(np.ascontiguousarray(np.asarray(raw.src, np.float32)[None, :])).to(self.dev)
        self.obs_band = self.obs_raw.clone()
        self.src_band = self.src_raw.clone()
        self.survey = None
        self.cur = None  # (dt, nt, band id) of the data in the survey
        self.band_id = 0
        self.calls = 0
        # wall time (s): resampling the data to a new time axis, moving the
        # survey to it (fwi_survey_set_time: re-plan when nt changes), the
        # first run on each axis (direct launches) and the later runs
        self.times = {"resample": 0.0, "set_time": 0.0, "first_runs": 0.0, "runs": 0.0}
        self.axes = 0
        self._fresh = False

    def set_source(self, wavelet):
        """Replace the source wavelet S0(nt_data) (source estimation); the
        next set_band filters it."""
        w = np.asarray(wavelet, np.float32).reshape(1, -1)
        self.src_raw = self.torch.from_numpy(np.ascontiguousarray(w)).to(self.dev)
        self.src_band = self.src_raw.clone()

    def set_band(self, f1, f2):
        torch = self.torch
        self.obs_band.copy_(self.obs_raw)
        self.src_band.copy_(self.src_raw)
        nt, dt = self.raw.nt_data, self.raw.dt_data
        api.time_filter(self.obs_band.data_ptr(), nt, dt, self.ntr, self.typef, f1, f2)
        api.time_filter(self.src_band.data_ptr(), nt, dt, 1, self.typef, f1, f2)
        torch.cuda.synchronize(self.dev)
        self.band_id += 1

    def _prepare(self, lam):
        import time
        torch = self.torch
        t0 = time.perf_counter()
        dt, nt, _ = api.time_rules(lam, self.spec.d, self.raw.tfin, self.store_snap)
        key = (float(dt), int(nt), self.band_id)
        if key == self.cur:
            return
        obs = torch.empty((self.ntr, nt), dtype=torch.float32, device=self.dev)
        api.interpolation_akima(self.obs_band.data_ptr(), self.raw.dt_data, self.raw.nt_data, self.ntr, dt, nt,
                                out=obs.data_ptr())
        s1 = torch.empty((1, nt), dtype=torch.float32, device=self.dev)
        api.interpolation_akima(self.src_band.data_ptr(), self.raw.dt_data, self.raw.nt_data, 1, dt, nt,
                                out=s1.data_ptr())
        src = s1.expand(sum(self.nsou), nt).contiguous()
        torch.cuda.synchronize(self.dev)
        t1 = time.perf_counter()
        self.times["resample"] += t1 - t0
        if self.survey is None:
            shots = [dataclasses.replace(sh, obs=None, src=None) for sh in self.spec.shots]
            spec = dataclasses.replace(self.spec, nt=int(nt), dt=float(dt), shots=shots)
            self.survey = api.Survey(spec, snap_form=self.snap_form, grad_form=self.grad_form,
                                     hbm_budget=self.hbm_budget)
        self.survey.set_time(float(dt), int(nt), src.data_ptr(), obs.data_ptr())
        self._keep = (obs, src)
        self.cur = key
        self.times["set_time"] += time.perf_counter() - t1
        self.axes += 1
        self._fresh = True

    def __call__(self, lam: np.ndarray, step: int, grad: Optional[np.ndarray] = None) -> Tuple[float, Optional[np.ndarray]]:
        import time
        lam = np.asfortranarray(lam, dtype=np.float32)
        self._prepare(lam)
        t0 = time.perf_counter()
        self.survey.set_lambda(lam)
        m, g = self.survey.run(step, grad if step == 1 else None)
        self.times["first_runs" if self._fresh else "runs"] += time.perf_counter() - t0
        self._fresh = False
        self.calls += 1
        return m, g

    def close(self):
        if self.survey is not None:
            self.survey.close()
            self.survey = None


# ---------------------------------------------------------------------------
# FWI.f90 and the band loop
# ---------------------------------------------------------------------------

@dataclasses.dataclass
class IterationLog:
    iter: int
    band: Tuple[float, float]
    misfit: float              # misfit of the model at the start of the iteration
    step: float                # EndStep of the line search
    trials: List[Tuple[float, float]]  # (nut, misfit) of every line-search trial
    beta: Optional[float]
    model_error: Optional[float] = None


def _beta(grad: np.ndarray, old: np.ndarray) -> float:
    ny, nx = grad.shape
    return float(api.Beta_calculous(grad, old, nx, ny)[0])


class DeviceModelOps:
    """The model arithmetic of FWI.f90 on the device: the first trial step
    1/100/maxval(abs(Search/log(var_orig))) (FWI.f90:175, fwi_first_step) and
    the update exp(Search*step)*var_orig (FWI.f90:227, :315,
    fwi_model_update), in the reference's FP32 operations with exp and log
    rounded once from FP64."""

    @staticmethod
    def first_step(search: np.ndarray, var_orig: np.ndarray) -> np.float32:
        return api.first_step(search, var_orig)

    @staticmethod
    def update(search: np.ndarray, var_orig: np.ndarray, step) -> np.ndarray:
        return api.model_update(search, var_orig, step)


def fwi_band(lam: np.ndarray, gradient: Callable, f1: float, f2: float, n_iter: int, iter0: int = 1,
             method: int = 1, beta_fn: Callable = _beta, vp_true: Optional[np.ndarray] = None,
             log: Optional[List[IterationLog]] = None, ops=DeviceModelOps) -> Tuple[np.ndarray, int]:
    """FWI(iter, f1, f2) (FWI.f90:1-368) for one band: n_iter NLCG iterations
    with the reference's line search.  lam (ny, nx) FP32 is the starting
    model (the reference's global lambda); returns the final model and the
    next global iteration number.  ``gradient(lam, step, grad)`` is
    calculate_misfit_gradient over all shots (step 1: misfit and gradient,
    step 2: misfit only); ``ops`` the model arithmetic (first trial step and
    exponential update), on the device by default."""
    lam = np.asfortranarray(lam, dtype=np.float32).copy()
    ny, nx = lam.shape
    var_orig = lam.copy()
    old_grad = np.zeros((ny, nx), np.float32, order="F")
    search = np.zeros((ny, nx), np.float32, order="F")
    end_step = F32(0.0)
    irep = 0
    it = iter0
    i_fwi = 1
    while i_fwi <= n_iter:
        i_fwi += 1
        grad = np.zeros((ny, nx), np.float32, order="F")
        misfit, _ = gradient(lam, 1, grad)
        misfit = F32(misfit)
        beta = None
        if method == 1:                                   # NLCG (FWI.f90:158-171)
            if i_fwi - 1 == 1:
                search = -grad
            else:
                beta = beta_fn(grad, old_grad)
                search = (-grad + F32(beta) * search) if beta > 0.0 else -grad
        else:
            search = -grad
        search = np.asfortranarray(search, dtype=np.float32)
        old_grad = grad
        # first trial step: 1 % of the largest relative model change (FWI.f90:186-190)
        if end_step == 0.0:
            nut = F32(ops.first_step(search, var_orig))
        else:
            nut = end_step
        m_test0 = m_test1 = misfit
        m_test = misfit
        loopind = looptotal = 0
        looptest = False
        trials = []
        restart = False
        while not looptest:                               # line search (FWI.f90:206-274)
            loopind += 1
            looptotal += 1
            lam = ops.update(search, var_orig, nut)
            if loopind >= 2:
                m_test0 = m_test1
                m_test1 = m_test
            m_test, _ = gradient(lam, 2, None)
            m_test = F32(m_test)
            trials.append((float(nut), float(m_test)))
            if looptotal > 6:                             # give up: repeat the iteration once, then stop
                end_step = F32(0.0)
                search = np.zeros_like(search)
                irep += 1
                if irep >= 2:
                    i_fwi = n_iter + 1
                else:
                    i_fwi -= 1
                restart = True
                break
            if F32(m_test - misfit) >= 0.0 and loopind == 1:
                nut = F32(nut / F32(2.0))
                loopind = 0
                continue
            if F32(m_test - m_test1) <= 0.0:
                nut = F32(nut * F32(2.0))
            else:
                looptest = True
        if restart:
            continue
        end_step = polyfit(nut, misfit if loopind == 2 else m_test0, m_test1, m_test, loopind)
        lam = ops.update(search, var_orig, end_step)
        var_orig = lam.copy()
        err = None
        if vp_true is not None:
            vp = np.sqrt(lam / F32(1000.0))
            err = float(np.linalg.norm(vp - vp_true) / np.linalg.norm(vp_true))
        if log is not None:
            log.append(IterationLog(it, (f1, f2), float(misfit), float(end_step), trials, beta, err))
        it += 1
    return lam, it


def invert(lam0: np.ndarray, gradient, bands: List[Tuple[float, float]], n_iter: int,
           estimate_source: Optional[Callable] = None, **kw):
    """Frequency continuation (00-main_Inversion.f90:83-98): fwi_band for every
    (f1, f2) band in turn, the model and the global iteration count carried
    over.  ``gradient.set_band(f1, f2)`` (when present) re-filters the data.
    ``estimate_source(lam, f1, f2)`` (inv_source = 1, FWI.f90:103-107) gives
    the band's wavelet, handed to ``gradient.set_source`` before filtering.
    Returns (final model, list of IterationLog)."""
    log: List[IterationLog] = []
    lam, it = np.asfortranarray(lam0, dtype=np.float32), 1
    for f1, f2 in bands:
        if estimate_source is not None:
            gradient.set_source(estimate_source(lam, f1, f2))
        if hasattr(gradient, "set_band"):
            gradient.set_band(f1, f2)
        lam, it = fwi_band(lam, gradient, f1, f2, n_iter, iter0=it, log=log, **kw)
    return lam, log
