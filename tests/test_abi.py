"""The C-ABI library: it loads, exports every entry point the header
declares, rejects use without a device cleanly, and its host-side FP32
arithmetic (geometry, Ricker, time rules) is bit-exact against the golden
vectors from the reference source.  No kernel is launched here."""
import ctypes
import os
import re

import numpy as np
import pytest

from tests.conftest import ROOT

HEADER = os.path.join(ROOT, "include", "fwi_gb300.h")


def declared_symbols():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(fwi_[a-z0-9_]+)\s*\(", txt)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("fwi_solver_acoustic_ss", "fwi_misfit_function", "fwi_beta_calculous", "fwi_misfit_gradient_batch"):
        assert s in syms


def test_library_exports_every_declared_symbol():
    import fwi_gb300._native as N
    lib = N.load()
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    assert set(N.EXPORTS) == set(declared_symbols())


def test_library_has_no_torch_dependency():
    # the product library is self-contained: plain C ABI over the CUDA runtime
    so = open(os.path.join(ROOT, "fwi_gb300", "_lib", "libfwi_gb300.so"), "rb").read()
    assert b"libtorch" not in so and b"libc10" not in so


def test_geometry_ricker_time_rules_bit_exact(golden):
    from fwi_gb300 import api
    g = golden("geometry")
    for t in "abc":
        f0, dtm, ntm = g[f"ricker_{t}_par"]
        assert np.array_equal(api.Ricker_mcs(float(f0), float(dtm), int(ntm)), g[f"ricker_{t}"])
    for t in "abcd":
        xs, sd, rd, near, drec, dm = (float(v) for v in g[f"geom_{t}_par"])
        a, b, c, d = api.mcs_geometry(xs, sd, rd, near, drec, dm, int(g[f"geom_{t}_nrec"]))
        assert a == g[f"geom_{t}_nxSou"] and b == g[f"geom_{t}_nySou"]
        assert np.array_equal(c, g[f"geom_{t}_nxRec"]) and np.array_equal(d, g[f"geom_{t}_nyRec"])
        dm, tf = (float(v) for v in g[f"time_{t}_par"])
        dt, nt, nts = api.time_rules(g[f"time_{t}_lambda"], dm, tf)
        assert dt == g[f"time_{t}_dt"] and nt == g[f"time_{t}_nt"] and nts == g[f"time_{t}_ntstore"]


def test_was_geometry_bit_exact(golden):
    """fwi_was_geometry (host FP32) against the statements of
    get_was_data.f90 executed from the reference: shot and OBS columns, the
    bathymetry model by INTRPL and its rows, the OBS relocated to it."""
    from fwi_gb300 import api
    z = golden("was_geometry")
    args = (z["xobs"], z["zobs"], z["xs"], z["bat"], float(z["shot_depth"]), float(z["dmodel"]), int(z["nxmodel"]))
    g = api.was_geometry(*args)
    assert np.array_equal(g["bat_model"], z["bat_model_was"])
    assert np.array_equal(g["bat_model_grid"], z["bat_model_grid_was"])
    assert np.array_equal(g["nxSou"], z["nxsou_was"]) and np.array_equal(g["nySou"], z["nysou_was"])
    assert np.array_equal(g["nxRec"], z["nxrec_was"][:, 0]) and g["nyRec"] == z["nyrec_was"][0, 0]
    assert np.array_equal(api.was_geometry(*args, relocate=False)["nySou"], z["zobs_grid_nav"])


def test_argument_errors_are_reported():
    from fwi_gb300 import _native as N
    lib = N.load()
    assert lib.fwi_set_solver_options(5, 20) == N.FWI_ERR_ARG
    assert b"acc" in lib.fwi_last_error()
    assert lib.fwi_set_solver_options(3, 0) == N.FWI_ERR_ARG
    assert lib.fwi_set_solver_options(3, 20) == 0
    assert lib.fwi_ricker(ctypes.c_float(-1.0), ctypes.c_float(0.001), 10, None) == N.FWI_ERR_ARG


def test_corner_factor_rule_matches_reference_matrices(golden):
    """The kernels index the corner CPML factors as A(max(j, dn-1-i)) (left
    corner) and A(max(i, j)) (right corner), 0-based; check the rule against
    the reference's ld/rd matrices (solver_PML_coeffs.f90:240-267)."""
    g = golden("coeffs")
    for tag in "abc":
        fA = g[f"pml_{tag}_fA"]
        ld, rd, lu, ru = g[f"pml_{tag}_cornA"]
        dn = fA.size
        j, i = np.meshgrid(np.arange(dn), np.arange(dn), indexing="ij")
        assert np.array_equal(ld, fA[np.maximum(j, dn - 1 - i)])
        assert np.array_equal(rd, fA[np.maximum(i, j)])


def test_no_device_is_an_error_not_a_crash():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    from fwi_gb300 import _native as N
    rc = N.load().fwi_init(0)
    assert rc in (N.FWI_ERR_CUDA, N.FWI_ERR_ARG)
    assert N.load().fwi_last_error()
