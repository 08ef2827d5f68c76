"""The allocation-free forward solver (fwi_solver_forward_noalloc).

It exists for callers that cannot call cudaMalloc -- code inside a framework
that owns the device memory pool, or code that must not allocate once set
up -- and keeps all of its working state in one fixed 16 MiB device array.
This file is collected last so that, if it fails, every other test has run.
Device buffers here come from torch (the test allocates; the entry point
does not).  Its traces must equal the drop-in solver's (iprop = 3), bit for
bit like every solver test, on two calls in a row: the shared array keeps
the previous call's contents, so the second call checks the clearing.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(seed, ny, nx, nt, nsou=2, nrec=30, acc=3, dpml=20):
    rng = np.random.default_rng(seed)
    dn = dpml + 2 * acc
    return dict(
        ny=ny, nx=nx, nt=nt, acc=acc, dpml=dpml, d=12.5, dt=0.001,
        ctmp=np.asfortranarray((1500 + 1500 * rng.random((ny, nx))).astype(np.float32)),
        S=np.asfortranarray(rng.standard_normal((nt, nsou)).astype(np.float32)),
        nxSou=np.array([nx // 2] + list(rng.integers(1, nx + 1, nsou - 1)), np.int32),
        nySou=np.array([3] + list(rng.integers(1, ny + 1, nsou - 1)), np.int32),
        nxRec=rng.integers(-dn + 1, nx + dn, nrec).astype(np.int32),
        nyRec=rng.integers(1, ny + dn, nrec).astype(np.int32))


def _reference_entry(z):
    import fwi_gb300 as F
    F.set_solver_options(z["acc"], z["dpml"])
    nrec = len(z["nxRec"])
    rec = np.zeros((z["nt"], nrec), np.float32, order="F")
    F.solver_acoustic_SS(0, 3, len(z["nxSou"]), nrec, z["nxSou"], z["nySou"], z["nxRec"], z["nyRec"], z["S"], None,
                         z["d"], z["dt"], z["ny"], z["nx"], z["ctmp"], 10, z["nt"] // 10, z["nt"], None, None, rec)
    return rec


def _noalloc(z, calls=1):
    """Device buffers from torch, then `calls` calls of the entry point.
    Returns the traces and the device's free bytes (cudaMemGetInfo) before
    and after each call."""
    import torch

    import fwi_gb300 as F
    F.set_solver_options(z["acc"], z["dpml"])
    lib = F.load()
    dev = torch.device("cuda", 0)
    S = torch.from_numpy(z["S"].reshape(-1, order="F").copy()).to(dev)
    ct = torch.from_numpy(z["ctmp"].reshape(-1, order="F").copy()).to(dev)
    nrec = len(z["nxRec"])
    rec = torch.full((nrec * z["nt"],), 5.0, dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    free = []
    for _ in range(calls):
        f0 = torch.cuda.mem_get_info(dev)[0]
        rc = lib.fwi_solver_forward_noalloc(len(z["nxSou"]), nrec, p(z["nxSou"]), p(z["nySou"]), p(z["nxRec"]),
                                            p(z["nyRec"]), C.c_void_p(S.data_ptr()), z["d"], z["dt"], z["ny"],
                                            z["nx"], C.c_void_p(ct.data_ptr()), z["nt"], C.c_void_p(rec.data_ptr()))
        assert rc == 0, lib.fwi_last_error()
        torch.cuda.synchronize()
        free.append((f0, torch.cuda.mem_get_info(dev)[0]))
    return rec.cpu().numpy().reshape(z["nt"], nrec, order="F"), free


def test_noalloc_matches_drop_in_on_two_calls():
    import fwi_gb300 as F
    F.init(0)
    for z in (_case(1, 60, 150, 300), _case(2, 40, 333, 250, acc=4)):
        ref = _reference_entry(z)
        first, _ = _noalloc(z)
        second, _ = _noalloc(z)
        assert np.abs(ref).max() > 0
        np.testing.assert_array_equal(first, ref)
        np.testing.assert_array_equal(second, ref)


def test_noalloc_leaves_device_memory_untouched():
    """The property the entry point exists for: once the library is set up
    and a first call has been made, a call takes no device memory -- the free
    bytes the driver reports are the same before and after it."""
    import fwi_gb300 as F
    F.init(0)
    z = _case(4, 50, 200, 200)
    traces, free = _noalloc(z, calls=3)
    np.testing.assert_array_equal(traces, _reference_entry(z))
    for before, after in free[1:]:
        assert before == after, f"free device memory changed across a call: {before} -> {after}"


def test_noalloc_rejects_grids_beyond_its_scratch():
    import fwi_gb300 as F
    F.init(0)
    z = _case(3, 400, 2000, 20)
    with pytest.raises(AssertionError, match="fixed limit"):
        _noalloc(z)
