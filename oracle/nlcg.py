"""FWI.f90's model arithmetic restated in numpy FP32 (TEST INFRASTRUCTURE ONLY:
the checker of fwi_first_step / fwi_model_update and the model arithmetic of
the CPU-only NLCG tests; the product runs it on the device).

    first_step: nut = 1/100/maxval(abs(Search/log(var_orig)))   FWI.f90:175
    update:     lambda = exp(Search*step)*var_orig              FWI.f90:227, :315

The reference evaluates log and exp in FP32 (REAL); numpy's float32 log/exp
stand in for them here, and may differ from a correctly rounded result in the
last place.
"""
import numpy as np

F32 = np.float32


class HostModelOps:
    @staticmethod
    def first_step(search, var_orig):
        with np.errstate(divide="ignore", invalid="ignore"):
            q = np.abs(np.asarray(search, F32) / np.log(np.asarray(var_orig, F32)))
        return F32(F32(F32(1.0) / F32(100.0)) / np.nanmax(q))

    @staticmethod
    def update(search, var_orig, step):
        with np.errstate(over="ignore"):
            return np.asfortranarray((np.exp(np.asarray(search, F32) * F32(step)) * np.asarray(var_orig, F32))
                                     .astype(F32))


def first_step_rounded(search, var_orig):
    """first_step with log evaluated in float64 and rounded once to FP32."""
    lg = np.log(np.asarray(var_orig, F32).astype(np.float64)).astype(F32)
    with np.errstate(divide="ignore", invalid="ignore"):
        q = np.abs(np.asarray(search, F32) / lg)
    return F32(F32(F32(1.0) / F32(100.0)) / np.nanmax(q))


def update_rounded(search, var_orig, step):
    """update with exp evaluated in float64 and rounded once to FP32."""
    t = (np.asarray(search, F32) * F32(step)).astype(F32)
    with np.errstate(over="ignore"):
        e = np.exp(t.astype(np.float64)).astype(F32)
        return np.asfortranarray((e * np.asarray(var_orig, F32)).astype(F32))
