"""Oracle pin for temporal accumulation: vo_taa against the reference's own
LightTAA.frag main compiled on the host (oracle/_ref), with the sampler and
sin/cos this library defines for the pass, bit for bit (NaN == NaN)."""
import ctypes as C

import numpy as np

import oracle
from tests import taa_cases
from tests.gpu_util import same_bits

fp = C.POINTER(C.c_float)


def test_taa_matches_reference(ref_lib):
    R = ref_lib
    R.ref_taa.argtypes = [fp] * 8 + [C.c_int, C.c_int, fp]
    R.ref_taa_set_sincos.argtypes = [C.c_void_p]
    R.ref_taa_set_sincos(C.cast(oracle.lib().vo_sincos, C.c_void_p))
    for seed, (W, H) in enumerate([(48, 32), (67, 41)]):
        fr = taa_cases.frame(W, H, seed)
        keys = ("light", "last", "color", "normal", "material", "depth", "motion", "noise")
        want = np.zeros((H, W, 4), np.float32)
        R.ref_taa(*[fr[k].ctypes.data_as(fp) for k in keys], W, H, want.ctypes.data_as(fp))
        got = oracle.taa(*[fr[k] for k in keys])
        assert same_bits(got, want).all()
        # every branch ran: sky (copied light; rows 0-1 sample only sky), disocclusion
        # (alpha 1), spiral (alpha in [0, 1])
        assert np.allclose(got[:2], fr["light"][:2], atol=1e-5)  # the sampled light, unfiltered
        assert (got[3:, :4, 3] == 1.0).all()
        assert np.isfinite(got[3:, 8:]).all() and (got[3:, 8:, 3] < 1.0).any()
