"""Temporal accumulation on the GPU (vxl_light_taa) against the oracle (which
is pinned to LightTAA.frag's own main), bit for bit, NaN == NaN; a second
frame fed back through last_light. Disoccluded bands of 4 columns (a few
such pixels per warp, whose taps the warp shares) and of 24 (most of a warp,
one pixel per lane)."""
import numpy as np
import pytest

import oracle
from tests import taa_cases
from tests.gpu_util import dev, same_bits

pytestmark = pytest.mark.gpu

KEYS = ("light", "last", "color", "normal", "material", "depth", "motion", "noise")


@pytest.mark.parametrize("W,H,band", [(64, 40, 4), (197, 113, 4), (96, 37, 24)])
def test_taa_matches_oracle(vxl, ctx, W, H, band):
    import torch

    fr = taa_cases.frame(W, H, W, band)
    d = {k: dev(fr[k]) for k in KEYS}
    out = torch.empty(W * H * 4, dtype=torch.float32, device="cuda")
    vxl.light_taa(ctx, *[d[k] for k in KEYS], W, H, out)
    torch.cuda.synchronize()
    got = out.cpu().numpy().reshape(H, W, 4)
    want = oracle.taa(*[fr[k] for k in KEYS])
    assert same_bits(got, want).all()
    # next frame: the output becomes last_light
    fr2 = taa_cases.frame(W, H, W + 1, band)
    fr2["last"] = want
    d2 = {k: dev(fr2[k]) for k in KEYS}
    out2 = torch.empty_like(out)
    vxl.light_taa(ctx, *[d2[k] for k in KEYS], W, H, out2)
    torch.cuda.synchronize()
    assert same_bits(out2.cpu().numpy().reshape(H, W, 4), oracle.taa(*[fr2[k] for k in KEYS])).all()
