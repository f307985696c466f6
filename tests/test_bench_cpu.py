"""bench.py's CPU leg on a small frame, no GPU: the oracle is timed on bands
of rows, and the comparison of its outputs with a frame's output buffers
(the benchmark's error against the CPU oracle) counts exactly the values
whose bits differ."""
import os
import sys

import numpy as np

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_cpu_leg_compares_each_sampled_band():
    import bench

    n, W, H = 32, 24, 70
    g = oracle.scene_noise(n, n, n, seed=4, threads=2)
    cam, tgt = bench.camera(n)
    pos, nrm, rough = oracle.gbuffer(g, cam, tgt, W, H, 4, threads=2)
    P = oracle.make_params(light_dir=bench.light_dir(4), cam_pos=cam, n_ao=4, ao_len=16.0, n_spec=1, seed=4)
    full = oracle.occlusion(g, pos, nrm, rough, P, threads=2)
    same = {k: full[k].copy() for k in ("shadow", "ao", "ao_vis", "spec", "spec_t")}
    v, rows, dt, th, chk = bench.cpu_sample_rays_per_s(g, pos, nrm, rough, P, W, H, budget_s=60.0, threads=2,
                                                        band=32, against=same)
    assert rows == H and v > 0 and th == 2
    assert chk["values"] == 5 * W * H and chk["bit_mismatches"] == 0 and chk["max_abs_diff"] == 0.0
    bad = {k: a.copy() for k, a in same.items()}
    i = int(np.flatnonzero(np.abs(nrm).reshape(-1, 3).sum(1) > 0)[5])
    bad["ao"][i] += np.float32(0.25)
    _, _, _, _, chk2 = bench.cpu_sample_rays_per_s(g, pos, nrm, rough, P, W, H, budget_s=60.0, threads=2, band=32,
                                                   against=bad)
    assert chk2["bit_mismatches"] == 1 and abs(chk2["max_abs_diff"] - 0.25) < 1e-6
    _, _, _, _, none = bench.cpu_sample_rays_per_s(g, pos, nrm, rough, P, W, H, budget_s=60.0, threads=2, band=32)
    assert none is None


def test_oracle_s_ref_is_the_records_mean():
    import bench

    n, W, H = 32, 20, 300
    g = oracle.scene_noise(n, n, n, seed=6, threads=2)
    cam, tgt = bench.camera(n)
    pos, nrm, rough = oracle.gbuffer(g, cam, tgt, W, H, 6, threads=2)
    P = oracle.make_params(light_dir=bench.light_dir(6), cam_pos=cam, n_ao=4, ao_len=16.0, n_spec=1, seed=6)
    full = oracle.occlusion(g, pos, nrm, rough, P, with_recs=True, threads=2)
    R = 6
    valid = np.abs(nrm).reshape(-1, 3).sum(1) > 0
    rows = [y for y in range(H) if (y // 32) % 8 == 0]
    pix = np.array([y * W + x for y in rows for x in range(W)])
    steps = full["recs"]["steps"].reshape(-1, R)[pix[valid[pix]]]
    sref, nrows = bench.oracle_s_ref(g, pos, nrm, rough, P, W, H, threads=2)
    assert nrows == len(rows) == 64 and sref == steps.sum() / steps.size
