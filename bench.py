#!/usr/bin/env python3
"""Throughput of the voxel occlusion path in Grays/s (giga-rays per second).

Workload (default "c2", the plain path at scale): 512^3 fine-voxel grid from
seeded 3-octave value noise (threshold 0.55, frequency 1/32, ground slab y < 8)
plus 2000 seeded boxes of 4-48 voxels per side; 1920x1080 primary-hit G-buffer
(fp32 position, normal, roughness U[0.05,1]) from a seeded pinhole camera
outside the grid; per pixel 1 shadow ray (maxt 100), 8 cosine-weighted AO rays
(maxt 32) and 1 GGX specular-occlusion ray (maxt 256), all through the exact
reference DDA (Light.frag:29-81). One step = one vxl_trace_occlusion call over
the frame. Inputs are generated on the device and are not timed.

Arms: default = libvxl CUDA path; --impl reference = the CPU restatement of
the reference path (oracle/) on all host cores, over a bounded sample of the
same frame per step.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# storage: "palette4" = bit-packed occupancy with the grid's 4-bit palette plane (seeded indices for the set
# voxels); "palette8" = the grid imported from a dense uint8 palette-index volume (voxel set where the index is
# >= 16, as ShadowVoxSystem.cpp:145 sets it); "occupancy" = bit-packed occupancy only
WORKLOADS = {
    "c2": dict(n=512, W=1920, H=1080, boxes=2000, n_shadow=1, n_ao=8, ao_len=32.0, n_spec=1, spec_len=256.0,
               shadow_len=100.0, seed=2024, storage="palette4"),
    "c1": dict(n=256, W=640, H=360, boxes=0, n_shadow=1, n_ao=4, ao_len=16.0, n_spec=0, spec_len=256.0,
               shadow_len=100.0, seed=2024, storage="palette8"),
    # stress: 2048^3 terrain (amplitude 512) + 50,000 instances of edge 16-128, 4K frame
    "c5": dict(kind="terrain", n=2048, W=3840, H=2160, boxes=0, instances=50000, n_shadow=1, n_ao=16, ao_len=64.0,
               n_spec=1, spec_len=256.0, shadow_len=256.0, seed=5, storage="occupancy"),
    # the stress workload's kernel on a quarter of its area (1024^3 terrain, 12,500 instances, 1920x1080), small
    # enough for a multi-pass ncu capture (under 1 GB on the device); the grid's bit addresses need 34 bits, so it
    # takes the same wide trace layout as 2048^3
    "c5s": dict(kind="terrain", n=1024, W=1920, H=1080, boxes=0, instances=12500, n_shadow=1, n_ao=16, ao_len=64.0,
                n_spec=1, spec_len=256.0, shadow_len=256.0, seed=5, storage="occupancy"),
}
L2_BYTES = 129 * 1024 * 1024


def camera(n):
    # outside the grid (above and in front), looking at its centre
    cam = np.array([0.5 * n, 1.15 * n, -0.1 * n], np.float32)
    tgt = np.array([0.5 * n, 0.5 * n, 0.5 * n], np.float32)
    return cam, tgt


def light_dir(seed):
    rng = np.random.default_rng(seed)
    v = rng.normal(size=3)
    v[1] = abs(v[1]) + 0.8  # above the horizon
    return (v / np.linalg.norm(v)).astype(np.float32)


def kernel_profile(workload):
    """Figures of the occlusion kernel from the committed ncu summary of this
    workload (profiles/k_occl_lean_<workload>.md): the kernel it covers, DRAM
    and L2 bytes per launch and pipe utilisation, or None where absent."""
    p = os.path.join(ROOT, "profiles", "k_occl_lean_%s.md" % workload)
    if not os.path.exists(p):
        return None
    out = {"file": os.path.relpath(p, ROOT)}
    for line in open(p):
        for key in ("kernel", "traffic_bytes_per_launch", "l2_bytes_per_launch"):
            if line.startswith(key + ":"):
                v = line.split(":", 1)[1].strip()
                out[key] = int(v) if key != "kernel" else v
        for key, name in (("sm__pipe_alu_cycles_active.avg.pct_of_peak_sustained_active", "alu_pipe"),
                          ("smsp__issue_active.avg.pct_of_peak_sustained_active", "issue_active"),
                          ("smsp__sass_branch_targets_threads_divergent.sum", "divergent_branch_targets"),
                          ("smsp__thread_inst_executed_per_inst_executed.ratio", "threads_per_instruction"),
                          ("sm__warps_active.avg.pct_of_peak_sustained_active", "warps_active")):
            if line.startswith("| `%s` |" % key):
                v = float(line.split("|")[2].split()[0])
                out[name] = v / 100.0 if "pct" in key else v
    return out


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.Q,
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0 and out.stdout.strip():
                    self.rows.append([c.strip() for c in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.02)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, name in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
        return rank, world, local, dist
    return 0, 1, 0, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, x):
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(dist, x):
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# --------------------------------------------------------------- CPU oracle
def cpu_sample_rays_per_s(g_r8, pos, nrm, rough, P, W, H, budget_s=12.0, threads=None, band=32, against=None):
    """Time the oracle on bands of `band` whole image rows, taken in seeded
    random order, until about budget_s of oracle time (one oracle call per
    band, so thread start-up is paid per band rather than per row). With
    `against` (the CUDA path's output buffers for the same frame, as numpy
    arrays) each band's oracle outputs are also compared with them, outside
    the timed calls. Returns (rays/s, rows, seconds, threads, check): check is
    None without `against`, else the values compared, those whose bits differ
    (any NaN equals any NaN) and the largest absolute difference."""
    import oracle

    threads = threads or (os.cpu_count() or 1)
    R = P.n_shadow + P.n_ao + P.n_spec
    valid = (np.abs(nrm).reshape(-1, 3).sum(1) > 0).reshape(H, W)
    starts = np.arange(0, H, band)
    order = np.random.default_rng(1).permutation(len(starts))
    rays = 0
    rows = 0
    busy = 0.0
    check = None if against is None else {"outputs": sorted(against), "values": 0, "bit_mismatches": 0,
                                          "max_abs_diff": 0.0}
    for b in order:
        y0 = int(starts[b])
        y1 = min(H, y0 + band)
        t1 = time.perf_counter()
        o = oracle.occlusion(g_r8, pos, nrm, rough, P, p0=y0 * W, p1=y1 * W, threads=threads)
        busy += time.perf_counter() - t1
        rays += int(valid[y0:y1].sum()) * R
        rows += y1 - y0
        if against is not None:
            for k, gpu in against.items():
                a = np.asarray(gpu[y0 * W:y1 * W], np.float32)
                w = o[k][y0 * W:y1 * W]
                both_nan = np.isnan(a) & np.isnan(w)
                differ = (a.view(np.int32) != w.view(np.int32)) & ~both_nan
                check["values"] += a.size
                check["bit_mismatches"] += int(differ.sum())
                d = np.abs(a.astype(np.float64) - w.astype(np.float64))[~(np.isnan(a) | np.isnan(w))]
                if d.size:
                    check["max_abs_diff"] = max(check["max_abs_diff"], float(d.max()))
        if busy > budget_s:
            break
    return rays / busy, rows, busy, threads, check


def oracle_s_ref(g_r8, pos, nrm, rough, P, W, H, every=8, band=32, threads=None):
    """Mean reference-DDA fetches per ray (S_ref) from the oracle's records
    on a stratified sample: every `every`-th band of `band` image rows, over
    the pixels that see geometry. Returns (S_ref, rows)."""
    import oracle

    R = P.n_shadow + P.n_ao + P.n_spec
    valid = np.abs(nrm).reshape(-1, 3).sum(1) > 0
    steps = 0
    rays = 0
    rows = 0
    for y0 in range(0, H, band * every):
        y1 = min(H, y0 + band)
        o = oracle.occlusion_range(g_r8, pos, nrm, rough, P, y0 * W, y1 * W, threads=threads)
        st = o["recs"]["steps"].reshape(-1, R)[valid[y0 * W:y1 * W]]
        steps += int(st.sum())
        rays += st.size
        rows += y1 - y0
    return steps / max(rays, 1), rows


def run_reference(args, wl):
    """--impl reference: the oracle port on the host cores (no GPU work)."""
    import oracle

    # no collective on this arm: rank 0 alone works and prints, the other ranks leave
    # before any process group exists, so nothing else reaches stdout
    if int(os.environ.get("RANK", "0")) != 0:
        return
    if wl.get("kind") == "terrain":
        print(json.dumps({"impl": "reference", "unavailable": "stress scene: voxelizing 50,000 instances on the "
                                                             "host cores exceeds the bounded reference run"}))
        return
    n, W, H = wl["n"], wl["W"], wl["H"]
    threads = os.cpu_count() or 1
    g = oracle.scene_noise(n, n, n, seed=wl["seed"], threads=threads)
    if wl["boxes"]:
        oracle.scene_boxes(g, wl["seed"], wl["boxes"], 4, 48)
    cam, tgt = camera(n)
    pos, nrm, rough = oracle.gbuffer(g, cam, tgt, W, H, wl["seed"], threads=threads)
    P = oracle.make_params(light_dir=light_dir(wl["seed"]), cam_pos=cam, bias=0.5, shadow_len=wl["shadow_len"],
                           ao_len=wl["ao_len"], spec_len=wl["spec_len"], n_shadow=wl["n_shadow"], n_ao=wl["n_ao"],
                           n_spec=wl["n_spec"], seed=wl["seed"])
    per_step = []
    # each step is a bounded sample; the whole run stays within ~150 s of CPU work
    budget = min(args.ref_step_seconds, 150.0 / max(1, args.warmup + args.steps))
    for s in range(args.warmup + args.steps):
        v, rows, dt, th, _ = cpu_sample_rays_per_s(g, pos, nrm, rough, P, W, H, budget_s=budget, threads=threads)
        if s >= args.warmup:
            per_step.append((v, rows, dt))
    rays_s = sum(v * dt for v, _, dt in per_step) / sum(dt for _, _, dt in per_step)
    val = rays_s / 1e9
    R = wl["n_shadow"] + wl["n_ao"] + wl["n_spec"]
    line = {
        "impl": "reference", "metric": "Grays/s shadow+AO+spec occlusion (exact voxel DDA)", "value": val,
        "unit": "Grays/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * statistics.mean(dt for _, _, dt in per_step), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": config_dict(wl),
        "cpu_baseline": {"value": val, "unit": "Grays/s", "cores": threads, "kind": "port",
                         "sample": "per step: bands of 32 whole image rows in seeded random order until %.0f s "
                                   "of wall time "
                                   "(%d rows of %d on average), %d rays per pixel" % (
                                       budget, statistics.mean(r for _, r, _ in per_step), H, R)},
        "e2e": {"value": val, "unit": "Grays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


STORAGE_TEXT = {
    "palette4": "bit-packed occupancy in 4^3 bricks with a 4-bit palette plane (seeded indices 1-15 for the set "
                "voxels; the occlusion traversal reads occupancy only), 8^3 tile map, trace layout",
    "palette8": "imported from a dense uint8 palette-index volume (voxel set where the index is >= 16) into "
                "bit-packed occupancy in 4^3 bricks, 8^3 tile map, trace layout",
    "occupancy": "bit-packed occupancy in 4^3 bricks, 8^3 tile map, wide trace layout (bit addresses of 33-37 "
                 "bits: the z term in 64 bits)",
}


def palette8_volume(G, n, seed):
    """The dense uint8 palette-index volume behind a grid's occupancy: seeded
    indices 16-255 where a voxel is set, 0-15 where it is not."""
    import torch

    import voxelengine_gb300 as V

    r8 = torch.empty((n // 2) ** 3, dtype=torch.uint8, device="cuda")
    G.export_r8(r8)
    r8 = r8.view(n // 2, n // 2, n // 2)
    occ = torch.zeros((n, n, n), dtype=torch.bool, device="cuda")
    for b in range(8):
        occ[(b >> 2) & 1::2, (b >> 1) & 1::2, b & 1::2] = ((r8 >> b) & 1).bool()
    gen = torch.Generator(device="cuda").manual_seed(seed)
    hi = torch.randint(16, 256, (n, n, n), dtype=torch.uint8, device="cuda", generator=gen)
    lo = torch.randint(0, 16, (n, n, n), dtype=torch.uint8, device="cuda", generator=gen)
    return torch.where(occ, hi, lo).contiguous()


def config_dict(wl):
    terrain = wl.get("kind") == "terrain"
    d = {"workload": "%s-%d^3-%dx%d-%dshadow+%dao(L%g)+%dspec" % (
        "terrain" if terrain else "plain", wl["n"], wl["W"], wl["H"], wl["n_shadow"], wl["n_ao"], wl["ao_len"],
        wl["n_spec"]),
        "grid": [wl["n"]] * 3, "image": [wl["W"], wl["H"]],
        "rays_per_pixel": wl["n_shadow"] + wl["n_ao"] + wl["n_spec"],
        "storage": STORAGE_TEXT[wl["storage"]],
        "l2": "flushed between timed steps (256 MiB write outside the per-step events)"}
    if terrain:
        d.update(terrain={"base": wl["n"] / 16.0, "amplitude": 512.0, "octaves": 6}, instances=wl["instances"],
                 instance_edges=[16, 128])
    else:
        d.update(boxes=wl["boxes"], noise_threshold=0.55)
    return d


# ------------------------------------------------------------------ GPU arm
def run_gpu(args, wl):
    import torch

    import voxelengine_gb300 as V

    rank, world, local, dist = dist_setup(args)
    torch.cuda.set_device(local)
    V.build()
    ctx = V.Context(local)
    from voxelengine_gb300 import autotune

    autotune.apply_cached(ctx, args.workload)
    if args.tuning:
        ctx.set_tuning(*[int(x) for x in args.tuning.split(",")])
    n, W, H = wl["n"], wl["W"], wl["H"]
    npix = W * H
    R = wl["n_shadow"] + wl["n_ao"] + wl["n_spec"]
    P_kw = dict(light_dir=light_dir(wl["seed"]), bias=0.5, shadow_len=wl["shadow_len"], ao_len=wl["ao_len"],
                spec_len=wl["spec_len"], n_shadow=wl["n_shadow"], n_ao=wl["n_ao"], n_spec=wl["n_spec"],
                seed=wl["seed"])
    scene_extra = {}
    if wl.get("kind") == "terrain":
        from voxelengine_gb300 import scenes as S

        sc = S.make_terrain_scene(ctx, n, W, H, seed=wl["seed"], n_instances=wl["instances"])
        G, pos, nrm, rough, cam = sc["grid"], sc["pos"], sc["nrm"], sc["rough"], sc["cam"]
        P = V.make_params(cam_pos=cam, **P_kw)
        scene_extra["voxelize"] = {"seconds": sc["voxelize_seconds"], "instances": wl["instances"],
                                   "source_voxels": sc["source_voxels"],
                                   "gvoxels_per_s": sc["source_voxels"] / sc["voxelize_seconds"] / 1e9}
    else:
        G = V.Grid(ctx, n, n, n)
        G.scene_noise(wl["seed"], 0.55, 1.0 / 32.0, 8)
        if wl["boxes"]:
            G.scene_boxes(wl["seed"], wl["boxes"], 4, 48)
        if wl["storage"] == "palette4":
            G.palette_alloc()
            G.scene_palette(wl["seed"])
        elif wl["storage"] == "palette8":
            vol = palette8_volume(G, n, wl["seed"])
            G.clear()
            G.import_palette(vol, opaque_min=16)
            del vol
        cam, tgt = camera(n)
        pos = torch.empty(npix * 3, dtype=torch.float32, device="cuda")
        nrm = torch.empty_like(pos)
        rough = torch.empty(npix, dtype=torch.float32, device="cuda")
        V.scene_gbuffer(ctx, G, cam, tgt, W, H, wl["seed"], pos, nrm, rough)
        P = V.make_params(cam_pos=cam, **P_kw)
    outs = {k: torch.empty(npix, dtype=torch.float32, device="cuda") for k in ("shadow", "ao", "ao_vis", "spec", "spec_t")}
    valid = int((nrm.view(-1, 3).abs().sum(1) > 0).sum().item())
    rays_per_step = valid * R

    # per-ray fetch counts (S_ref) from one untimed pass with records
    rec = torch.empty(npix * R * 6, dtype=torch.int32, device="cuda")
    V.trace_occlusion(ctx, G, pos, nrm, rough, npix, P, records=rec, width=W, height=H, **outs)
    torch.cuda.synchronize()
    steps_col = rec.view(-1, 6)[:, 4].view(npix, R)
    vmask = (nrm.view(-1, 3).abs().sum(1) > 0)
    s_ref = float(steps_col[vmask].double().mean().item())
    hits = float(((rec.view(-1, 6)[:, 5] & 1).view(npix, R)[vmask]).double().mean().item())
    del rec

    if args.autotune:
        autotune.tune(ctx, lambda: (lambda: V.trace_occlusion(ctx, G, pos, nrm, rough, npix, P, width=W, height=H, **outs)),
                      args.workload, log=lambda m: print(m, file=sys.stderr))
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    # clocks are sampled from the start of the warm-up (same load) to the end
    # of the timed steps: the timed region alone is often shorter than one
    # nvidia-smi query
    with ClockSampler(local) as clk:
        for _ in range(args.warmup):
            V.trace_occlusion(ctx, G, pos, nrm, rough, npix, P, width=W, height=H, **outs)
        torch.cuda.synchronize()
        l0 = ctx.launch_count()
        barrier(dist)
        torch.cuda.synchronize()
        for s in range(args.steps):
            flush.fill_(float(s))
            ev[s][0].record(stream)
            V.trace_occlusion(ctx, G, pos, nrm, rough, npix, P, width=W, height=H, **outs)
            ev[s][1].record(stream)
        torch.cuda.synchronize()
        barrier(dist)
    launches = ctx.launch_count() - l0
    times = [a.elapsed_time(b) for a, b in ev]  # ms
    t_total = max_over_ranks(dist, sum(times) / 1e3)
    rays_total = sum_over_ranks(dist, rays_per_step * args.steps)
    value = rays_total / t_total / 1e9

    # end to end through the host-memory entry point (pinned buffers)
    hp, hn, hr = pos.cpu().pin_memory(), nrm.cpu().pin_memory(), rough.cpu().pin_memory()
    hout = {k: torch.empty(npix, dtype=torch.float32).pin_memory() for k in outs}
    for _ in range(max(1, args.warmup)):
        V.trace_occlusion_host(ctx, G, hp, hn, hr, npix, P, h_shadow=hout["shadow"], h_ao=hout["ao"],
                               h_ao_vis=hout["ao_vis"], h_spec=hout["spec"], h_spec_t=hout["spec_t"])
    torch.cuda.synchronize()
    barrier(dist)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for s in range(args.steps):
        V.trace_occlusion_host(ctx, G, hp, hn, hr, npix, P, h_shadow=hout["shadow"], h_ao=hout["ao"],
                               h_ao_vis=hout["ao_vis"], h_spec=hout["spec"], h_spec_t=hout["spec_t"])
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(dist)
    t_e2e = max_over_ranks(dist, e0.elapsed_time(e1) / 1e3)
    e2e = rays_total / t_e2e / 1e9
    h2d = npix * (3 + 3 + 1) * 4
    d2h = npix * 5 * 4

    if rank != 0:
        return
    hbm, peak_kind = measured_peaks()
    # the L2 side: this GPU's L2 read bandwidth, measured here by a streaming kernel
    l2_gbs, l2_ms = V.l2_read_gbs(ctx, 64 << 20, 50)
    b_pix_in = 24 + (4 if wl["n_spec"] else 0)
    b_pix_out = 4 * 5
    b_ray = (b_pix_in + b_pix_out) / R + 4.0 * s_ref
    ms = statistics.mean(times)
    achieved = b_ray * rays_per_step / (ms / 1e3) / 1e9
    prof = kernel_profile(args.workload)
    line = {
        "metric": "Grays/s shadow+AO+spec occlusion (exact voxel DDA)", "value": value, "unit": "Grays/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "ms_per_step_median": statistics.median(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene and G-buffer)",
        "config": config_dict(wl),
        "rays_per_step": rays_per_step, "valid_pixels": valid, "s_ref_mean_fetches_per_ray": s_ref,
        "hit_fraction": hits,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "frac_hbm": achieved / hbm, "l2_peak": l2_gbs, "frac_l2": achieved / l2_gbs,
                     "l2_peak_how": "best of 50 timed reads of a 64 MiB L2-resident buffer (vxl_diag_l2_read_gbs), "
                                    "this run",
                     "traffic": prof.get("traffic_bytes_per_launch") if prof else None,
                     "l2_traffic": prof.get("l2_bytes_per_launch") if prof else None,
                     "peak_kind": peak_kind, "profile": prof,
                     "bytes_per_ray": b_ray,
                     "note": "algorithmic bytes = ((28 B in + 20 B out) per pixel)/R + 4 B x S_ref per ray; "
                             "per-launch time from CUDA events on the launch stream; traffic from the ncu "
                             "summary named in profile"},
        "e2e": {"value": e2e, "unit": "Grays/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "path": "vxl_trace_occlusion_host, pinned host G-buffer and outputs"},
        "gpu_launches": int(launches),
        "tuning": ctx.get_tuning(),
        "clocks": clk.summary(),
    }
    line.update(scene_extra)
    if not args.no_cpu_baseline:
        g8 = torch.zeros((n // 2) ** 3, dtype=torch.uint8, device="cuda")
        G.export_r8(g8)
        torch.cuda.synchronize()
        g_np = g8.cpu().numpy().reshape(n // 2, n // 2, n // 2)
        import oracle

        OP = oracle.make_params(cam_pos=cam, **P_kw)
        gpu_out = {k: t.cpu().numpy() for k, t in outs.items()}
        v, rows, dt, th, chk = cpu_sample_rays_per_s(g_np, pos.cpu().numpy(), nrm.cpu().numpy(), rough.cpu().numpy(),
                                                     OP, W, H, budget_s=args.cpu_seconds, against=gpu_out)
        # the error against the CPU oracle on the sampled rows (bit-exact is expected)
        line["oracle_check"] = dict(chk, sample="the cpu_baseline rows")
        sref, srows = oracle_s_ref(g_np, pos.cpu().numpy(), nrm.cpu().numpy(), rough.cpu().numpy(), OP, W, H)
        line["oracle_check"]["s_ref_oracle"] = sref
        line["oracle_check"]["s_ref_sample"] = "oracle records of every 8th band of 32 rows: %d of %d rows" % (srows, H)
        line["cpu_baseline"] = {"value": v / 1e9, "unit": "Grays/s", "cores": th, "kind": "port",
                                "sample": "%d whole image rows of %d in bands of 32, seeded random order (%.1f s), %d rays/px" % (
                                    rows, H, dt, R)}
        v1, rows1, dt1, _, _ = cpu_sample_rays_per_s(g_np, pos.cpu().numpy(), nrm.cpu().numpy(),
                                                  rough.cpu().numpy(), OP, W, H,
                                                  budget_s=min(4.0, args.cpu_seconds), threads=1)
        line["cpu_baseline"]["one_core"] = {"value": v1 / 1e9, "unit": "Grays/s", "cores": 1,
                                            "sample": "%d whole image rows (%.1f s)" % (rows1, dt1)}
    if not args.no_extras and args.workload == "c2":
        # the batched and differentiable forms, compact, on the same GPU
        n_ex = max(3, min(args.steps, 10))
        c3 = c3_result(args, n_ex, 3, check=not args.no_cpu_baseline)
        line["c3_batched"] = {k: c3[k] for k in ("value", "unit", "ms_per_step", "plain_value", "plain_ms_per_step",
                                                 "batched_over_plain", "rays_per_step", "clocks")}
        line["c3_batched"]["voxelize_gvoxels_per_s"] = c3["voxelize"]["gvoxels_per_s"]
        if "oracle_check" in c3:
            line["c3_batched"]["oracle_check"] = c3["oracle_check"]
        c4 = c4_result(args, n_ex, 3, fd_check=not args.no_cpu_baseline, cpu_baseline=False)
        line["c4_adjoint"] = {k: c4[k] for k in ("value", "unit", "forward_ms", "adjoint_ms", "adjoint_over_forward",
                                                 "clocks")}
        if "fd_check" in c4:
            line["c4_adjoint"]["fd_check"] = c4["fd_check"]
    print(json.dumps(line))


def c3_result(args, steps, warmup, check=True):
    """C3: 64 scenes (edges log-uniform 64-512, noise threshold U[0.45,0.65],
    rays per scene log-uniform 64K-2M at 1 shadow + 8 AO + 1 spec per pixel),
    10,000 Vox instances (edge 8-64, ~40% fill, uniform rotations) voxelized
    into the scene grids first (timed on its own). One step = all 64 scenes:
    the batched form (one persistent launch, CUDA-graph replay) against the
    plain form (one vxl_trace_occlusion per scene). With `check`, the batch's
    output buffers of 8 of the scenes are compared with the oracle on bands
    of their image rows."""
    import torch

    import voxelengine_gb300 as V
    from voxelengine_gb300 import scenes as S

    V.build()
    ctx = V.Context(0)
    from voxelengine_gb300 import autotune

    autotune.apply_cached(ctx, "c3")
    if args.tuning:
        ctx.set_tuning(*[int(x) for x in args.tuning.split(",")])
    scenes = [S.add_outputs(sc) for sc in S.batch_set(ctx, 64, seed=7, palette=True)]
    models = S.vox_models(11, 32)
    d_models = [torch.from_numpy(m).cuda() for m in models]
    mdesc = [(d.data_ptr(),) + m.shape[::-1] for m, d in zip(models, d_models)]
    per = S.instance_set(scenes, 10000, models, seed=13)
    src_voxels = sum(int(np.prod(models[mi].shape)) for lst in per for _, mi, _ in lst)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for sc, lst in zip(scenes, per):
        if lst:
            V.voxelize(ctx, sc["grid"], mdesc, lst)
    e1.record()
    torch.cuda.synchronize()
    t_vox = e0.elapsed_time(e1) / 1e3
    # re-render the G-buffers now that the instances are in the grids
    for sc in scenes:
        V.scene_gbuffer(ctx, sc["grid"], sc["cam"], np.array([sc["n"] / 2] * 3, np.float32), sc["W"], sc["H"],
                        sc["seed"], sc["pos"], sc["nrm"], sc["rough"])
    rays = sum(sc["npix"] * 10 for sc in scenes)
    valid = sum(int((sc["nrm"].view(-1, 3).abs().sum(1) > 0).sum().item()) for sc in scenes)
    traced = valid * 10

    def plain():
        for sc in scenes:
            V.trace_occlusion(ctx, sc["grid"], sc["pos"], sc["nrm"], sc["rough"], sc["npix"], sc["params"],
                              shadow=sc["shadow"], ao=sc["ao"], ao_vis=sc["ao_vis"], spec=sc["spec"],
                              spec_t=sc["spec_t"])

    if getattr(args, "autotune", False):
        def make_step():
            b = V.Batch(ctx, scenes, use_graph=True)
            return b.run

        autotune.tune(ctx, make_step, "c3", log=lambda m: print(m, file=sys.stderr))
    batch = V.Batch(ctx, scenes, use_graph=True)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")

    def timed(fn):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        ts = []
        for s in range(steps):
            flush.fill_(float(s))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            ts.append((a, b))
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in ts) / 1e3 / steps

    with ClockSampler(0) as clk:
        t_plain = timed(plain)
        t_batch = timed(batch.run)
    out = {
        "value": traced / t_batch / 1e9, "unit": "Grays/s", "ms_per_step": t_batch * 1e3,
        "plain_value": traced / t_plain / 1e9, "plain_ms_per_step": t_plain * 1e3,
        "batched_over_plain": t_plain / t_batch, "rays_per_step": traced, "rays_nominal": rays,
        "edges": [int(sc["n"]) for sc in scenes], "pixels": [int(sc["npix"]) for sc in scenes],
        "voxelize": {"seconds": t_vox, "instances": 10000, "source_voxels": src_voxels,
                     "gvoxels_per_s": src_voxels / t_vox / 1e9},
        "tuning": ctx.get_tuning(), "clocks": clk.summary(),
    }
    if check:
        # the last batch run's buffers against the oracle, on bands of rows of every 8th scene
        batch.run()
        torch.cuda.synchronize()
        import ctypes

        import oracle

        chk = {"scenes": [], "values": 0, "bit_mismatches": 0}
        for i in range(0, len(scenes), 8):
            sc = scenes[i]
            n, W, H = sc["n"], sc["W"], sc["H"]
            g8 = torch.zeros((n // 2) ** 3, dtype=torch.uint8, device="cuda")
            sc["grid"].export_r8(g8)
            torch.cuda.synchronize()
            g_np = g8.cpu().numpy().reshape(n // 2, n // 2, n // 2)
            op = oracle.Params()
            ctypes.memmove(ctypes.byref(op), ctypes.byref(sc["params"]), ctypes.sizeof(op))
            pos, nrm, rough = sc["pos"].cpu().numpy(), sc["nrm"].cpu().numpy(), sc["rough"].cpu().numpy()
            bands = [(int(y), int(min(H, y + 16))) for y in np.linspace(0, max(0, H - 16), 4).astype(int)]
            for y0, y1 in sorted(set(bands)):
                o = oracle.occlusion_range(g_np, pos, nrm, rough, op, y0 * W, y1 * W)
                for k in ("shadow", "ao", "ao_vis", "spec", "spec_t"):
                    a = sc[k][y0 * W:y1 * W].cpu().numpy()
                    w = o[k]
                    same = (a.view(np.int32) == w.view(np.int32)) | (np.isnan(a) & np.isnan(w))
                    chk["values"] += a.size
                    chk["bit_mismatches"] += int((~same).sum())
            chk["scenes"].append(i)
        chk["sample"] = "4 bands of 16 image rows of every 8th scene, all five buffers of the batched run"
        out["oracle_check"] = chk
    batch.close()
    return out


def run_gpu_c3(args):
    r = c3_result(args, args.steps, args.warmup, check=not args.no_cpu_baseline)
    line = {
        "metric": "Grays/s shadow+AO+spec occlusion, 64-scene batch (exact voxel DDA)",
        "value": r["value"], "unit": "Grays/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded scenes, G-buffers and Vox instances)",
        "config": {"workload": "batch-64-scenes", "edges": r.pop("edges"), "pixels": r.pop("pixels"),
                   "rays_per_pixel": 10, "instances": 10000, "storage": STORAGE_TEXT["palette4"],
                   "l2": "flushed between timed steps"},
    }
    line.update({k: v for k, v in r.items() if k not in ("value", "unit", "ms_per_step")})
    print(json.dumps(line))


def c4_result(args, steps, warmup, fd_check=True, cpu_baseline=True):
    """C4, the differentiable variant: 128^3 soft grid (opacity
    sigmoid(8 (noise - 0.55)), albedo U[0,1)), 512x512 G-buffer of the matching
    binary scene, 1 shadow + 16 AO rays per pixel of length 24; loss = MSE
    against a target rendered with a second albedo seed. One step = forward,
    dL/dimage, zeroing the gradient and the adjoint. Reports the forward and
    adjoint times and their ratio. With `fd_check`, the adjoint of a loss on
    every 64th pixel is compared with FP64 central finite differences
    (h = 1e-4, the oracle) at the 64 voxels of largest gradient."""
    import torch

    import voxelengine_gb300 as V
    from voxelengine_gb300 import scenes as S

    V.build()
    ctx = V.Context(0)
    n, W, H, seed = 128, 512, 512, 2024
    P = V.make_soft_params(light_dir=S.light_dir(seed), bias=0.5, length=24.0, k_sun=0.7, k_amb=0.5, n_shadow=1,
                           n_ao=16, seed=seed)
    sc = S.make_soft_scene(ctx, n, W, H, seed, albedo_seed=1, params=P)
    tg = S.make_soft_scene(ctx, n, W, H, seed, albedo_seed=2, params=P)
    npix = sc["npix"]
    img = torch.empty((npix, 3), dtype=torch.float32, device="cuda")
    light = torch.empty_like(img)
    target = torch.empty_like(img)
    V.trace_soft_fwd(ctx, tg["soft"], tg["pos"], tg["nrm"], npix, P, target)
    grad = torch.zeros_like(sc["soft"])
    gi = torch.empty_like(img)
    valid = int((sc["nrm3"].abs().sum(1) > 0).sum().item())
    rays = valid * 17
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")

    def fwd():
        V.trace_soft_fwd(ctx, sc["soft"], sc["pos"], sc["nrm"], npix, P, img, light)

    def bwd():
        V.trace_soft_bwd(ctx, sc["soft"], sc["pos"], sc["nrm"], npix, P, gi, light, grad)

    def step():
        fwd()
        torch.sub(img, target, out=gi)
        gi.mul_(2.0 / img.numel())
        grad.zero_()
        bwd()

    def timed(fn):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        ts = []
        for k in range(steps):
            flush.fill_(float(k))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            ts.append((a, b))
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in ts) / 1e3 / steps

    step()
    with ClockSampler(0) as clk:
        t_fwd = timed(fwd)
        t_bwd = timed(bwd)
        t_step = timed(step)
    loss = float(((img - target) ** 2).mean())
    out = {"value": rays / t_step / 1e9, "unit": "Grays/s", "ms_per_step": t_step * 1e3,
           "forward_ms": t_fwd * 1e3, "adjoint_ms": t_bwd * 1e3, "adjoint_over_forward": t_bwd / t_fwd,
           "rays_per_step": rays, "loss": loss, "clocks": clk.summary()}
    if fd_check or cpu_baseline:
        import oracle

        vox = sc["soft"].cpu().numpy()
        pos, nrm = sc["pos3"].cpu().numpy(), sc["nrm3"].cpu().numpy()
        op = oracle.make_soft_params(light_dir=list(P.light_dir), bias=P.bias, length=P.len, k_sun=P.k_sun,
                                     k_amb=P.k_amb, n_shadow=P.n_shadow, n_ao=P.n_ao, seed=P.seed)
        sel = np.arange(0, npix, 64)
    if fd_check:
        # the adjoint of L = sum(image[sel] * g) for a seeded g on every 64th pixel
        rng = np.random.default_rng(5)
        g_sel = rng.standard_normal((len(sel), 3)).astype(np.float32)
        g_full = np.zeros((npix, 3), np.float32)
        g_full[sel] = g_sel
        fwd()
        gi.copy_(torch.from_numpy(g_full))
        grad.zero_()
        bwd()
        torch.cuda.synchronize()
        got = grad.cpu().numpy()[..., 0].ravel().astype(np.float64)
        a = vox[..., 0].ravel()
        amax = 1.0 - 1.0 / 4096.0
        cand = np.flatnonzero((a > 2e-4) & (a < amax - 2e-4) & (got != 0))
        pick = cand[np.argsort(-np.abs(got[cand]))[:64]]
        h = 1e-4
        threads = os.cpu_count() or 1

        # the oracle seeds each pixel's rays with its index: render the whole frame
        # with the unselected pixels' normals zeroed (they trace nothing)
        nrm_sel = np.zeros_like(nrm)
        nrm_sel[sel] = nrm[sel]

        def lossv(v, d):
            return float((oracle.soft_render(vox, pos, nrm_sel, op, perturb_voxel=v, perturb_delta=d,
                                             threads=threads)[sel] * g_sel).sum())

        fd = np.array([(lossv(v, h) - lossv(v, -h)) / (2 * h) for v in pick])
        err = np.abs(got[pick] - fd) / np.maximum(np.abs(fd), 1e-3 * np.abs(fd).max())
        out["fd_check"] = {"voxels": int(len(pick)), "max_rel_err": float(err.max()), "h": h,
                           "sample": "opacity gradient of a loss on every 64th pixel, 64 voxels of largest "
                                     "gradient, FP64 central differences by the oracle"}
    if cpu_baseline:
        gih = gi.cpu().numpy()
        live = int((np.abs(nrm[sel]).sum(1) > 0).sum())
        threads = min(4, os.cpu_count() or 1)
        t0 = time.perf_counter()
        oracle.soft_render(vox, pos[sel], nrm[sel], op, gih[sel], threads=threads)
        t = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": live * 17 / t / 1e9, "unit": "Grays/s", "cores": threads, "kind": "port",
                               "sample": "FP64 oracle forward+adjoint on every 64th pixel (%d rays)" % (live * 17)}
    return out


def run_gpu_c4(args):
    r = c4_result(args, args.steps, args.warmup, fd_check=not args.no_cpu_baseline,
                  cpu_baseline=not args.no_cpu_baseline)
    line = {
        "metric": "Grays/s soft-opacity forward + adjoint (exact voxel DDA cells)",
        "value": r["value"], "unit": "Grays/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded soft grid and G-buffer)",
        "config": {"workload": "soft-128^3-512x512-1shadow+16ao(L24)-mse", "l2": "flushed between timed steps"},
        "gpu_launches": 2,
    }
    line.update({k: v for k, v in r.items() if k not in ("value", "unit", "ms_per_step")})
    print(json.dumps(line))


def run_gpu_frame(args):
    """Whole frame on the GPU: 4096 Vox instances (the reference's per-frame
    cap, GeometryVoxelPipeline.h:17; edges 16-64, uniform rotations) spread
    over a 512^3 world, voxelized into the ShadowVox grid, primary visibility
    at 1920x1080 (vxl_trace_primary), then occlusion rays (1 shadow + 8 AO +
    1 spec) from that G-buffer. One step = primary + occlusion; the
    voxelization is timed once on its own."""
    import torch

    import voxelengine_gb300 as V
    from voxelengine_gb300 import scenes as S

    V.build()
    ctx = V.Context(0)
    n, W, H, seed, ninst = 512, 1920, 1080, 7, 4096
    rng = np.random.default_rng(seed)
    vols = S.vox_models(seed, 48, 16, 64, fill=0.4)
    vol_of = rng.integers(0, len(vols), ninst).astype(np.int32)
    worlds = np.array([S.instance_matrix(rng, n, vols[v].shape) for v in vol_of], np.float32)
    G = V.Grid(ctx, n, n, n)
    d_models = [torch.from_numpy(v).cuda() for v in vols]
    mdesc = [(d.data_ptr(),) + v.shape[::-1] for v, d in zip(vols, d_models)]
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    V.voxelize(ctx, G, mdesc, [(worlds[k], int(vol_of[k]), V.OP_SET) for k in range(ninst)])
    e1.record()
    torch.cuda.synchronize()
    t_vox = e0.elapsed_time(e1) / 1e3
    vs = V.VolumeSet(ctx, vols)
    cam_fine, tgt_fine = camera(n)
    cam, tgt = cam_fine * np.float32(0.1), tgt_fine * np.float32(0.1)
    npix = W * H
    pos = torch.empty(npix * 3, dtype=torch.float32, device="cuda")
    nrm = torch.empty_like(pos)
    rough = torch.full((npix,), 0.5, dtype=torch.float32, device="cuda")
    P = V.make_params(light_dir=light_dir(seed), cam_pos=cam_fine, bias=0.5, shadow_len=100.0, ao_len=32.0,
                      spec_len=256.0, n_shadow=1, n_ao=8, n_spec=1, seed=seed)
    outs = {k: torch.empty(npix, dtype=torch.float32, device="cuda") for k in ("shadow", "ao", "ao_vis", "spec",
                                                                                "spec_t")}
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")

    cmd_table = V.voxcmds(worlds, vol_of)  # the engine's per-frame command buffer (GeometryVoxelPipeline::Cmd)

    def primary():
        V.trace_primary(ctx, vs, None, None, cam, tgt, W, H, pos, nrm, cmds=cmd_table)

    def occl():
        V.trace_occlusion(ctx, G, pos, nrm, rough, npix, P, width=W, height=H, **outs)

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        ts = []
        for k in range(args.steps):
            flush.fill_(float(k))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            ts.append((a, b))
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in ts) / 1e3 / args.steps

    # 64 point / spot lights over the scene (every third a spot), shadows fused in one launch
    lrng = np.random.default_rng(seed + 1)
    lights = [(lrng.uniform(0.0, n / 10.0, 3).astype(np.float32), float(lrng.uniform(4.0, 12.0)), l % 3 == 2)
              for l in range(64)]
    wpos = torch.empty_like(pos)
    noise = torch.rand(npix * 4, dtype=torch.float32, device="cuda")
    lit = torch.empty(npix, dtype=torch.int64, device="cuda")
    inr = torch.empty_like(lit)

    def lights_pass():
        torch.mul(pos, 0.1, out=wpos)
        V.light_points(ctx, G, wpos, nrm, noise, npix, lights, lit, inr)

    # temporal accumulation of a lighting buffer built from the occlusion terms
    depth_t = torch.empty(npix, dtype=torch.float32, device="cuda")
    light4 = torch.zeros(npix * 4, dtype=torch.float32, device="cuda")
    last4 = torch.rand(npix * 4, dtype=torch.float32, device="cuda")
    color3 = torch.full((npix * 3,), 0.5, dtype=torch.float32, device="cuda")
    mat4 = torch.zeros(npix * 4, dtype=torch.float32, device="cuda")
    motion2 = (torch.rand(npix * 2, dtype=torch.float32, device="cuda") - 0.5) * 2e-3
    taa_out = torch.empty(npix * 4, dtype=torch.float32, device="cuda")

    def taa_pass():
        V.trace_primary(ctx, vs, None, None, cam, tgt, W, H, pos, nrm, depth=depth_t, cmds=cmd_table)
        occl()
        lv = light4.view(npix, 4)
        lv[:, 0] = outs["shadow"]
        lv[:, 1] = outs["ao"]
        lv[:, 2] = outs["spec"]
        depth_t.div_(4096.0)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        V.light_taa(ctx, light4, last4, color3, nrm, mat4, depth_t, motion2, noise, W, H, taa_out)
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b)

    primary()
    torch.cuda.synchronize()
    valid = int((nrm.view(-1, 3).abs().sum(1) > 0).sum().item())
    with ClockSampler(0) as clk:
        t_p = timed(primary)
        t_o = timed(occl)
        t_l = timed(lights_pass)
        t_taa = statistics.median([taa_pass() for _ in range(max(3, args.steps // 4))]) / 1e3
        t_f = timed(lambda: (primary(), occl()))
    pairs = int(sum(bin(int(x)).count("1") for x in inr.cpu().numpy().view(np.uint64)))
    line = {
        "metric": "frame ms: primary visibility + shadow/AO/spec occlusion, 4096 instances, 1080p",
        "value": t_f * 1e3, "unit": "ms", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_f * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded Vox models and placements)",
        "config": {"workload": "frame-512^3-4096inst-1920x1080-1shadow+8ao+1spec", "instances": ninst,
                   "model_edges": [16, 64], "l2": "flushed between timed steps"},
        "primary_ms": t_p * 1e3, "primary_mpix_per_s": npix / t_p / 1e6, "occlusion_ms": t_o * 1e3,
        "occlusion_grays_per_s": valid * 10 / t_o / 1e9, "covered_pixels": valid,
        "taa_ms": t_taa * 1e3, "lights64_ms": t_l * 1e3, "light_rays": pairs, "light_grays_per_s": pairs / t_l / 1e9,
        "voxelize": {"seconds": t_vox, "instances": ninst}, "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline:
        import oracle

        sub_w, sub_h = 64, 36  # a 64x36 frame of the same camera: the oracle tests every instance per pixel
        t0 = time.perf_counter()
        oracle.primary(vols, worlds, vol_of, cam, tgt, sub_w, sub_h, threads=os.cpu_count())
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": sub_w * sub_h / dt / 1e6, "unit": "Mpix/s (primary only)",
                                "cores": os.cpu_count(), "kind": "port",
                                "sample": "oracle primary visibility on a 64x36 frame, every instance per pixel"}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="vxl", choices=["vxl", "reference"])
    ap.add_argument("--workload", default="c2", choices=sorted(WORKLOADS) + ["c3", "c4", "frame"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--ref-step-seconds", type=float, default=4.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="leave the C3 batched and C4 adjoint figures out of "
                                                              "the default line")
    ap.add_argument("--tuning", default="", help="tile_px,kstep,leap,order,tile_w,grab for the occlusion kernel")
    ap.add_argument("--autotune", action="store_true", help="search the launch shape first and cache it")
    args = ap.parse_args()
    if args.workload == "c3":
        run_gpu_c3(args)
        return
    if args.workload == "c4":
        run_gpu_c4(args)
        return
    if args.workload == "frame":
        run_gpu_frame(args)
        return
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        run_reference(args, wl)
    else:
        run_gpu(args, wl)


if __name__ == "__main__":
    main()
