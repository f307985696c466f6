"""Helpers for GPU parity tests: device buffers are torch tensors, calls go
through libvxl's C ABI (voxelengine_gb300)."""
import numpy as np


def dev(a, dtype=None):
    import torch

    t = torch.from_numpy(np.ascontiguousarray(a))
    if dtype is not None:
        t = t.to(dtype)
    return t.cuda()


def empty(n, dtype):
    import torch

    return torch.empty(n, dtype=dtype, device="cuda")


def recs_np(t):
    from voxelengine_gb300 import REC_DTYPE

    return t.cpu().numpy().view(REC_DTYPE).reshape(-1)


def rec_buffer(n):
    import torch

    return torch.zeros(n * 6, dtype=torch.int32, device="cuda")


def grid_from_r8(V, ctx, g_r8):
    sz, sy, sx = g_r8.shape
    G = V.Grid(ctx, 2 * sx, 2 * sy, 2 * sz)
    G.import_r8(dev(g_r8))
    return G


def export_r8(G):
    import torch

    out = torch.zeros((G.nz // 2) * (G.ny // 2) * (G.nx // 2), dtype=torch.uint8, device="cuda")
    G.export_r8(out)
    torch.cuda.synchronize()
    return out.cpu().numpy().reshape(G.nz // 2, G.ny // 2, G.nx // 2)


def same_bits(a, b):
    """float32 arrays equal bit for bit, except that any NaN equals any NaN
    (the payload of a generated NaN differs between x86, Arm and the GPU)"""
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    return (a.view(np.int32) == b.view(np.int32)) | (np.isnan(a) & np.isnan(b))


def assert_recs_equal(got, want, what=""):
    """bitwise equality of ray records (t compared as raw bits, NaN == NaN)"""
    assert got.shape == want.shape
    gv = got.view(np.int32).reshape(-1, 6)
    wv = want.view(np.int32).reshape(-1, 6)
    diff = gv != wv
    diff[:, 3] = ~same_bits(got["t"], want["t"])
    bad = np.nonzero(diff.any(axis=1))[0]
    assert bad.size == 0, "%s: %d of %d records differ; first %s: got %s want %s" % (
        what, bad.size, len(gv), bad[:5], got[bad[:3]], want[bad[:3]])
