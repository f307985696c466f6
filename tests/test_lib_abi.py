"""libvxl.so loads without a GPU and exports every function include/vxl.h
declares; host-only entry points behave (no device work is started here)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "vxl.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:vxl_status|int|uint64_t|const char\*)\s+(vxl_\w+)\s*\(", src, flags=re.M)))


@pytest.fixture(scope="module")
def V():
    import voxelengine_gb300 as V

    V.build()
    return V


def test_every_declared_symbol_is_exported(V):
    names = declared_functions()
    assert len(names) >= 30
    L = C.CDLL(V.LIB_PATH)
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert sorted(V.EXPORTED) == names


def test_binding_declares_every_argument_list(V):
    """ctypes passes an undeclared argument as a C int: a 64-bit device pointer
    would be cut to 32 bits. Every entry point that takes arguments declares them."""
    L = V.lib()
    no_args = {"vxl_abi_version", "vxl_last_error_string"}
    undeclared = [n for n in V.EXPORTED if n not in no_args and getattr(L, n).argtypes is None]
    assert not undeclared, undeclared


def test_abi_version_and_status_strings(V):
    L = V.lib()
    assert L.vxl_abi_version() == 2
    assert L.vxl_status_string(0) == b"VXL_OK"
    assert L.vxl_status_string(5) == b"VXL_ERR_OUT_OF_RANGE"


def test_null_arguments_are_rejected_without_device_work(V):
    L = V.lib()
    assert L.vxl_ctx_create(0, None) == 1
    assert L.vxl_grid_describe(None, None) == 1
    assert L.vxl_trace_rays(None, None, None, 0, 0, None, None) == 1
    assert b"NULL" in L.vxl_last_error_string() or b"bad" in L.vxl_last_error_string()
    assert L.vxl_voxelize_noalloc(None, None, 0, None, 0, None, None) == 1


def test_context_on_a_missing_device_fails_with_a_status(V):
    """Failure on the host, no GPU fault: a context on a device that does not
    exist comes back as a status and a message (no exception across the ABI,
    no context). Without a GPU the device count itself fails (VXL_ERR_CUDA);
    with one, the index is out of range (VXL_ERR_INVALID_ARG)."""
    import ctypes as C

    L = V.lib()
    out = C.c_void_p(12345)
    st = L.vxl_ctx_create(1000, C.byref(out))
    assert st in (1, 3), st
    assert out.value is None
    msg = L.vxl_last_error_string()
    assert msg and (b"device" in msg or b"cuda" in msg.lower())


def test_read_v_fixture_and_errors(V, tmp_path):
    from tests import vox_cases

    m = vox_cases.random_model(np.random.default_rng(0), 5, 7, 9)
    p = tmp_path / "m.v"
    p.write_bytes(np.array([5, 7, 9], np.uint32).tobytes() + m.tobytes())
    got = V.read_v(str(p))
    assert np.array_equal(got, m)
    (tmp_path / "t.v").write_bytes(np.array([5, 7, 9], np.uint32).tobytes() + m.tobytes()[:100])
    with pytest.raises(V.VxlError) as e:
        V.read_v(str(tmp_path / "t.v"))
    assert e.value.status == 6 and "truncated" in str(e.value)
    (tmp_path / "h.v").write_bytes(b"\x01\x00")
    with pytest.raises(V.VxlError):
        V.read_v(str(tmp_path / "h.v"))
    with pytest.raises(V.VxlError):
        V.read_v(str(tmp_path / "missing.v"))


def test_read_v_shipped_assets(V):
    from oracle.ref.build_ref import reference_dir

    d = os.path.join(reference_dir(), "Assets", "Mods", "default", "FarmHouse")
    if not os.path.isdir(d):
        pytest.skip("reference assets not present")
    from tests import vox_cases

    for name in ("0.v", "1.v", "10.v"):
        assert np.array_equal(V.read_v(os.path.join(d, name)), vox_cases.read_v(os.path.join(d, name)))
