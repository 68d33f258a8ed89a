"""C-ABI checks that need no GPU: the library loads, exports everything include/lsdg.h declares,
shares the oracle's parameter table, and rejects bad arguments with a status (no crash)."""
import ctypes as C

import numpy as np
import pytest

import lsdg
import lsdg_types as T
import lsdo


def test_library_exports_every_declared_symbol():
    L = lsdg.lib()
    declared = lsdg.declared_symbols()
    assert len(declared) >= 25
    missing = [s for s in declared if not hasattr(L, s)]
    assert not missing, missing


def test_abi_version():
    assert lsdg.lib().lsdg_abi_version() == 1


def test_default_params_match_oracle_table():
    assert lsdg.default_params().as_bytes() == lsdo.default_params().as_bytes()


def test_struct_sizes():
    assert C.sizeof(T.Intrinsics) == 16
    assert C.sizeof(T.TrackStats) % 8 == 0


def test_create_rejects_bad_params():
    p = lsdg.default_params()
    p.levels = 0
    h = C.c_void_p()
    assert lsdg.lib().lsdg_create(C.byref(h), C.byref(p), 0) == T.INVALID_ARG
    p = lsdg.default_params()
    p.max_search_len = 5000
    assert lsdg.lib().lsdg_create(C.byref(h), C.byref(p), 0) == T.INVALID_ARG


def test_null_arguments_return_status():
    L = lsdg.lib()
    assert L.lsdg_create(None, None, 0) == T.INVALID_ARG
    assert L.lsdg_destroy(None) == T.INVALID_ARG
    assert L.lsdg_sync(None) == T.INVALID_ARG
    assert L.lsdg_last_error(None) == b"null context"
    k = T.Intrinsics(500, 500, 320, 240)
    h = C.c_void_p()
    assert L.lsdg_frame_create(None, 640, 480, C.byref(k), C.byref(h)) == T.INVALID_ARG


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-GPU failure path")
def test_create_without_gpu_fails_cleanly():
    h = C.c_void_p()
    rc = lsdg.lib().lsdg_create(C.byref(h), None, 0)
    assert rc in (T.CUDA_ERROR, T.NOT_SUPPORTED)
    assert not h.value


def test_sim3_pose_packing():
    """(R|t, s) tuples map onto the ABI's 13-double {R, t, s} layout."""
    import lsdg
    M = np.arange(12, dtype=np.float64).reshape(3, 4)
    a = lsdg._pose13((M, 2.5))
    np.testing.assert_array_equal(a[:9], M[:, :3].ravel())
    np.testing.assert_array_equal(a[9:12], M[:, 3])
    assert a[12] == 2.5


def test_sim3_pose_unpacking_inverts_packing():
    import lsdg
    M = np.arange(12, dtype=np.float64).reshape(3, 4)
    M2, s = lsdg.unpack13(lsdg._pose13((M, 1.7)))
    np.testing.assert_array_equal(M2, M)
    assert s == 1.7
