"""lsdg_depth_propagate_noalloc: propagateDepth for callers that cannot allocate device memory when a
keyframe changes (an application that reserves all GPU memory up front and forbids allocation in its
real-time mapping thread, or that records the mapping step inside its own stream capture).  It must
give exactly what the context-based lsdg_depth_create_keyframe gives (the depth tests' bar is
bit-identity), on two calls in a row through the same shared z-buffer.

This file is collected last on purpose; it runs alone in a fresh process as well as after the
other tests."""
import ctypes as C

import numpy as np
import pytest

import lsdg
import lsdg_types as T
import lsdo
import synth

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _entry():
    f = lsdg.lib().lsdg_depth_propagate_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(T.Intrinsics), C.POINTER(T.Params),
                  np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")] + [C.c_void_p] * 11
    return f


def test_propagate_noalloc_matches_create_keyframe():
    torch = pytest.importorskip("torch")
    seq = synth.depth_sequence(11, 640, 480)
    key_to_new = lsdo._inv(seq.next_to_key)
    ctx = lsdg.Context()
    dm = lsdg.DepthMap(ctx, seq.w, seq.h, seq.intr).set_keyframe(seq.key_image, seq.init_idepth, seq.init_var)
    dm.updateKeyframe(seq.ref_images, [lsdo._inv(T_) for T_ in seq.ref_frame_to_key], regularize=True)
    old = dm.get()
    dm.createKeyFrame(seq.next_image, key_to_new, regularize=False)
    want = dm.get()
    dm.close()

    f = _entry()
    intr = lsdg.intrinsics(seq.intr)
    params = lsdg.default_params()
    ins = [_dev(torch, x) for x in (seq.key_image.astype(np.float32), seq.next_image.astype(np.float32),
                                    old["idepth"], old["var"], old["validity"])]
    names = ("idepth", "var", "idepth_smoothed", "var_smoothed", "validity", "blacklist")
    stream = torch.cuda.current_stream()
    for call in range(2):
        outs = {n: torch.full((seq.h, seq.w), 7 + call, dtype=torch.int32 if n in ("validity", "blacklist")
                              else torch.float32, device="cuda") for n in names}
        rc = f(stream.cuda_stream, seq.w, seq.h, C.byref(intr), C.byref(params),
               np.ascontiguousarray(key_to_new, np.float64).ravel(),
               *[t.data_ptr() for t in ins], *[outs[n].data_ptr() for n in names])
        assert rc == T.OK
        stream.synchronize()
        for n in names:
            np.testing.assert_array_equal(outs[n].cpu().numpy(), want[n], err_msg=f"call {call}: {n}")


def test_propagate_noalloc_rejects_oversized_keyframes():
    f = _entry()
    intr = T.Intrinsics(500, 500, 320, 240)
    params = lsdg.default_params()
    pose = np.ascontiguousarray(np.eye(3, 4), np.float64).ravel()
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = f(None, 2048, 2048, C.byref(intr), C.byref(params), pose, *([dummy] * 11))
    assert rc == T.INVALID_ARG
