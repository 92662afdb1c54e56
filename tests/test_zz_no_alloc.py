"""kzg_state_hash_noalloc (the allocation-free state hash) against kzg_state_hash, through the C-ABI.

The file name sorts last so that the run also covers the entry point after every other test has
used the device; it passes on its own as well.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KZG_ERR_CAPACITY = -3
MAX_BODIES = 16384
FNV_OFFSET = 1469598103934665603


def _entry():
    from kizuriphysics3d_gb300 import capi
    f = capi.load().kzg_state_hash_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p,
                  ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_char_p)]
    return f


def _noalloc_hash(state_ptr, ids_ptr, n):
    out, err = ctypes.c_uint64(), ctypes.c_char_p()
    status = _entry()(state_ptr, ids_ptr, n, None, ctypes.byref(out), ctypes.byref(err))
    return status, out.value, (err.value or b"").decode()


def _device_copy(world):
    import torch
    state = torch.from_numpy(np.ascontiguousarray(world.state(), np.float32)).cuda()
    ids = torch.arange(world.n, dtype=torch.int32, device="cuda")  # BodyID(slot, 0).Packed()
    torch.cuda.synchronize()
    return state, ids


def test_matches_state_hash_on_two_calls_in_a_row():
    """A large world then a smaller one: the second call must not see the first call's words."""
    from kizuriphysics3d_gb300 import World, scenes
    with World(scenes.pile(3000, seed=99)) as big, World(scenes.pyramid(6)) as small:
        big.step_fixed(n=40)
        small.step_fixed(n=40)
        results = []
        for w in (big, small):
            state, ids = _device_copy(w)
            status, h, err = _noalloc_hash(state.data_ptr(), ids.data_ptr(), w.n)
            assert status == 0, err
            results.append((h, w.compute_state_hash()))
        for got, want in results:
            assert got == want
        assert results[0][0] != results[1][0]


def test_empty_state_is_the_fnv_offset_basis():
    status, h, err = _noalloc_hash(None, None, 0)
    assert status == 0, err
    assert h == FNV_OFFSET


def test_rejects_more_bodies_than_the_scratch_holds():
    import torch
    state = torch.zeros((MAX_BODIES + 1) * 13, dtype=torch.float32, device="cuda")
    ids = torch.zeros(MAX_BODIES + 1, dtype=torch.int32, device="cuda")
    status, _, err = _noalloc_hash(state.data_ptr(), ids.data_ptr(), MAX_BODIES + 1)
    assert status == KZG_ERR_CAPACITY
    assert "16384" in err
