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


def _noalloc_hash(state_ptr, ids_ptr, n, stream=None):
    out, err = ctypes.c_uint64(), ctypes.c_char_p()
    status = _entry()(state_ptr, ids_ptr, n, stream, ctypes.byref(out), ctypes.byref(err))
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


def test_allocates_nothing_across_repeated_calls():
    """After a first call (which does the per-device set-up), further calls leave the device's free
    memory and torch's allocator exactly as they were: nothing is allocated or freed."""
    import torch
    from kizuriphysics3d_gb300 import World, scenes
    with World(scenes.pile(2000, seed=5)) as w:
        w.step_fixed(n=20)
        state, ids = _device_copy(w)
        status, first, err = _noalloc_hash(state.data_ptr(), ids.data_ptr(), w.n)
        assert status == 0, err
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info()
        alloc0, reserved0 = torch.cuda.memory_allocated(), torch.cuda.memory_reserved()
        for _ in range(5):
            status, h, err = _noalloc_hash(state.data_ptr(), ids.data_ptr(), w.n)
            assert status == 0, err
            assert h == first
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        assert free1 == free0
        assert torch.cuda.memory_allocated() == alloc0 and torch.cuda.memory_reserved() == reserved0
        assert first == w.compute_state_hash()


def test_exactly_the_maximum_on_a_caller_stream():
    """n == KZG_NOALLOC_HASH_MAX_BODIES on a non-default stream, against kzg_state_hash."""
    import torch
    from kizuriphysics3d_gb300 import World, scenes
    with World(scenes.stacks(8, 8, MAX_BODIES // 64 - 1)) as w:
        assert w.n <= MAX_BODIES
        w.step_fixed(n=3)
        state, ids = _device_copy(w)
        # pad to exactly the maximum with copies of the last body (same words in both hashes)
        pad = MAX_BODIES - w.n
        st_full = torch.cat([state, state[-1:].repeat(pad, 1)]).contiguous()
        id_full = torch.cat([ids, ids[-1:].repeat(pad)]).contiguous()
        s = torch.cuda.Stream()
        torch.cuda.synchronize()
        status, h, err = _noalloc_hash(st_full.data_ptr(), id_full.data_ptr(), MAX_BODIES, ctypes.c_void_p(s.cuda_stream))
        assert status == 0, err
        words = np.zeros((MAX_BODIES, 14), np.uint64)
        host = st_full.cpu().numpy()
        words[:, 0] = id_full.cpu().numpy().astype(np.uint64)
        words[:, 1:] = (host * np.float32(100000.0)).astype(np.int64).astype(np.uint64)
        want = FNV_OFFSET
        for v in words.reshape(-1).tolist():
            want = ((want ^ v) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
        assert h == want
        status, h2, err = _noalloc_hash(state.data_ptr(), ids.data_ptr(), w.n, ctypes.c_void_p(s.cuda_stream))
        assert status == 0, err
        assert h2 == w.compute_state_hash()


def test_rejects_host_memory():
    """A host pointer (pageable or pinned) is refused before any kernel could read it."""
    import torch
    host = np.zeros((4, 13), np.float32)
    ids = np.zeros(4, np.uint32)
    status, _, err = _noalloc_hash(host.ctypes.data, ids.ctypes.data, 4)
    assert status == -1 and "device pointers" in err
    pinned = torch.zeros((4, 13), dtype=torch.float32).pin_memory()
    dev_ids = torch.zeros(4, dtype=torch.int32, device="cuda")
    status, _, err = _noalloc_hash(pinned.data_ptr(), dev_ids.data_ptr(), 4)
    assert status == -1 and "current device" in err
