"""flock_ntt_noalloc (the NTT for callers that cannot allocate device memory)
against flock_ntt, through the C ABI, bit-exact, on consecutive calls that
share the library's fixed twiddle array."""
import ctypes

import numpy as np
import pytest

import flock_challenge_gb300 as F

pytestmark = pytest.mark.gpu

FLOCK_ERR_LIMIT = -8


def _lib():
    L = F.lib()
    P, i32 = ctypes.c_void_p, ctypes.c_int
    L.flock_ntt_noalloc.argtypes = [P, i32, i32, i32, P]
    L.flock_ntt_noalloc.restype = i32
    L.flock_ntt.argtypes = [P, P, i32, i32, i32, P]
    L.flock_ntt.restype = i32
    return L


def _data(log_d, log_lanes, seed):
    import torch
    rng = np.random.default_rng(seed)
    words = rng.integers(0, 2**63, (1 << (log_d + log_lanes)) * 2, dtype=np.uint64)
    words |= rng.integers(0, 2, words.shape, dtype=np.uint64) << np.uint64(63)
    return torch.from_numpy(words.view(np.uint8).copy()).cuda()


def test_noalloc_ntt_matches_ntt_on_consecutive_calls(cuda_device):
    import torch
    L = _lib()
    ctx = F.Context(0)
    # Sizes change from call to call, so each call runs on the table the
    # previous one left behind; the last case repeats the first.
    cases = [(12, 4, 1, 11), (16, 6, 0, 12), (9, 3, 2, 13), (12, 4, 1, 14)]
    for log_d, log_lanes, start, seed in cases:
        ref = _data(log_d, log_lanes, seed)
        out = ref.clone()
        assert L.flock_ntt(ctx.handle, ctypes.c_void_p(ref.data_ptr()), log_d, log_lanes, start, None) == 0
        assert L.flock_ntt_noalloc(ctypes.c_void_p(out.data_ptr()), log_d, log_lanes, start, None) == 0
        torch.cuda.synchronize()
        assert torch.equal(out, ref), (log_d, log_lanes, start)


def test_noalloc_ntt_rejects_sizes_above_limit(cuda_device):
    import torch
    L = _lib()
    buf = torch.zeros(16 << (17 + 3), dtype=torch.uint8, device="cuda")
    before = buf.clone()
    assert L.flock_ntt_noalloc(ctypes.c_void_p(buf.data_ptr()), 17, 3, 0, None) == FLOCK_ERR_LIMIT
    torch.cuda.synchronize()
    assert torch.equal(buf, before)


def test_noalloc_ntt_takes_no_device_memory(cuda_device):
    # The point of the entry point: after a first call of a shape (which loads
    # its kernels), further calls leave the device's free memory unchanged. A
    # cudaMalloc on this path would take at least one 2 MiB page.
    import torch
    L = _lib()
    data = _data(14, 5, 21)
    ptr = ctypes.c_void_p(data.data_ptr())
    assert L.flock_ntt_noalloc(ptr, 14, 5, 1, None) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert L.flock_ntt_noalloc(ptr, 14, 5, 1, None) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
