"""spp_pairs_noalloc: the pair search for callers that cannot allocate GPU
memory (a component under another owner's fixed memory budget, or a loop in
which cudaMalloc/cudaFree would synchronise the device).

The caller owns every buffer (here: torch tensors standing in for memory the
host application already has); the entry point's own scratch is a static
device array inside the library.  Its output must equal that of the existing
entry point, spp_pairs, on two calls in a row -- the second call reuses the
scratch the first one left behind.  This file is collected last so that a
run stopping at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from spp_gb300 import System, abi, configs

pytestmark = pytest.mark.gpu


def pairs_via_system(x, y, n, L, r):
    p = configs.abp_config(n=n, L=L, seed=1)
    _, _, th = configs.random_state(n, L, seed=1)
    with System(p) as s:
        s.upload(x, y, th)
        return s.pairs(r)


def pairs_noalloc(lib, x, y, L, r, cap, stream=None):
    import torch
    n = len(x)
    dx = torch.from_numpy(np.ascontiguousarray(x, np.float32)).cuda()
    dy = torch.from_numpy(np.ascontiguousarray(y, np.float32)).cuda()
    pi = torch.empty(cap, dtype=torch.int32, device="cuda")
    pj = torch.empty(cap, dtype=torch.int32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    handle = C.c_void_p(stream.cuda_stream) if stream is not None else None
    rc = lib.spp_pairs_noalloc(C.c_void_p(dx.data_ptr()), C.c_void_p(dy.data_ptr()), n, float(L),
                               float(r), C.c_void_p(pi.data_ptr()), C.c_void_p(pj.data_ptr()),
                               cap, C.c_void_p(cnt.data_ptr()), handle)
    assert rc == abi.SPP_OK, lib.spp_last_error()
    if stream is not None:
        stream.synchronize()
    torch.cuda.synchronize()
    total = int(cnt.item())
    m = min(total, cap)
    a = pi[:m].cpu().numpy().astype(np.int64)
    b = pj[:m].cpu().numpy().astype(np.int64)
    return total, np.sort(np.minimum(a, b) * (1 << 32) + np.maximum(a, b))


def test_noalloc_pairs_match_spp_pairs_twice(gpu_lib):
    n, L, r = 4096, 32.0, 1.0
    x1, y1, _ = configs.random_state(n, L, seed=11)
    x2, y2, _ = configs.random_state(n, L, seed=12)
    ref1 = pairs_via_system(x1, y1, n, L, r)
    ref2 = pairs_via_system(x2, y2, n, L, r)
    cap = 8 * n
    t1, got1 = pairs_noalloc(gpu_lib, x1, y1, L, r, cap)
    assert t1 == ref1.size and np.array_equal(got1, ref1)
    t2, got2 = pairs_noalloc(gpu_lib, x2, y2, L, r, cap)  # second call in a row, new inputs
    assert t2 == ref2.size and np.array_equal(got2, ref2)
    t3, got3 = pairs_noalloc(gpu_lib, x1, y1, L, r, cap)  # and back: nothing stale survives
    assert t3 == ref1.size and np.array_equal(got3, ref1)


def test_noalloc_reports_total_beyond_capacity(gpu_lib):
    n, L, r = 2048, 16.0, 1.0
    x, y, _ = configs.random_state(n, L, seed=13)
    ref = pairs_via_system(x, y, n, L, r)
    total, got = pairs_noalloc(gpu_lib, x, y, L, r, cap=100)
    assert total == ref.size and got.size == 100
    assert np.all(np.isin(got, ref))


def test_noalloc_rejects_sizes_beyond_the_limit(gpu_lib):
    big = abi.lib().spp_pairs_noalloc(C.c_void_p(1), C.c_void_p(1), 65537, 512.0, 1.0, None,
                                      None, 0, C.c_void_p(1), None)
    assert big == 1
    assert b"65536" in gpu_lib.spp_last_error()
    small_box = gpu_lib.spp_pairs_noalloc(C.c_void_p(1), C.c_void_p(1), 10, 1.0, 1.0, None, None, 0,
                                          C.c_void_p(1), None)
    assert small_box == 1


def test_noalloc_clamped_grid_smallest_grid_and_a_stream(gpu_lib):
    """Grid edge cases against the existing pair search: a sparse box whose
    2L/r (1024) is clamped to 256 cells per side (wider cells, more
    candidates, the same pairs), the smallest grid of 3 x 3 cells, where every
    wrapped neighbour cell is distinct (checked against the oracle's FP32
    pair predicate, since a system handle needs cells wider than its list
    radius), and a call enqueued on a non-default stream."""
    import torch
    from oracle import oracle as O
    n, L, r = 4096, 512.0, 1.0
    x, y, _ = configs.random_state(n, L, seed=21)
    # a cluster as well, so that the sparse box has pairs to find
    x[:512] = (x[:512] / L * 4.0).astype(np.float32)
    y[:512] = (y[:512] / L * 4.0).astype(np.float32)
    ref = pairs_via_system(x, y, n, L, r)
    assert ref.size > 100
    total, got = pairs_noalloc(gpu_lib, x, y, L, r, 8 * n)
    assert total == ref.size and np.array_equal(got, ref)
    side = torch.cuda.Stream()
    total, got = pairs_noalloc(gpu_lib, x, y, L, r, 8 * n, stream=side)
    assert total == ref.size and np.array_equal(got, ref)

    n3, L3 = 60, 1.6      # floor(2L / (1.001 r)) = 3 cells per side
    x3, y3, _ = configs.random_state(n3, L3, seed=22)
    ref3 = O.pairs32(configs.abp_config(n=n3, L=L3, seed=1), x3, y3, r)
    assert ref3.size > 0
    total, got = pairs_noalloc(gpu_lib, x3, y3, L3, r, 8 * n3 * n3)
    assert total == ref3.size and np.array_equal(got, ref3)


def test_noalloc_calls_take_no_device_memory(gpu_lib):
    """The promise itself: after one warm call (the context, the library's
    device code and the caller's buffers exist), further calls leave the
    device's free memory unchanged."""
    import torch
    n, L, r = 8192, 64.0, 1.0
    x, y, _ = configs.random_state(n, L, seed=23)
    dx = torch.from_numpy(x).cuda()
    dy = torch.from_numpy(y).cuda()
    cap = 8 * n
    pi = torch.empty(cap, dtype=torch.int32, device="cuda")
    pj = torch.empty(cap, dtype=torch.int32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int64, device="cuda")

    def call():
        rc = gpu_lib.spp_pairs_noalloc(C.c_void_p(dx.data_ptr()), C.c_void_p(dy.data_ptr()), n,
                                       float(L), float(r), C.c_void_p(pi.data_ptr()),
                                       C.c_void_p(pj.data_ptr()), cap, C.c_void_p(cnt.data_ptr()),
                                       None)
        assert rc == abi.SPP_OK, gpu_lib.spp_last_error()

    call()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(5):
        call()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert int(cnt.item()) > 0
