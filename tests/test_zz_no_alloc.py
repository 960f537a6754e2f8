"""The allocation-free schedule generator against the allocating one.

knp_gb300_generate_bernoulli_schedule_noalloc exists for callers that cannot allocate GPU memory
when they need a spike schedule (another component owns the memory pool, or the allocator forbids
cudaMalloc/cudaFree in the calling phase). It writes into buffers the caller already holds and keeps
its scratch in a fixed device array. This test compares two consecutive calls with the schedule
that knp_gb300_generate_bernoulli_schedule builds for the same seed, observed through a one-to-one
projection (weight 1.0, delay 1): every scheduled spike of step t makes its neuron fire at step t + 1.
The comparison is exact (integer indexes). The file is collected last so that a failure here
leaves every other test already run.
"""
import ctypes

import numpy as np
import pytest

from knp_gb300 import network as N
from knp_gb300 import types as T

pytestmark = pytest.mark.gpu

N_SRC, STEPS, P, SEED = 5000, 40, 0.05, 11


def _expected_from_allocating_generator():
    from knp_gb300 import backend as B

    pop = N.Population(T.uid_from_int(701), T.BLIFAT, T.blifat_defaults(N_SRC))
    chan = T.uid_from_int(709)
    ar = np.arange(N_SRC, dtype=np.uint32)
    one = N.Projection(T.uid_from_int(702), T.DELTA, T.NULL_UID, pop.uid, ar, ar.copy(),
                       np.ones(N_SRC, np.float32), np.ones(N_SRC, np.uint32))
    b = B.GB300Backend()
    b.load_network(N.Network([pop], [one], [(one.uid, chan)]))
    b._init()
    b.generate_bernoulli_schedule(chan, N_SRC, P, 0, STEPS, seed=SEED)
    b.step(STEPS + 1)
    exp = [b.spikes(pop.uid, t + 1) for t in range(STEPS)]
    b.close()
    return exp


def test_noalloc_schedule_matches_allocating_generator_twice():
    import torch

    from knp_gb300 import _capi

    expected = _expected_from_allocating_generator()
    lib = _capi.lib()
    cap = 40_000
    offs = torch.empty(STEPS + 1, dtype=torch.int64, device="cuda")
    idx = torch.empty(cap, dtype=torch.int32, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        offs.fill_(-1)
        idx.fill_(-1)
        n = ctypes.c_uint64(0)
        rc = lib.knp_gb300_generate_bernoulli_schedule_noalloc(
            N_SRC, P, 0, STEPS, SEED, N.S_INPUT, ctypes.c_void_p(offs.data_ptr()), ctypes.c_void_p(idx.data_ptr()),
            cap, ctypes.byref(n), stream)
        assert rc == 0, lib.knp_gb300_last_error()
        torch.cuda.synchronize()
        o = offs.cpu().numpy()
        ix = idx.cpu().numpy().astype(np.uint32)
        assert o[0] == 0 and o[-1] == n.value
        for t in range(STEPS):
            np.testing.assert_array_equal(ix[o[t]:o[t + 1]], expected[t], err_msg=f"call {call}, step {t}")


def test_noalloc_schedule_rejects_sizes_beyond_its_scratch():
    import torch

    from knp_gb300 import _capi

    lib = _capi.lib()
    offs = torch.empty(1001, dtype=torch.int64, device="cuda")
    idx = torch.empty(16, dtype=torch.int32, device="cuda")
    n = ctypes.c_uint64(0)
    # 1000 steps x 1024 chunks of 4096 sources > 2^18 scratch cells.
    rc = lib.knp_gb300_generate_bernoulli_schedule_noalloc(
        1024 * 4096, 0.01, 0, 1000, 1, N.S_INPUT, ctypes.c_void_p(offs.data_ptr()), ctypes.c_void_p(idx.data_ptr()),
        16, ctypes.byref(n), None)
    assert rc == -1 and b"scratch" in lib.knp_gb300_last_error()
    assert n.value == 0  # argument errors report no count
    # Capacity too small: the needed count comes back, nothing is written.
    rc = lib.knp_gb300_generate_bernoulli_schedule_noalloc(
        N_SRC, P, 0, STEPS, SEED, N.S_INPUT, ctypes.c_void_p(offs.data_ptr()), ctypes.c_void_p(idx.data_ptr()),
        16, ctypes.byref(n), None)
    assert rc == -1 and n.value > 16
    # A probability that is not a finite number is refused (and reports no count).
    rc = lib.knp_gb300_generate_bernoulli_schedule_noalloc(
        N_SRC, float("nan"), 0, STEPS, SEED, N.S_INPUT, ctypes.c_void_p(offs.data_ptr()),
        ctypes.c_void_p(idx.data_ptr()), 16, ctypes.byref(n), None)
    assert rc == -1 and n.value == 0 and b"finite" in lib.knp_gb300_last_error()


def test_noalloc_schedule_later_calls_allocate_no_device_memory():
    """After the first call in a process (which loads the entry point's kernels and scratch array),
    a later call leaves the device's free memory unchanged."""
    import torch

    from knp_gb300 import _capi

    lib = _capi.lib()
    offs = torch.empty(STEPS + 1, dtype=torch.int64, device="cuda")
    idx = torch.empty(40_000, dtype=torch.int32, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    n = ctypes.c_uint64(0)

    def call():
        rc = lib.knp_gb300_generate_bernoulli_schedule_noalloc(
            N_SRC, P, 0, STEPS, SEED, N.S_INPUT, ctypes.c_void_p(offs.data_ptr()), ctypes.c_void_p(idx.data_ptr()),
            idx.numel(), ctypes.byref(n), stream)
        assert rc == 0, lib.knp_gb300_last_error()
        torch.cuda.synchronize()

    call()  # set-up call
    free_before, _ = torch.cuda.mem_get_info()
    call()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before
