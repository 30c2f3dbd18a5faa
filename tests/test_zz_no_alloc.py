"""faco_pheromone_step_noalloc: the pheromone step on device buffers with a
fixed file-scope scratch.  Its results equal faco_pheromone_step's (host
buffers, per-call device allocations) bit for bit, call after call, so no
state leaks through the shared scratch.  This file sorts last so that the
entry point also runs after every other GPU test in the session."""
import ctypes as C

import numpy as np
import pytest

from tests import _cases

pytestmark = pytest.mark.gpu

MAX_NODES = 65535


def _case(oracle, n, k, seed):
    rng = np.random.default_rng(seed)
    xy = _cases.uniform_instance(n, seed=seed)
    primary = np.ascontiguousarray(oracle.prepare(xy, k, 0, min(20, n - 1))["primary"], dtype=np.uint32)
    d = oracle.euc2d_matrix(xy)[np.arange(n)[:, None], primary]
    eta = (1.0 / np.maximum(1, d)).astype(np.float32)
    trails = rng.uniform(1e-7, 2e-6, (n, k)).astype(np.float32)
    parent = rng.permutation(n).astype(np.uint32)
    return primary, parent, eta, trails


def _host_step(lib, primary, parent, eta, trails, ret, tmin, tmax, inc):
    n, k = primary.shape
    t = trails.copy()
    p = np.zeros_like(trails)
    code = lib.faco_pheromone_step(n, k, primary.ctypes.data, parent.ctypes.data, ret, tmin, tmax, inc,
                                   eta.ctypes.data, t.ctypes.data, p.ctypes.data)
    assert code == 0, lib.faco_last_error()
    return t, p


class _Device:
    """The case's arrays as device tensors (torch is only the allocator)."""

    def __init__(self, primary, parent, eta, trails):
        import torch
        dev = torch.device("cuda", 0)
        self.primary = torch.from_numpy(primary.astype(np.int32)).to(dev)   # same bits as u32 (< 2^31)
        self.parent = torch.from_numpy(parent.astype(np.int32)).to(dev)
        self.eta = torch.from_numpy(eta).to(dev)
        self.trails = torch.from_numpy(trails).to(dev)
        self.products = torch.zeros_like(self.trails)
        self.n, self.k = primary.shape

    def step(self, lib, ret, tmin, tmax, inc, stream=None, parent_ptr=None):
        return lib.faco_pheromone_step_noalloc(self.n, self.k, self.primary.data_ptr(),
                                               parent_ptr or self.parent.data_ptr(), ret, tmin, tmax, inc,
                                               self.eta.data_ptr(), self.trails.data_ptr(),
                                               self.products.data_ptr(), stream)

    def result(self):
        return self.trails.cpu().numpy(), self.products.cpu().numpy()


def test_no_alloc_matches_allocating_step_on_consecutive_calls(engine_lib, oracle):
    import torch
    lib = engine_lib
    ret, tmin, tmax, inc = float(np.float32(0.98)), float(np.float32(1e-7)), float(np.float32(2e-6)), \
        float(np.float32(1 / 7.3e7))
    # a caller's own non-blocking stream for the second call of each case
    # (the first runs on the legacy default stream, NULL)
    side = torch.cuda.Stream(device=0)
    assert side.cuda_stream != 0
    # a large vectorised case (k % 4 == 0), then a smaller scalar one (k odd)
    # that reads the scratch after the larger call left its entries behind
    for n, k, seed in ((1000, 16, 5), (537, 7, 6)):
        primary, parent, eta, trails = _case(oracle, n, k, seed)
        dev = _Device(primary, parent, eta, trails)
        torch.cuda.synchronize()
        ref_t, ref_p = trails, None
        for call in range(2):   # two calls in a row on the same buffers
            ref_t, ref_p = _host_step(lib, primary, parent, eta, ref_t, ret, tmin, tmax, inc)
            if call:
                with torch.cuda.stream(side):
                    code = dev.step(lib, ret, tmin, tmax, inc, C.c_void_p(side.cuda_stream))
            else:
                code = dev.step(lib, ret, tmin, tmax, inc, None)
            assert code == 0, lib.faco_last_error()
            got_t, got_p = dev.result()
            assert np.array_equal(got_t, ref_t) and np.array_equal(got_p, ref_p), (n, k, call)
        # and the oracle's FP32 restatement of the same two steps
        o_t = trails.reshape(-1).copy()
        o_p = np.zeros(n * k, np.float32)
        for _ in range(2):
            d = C.c_float(tmax)
            oracle.lib().orc_pheromone32(n, k, primary, parent, np.float32(ret), np.float32(tmin),
                                         np.float32(tmax), np.float32(inc), eta.reshape(-1), o_t, o_p, C.byref(d))
        assert np.array_equal(dev.result()[0].reshape(-1), o_t)


def test_no_alloc_rejects_invalid_inputs_and_recovers(engine_lib, oracle):
    import torch
    lib = engine_lib
    ret, tmin, tmax, inc = 0.5, 1e-7, 2e-6, 1e-8
    primary, parent, eta, trails = _case(oracle, 300, 8, 9)
    dev = _Device(primary, parent, eta, trails)
    # a parent that repeats a node: found on the device, buffers untouched
    bad = parent.copy()
    bad[1] = bad[0]
    bad_dev = torch.from_numpy(bad.astype(np.int32)).cuda()
    assert dev.step(lib, ret, tmin, tmax, inc, parent_ptr=bad_dev.data_ptr()) == -1
    assert b"permutation" in lib.faco_last_error()
    assert np.array_equal(dev.result()[0], trails)
    # a parent entry out of range: also found on the device
    bad[1] = 300
    bad_dev = torch.from_numpy(bad.astype(np.int32)).cuda()
    assert dev.step(lib, ret, tmin, tmax, inc, parent_ptr=bad_dev.data_ptr()) == -1
    assert b"out of range" in lib.faco_last_error()
    assert np.array_equal(dev.result()[0], trails)
    # the next valid call is exact again (the error word is cleared per call)
    assert dev.step(lib, ret, tmin, tmax, inc) == 0, lib.faco_last_error()
    ref_t, ref_p = _host_step(lib, primary, parent, eta, trails, ret, tmin, tmax, inc)
    got_t, got_p = dev.result()
    assert np.array_equal(got_t, ref_t) and np.array_equal(got_p, ref_p)
    # host pointers and sizes beyond the scratch are refused before any work
    host = trails.copy()
    code = lib.faco_pheromone_step_noalloc(300, 8, dev.primary.data_ptr(), dev.parent.data_ptr(), ret, tmin, tmax,
                                           inc, dev.eta.data_ptr(), host.ctypes.data, dev.products.data_ptr(), None)
    assert code == -1 and b"device pointers" in lib.faco_last_error()
    code = lib.faco_pheromone_step_noalloc(MAX_NODES + 1, 1, dev.primary.data_ptr(), dev.parent.data_ptr(), ret,
                                           tmin, tmax, inc, dev.eta.data_ptr(), dev.trails.data_ptr(),
                                           dev.products.data_ptr(), None)
    assert code == -1 and b"65535" in lib.faco_last_error()
