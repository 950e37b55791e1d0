"""gbmie_s12_noalloc: S1/S2 for callers that cannot allocate device memory.

Some callers of this library run inside another framework's memory pool or
allocator-owned region, or must not grow the device footprint after
start-up, so they cannot let the library call cudaMalloc.
gbmie_s12_noalloc computes the same S1/S2 as gbmie_s12 from caller-owned
inputs and outputs, keeping its angular table in a fixed device array inside
the library.  This test calls it through the C ABI twice in a row (different
sizes, cosines and angle counts, so the second call must not depend on what
the first left in the shared array) and checks both against gbmie_s12 within
1e-13 of each instance's largest |S|; then that a call allocates nothing,
that an invalid call is reported and does not disturb the next one, and the
capacity limit.

The file name makes pytest collect it last.
"""
import ctypes

import numpy as np
import pytest

P = ctypes.c_void_p


def _case(seed, n, nang):
    import torch
    from geosmie_gb300.mie import coefficients, s12
    rng = np.random.default_rng(seed)
    x = np.sort(10.0 ** rng.uniform(-2.0, 2.2, n))
    m = 1.45 + 0.1 * rng.random() + 1j * 10.0 ** rng.uniform(-6, -1)
    off, an, bn, _ = coefficients(x, m * m)
    cost = np.cos(np.radians(np.sort(rng.uniform(0.0, 180.0, nang))))
    ref1, ref2 = s12(off, an, bn, cost)
    nmax_max = int(np.max(np.diff(off.cpu().numpy())))
    dcost = torch.as_tensor(cost).cuda()
    return off, an, bn, nmax_max, dcost, ref1, ref2


@pytest.mark.gpu
def test_s12_noalloc_matches_s12_twice():
    import torch
    from geosmie_gb300 import _native
    lib = _native.load()
    stream = torch.cuda.current_stream().cuda_stream
    for seed, n, nang in [(1, 300, 181), (2, 57, 37)]:
        off, an, bn, nmax_max, dcost, ref1, ref2 = _case(seed, n, nang)
        s1 = torch.full_like(ref1, float("nan"))
        s2 = torch.full_like(ref2, float("nan"))
        st = lib.gbmie_s12_noalloc(P(stream), n, P(off.data_ptr()), P(an.data_ptr()), P(bn.data_ptr()),
                                   nmax_max, nang, P(dcost.data_ptr()), P(s1.data_ptr()), P(s2.data_ptr()))
        assert st == 0, lib.gbmie_status_string(st)
        r1, r2 = ref1.cpu().numpy(), ref2.cpu().numpy()
        g1, g2 = s1.cpu().numpy(), s2.cpu().numpy()
        scale = np.maximum(np.abs(r1).max(axis=1, keepdims=True), np.abs(r2).max(axis=1, keepdims=True))
        assert np.max(np.abs(g1 - r1) / scale) < 1e-13
        assert np.max(np.abs(g2 - r2) / scale) < 1e-13


@pytest.mark.gpu
def test_s12_noalloc_allocates_nothing_and_clears_status():
    """After a first call (which looks up the array's device address), a call
    leaves torch's allocator and the device's free memory unchanged.  A call
    with an invalid cosine (|u| > 1, NaN) returns GBMIE_ERR_INVALID; the next
    valid call matches gbmie_s12 again, so the status word and the table rows
    the invalid call skipped do not leak into it."""
    import torch
    from geosmie_gb300 import _native
    lib = _native.load()
    stream = torch.cuda.current_stream().cuda_stream
    off, an, bn, nmax_max, dcost, ref1, ref2 = _case(4, 120, 91)
    s1 = torch.empty_like(ref1)
    s2 = torch.empty_like(ref2)

    def call(cost):
        return lib.gbmie_s12_noalloc(P(stream), 120, P(off.data_ptr()), P(an.data_ptr()), P(bn.data_ptr()),
                                     nmax_max, 91, P(cost.data_ptr()), P(s1.data_ptr()), P(s2.data_ptr()))
    assert call(dcost) == 0
    torch.cuda.synchronize()
    alloc0 = torch.cuda.memory_allocated()
    free0, _ = torch.cuda.mem_get_info()
    assert call(dcost) == 0
    torch.cuda.synchronize()
    assert torch.cuda.memory_allocated() == alloc0
    assert torch.cuda.mem_get_info()[0] == free0
    for bad in (1.5, float("nan")):
        badcost = dcost.clone()
        badcost[45] = bad
        assert call(badcost) == 1   # GBMIE_ERR_INVALID
    assert call(dcost) == 0
    r1, r2 = ref1.cpu().numpy(), ref2.cpu().numpy()
    scale = np.maximum(np.abs(r1).max(axis=1, keepdims=True), np.abs(r2).max(axis=1, keepdims=True))
    assert np.max(np.abs(s1.cpu().numpy() - r1) / scale) < 1e-13
    assert np.max(np.abs(s2.cpu().numpy() - r2) / scale) < 1e-13


@pytest.mark.gpu
def test_s12_noalloc_rejects_oversize():
    import torch
    from geosmie_gb300 import _native
    lib = _native.load()
    stream = torch.cuda.current_stream().cuda_stream
    off, an, bn, nmax_max, dcost, ref1, ref2 = _case(3, 20, 19)
    s1 = torch.empty_like(ref1)
    s2 = torch.empty_like(ref2)
    # 4 MiB of (p, q) pairs hold 262144 (order, angle) entries
    st = lib.gbmie_s12_noalloc(P(stream), 20, P(off.data_ptr()), P(an.data_ptr()), P(bn.data_ptr()),
                               262144 // 19 + 1, 19, P(dcost.data_ptr()), P(s1.data_ptr()), P(s2.data_ptr()))
    assert st == 7   # GBMIE_ERR_CAPACITY
    # an instance with more orders than nmax_max is refused, not read past the table
    st = lib.gbmie_s12_noalloc(P(stream), 20, P(off.data_ptr()), P(an.data_ptr()), P(bn.data_ptr()),
                               max(2, nmax_max - 1), 19, P(dcost.data_ptr()), P(s1.data_ptr()), P(s2.data_ptr()))
    assert st == 2   # GBMIE_ERR_NMAX
