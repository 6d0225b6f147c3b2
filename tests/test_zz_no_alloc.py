"""dm_nbasis_probs_noalloc: the basis-N measurement with no device allocation.

Some callers of this library cannot call cudaMalloc: their device memory is
already handed to another allocator (a framework's caching pool) where raw
allocations fail or are not allowed, or they sit on a latency-critical path
where cudaMalloc/cudaFree would synchronise the device.  For them the
library offers one entry point whose scratch lives in a file-scope device
array (1.5 MiB, n <= 10).  This file checks it through the C ABI against
the allocating entry point dm_nbasis_probs, on two calls in a row (the
second call must not see anything the first one left in the shared array).
It is collected last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes

import numpy as np
import pytest

from qiskit_aakash_gb300 import _native as N

pytestmark = pytest.mark.gpu

TOL = 1e-12          # the FP64 tolerance of the other measurement tests


@pytest.fixture(scope='module')
def torch():
    import torch
    if not torch.cuda.is_available():
        pytest.fail('CUDA device required for the gpu tests')
    N.build()
    N.lib()
    return torch


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


def _allocating(torch, state, n, nvec, err, stream):
    L = N.lib()
    scratch = torch.empty(max(8, L.dm_nbasis_probs_scratch_bytes(n)), dtype=torch.uint8, device='cuda')
    out = torch.empty(2 ** n, dtype=torch.float64, device='cuda')
    v = N.f64_array(nvec)
    N.call('dm_nbasis_probs', _vp(state), n, N.DM_F64, v, err, _vp(out), _vp(scratch), stream)
    return out.cpu().numpy()


@pytest.mark.parametrize('n', [2, 4, 7, 10])
def test_noalloc_matches_allocating_entry_point_twice(torch, n):
    rng = np.random.default_rng(4242 + n)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        st = torch.from_numpy(rng.normal(size=4 ** n) / 2 ** n).cuda()
        nvec = rng.normal(size=3)
        nvec /= np.linalg.norm(nvec)
        err = float(rng.uniform(0.9, 1.0))
        out = torch.full((2 ** n,), float('nan'), dtype=torch.float64, device='cuda')
        v = N.f64_array(nvec)
        N.call('dm_nbasis_probs_noalloc', _vp(st), n, N.DM_F64, v, err, _vp(out), stream)
        got = out.cpu().numpy()
        ref = _allocating(torch, st, n, nvec, err, stream)
        assert np.isfinite(got).all(), 'call %d' % call
        np.testing.assert_allclose(got, ref, rtol=0, atol=TOL * max(1.0, np.abs(ref).max()))


def test_noalloc_rejects_registers_beyond_its_array(torch):
    n = 11
    st = torch.zeros(4 ** n, dtype=torch.float64, device='cuda')
    out = torch.zeros(2 ** n, dtype=torch.float64, device='cuda')
    rc = N.lib().dm_nbasis_probs_noalloc(_vp(st), n, N.DM_F64, N.f64_array([0, 0, 1]), 1.0, _vp(out),
                                         ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == N.DM_ERR_RANGE
