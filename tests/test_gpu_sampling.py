"""Shot counts drawn on the device from outcome probabilities (dm_sample_counts, counts_shots option)."""
import ctypes

import numpy as np
import pytest

from qiskit_aakash_gb300 import _native as N

pytestmark = pytest.mark.gpu


def draw(torch, p, shots, seed):
    m = int(np.log2(len(p)))
    pd = torch.from_numpy(np.asarray(p, dtype=np.float64)).cuda()
    counts = torch.empty(2 ** m, dtype=torch.int64, device='cuda')
    scratch = torch.empty(N.lib().dm_sample_counts_scratch_bytes(m), dtype=torch.uint8, device='cuda')
    N.call('dm_sample_counts', ctypes.c_void_p(pd.data_ptr()), m, ctypes.c_int64(shots), ctypes.c_uint64(seed),
           ctypes.c_void_p(counts.data_ptr()), ctypes.c_void_p(scratch.data_ptr()), None)
    return counts.cpu().numpy()


@pytest.mark.parametrize('m', [1, 4, 11, 16])
def test_counts_follow_the_distribution(m):
    import torch
    rng = np.random.default_rng(m)
    p = rng.dirichlet(np.ones(2 ** m) * 0.5)
    p[rng.random(2 ** m) < 0.2] = 0.0          # impossible outcomes
    p[0] -= 1e-17                               # rounding noise below zero counts as zero
    p /= p.sum()
    shots = 2_000_000
    c = draw(torch, p, shots, 7)
    assert c.sum() == shots and (c >= 0).all()
    assert c[p <= 0].sum() == 0
    # every outcome within 6 standard deviations of its expectation
    sd = np.sqrt(shots * p * (1 - p)) + 1
    assert np.all(np.abs(c - shots * p) <= 6 * sd)
    assert np.array_equal(c, draw(torch, p, shots, 7))        # deterministic in the seed
    assert not np.array_equal(c, draw(torch, p, shots, 8))


def test_backend_counts_option():
    import copy
    from qiskit_aakash_gb300 import BasicAer, execute, random_layer_circuit, noise_options
    qc = random_layer_circuit(5, 3, 2)
    opts = noise_options(depolarisation=1e-2, decoherence=0.99, decay=0.99)
    res = execute(qc, BasicAer.get_backend('dm_simulator'), counts_shots=100000, counts_seed=3,
                  **copy.deepcopy(opts)).result()['results'][0]['data']
    probs, counts = res['ensemble_probability'], res['counts']
    assert sum(counts.values()) == 100000 and set(counts) <= set(probs)
    for k, c in counts.items():
        assert abs(c - 1e5 * probs[k]) <= 6 * np.sqrt(1e5 * probs[k]) + 2
    res2 = execute(qc, BasicAer.get_backend('dm_simulator'), **copy.deepcopy(opts)).result()['results'][0]['data']
    assert 'counts' not in res2


def test_no_positive_probability_draws_nothing():
    """All-zero (or negative) probabilities: no shot is drawn, every count is 0."""
    import torch
    p = np.zeros(16)
    p[3] = -1e-18
    c = draw(torch, p, 1000, 5)
    assert c.sum() == 0
