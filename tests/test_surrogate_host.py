"""Host helpers of the noise surrogate (no GPU): noise sampling, features, parameter vectors."""
import numpy as np

from qiskit_aakash_gb300 import surrogate as S
from qiskit_aakash_gb300 import template as TP


def test_noise_samples_stay_in_their_ranges_and_features_in_unit_box():
    raw = S.sample_noise(5000, seed=0)
    for d in S.LOG_DIMS:
        assert raw[:, d].min() >= 1e-4 and raw[:, d].max() <= 1e-2
    assert raw[:, 3].min() >= 0.8 and raw[:, 3].max() <= 1.0
    assert raw[:, 4].min() >= 0.0 and raw[:, 4].max() <= 0.05
    x = S.features(raw)
    assert x.dtype == np.float32 and x.min() >= -1.0 - 1e-6 and x.max() <= 1.0 + 1e-6
    # log-uniform dimensions fill the box evenly in log space
    assert abs(np.mean(x[:, 0])) < 0.05


def test_param_vectors_equal_the_backend_option_mapping():
    raw = S.sample_noise(50, seed=3)
    v = S.param_vectors(raw)
    for i in range(len(raw)):
        assert np.allclose(v[i], TP.param_vector(S.options_of(raw[i])), rtol=0, atol=1e-15)


def test_layer_offsets_are_aligned_for_the_bf16_gemm():
    layers, P = S._layer_offsets(S.WIDTHS)
    assert P == sum(o * i + o for (_, _, o, i) in layers)
    for w0, b0, out, inp in layers:
        assert w0 % 8 == 0 and inp % 64 == 0 and out % 64 == 0
    assert P % 8 == 0
