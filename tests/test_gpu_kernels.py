"""Each C-ABI entry point on the GPU against the CPU oracle's numpy kernels."""
import ctypes

import numpy as np
import pytest

from oracle import dm_oracle as O
from qiskit_aakash_gb300 import _native as N
from qiskit_aakash_gb300 import program as P

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def torch():
    import torch
    if not torch.cuda.is_available():
        pytest.fail('CUDA device required for the gpu tests')
    N.build()
    N.lib()
    return torch


def dev(torch, a, dtype=np.float64):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).cuda()


def vp(t):
    return ctypes.c_void_p(t.data_ptr())


def stream(torch):
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def dparr(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


@pytest.mark.parametrize('n', [1, 2, 3, 5, 8])
@pytest.mark.parametrize('dtype', [N.DM_F64, N.DM_F32])
def test_map1_cx_noise(torch, n, dtype):
    rng = np.random.default_rng(n)
    npdt = np.float64 if dtype == N.DM_F64 else np.float32
    tol = 1e-13 if dtype == N.DM_F64 else 2e-6
    st = rng.normal(size=4 ** n)
    t = dev(torch, st, npdt)
    ref = st.copy()
    for q in range(n):
        m = rng.normal(size=(4, 4))
        keep, ptr = dparr(m.reshape(16))
        N.call('dm_apply_map1', vp(t), n, dtype, q, ptr, stream(torch))
        v = ref.reshape(4 ** q, 4, 4 ** (n - q - 1))
        ref = np.einsum('ij,ajb->aib', m, v).reshape(-1)
    if n >= 2:
        for (c, tq) in [(0, n - 1), (n - 1, 0), (n // 2, (n // 2 + 1) % n)]:
            if c == tq:
                continue
            for tsp in ([1.0, 0.0], [0.96, 0.07]):
                keep, ptr = dparr(tsp)
                N.call('dm_apply_cx', vp(t), n, dtype, c, tq, ptr, stream(torch))
                ref = O.cx_apply(ref, n, c, tq, tsp)
    N.call('dm_apply_memory_noise', vp(t), n, dtype, 0.97, 0.2, 0.93, stream(torch))
    ref = O.memory_noise(ref, n, 0.97, 0.2, 0.93)
    got = t.double().cpu().numpy()
    np.testing.assert_allclose(got, ref, rtol=0, atol=tol * np.abs(ref).max() * 10)


@pytest.mark.parametrize('n,k,low', [(4, 4, 2), (6, 6, 2), (7, 5, 2), (8, 6, 2), (9, 7, 2), (9, 7, 3), (10, 6, 0)])
@pytest.mark.parametrize('dtype', [N.DM_F64, N.DM_F32])
@pytest.mark.parametrize('rounds', [False, True])
def test_fused_pass_equals_program_order(torch, n, k, low, dtype, rounds):
    from test_planner import apply_op, random_ops
    rng = np.random.default_rng(1000 + n * 7 + k)
    npdt = np.float64 if dtype == N.DM_F64 else np.float32
    ops = random_ops(rng, n, 80)
    if rounds:
        ops = [op for op in ops if op.kind != 'map2']
    for op in ops:                       # keep magnitudes bounded
        if op.kind == 'map1':
            op.data = op.data / np.abs(op.data).sum(axis=1, keepdims=True)
        elif op.kind == 'diag2':
            op.data = np.clip(op.data, -1, 1)
    st = rng.normal(size=4 ** n)
    ref = st.copy()
    for op in ops:
        ref = apply_op(ref, n, op)
    passes = P.plan_passes(ops, n, k, low)
    mats = []
    descs = [P.encode_pass(p, mats, npdt, N.DM_ROUND_AXES[dtype] if rounds else None, n) for p in passes]
    if rounds and low > 0 and k <= P.ROUND_MAX_AXES[np.dtype(npdt)]:
        assert any(d.nrounds > 0 for d in descs)
    m = np.concatenate(mats)
    md = dev(torch, m, npdt)
    t = dev(torch, st, npdt)
    for d in descs:
        N.call('dm_apply_pass', vp(t), n, dtype, ctypes.byref(d), vp(md), ctypes.c_size_t(m.size), stream(torch))
    got = t.double().cpu().numpy()
    tol = 1e-12 if dtype == N.DM_F64 else 1e-4
    np.testing.assert_allclose(got, ref, rtol=0, atol=tol * np.abs(ref).max())


@pytest.mark.parametrize('n', [1, 3, 6, 11, 12, 13])
def test_axis_probs_and_partial(torch, n):
    rng = np.random.default_rng(n + 50)
    st = rng.normal(size=4 ** n) / 2 ** n
    t = dev(torch, st)
    for basis, col in (('X', 1), ('Y', 2), ('Z', 3)):
        out = torch.empty(2 ** n, dtype=torch.float64, device='cuda')
        mode = (ctypes.c_int * n)(*([col] * n))
        N.call('dm_axis_probs', vp(t), n, N.DM_F64, mode, 0.97, vp(out), stream(torch))
        ref = O.ensemble_probabilities(st, n, basis, None, 0.97)
        np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=0, atol=1e-12 * max(1, np.abs(ref).max()))
    # marginal over a random subset of measured qubits
    meas = sorted(int(x) for x in rng.choice(n, max(1, n // 2), replace=False))
    full = O.ensemble_probabilities(st, n, 'Z', None, 0.9)
    others = tuple(sorted(set(range(n)) - set(meas)))
    ref = np.sum(full.reshape([2] * n), axis=others).reshape(-1)
    out = torch.empty(2 ** len(meas), dtype=torch.float64, device='cuda')
    mode = (ctypes.c_int * n)(*[3 if q in meas else 0 for q in range(n)])
    N.call('dm_axis_probs', vp(t), n, N.DM_F64, mode, 0.9, vp(out), stream(torch))
    np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=0, atol=1e-12 * max(1, np.abs(ref).max()))


@pytest.mark.parametrize('n', [1, 2, 3, 4, 7, 10])
def test_nbasis_probs(torch, n):
    rng = np.random.default_rng(n + 70)
    st = rng.normal(size=4 ** n) / 2 ** n
    nvec = rng.normal(size=3)
    nvec /= np.linalg.norm(nvec)
    t = dev(torch, st)
    L = N.lib()
    scratch = torch.empty(max(8, L.dm_nbasis_probs_scratch_bytes(n)), dtype=torch.uint8, device='cuda')
    out = torch.empty(2 ** n, dtype=torch.float64, device='cuda')
    keep, ptr = dparr(nvec)
    N.call('dm_nbasis_probs', vp(t), n, N.DM_F64, ptr, 0.95, vp(out), vp(scratch), stream(torch))
    ref = O.ensemble_probabilities(st, n, 'N', nvec, 0.95)
    np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=0, atol=1e-12 * max(1, np.abs(ref).max()))


@pytest.mark.parametrize('n', [1, 2, 5, 7])
def test_pauli_to_matrix_chop_gather_overlap(torch, n):
    rng = np.random.default_rng(n + 90)
    st = rng.normal(size=4 ** n)
    st[rng.random(4 ** n) < 0.3] *= 1e-17
    t = dev(torch, st)
    L = N.lib()
    scratch = torch.empty(L.dm_pauli_to_matrix_scratch_bytes(n), dtype=torch.uint8, device='cuda')
    out = torch.empty((2 ** n, 2 ** n), dtype=torch.complex128, device='cuda')
    N.call('dm_pauli_to_matrix', vp(t), n, N.DM_F64, vp(out), vp(scratch), stream(torch))
    np.testing.assert_allclose(out.cpu().numpy(), O.pauli_to_matrix(st, n), rtol=0, atol=1e-12)
    ch = torch.empty(4 ** n, dtype=torch.float64, device='cuda')
    N.call('dm_chop_copy', vp(t), n, N.DM_F64, 1e-15, vp(ch), stream(torch))
    ref = st.copy()
    ref[np.abs(ref) < 1e-15] = 0
    assert np.array_equal(ch.cpu().numpy(), ref)
    idx = rng.integers(0, 4 ** n, size=min(64, 4 ** n))
    g = torch.empty(len(idx), dtype=torch.float64, device='cuda')
    N.call('dm_gather', vp(t), n, N.DM_F64, (ctypes.c_int64 * len(idx))(*idx.tolist()), len(idx), vp(g),
           stream(torch))
    assert np.array_equal(g.cpu().numpy(), st[idx])
    other = rng.normal(size=4 ** n)
    o = dev(torch, other)
    sc = torch.empty(L.dm_overlap_scratch_bytes(n), dtype=torch.uint8, device='cuda')
    res = torch.empty(1, dtype=torch.float64, device='cuda')
    N.call('dm_overlap', vp(t), vp(o), n, N.DM_F64, vp(res), vp(sc), stream(torch))
    ref = np.dot(st, other) * 2 ** n
    assert abs(res.item() - ref) <= 1e-12 * np.abs(st * other).sum() * 2 ** n


@pytest.mark.parametrize('n', [1, 4, 9])
def test_init_product(torch, n):
    rng = np.random.default_rng(n + 110)
    vecs = rng.normal(size=(n, 4))
    vecs[rng.random((n, 4)) < 0.4] = 0
    t = torch.empty(4 ** n, dtype=torch.float64, device='cuda')
    keep, ptr = dparr(vecs.reshape(-1))
    N.call('dm_init_product', vp(t), n, N.DM_F64, ptr, 0.5 ** n, stream(torch))
    ref = np.array([1.0])
    for q in range(n):
        ref = np.kron(ref, vecs[q])
    np.testing.assert_allclose(t.cpu().numpy(), ref * 0.5 ** n, rtol=1e-15, atol=0)


def _tc_launch(torch, kernel, p, n, t, status, compose, images):
    """Run pass ``p`` on ``t`` with dm_apply_pass_tma (kernel 'tma') or dm_apply_pass_tc ('tc'), the
    round images composed on the host and uploaded, or by dm_compose_rounds into ``images``.
    False when the pass does not fit that kernel."""
    name = 'dm_apply_pass_tma' if kernel == 'tma' else 'dm_apply_pass_tc'
    try:
        if compose == 'host':
            umats = []
            d = (P.encode_pass_tma if kernel == 'tma' else P.encode_pass_tc)(p, n, umats)
            m = np.concatenate(umats)
            md = torch.from_numpy(m.view(np.int16)).cuda()
        else:
            coefs = []
            d, bp = P.encode_pass_tc_ops(p, n, coefs, kernel)
            c = dev(torch, np.concatenate(coefs))
            md = images
            N.call('dm_compose_rounds', N.DM_IMAGE_TMA if kernel == 'tma' else N.DM_IMAGE_TC, ctypes.byref(bp),
                   vp(c), ctypes.c_size_t(c.numel()), vp(md), ctypes.c_size_t(md.numel()), stream(torch))
    except P.TcPlanError:
        return False
    N.call(name, vp(t), n, ctypes.byref(d), vp(md), ctypes.c_size_t(md.numel()), vp(status), stream(torch))
    torch.cuda.synchronize()
    return True


def _image_buffer(torch):
    return torch.empty(N.DM_MAX_ROUNDS * P.TC_IMAGE_HALVES, dtype=torch.int16, device='cuda')


@pytest.mark.parametrize('compose', ['host', 'device'])
@pytest.mark.parametrize('n', [7, 8, 10])
def test_tensor_core_pass_equals_program_order(torch, n, compose):
    """dm_apply_pass_tc (FP16-split tcgen05 rounds) against the ops applied one by one in FP64.

    The FP16 form holds the tile in units of 2**-n with an absolute floor of
    about 2**-35 in those units, so the check uses what circuits produce:
    trace-preserving maps (I row (1, 0, 0, 0), other rows of absolute sum
    <= 1) on a state with a = 2**-n on the identity and |a| <= 2**-n
    elsewhere, and measures the error in units of 2**-n."""
    from test_planner import apply_op, random_ops
    rng = np.random.default_rng(3000 + n)
    ops = random_ops(rng, n, 60)
    for op in ops:
        if op.kind == 'map1':
            m = op.data / np.abs(op.data).sum(axis=1, keepdims=True)
            m[0] = (1.0, 0.0, 0.0, 0.0)
            op.data = m
        elif op.kind == 'diag2':
            op.data = np.clip(op.data, -1, 1)
            op.data[0] = 1.0
        elif op.kind == 'map2':
            m = op.data / np.abs(op.data).sum(axis=1, keepdims=True)
            m[0] = 0.0
            m[0, 0] = 1.0
            op.data = m
    st = rng.uniform(-1, 1, size=4 ** n) * 2.0 ** -n
    st[0] = 2.0 ** -n
    ref = st.copy()
    for op in ops:
        ref = apply_op(ref, n, op)
    passes = P.plan_passes(ops, n, 7, 2)
    t = dev(torch, st, np.float32)
    status = torch.zeros(1, dtype=torch.int32, device='cuda')
    images = _image_buffer(torch)
    for p in passes:
        assert _tc_launch(torch, 'tc', p, n, t, status, compose, images)
    got = t.double().cpu().numpy()
    assert status.item() == 0
    assert np.max(np.abs(got - ref)) * 2.0 ** n < 2e-6


def _physical_ops(rng, n, count):
    """Random ops made trace-preserving and contractive (see test_tensor_core_pass_equals_program_order)."""
    from test_planner import random_ops
    ops = random_ops(rng, n, count)
    for op in ops:
        if op.kind == 'map1':
            m = op.data / np.abs(op.data).sum(axis=1, keepdims=True)
            m[0] = (1.0, 0.0, 0.0, 0.0)
            op.data = m
        elif op.kind == 'diag2':
            op.data = np.clip(op.data, -1, 1)
            op.data[0] = 1.0
        elif op.kind == 'map2':
            m = op.data / np.abs(op.data).sum(axis=1, keepdims=True)
            m[0] = 0.0
            m[0, 0] = 1.0
            op.data = m
    return ops


def _tma_case(kind, n):
    """(ops, state) for the TMA-pass test: random physical ops off the two lowest-stride qubits, or the
    recorded operations of a noisy layered circuit."""
    rng = np.random.default_rng(4000 + n)
    if kind == 'random':
        ops = [op for op in _physical_ops(rng, n, 60) if all(q < n - 2 for q in op.axes)]
    elif kind == 'dense':      # every qubit: long passes (streamed round images), axis 0 in first / last rounds
        ops = _physical_ops(rng, n, 90)
    else:
        from qiskit_aakash_gb300 import batch as B
        import qiskit_aakash_gb300 as dmg
        qc = dmg.random_layer_circuit(n, 4, 5, barrier_after_gate=(n < 10))
        opts = dmg.noise_options(depolarisation=1e-3, decoherence=0.995, decay=0.998, rotation_sigma=1e-3)
        rec = B.compile_experiment(qc.to_experiment(), opts)
        st = np.array([1.0])
        for v in rec.init[0]:
            st = np.kron(st, v)
        return rec.ops, st * rec.init[1]          # the circuit's own start: |0...0>
    st = rng.uniform(-1, 1, size=4 ** n) * 2.0 ** -n
    st[0] = 2.0 ** -n
    return ops, st


@pytest.mark.parametrize('compose', ['host', 'device'])
@pytest.mark.parametrize('kind,n', [('random', 7), ('random', 9), ('layered', 8), ('layered', 9), ('layered', 10),
                                    ('dense', 7), ('dense', 9)])
def test_tma_pass_equals_program_order(torch, kind, n, compose):
    """dm_apply_pass_tma (TMA-fed tiles, resident round images, last round straight to global memory)
    against the ops applied in FP64, and against dm_apply_pass_tc on the same passes."""
    from test_planner import apply_op
    ops, st = _tma_case(kind, n)
    ref = st.copy()
    for op in ops:
        ref = apply_op(ref, n, op)
    passes = P.plan_passes(ops, n, 7, 2)
    status = torch.zeros(1, dtype=torch.int32, device='cuda')
    t_tma = dev(torch, st, np.float32)
    t_tc = dev(torch, st, np.float32)
    images = _image_buffer(torch)
    used = 0
    for p in passes:
        if _tc_launch(torch, 'tma', p, n, t_tma, status, compose, images):
            used += 1
        else:     # a pass the TMA kernel does not take: the cp.async kernel for both
            assert _tc_launch(torch, 'tc', p, n, t_tma, status, compose, images)
        assert _tc_launch(torch, 'tc', p, n, t_tc, status, compose, images)
    assert used > 0
    assert status.item() == 0
    got = t_tma.double().cpu().numpy()
    other = t_tc.double().cpu().numpy()
    assert np.max(np.abs(got - ref)) * 2.0 ** n < 2e-6
    assert np.max(np.abs(got - other)) * 2.0 ** n < 1e-6


@pytest.mark.parametrize('kernel', ['tc', 'tma'])
def test_device_composed_round_images(torch, kernel):
    """dm_compose_rounds (FP64 on the device) against the host composition (numpy FP64 products):
    Uh + 2**-11 Ul within the split's own rounding of U, and the FP16 values equal except where
    the last FP64 bit of an entry moves it across an FP16 rounding boundary.  (Values, not bits:
    the device's op-by-op columns keep the sign of a zero that a negated or negatively scaled
    zero gets, -0.0, where the host's matrix products sum it into +0.0.)"""
    rng = np.random.default_rng(77)
    n = 10
    ops = _physical_ops(rng, n, 120)
    halves = P.TMA_IMAGE_HALVES if kernel == 'tma' else P.TC_IMAGE_HALVES
    host_image = P.tc_round_image_tma if kernel == 'tma' else P.tc_round_image
    uh_at = 0 if kernel == 'tma' else 8192
    images = _image_buffer(torch)
    checked, differ, total = 0, 0, 0
    for p in P.plan_passes(ops, n, 7, 2):
        coefs = []
        try:
            dp, bp = P.encode_pass_tc_ops(p, n, coefs, kernel)
        except P.TcPlanError:
            continue
        c = dev(torch, np.concatenate(coefs))
        N.call('dm_compose_rounds', N.DM_IMAGE_TMA if kernel == 'tma' else N.DM_IMAGE_TC, ctypes.byref(bp),
               vp(c), ctypes.c_size_t(c.numel()), vp(images), ctypes.c_size_t(images.numel()), stream(torch))
        got = images[:bp.nrounds * halves].cpu().numpy().view(np.uint16)
        _, rounds, layouts = P.plan_tc_rounds(p, n, 'tma' if kernel == 'tma' else 'xor')
        for r, U in enumerate(P.compose_round_matrices(rounds, layouts)):
            g = got[r * halves:(r + 1) * halves]
            want = host_image(U)
            differ += int(np.count_nonzero(g.view(np.float16) != want.view(np.float16)))
            total += g.size
            uh = g[uh_at + P._KMAJOR].view(np.float16).astype(np.float64).reshape(64, 64)
            ul = g[4096 + P._KMAJOR].view(np.float16).astype(np.float64).reshape(64, 64)
            assert np.all(np.abs(uh + ul * 2.0 ** -11 - U) <= 2.0 ** -21 * np.abs(U) + 2.0 ** -34)
            if kernel == 'tc':
                big = g[P._KMAJOR].view(np.float16).astype(np.float64).reshape(64, 64)
                np.testing.assert_array_equal(big, uh * 2048.0)
        checked += 1
    assert checked > 0
    assert differ <= 1e-4 * total


def test_tensor_core_pass_rejects_bad_programs(torch):
    """Malformed tensor-core descriptors are refused on the host (no launch)."""
    n = 8
    t = torch.zeros(4 ** n, dtype=torch.float32, device='cuda')
    u = torch.zeros(3 * 4096, dtype=torch.int16, device='cuda')
    status = torch.zeros(1, dtype=torch.int32, device='cuda')
    rng = np.random.default_rng(0)
    from test_planner import random_ops
    ops = random_ops(rng, n, 10)
    good = P.encode_pass_tc(P.plan_passes(ops, n, 7, 2)[0], n, [])

    def rc_of(mutate):
        d = N.DmTcPass.from_buffer_copy(good)
        mutate(d)
        return N.lib().dm_apply_pass_tc(vp(t), n, ctypes.byref(d), vp(u), 3 * 4096, vp(status), stream(torch))

    def bad_axes(d):
        d.axes[1], d.axes[2] = d.axes[2], d.axes[1]           # not decreasing
    def bad_umoff(d):
        d.rounds[0].umoff = 8                                 # images overrun the 12288-value buffer
    def bad_row(d):
        d.rounds[0].rowc[0] = 3 if d.nrounds > 1 else 20000   # not a power of two / outside the tile
    def bad_vec(d):
        d.vec0 = 0
        d.natk[0], d.natk[1] = 2, 1                           # vector loads need offsets 1, 2
    for mut in (bad_axes, bad_umoff, bad_row, bad_vec):
        assert rc_of(mut) == N.DM_ERR_PROGRAM, mut.__name__
    assert status.item() == 0


@pytest.mark.parametrize('dtype', [N.DM_F64, N.DM_F32])
def test_chunked_copy_out_equals_one_shot(torch, dtype, monkeypatch):
    """DeviceState.coefficients: written by the chop kernel straight into a mapped page-locked result
    block, or in chunks through pinned staging buffers when the blocks are held, = dm_chop_copy."""
    from qiskit_aakash_gb300 import engine
    n = 7
    rng = np.random.default_rng(5)
    st = rng.normal(size=4 ** n) * 2.0 ** -n
    st[rng.random(4 ** n) < 0.3] *= 1e-17
    ds = engine.DeviceState(n, precision='double' if dtype == N.DM_F64 else 'single')
    ds.load(st)
    one = ds.coefficients(1e-15)
    monkeypatch.setattr(engine, '_COPY_CHUNK', 1000)     # 17 chunks, the last one ragged
    monkeypatch.setattr(engine, '_HOST_SLICE', 96)
    engine._RESULT_BLOCKS.pop(8 * 4 ** n, None)
    chunked = ds.coefficients(1e-15)                     # page-locked block 1, device -> block copies
    assert np.array_equal(one, chunked)
    blocks = engine._RESULT_BLOCKS[8 * 4 ** n]
    assert len(blocks) == 1 and blocks[0].dev and not blocks[0].free     # mapped into the device's space
    second = ds.coefficients(1e-15)                      # block 1 held: block 2
    third = ds.coefficients(1e-15)                       # both held: staging buffers + host copies
    assert len(blocks) == 2 and blocks[1].dev
    for got in (chunked, second, third):
        assert np.array_equal(one, got)
    del second
    import gc
    gc.collect()
    assert blocks[1].free
    again = ds.coefficients(1e-15)                       # released block 2 is reused
    assert np.array_equal(one, again) and not blocks[1].free
    del chunked, third, again
    engine._RESULT_BLOCKS.pop(8 * 4 ** n)
    gc.collect()
    with pytest.raises(N.NativeError):
        out = torch.empty(10, dtype=torch.float64, device='cuda')
        N.call('dm_chop_copy_range', ds.ptr, n, dtype, ctypes.c_int64(4 ** n - 5), ctypes.c_int64(10), 0.0,
               vp(out), stream(torch))


def test_bounded_wait_gives_up_and_the_engine_raises(torch):
    """A wait that nothing completes runs out after its limit and sets the status word; the engine
    turns a set status into BasicAerError at its next flush (no fault, no hang: 20 ms limit)."""
    from qiskit_aakash_gb300 import engine
    from qiskit_aakash_gb300.exceptions import BasicAerError
    from qiskit_aakash_gb300.program import IDENTITY4
    ds = engine.DeviceState(8, precision='single')
    assert ds.status is not None and int(ds.status.item()) == 0
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record()
    N.call('dm_tc_wait_selftest', vp(ds.status), ctypes.c_int64(20_000_000), stream(torch))
    t1.record()
    torch.cuda.synchronize()
    assert int(ds.status.item()) == 1
    assert t0.elapsed_time(t1) >= 19.0           # it waited its limit, then gave up
    ds.init_product(np.tile([1.0, 0.0, 0.0, 1.0], (8, 1)), 2.0 ** -8)
    ds.map1(3, IDENTITY4)
    with pytest.raises(BasicAerError, match='bounded wait'):
        ds.flush()


def test_tile_copy_probe_leaves_the_state(torch):
    """dm_tile_copy_probe rewrites every tile in place without changing a bit."""
    n = 9
    rng = np.random.default_rng(8)
    st = rng.normal(size=4 ** n).astype(np.float32)
    t = dev(torch, st, np.float32)
    for axes in ([8, 7, 6, 5, 4, 3, 2], [8, 7, 5, 3, 2, 1, 0]):
        a = (ctypes.c_int32 * 7)(*axes)
        N.call('dm_tile_copy_probe', vp(t), n, a, stream(torch))
    torch.cuda.synchronize()
    assert np.array_equal(t.cpu().numpy().view(np.uint32), st.view(np.uint32))
    bad = (ctypes.c_int32 * 7)(7, 6, 5, 4, 3, 2, 1)          # lowest qubit not resident
    assert N.lib().dm_tile_copy_probe(vp(t), n, bad, stream(torch)) == N.DM_ERR_ARG
