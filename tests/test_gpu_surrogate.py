"""Template sweeps and the surrogate network's kernels on the GPU.

* template sweep: every instance against the oracle run of the same template
  with that instance's noise options;
* tcgen05 BF16 GEMM: every epilogue against numpy on the same BF16 operands;
* one training step (forward, softmax/KL, backward) against the CPU oracle
  of the network, Adam and the BF16 weight copies bit for bit against the
  oracle's update of the same gradients, ensemble statistics;
* a small surrogate trained end to end beats the parameter-blind baseline.
"""
import ctypes

import numpy as np
import pytest

from oracle import dm_oracle as O
from oracle import mlp_oracle as MO
from qiskit_aakash_gb300 import _native as N
from qiskit_aakash_gb300 import surrogate as S
from qiskit_aakash_gb300 import template as TP
from qiskit_aakash_gb300.circuit import random_layer_circuit

pytestmark = pytest.mark.gpu


def _torch():
    import torch
    return torch


def bf16_tensor(a):
    """numpy float32 -> torch int16 tensor of BF16 bits (round to nearest even), on the GPU."""
    torch = _torch()
    r = MO.bf16(a).astype(np.float32).view(np.uint32) >> 16
    return torch.from_numpy(r.astype(np.uint16).view(np.int16)).cuda()


def bf16_to_float(t):
    u = t.cpu().numpy().view(np.uint16).astype(np.uint32) << 16
    return u.view(np.float32)


@pytest.mark.parametrize('precision', ['double', 'single'])
def test_template_sweep_matches_oracle(precision):
    n, layers = 6, 5
    qc = random_layer_circuit(n, layers, seed=3)
    raw = S.sample_noise(6, seed=1)
    prog = TP.TemplateProgram(qc.to_experiment(), S.options_of(raw[0]), precision)
    got = TP.TemplateRunner(prog, max_states_bytes=4 * 4 ** n * 4).run(S.param_vectors(raw)).cpu().numpy()
    tol = 1e-12 if precision == 'double' else 2e-6
    for i in range(len(raw)):
        res = O.OracleDmSimulator(dict(S.options_of(raw[i]), compute_densitymatrix=False)).run_experiment(
            qc.to_experiment())
        want = np.array([res['data']['ensemble_probability'][k] for k in O.bitstring_keys(n)])
        assert np.max(np.abs(got[i] - want)) < tol, i


def test_template_sweep_equals_batched_instances():
    from qiskit_aakash_gb300 import batch as B
    n, layers = 9, 8
    raw = S.sample_noise(5, seed=2)
    qc = random_layer_circuit(n, layers, seed=5)
    prog = TP.TemplateProgram(qc.to_experiment(), S.options_of(raw[0]), 'double')
    got = TP.TemplateRunner(prog).run(S.param_vectors(raw)).cpu().numpy()
    from qiskit_aakash_gb300.dm_simulator import DmSimulatorGPU
    for i in range(len(raw)):
        DmSimulatorGPU.DEFAULT_OPTIONS['rotation_error'] = {'rx': [1., 0.], 'ry': [1., 0.], 'rz': [1., 0.]}
        be = DmSimulatorGPU()
        be._set_options(backend_options=dict(S.options_of(raw[i]), compute_densitymatrix=False))
        res = be.run_experiment(qc.to_experiment())
        want = np.array([res['data']['ensemble_probability'][k] for k in O.bitstring_keys(n)])
        assert np.max(np.abs(got[i] - want)) < 1e-12
    DmSimulatorGPU.DEFAULT_OPTIONS['rotation_error'] = {'rx': [1., 0.], 'ry': [1., 0.], 'rz': [1., 0.]}


def test_tensor_core_template_sweep_matches_oracle_and_cuda_core_form():
    """FP32 template of 9 qubits on the tensor cores: every instance vs the oracle, and vs the
    CUDA-core template form of the same program."""
    n, layers = 9, 6
    qc = random_layer_circuit(n, layers, seed=4)
    raw = S.sample_noise(12, seed=3)
    tc = TP.TemplateProgram(qc.to_experiment(), S.options_of(raw[0]), 'single')
    cc = TP.TemplateProgram(qc.to_experiment(), S.options_of(raw[0]), 'single', tensor_cores=False)
    assert tc.tc and not cc.tc
    runner = TP.TemplateRunner(tc, max_states_bytes=5 * 4 ** n * 4)      # three chunks
    got = runner.run(S.param_vectors(raw)).cpu().numpy()
    ref = TP.TemplateRunner(cc).run(S.param_vectors(raw)).cpu().numpy()
    assert int(runner.status.item()) == 0
    for i in range(len(raw)):
        res = O.OracleDmSimulator(dict(S.options_of(raw[i]), compute_densitymatrix=False)).run_experiment(
            qc.to_experiment())
        want = np.array([res['data']['ensemble_probability'][k] for k in O.bitstring_keys(n)])
        assert np.max(np.abs(got[i] - want)) < 2e-6, i
        assert np.max(np.abs(got[i] - ref[i])) < 2e-6, i


def test_tensor_core_template_rejects_bad_tables():
    torch = _torch()
    n = 9
    qc = random_layer_circuit(n, 3, seed=1)
    raw = S.sample_noise(2, seed=1)
    prog = TP.TemplateProgram(qc.to_experiment(), S.options_of(raw[0]), 'single')
    runner = TP.TemplateRunner(prog)
    prm = torch.as_tensor(S.param_vectors(raw), dtype=torch.float64).cuda()
    states = torch.empty(2 * 4 ** n, dtype=torch.float32, device='cuda')
    out = torch.empty(2 * 2 ** n, dtype=torch.float64, device='cuda')
    vp = ctypes.c_void_p

    def call(passes):
        N.call('dm_batch_run_params_tc', ctypes.byref(runner.host), ctypes.byref(runner.dev_struct), passes,
               vp(runner.tc_passes_dev.data_ptr()), vp(prm.data_ptr()), prm.shape[1], 2, vp(states.data_ptr()),
               ctypes.c_size_t(states.numel()), vp(out.data_ptr()), ctypes.c_size_t(out.numel()),
               vp(runner.counter.data_ptr()), vp(runner.scratch.data_ptr()), ctypes.c_size_t(runner.scratch.numel()),
               vp(runner.status.data_ptr()), None)

    bad = (N.DmBatchTcPass * prog.npasses).from_buffer_copy(bytes(prog.passes))
    bad[0].ops.ops[1].moff = 0                       # op 1 must read coefficient slot 1
    with pytest.raises(N.NativeError) as e:
        call(bad)
    assert e.value.code == N.DM_ERR_PROGRAM
    bad = (N.DmBatchTcPass * prog.npasses).from_buffer_copy(bytes(prog.passes))
    bad[0].ops.nops -= 1                             # slots no longer line up with the ops
    bad[0].ops.round_end[bad[0].ops.nrounds - 1] -= 1
    with pytest.raises(N.NativeError) as e:
        call(bad)
    assert e.value.code == N.DM_ERR_PROGRAM
    call(prog.passes)                                # the good tables run
    torch.cuda.synchronize()
    assert int(runner.status.item()) == 0


def _gemm(epi, A, Bm, members, bias=None, pre=None, want_f32=True, want_bf=False, want_t=False):
    torch = _torch()
    M, K = A.shape[1], A.shape[2]
    Nn = Bm.shape[1]
    g = N.DmMlpGemm()
    g.epi, g.M, g.N, g.K, g.members = epi, M, Nn, K, members
    a, b = bf16_tensor(A), bf16_tensor(Bm)
    g.A, g.lda, g.a_ms = a.data_ptr(), K, M * K
    g.B, g.ldb, g.b_ms = b.data_ptr(), K, Nn * K
    keep = [a, b]
    out = {}
    if bias is not None:
        bt = torch.from_numpy(bias).cuda()
        keep.append(bt)
        g.bias, g.bias_ms = bt.data_ptr(), Nn
    if pre is not None:
        pt = torch.from_numpy(pre).cuda()
        keep.append(pt)
        g.pre, g.ld_pre, g.pre_ms = pt.data_ptr(), Nn, M * Nn
    if want_f32:
        out['f32'] = torch.zeros((members, M, Nn), dtype=torch.float32, device='cuda')
        g.out_f32, g.ld_f32, g.f32_ms = out['f32'].data_ptr(), Nn, M * Nn
    if want_bf:
        out['bf'] = torch.zeros((members, M, Nn), dtype=torch.int16, device='cuda')
        g.out_bf16, g.ld_bf16, g.bf16_ms = out['bf'].data_ptr(), Nn, M * Nn
    if want_t:
        out['t'] = torch.zeros((members, Nn, M), dtype=torch.int16, device='cuda')
        g.out_t, g.ld_t, g.t_ms = out['t'].data_ptr(), M, Nn * M
    status = torch.zeros(1, dtype=torch.int32, device='cuda')
    N.call('dm_mlp_gemm_run', ctypes.byref(g), ctypes.c_void_p(status.data_ptr()), None)
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    return {k: v for k, v in out.items()}


@pytest.mark.parametrize('M,Nn,K', [(128, 64, 64), (256, 256, 256), (384, 128, 1024)])
def test_gemm_epilogues(M, Nn, K):
    rng = np.random.default_rng(M + Nn + K)
    Z = 2
    A = rng.normal(size=(Z, M, K)).astype(np.float32)
    Bm = rng.normal(size=(Z, Nn, K)).astype(np.float32) / np.sqrt(K)
    bias = rng.normal(size=(Z, Nn)).astype(np.float32)
    acc = np.einsum('zmk,znk->zmn', MO.bf16(A).astype(np.float64), MO.bf16(Bm).astype(np.float64))
    o = _gemm(N.DM_MLP_EPI_F32, A, Bm, Z)
    assert np.max(np.abs(o['f32'].cpu().numpy() - acc)) < 1e-4 * np.abs(acc).max()
    o = _gemm(N.DM_MLP_EPI_BIAS_F32, A, Bm, Z, bias=bias)
    u = acc + bias[:, None, :]
    assert np.max(np.abs(o['f32'].cpu().numpy() - u)) < 1e-4 * np.abs(u).max()
    o = _gemm(N.DM_MLP_EPI_GELU_FWD, A, Bm, Z, bias=bias, want_bf=True, want_t=True)
    h = MO.gelu(o['f32'].cpu().numpy().astype(np.float64))
    hb = bf16_to_float(o['bf']).reshape(h.shape)
    assert np.max(np.abs(hb - h) / (np.abs(h) + 1e-3)) < 2 ** -7
    assert np.array_equal(o['bf'].cpu().numpy(), np.swapaxes(o['t'].cpu().numpy(), 1, 2))
    pre = rng.normal(size=(Z, M, Nn)).astype(np.float32)
    o = _gemm(N.DM_MLP_EPI_GELU_BWD, A, Bm, Z, pre=pre, want_f32=False, want_bf=True, want_t=True)
    d = acc * MO.gelu_grad(pre.astype(np.float64))
    db = bf16_to_float(o['bf']).reshape(d.shape)
    assert np.max(np.abs(db - d)) < 2 ** -7 * np.abs(d).max()
    assert np.array_equal(o['bf'].cpu().numpy(), np.swapaxes(o['t'].cpu().numpy(), 1, 2))


def _setup_step(members, B, nout, seed=0):
    torch = _torch()
    rng = np.random.default_rng(seed)
    ens = S.MLPEnsemble(members=members, batch=B, nout=nout)
    widths = S.WIDTHS[:4] + (nout,)
    host = [MO.init_params(seed + z, widths) for z in range(members)]
    flat = np.stack([np.concatenate([p.reshape(-1) for p in host[z]]) for z in range(members)])
    ens.set_params(torch.from_numpy(flat))
    feats = torch.from_numpy(rng.uniform(-1, 1, size=(2 * B, 6)).astype(np.float32)).cuda()
    targets = torch.from_numpy(rng.dirichlet(np.ones(nout) * 0.3, size=2 * B).astype(np.float32)).cuda()
    index = torch.from_numpy(np.stack([rng.permutation(2 * B)[:B] for _ in range(members)]).astype(np.int32)).cuda()
    return ens, host, flat, feats, targets, index


def test_training_step_matches_oracle():
    torch = _torch()
    members, B, nout = 2, 128, 256
    ens, host, flat, feats, targets, index = _setup_step(members, B, nout)
    ens.gather(feats, targets, index, B)
    ens.loss_and_grads(B)
    torch.cuda.synchronize()
    grads = ens.grads.cpu().numpy()
    for z in range(members):
        idx = index[z].cpu().numpy()
        x = MO.pad_features(feats.cpu().numpy()[idx])
        t = targets.cpu().numpy()[idx].astype(np.float64)
        _, _, q = MO.forward(host[z], x)
        loss, g_or = MO.backward(host[z], x, t)
        assert np.max(np.abs(ens.probs[z].cpu().numpy() - q)) < 2e-3 * q.max()
        assert abs(float(ens.loss_rows[z].mean()) - loss) < 2e-3 * abs(loss)
        g_gpu = ens.unpack(grads[z])
        for k, (a, b) in enumerate(zip(g_gpu, g_or)):
            err = np.linalg.norm(a - b) / (np.linalg.norm(b) + 1e-30)
            assert err < 3e-2, (z, k, err)


def test_adam_and_bf16_copies_match_oracle():
    torch = _torch()
    members, B, nout = 2, 128, 256
    ens, host, flat, feats, targets, index = _setup_step(members, B, nout, seed=3)
    rng = np.random.default_rng(4)
    g = rng.normal(size=flat.shape).astype(np.float32) * 1e-2
    ens.grads.copy_(torch.from_numpy(g))
    for step in (1, 2):
        ens._adam(step, 1e-3)
    torch.cuda.synchronize()
    for z in range(members):
        p = [a.copy() for a in host[z]]
        m = [np.zeros_like(a) for a in p]
        v = [np.zeros_like(a) for a in p]
        gz = ens.unpack(g[z])
        for step in (1, 2):
            MO.adam(p, gz, m, v, step, 1e-3)
        got = ens.unpack(ens.params[z].cpu().numpy())
        for a, b in zip(got, p):
            assert np.max(np.abs(a - b)) < 1e-6
        wb = ens.wb[z].cpu().numpy().view(np.uint16)
        wtb = ens.wtb[z].cpu().numpy().view(np.uint16)
        pz = ens.params[z].cpu().numpy()
        for (w0, b0, out, inp) in ens.layers:
            w = pz[w0:w0 + out * inp]
            want = (MO.bf16(w).view(np.uint32) >> 16).astype(np.uint16)
            assert np.array_equal(wb[w0:w0 + out * inp], want)
            assert np.array_equal(wtb[w0:w0 + out * inp].reshape(inp, out), want.reshape(out, inp).T)


def test_ensemble_stats_match_oracle():
    torch = _torch()
    rng = np.random.default_rng(7)
    qs = rng.dirichlet(np.ones(256), size=(5, 300)).astype(np.float32)
    ref = rng.dirichlet(np.ones(256), size=300).astype(np.float32)
    ens = S.MLPEnsemble(members=5, batch=128, nout=256)
    mean, spread, tv = ens.ensemble(torch.from_numpy(qs).cuda(), torch.from_numpy(ref).cuda())
    m_or, s_or = MO.ensemble_stats(qs)
    assert np.max(np.abs(mean.cpu().numpy() - m_or)) < 1e-6
    assert np.max(np.abs(spread.cpu().numpy() - s_or)) < 1e-5
    assert np.max(np.abs(tv.cpu().numpy() - MO.tv(m_or, ref))) < 1e-5


def test_surrogate_learns_and_beats_the_parameter_blind_baseline():
    torch = _torch()
    tmpl = S.Template(n=8, layers=6, seed=1)
    raw_tr, raw_te = S.sample_noise(8192, seed=10), S.sample_noise(1024, seed=11)
    y_tr = tmpl.simulate(raw_tr).float()
    y_te = tmpl.simulate(raw_te).float()
    f_tr = torch.from_numpy(S.features(raw_tr)).cuda()
    f_te = torch.from_numpy(S.features(raw_te)).cuda()
    ens = S.MLPEnsemble(members=3, batch=512, nout=256, seed=1)
    qs0 = ens.predict(f_te)
    _, _, tv0 = ens.ensemble(qs0, y_te)
    ens.fit(f_tr, y_tr, epochs=12, lr=2e-3)
    qs = ens.predict(f_te)
    mean, spread, tv = ens.ensemble(qs, y_te)
    # parameter-blind baseline: the mean training distribution for every point
    blind = y_tr.mean(dim=0, keepdim=True)
    tv_blind = 0.5 * (y_te - blind).abs().sum(dim=1)
    assert float(tv.mean()) < 0.5 * float(tv_blind.mean())
    assert float(tv.mean()) < float(tv0.mean())
    # the spread flags the worst points: the top-spread decile holds more error than the rest
    order = torch.argsort(spread, descending=True)
    top = order[: len(order) // 10]
    assert float(tv[top].mean()) > float(tv.mean())
