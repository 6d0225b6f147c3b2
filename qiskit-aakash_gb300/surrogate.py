"""Learned noise surrogate: an MLP ensemble from noise parameters to a template's outcome distribution.

The reference has no learned part; this is the engine's own extension.  A
fixed circuit template (by default 10 qubits, 30 random brick layers, Z
ensemble measurement) is simulated for many noise-parameter points by the
template sweep (``template.TemplateRunner``); an ensemble of small MLPs
(6 -> 256 -> 256 -> 256 -> 1024, GELU, softmax) learns the map from the six
noise parameters to the 1024 outcome probabilities.  At inference the
ensemble's spread (mean total-variation distance of the members to their
mean) decides where the surrogate is trusted: points above the threshold
fall back to the plain simulation.

Every step runs in libdmgb300.so: BF16 tensor-core GEMMs with fused
bias / GELU / GELU' epilogues (FP32 master weights), softmax with the KL
loss, bias gradients, Adam, the minibatch gather and the ensemble
statistics.  torch tensors are only device buffers.

Noise dimensions (the six inputs, and how each maps to backend options):
    depolarisation p   log-uniform [1e-4, 1e-2]  -> depolarization_factor = 1 - p (at measurement)
    decoherence 1 - f  log-uniform [1e-4, 1e-2]  -> decoherence_factor = f
    decay 1 - g        log-uniform [1e-4, 1e-2]  -> decay_factor = g
    thermal p_th       uniform [0.8, 1.0]        -> thermal_factor
    rotation sigma     uniform [0, 0.05]         -> rotation_error <cos> = exp(-sigma**2 / 2), mean 0
    CX error 1 - c     log-uniform [1e-4, 1e-2]  -> tsp_model_error = [c, 0]
"""
import ctypes
import math
import time

import numpy as np

from . import _native as N
from . import template as TP
from .circuit import noise_options, random_layer_circuit
from .exceptions import BasicAerError

NOISE_DIMS = ('depolarisation', 'decoherence_loss', 'decay_loss', 'thermal', 'rotation_sigma', 'cx_loss')
LOG_DIMS = (0, 1, 2, 5)
LOG_RANGE = (1e-4, 1e-2)
LIN_RANGES = {3: (0.8, 1.0), 4: (0.0, 0.05)}
WIDTHS = (64, 256, 256, 256, 1024)
N_FEATURES = 6


def sample_noise(count, seed):
    """Seeded noise points [count, 6] in the physical units of NOISE_DIMS."""
    rng = np.random.default_rng(seed)
    raw = np.empty((count, N_FEATURES))
    lo, hi = np.log(LOG_RANGE[0]), np.log(LOG_RANGE[1])
    for d in LOG_DIMS:
        raw[:, d] = np.exp(rng.uniform(lo, hi, count))
    for d, (a, b) in LIN_RANGES.items():
        raw[:, d] = rng.uniform(a, b, count)
    return raw


def features(raw):
    """Network inputs in [-1, 1]: log10 of the log-uniform dimensions, the others linearly."""
    raw = np.asarray(raw, dtype=np.float64)
    x = np.empty_like(raw)
    llo, lhi = np.log10(LOG_RANGE[0]), np.log10(LOG_RANGE[1])
    for d in LOG_DIMS:
        x[:, d] = 2 * (np.log10(raw[:, d]) - llo) / (lhi - llo) - 1
    for d, (a, b) in LIN_RANGES.items():
        x[:, d] = 2 * (raw[:, d] - a) / (b - a) - 1
    return x.astype(np.float32)


def options_of(row):
    """Backend options of one noise point."""
    return noise_options(depolarisation=row[0], decoherence=1 - row[1], decay=1 - row[2], thermal=row[3],
                         rotation_sigma=row[4], tsp=[1 - row[5], 0.0])


def param_vectors(raw):
    """Template-sweep parameter vectors [count, PARAM_STRIDE] of noise points (the options_of mapping)."""
    raw = np.asarray(raw, dtype=np.float64)
    v = np.zeros((raw.shape[0], TP.PARAM_STRIDE))
    v[:, 0] = 1 - raw[:, 1]
    v[:, 1] = raw[:, 3]
    v[:, 2] = 1 - raw[:, 2]
    c = np.exp(-0.5 * raw[:, 4] ** 2)
    v[:, 3] = v[:, 5] = v[:, 7] = c
    v[:, 9] = 1 - raw[:, 5]
    v[:, 11] = 1 - raw[:, 0]
    return v


class Template:
    """The fixed circuit of the surrogate and its template sweep on the device."""

    def __init__(self, n=10, layers=30, seed=0, precision='single', device=None):
        self.n, self.layers, self.seed = n, layers, seed
        self.circuit = random_layer_circuit(n, layers, seed)
        centre = sample_noise(1, 12345)[0]
        self.program = TP.TemplateProgram(self.circuit.to_experiment(), options_of(centre), precision)
        self.runner = TP.TemplateRunner(self.program, device)

    def simulate(self, raw):
        """Outcome distributions [count, 2**n] (FP64, device) of noise points, by the plain simulation."""
        return self.runner.run(param_vectors(raw))


def _layer_offsets(widths):
    offs, o = [], 0
    for li in range(4):
        out, inp = widths[li + 1], widths[li]
        offs.append((o, o + out * inp, out, inp))
        o += out * inp + out
    return offs, o


class MLPEnsemble:
    """``members`` networks trained together; every buffer is [members, ...] on the device."""

    def __init__(self, members=5, batch=1024, seed=0, nout=1024, device=None):
        import torch
        if not torch.cuda.is_available():
            raise BasicAerError('the surrogate needs a CUDA device')
        N.lib()
        if batch % 128:
            raise BasicAerError('the batch size must be a multiple of 128')
        if nout % 256 or not 256 <= nout <= 4096:
            raise BasicAerError('the output width must be a multiple of 256 up to 4096')
        self.M, self.B, self.nout = members, batch, nout
        self.widths = WIDTHS[:4] + (nout,)
        self.device = torch.device(device or 'cuda')
        self.layers, self.P = _layer_offsets(self.widths)
        self.shapes = (ctypes.c_int32 * 8)(*[v for (_, _, out, inp) in self.layers for v in (out, inp)])
        dev, f32, bf = self.device, torch.float32, torch.int16
        M, B, P = members, batch, self.P
        z = lambda *s, dt=f32: torch.zeros(*s, dtype=dt, device=dev)  # noqa: E731
        self.params, self.grads, self.m, self.v = z(M, P), z(M, P), z(M, P), z(M, P)
        self.wb, self.wtb = z(M, P, dt=bf), z(M, P, dt=bf)
        self.status = z(1, dt=torch.int32)
        self.step_count = 0
        self._alloc(B)
        self.init_params(seed)

    def _alloc(self, B):
        import torch
        dev, f32, bf = self.device, torch.float32, torch.int16
        M = self.M
        z = lambda *s, dt=f32: torch.empty(*s, dtype=dt, device=dev)  # noqa: E731
        self.bufB = B
        self.x, self.xt = z(M, B, 64, dt=bf), z(M, 64, B, dt=bf)
        self.pre = [z(M, B, 256) for _ in range(3)]
        self.h = [z(M, B, 256, dt=bf) for _ in range(3)]
        self.ht = [z(M, 256, B, dt=bf) for _ in range(3)]
        K = self.nout
        self.logits, self.t = z(M, B, K), z(M, B, K)
        self.dz, self.dzt = z(M, B, K, dt=bf), z(M, K, B, dt=bf)
        self.du = [z(M, B, 256, dt=bf) for _ in range(2)]
        self.dut = [z(M, 256, B, dt=bf) for _ in range(2)]
        self.loss_rows = z(M, B)
        self.probs = z(M, B, K)

    # -- parameters ------------------------------------------------------------
    def init_params(self, seed):
        """He-style normal initialisation (std sqrt(2 / fan_in); sqrt(1 / fan_in) for the output layer)."""
        import torch
        host = np.zeros((self.M, self.P), dtype=np.float32)
        for z in range(self.M):
            rng = np.random.default_rng([seed, z])
            for li, (w0, b0, out, inp) in enumerate(self.layers):
                real_in = N_FEATURES if li == 0 else inp
                std = math.sqrt((2.0 if li < 3 else 1.0) / real_in)
                w = np.zeros((out, inp), dtype=np.float32)
                w[:, :real_in] = rng.normal(0.0, std, size=(out, real_in))
                host[z, w0:w0 + out * inp] = w.reshape(-1)
        self.set_params(torch.from_numpy(host))

    def set_params(self, flat):
        """Load [members, P] FP32 parameters (W1 b1 ... W4 b4 per member); resets Adam."""
        import torch
        self.params.copy_(torch.as_tensor(flat, dtype=torch.float32))
        self.m.zero_()
        self.v.zero_()
        self.step_count = 0
        self._adam(0, 0.0)

    def unpack(self, flat):
        """[W1, b1, ..., W4, b4] numpy arrays of one member's flat parameter vector."""
        out = []
        for (w0, b0, o, i) in self.layers:
            out += [flat[w0:w0 + o * i].reshape(o, i), flat[b0:b0 + o]]
        return out

    # -- kernels -----------------------------------------------------------------
    def _stream(self):
        import torch
        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def _gemm(self, epi, M, Nn, K, A, lda, a_ms, Bm, ldb, b_ms, bias=None, pre=None, out_f32=None, ld_f32=0,
              f32_ms=0, out_bf16=None, out_t=None):
        g = N.DmMlpGemm()
        g.epi, g.M, g.N, g.K, g.members = epi, M, Nn, K, self.M
        g.A, g.lda, g.a_ms = A, lda, a_ms
        g.B, g.ldb, g.b_ms = Bm, ldb, b_ms
        if bias is not None:
            g.bias, g.bias_ms = bias, self.P
        if pre is not None:
            g.pre, g.ld_pre, g.pre_ms = pre.data_ptr(), pre.shape[2], pre.shape[1] * pre.shape[2]
        if out_f32 is not None:
            g.out_f32, g.ld_f32, g.f32_ms = out_f32, ld_f32, f32_ms
        if out_bf16 is not None:
            g.out_bf16, g.ld_bf16, g.bf16_ms = out_bf16.data_ptr(), out_bf16.shape[2], out_bf16.shape[1] * out_bf16.shape[2]
        if out_t is not None:
            g.out_t, g.ld_t, g.t_ms = out_t.data_ptr(), out_t.shape[2], out_t.shape[1] * out_t.shape[2]
        N.call('dm_mlp_gemm_run', ctypes.byref(g), ctypes.c_void_p(self.status.data_ptr()), self._stream())

    def _w(self, li, transposed=False):
        base = (self.wtb if transposed else self.wb).data_ptr()
        return base + 2 * self.layers[li][0]

    def _adam(self, step, lr, beta1=0.9, beta2=0.999, eps=1e-8):
        vp = ctypes.c_void_p
        N.call('dm_mlp_adam', vp(self.params.data_ptr()), vp(self.grads.data_ptr()), vp(self.m.data_ptr()),
               vp(self.v.data_ptr()), ctypes.c_int64(self.P), self.M, self.shapes, 4, ctypes.c_float(lr),
               ctypes.c_float(beta1), ctypes.c_float(beta2), ctypes.c_float(eps), step, vp(self.wb.data_ptr()),
               vp(self.wtb.data_ptr()), self._stream())

    def forward(self, rows, train):
        """Forward pass of the members on self.x (rows <= batch); logits in self.logits."""
        f32 = 4
        P, B, K = self.P, self.bufB, self.nout
        E = N.DM_MLP_EPI_GELU_FWD
        A, lda, ams = self.x.data_ptr(), 64, B * 64
        for li in range(3):
            inp = self.widths[li]
            self._gemm(E, rows, 256, inp, A, lda, ams, self._w(li), inp, P, bias=self.params.data_ptr() + f32 * self.layers[li][1],
                       out_f32=self.pre[li].data_ptr() if train else None, ld_f32=256, f32_ms=B * 256,
                       out_bf16=self.h[li], out_t=self.ht[li] if train else None)
            A, lda, ams = self.h[li].data_ptr(), 256, B * 256
        self._gemm(N.DM_MLP_EPI_BIAS_F32, rows, K, 256, A, lda, ams, self._w(3), 256, P,
                   bias=self.params.data_ptr() + f32 * self.layers[3][1], out_f32=self.logits.data_ptr(), ld_f32=K,
                   f32_ms=B * K)

    def backward(self, rows):
        """Gradients of the mean KL loss (self.dz / self.dzt already hold dL/dz) into self.grads."""
        vp = ctypes.c_void_p
        f32 = 4
        P, B, K = self.P, self.bufB, self.nout
        g0 = self.grads.data_ptr()
        # output layer
        self._gemm(N.DM_MLP_EPI_F32, K, 256, rows, self.dzt.data_ptr(), B, K * B, self.ht[2].data_ptr(), B,
                   256 * B, out_f32=g0 + f32 * self.layers[3][0], ld_f32=256, f32_ms=P)
        N.call('dm_mlp_bias_grad', vp(self.dzt.data_ptr()), ctypes.c_int64(B), ctypes.c_int64(K * B), K, rows,
               self.M, vp(g0 + f32 * self.layers[3][1]), ctypes.c_int64(P), self._stream())
        dA, lda, ams, inw = self.dz.data_ptr(), K, B * K, K
        for li in (2, 1, 0):
            cur = (2 - li) % 2
            # dU_li = (d_next @ W_{li+1}) * gelu'(pre_li)
            self._gemm(N.DM_MLP_EPI_GELU_BWD, rows, 256, inw, dA, lda, ams, self._w(li + 1, True), inw, P,
                       pre=self.pre[li], out_bf16=self.du[cur], out_t=self.dut[cur])
            prev_t = self.ht[li - 1].data_ptr() if li > 0 else self.xt.data_ptr()
            width_in = self.widths[li]
            self._gemm(N.DM_MLP_EPI_F32, 256, width_in, rows, self.dut[cur].data_ptr(), B, 256 * B, prev_t, B,
                       width_in * B, out_f32=g0 + f32 * self.layers[li][0], ld_f32=width_in, f32_ms=P)
            N.call('dm_mlp_bias_grad', vp(self.dut[cur].data_ptr()), ctypes.c_int64(B), ctypes.c_int64(256 * B), 256,
                   rows, self.M, vp(g0 + f32 * self.layers[li][1]), ctypes.c_int64(P), self._stream())
            dA, lda, ams, inw = self.du[cur].data_ptr(), 256, B * 256, 256

    def gather(self, feats, targets, index, rows):
        vp = ctypes.c_void_p
        N.call('dm_mlp_gather', vp(feats.data_ptr()), N_FEATURES, vp(targets.data_ptr()), self.nout,
               ctypes.c_int64(feats.shape[0]), vp(index.data_ptr()), rows, self.M, 64, vp(self.x.data_ptr()),
               vp(self.xt.data_ptr()), vp(self.t.data_ptr()), self._stream())

    def loss_and_grads(self, rows):
        """Forward + softmax/KL + backward on the gathered minibatch (self.x, self.t)."""
        vp = ctypes.c_void_p
        self.forward(rows, True)
        N.call('dm_mlp_softmax_xent', vp(self.logits.data_ptr()), vp(self.t.data_ptr()), rows, self.M, self.nout,
               ctypes.c_float(1.0 / rows), vp(self.probs.data_ptr()), vp(self.dz.data_ptr()),
               vp(self.dzt.data_ptr()), vp(self.loss_rows.data_ptr()), self._stream())
        self.backward(rows)

    def train_step(self, feats, targets, index, lr):
        self.gather(feats, targets, index, self.B)
        self.loss_and_grads(self.B)
        self.step_count += 1
        self._adam(self.step_count, lr)

    def fit(self, feats, targets, epochs, lr=2e-3, lr_min=2e-5, seed=0, log_every=0):
        """Train every member on (feats [S, 6], targets [S, 1024]) device tensors; own shuffles per member."""
        import torch
        S = feats.shape[0]
        steps_per_epoch = S // self.B
        if steps_per_epoch < 1:
            raise BasicAerError('fewer samples than one batch')
        total = epochs * steps_per_epoch
        rng = np.random.default_rng(seed)
        history = []
        t0 = time.perf_counter()
        for ep in range(epochs):
            perm = np.stack([rng.permutation(S)[:steps_per_epoch * self.B] for _ in range(self.M)]).astype(np.int32)
            perm_d = torch.from_numpy(perm).to(self.device)
            for s in range(steps_per_epoch):
                k = ep * steps_per_epoch + s
                lr_k = lr_min + 0.5 * (lr - lr_min) * (1 + math.cos(math.pi * k / total))
                idx = perm_d[:, s * self.B:(s + 1) * self.B].contiguous()
                self.train_step(feats, targets, idx, lr_k)
                if log_every and k % log_every == 0:
                    history.append((k, float(self.loss_rows.mean())))
        torch.cuda.synchronize(self.device)
        if int(self.status.item()) != 0:
            raise BasicAerError('a tensor-core GEMM abandoned a bounded wait')
        return {'steps': total, 'seconds': time.perf_counter() - t0, 'history': history}

    def predict(self, feats):
        """Member distributions [members, S, 1024] (FP32, device) of feature rows [S, 6] (device)."""
        import torch
        S = feats.shape[0]
        out = torch.empty((self.M, S, self.nout), dtype=torch.float32, device=self.device)
        vp = ctypes.c_void_p
        for s0 in range(0, S, self.B):
            rows = min(self.B, S - s0)
            padded = ((rows + 127) // 128) * 128
            idx = torch.arange(s0, s0 + padded, device=self.device, dtype=torch.int32).clamp_(max=S - 1)
            idx = idx.unsqueeze(0).expand(self.M, padded).contiguous()
            N.call('dm_mlp_gather', vp(feats.data_ptr()), N_FEATURES, None, self.nout, ctypes.c_int64(S),
                   vp(idx.data_ptr()), padded, self.M, 64, vp(self.x.data_ptr()), vp(self.xt.data_ptr()), None,
                   self._stream())
            self.forward(padded, False)
            N.call('dm_mlp_softmax_xent', vp(self.logits.data_ptr()), None, padded, self.M, self.nout, ctypes.c_float(1.0),
                   vp(self.probs.data_ptr()), None, None, None, self._stream())
            out[:, s0:s0 + rows] = self.probs[:, :rows]
        return out

    def ensemble(self, member_probs, ref=None):
        """(mean [S, 1024], spread [S], TV(mean, ref) [S] or None), all on the device."""
        import torch
        M, S, K = member_probs.shape
        mean = torch.empty((S, K), dtype=torch.float32, device=self.device)
        spread = torch.empty(S, dtype=torch.float32, device=self.device)
        tv = torch.empty(S, dtype=torch.float32, device=self.device) if ref is not None else None
        vp = ctypes.c_void_p
        N.call('dm_mlp_ensemble', vp(member_probs.data_ptr()), S, M, K, vp(ref.data_ptr()) if ref is not None else None,
               vp(mean.data_ptr()), vp(spread.data_ptr()), vp(tv.data_ptr()) if tv is not None else None,
               self._stream())
        return mean, spread, tv
