"""Parametric batched programs: one circuit template, many noise-parameter vectors.

A template experiment is recorded once through the backend's own run loop
(merge, levels, per-level memory noise, final Z ensemble measurement).  Each
recorded operation becomes a recipe that says how to rebuild it from an
instance's noise parameters: a gate's rotations (fixed angles, the
instance's rotation error), a memory-noise map (the instance's f, p, g), a
CX (the instance's transition-model error) or a constant map.  One pass /
round plan serves every instance; the batch kernel composes each pass's
coefficients from the recipes in FP64 on the GPU, so an instance costs the
host nothing but its 12 parameters.

Parameter vector (``PARAM_STRIDE`` doubles per instance):
    0 decoherence_factor f, 1 thermal_factor p, 2 decay_factor g,
    3-8 rotation_error (<cos>, mean) of rx, ry, rz,
    9-10 tsp_model_error (<cos>, mean), 11 depolarization_factor (the read-out's polarisation)
"""
import ctypes

import numpy as np

from . import _native as N
from . import program as P
from .exceptions import BasicAerError

PARAM_STRIDE = 16
_AXIS_CODE = {'rx': 0, 'ry': 1, 'rz': 2}


# The backend's option defaults (dm_simulator.py:120-130).
DEFAULTS = {'thermal_factor': 1.0, 'decoherence_factor': 1.0, 'depolarization_factor': 1.0, 'decay_factor': 1.0,
            'rotation_error': {'rx': [1.0, 0.0], 'ry': [1.0, 0.0], 'rz': [1.0, 0.0]}, 'tsp_model_error': [1.0, 0.0]}


def param_vector(options):
    """The parameter vector of backend options (missing options take the backend's defaults)."""
    o = dict(DEFAULTS)
    o.update(options)
    rot = dict(DEFAULTS['rotation_error'])
    rot.update(options.get('rotation_error', {}))
    v = np.zeros(PARAM_STRIDE)
    v[0], v[1], v[2] = o['decoherence_factor'], o['thermal_factor'], o['decay_factor']
    for ax, code in _AXIS_CODE.items():
        v[3 + 2 * code], v[4 + 2 * code] = rot[ax]
    v[9], v[10] = o['tsp_model_error']
    v[11] = o['depolarization_factor']
    return v


class TemplateProgram:
    """Host tables of one template: passes, slots, recipe chains, recipes, constants."""

    def __init__(self, experiment, options, precision='single', kmax=None, probe_options=None, tensor_cores=None):
        from .batch import compile_experiment
        self.precision = precision
        self.dtype = N.DM_F32 if precision == 'single' else N.DM_F64
        rec = compile_experiment(experiment, options)
        n = rec.n
        width = N.DM_ROUND_AXES[self.dtype]
        if not width <= n <= 12:
            raise BasicAerError('template programs hold %d..12 qubits' % width)
        self.n = n
        # a second recording with other parameters must keep the structure and every constant map
        probe = dict(options)
        probe.update(probe_options or {'decoherence_factor': 0.9, 'decay_factor': 0.8, 'thermal_factor': 0.7,
                                       'rotation_error': {'rx': [0.9, 0.01], 'ry': [0.8, 0.02], 'rz': [0.7, 0.03]},
                                       'tsp_model_error': [0.9, 0.05], 'depolarization_factor': 0.6})
        rec2 = compile_experiment(experiment, probe)
        if len(rec2.ops) != len(rec.ops):
            raise BasicAerError('the template changes structure with its noise parameters')
        recipes, consts = [], []
        for op, op2 in zip(rec.ops, rec2.ops):
            if op.kind != op2.kind or op.axes != op2.axes or op.tag != op2.tag:
                raise BasicAerError('the template changes structure with its noise parameters')
            r = N.DmRecipe()
            if op.kind == 'cx':
                r.kind = N.DM_RECIPE_CX
            elif op.kind == 'map1' and op.tag and op.tag[0] == 'rot':
                r.kind = N.DM_RECIPE_ROT
                r.nrot = len(op.tag[1])
                if not 1 <= r.nrot <= 3:
                    raise BasicAerError('a gate of more than three rotations')
                for k, (ax, ang) in enumerate(op.tag[1]):
                    r.axis[k] = _AXIS_CODE[ax]
                    r.angle[k] = ang
            elif op.kind == 'map1' and op.tag == ('noise',):
                r.kind = N.DM_RECIPE_NOISE
            elif op.kind in ('map1', 'diag2'):
                m = np.asarray(op.data, dtype=np.float64).reshape(16)
                if not np.array_equal(m, np.asarray(op2.data, dtype=np.float64).reshape(16)):
                    raise BasicAerError('a template operation depends on the noise parameters in a way '
                                        'the template program does not model')
                r.kind = N.DM_RECIPE_CONST
                r.const_off = len(consts) * 16
                consts.append(m)
            else:
                raise BasicAerError('template programs hold 4x4 maps, CX and diagonal pair maps only')
            recipes.append(r)
        self.meas_err_template = rec.readouts[0][3]
        self.recipes = (N.DmRecipe * max(len(recipes), 1))(*recipes)
        self.nrecipes = len(recipes)
        self.consts = np.concatenate(consts) if consts else np.zeros(16)
        self.nconsts = len(consts) * 16
        if tensor_cores is None:        # FP32 templates of >= 9 qubits run faster on the tensor cores
            tensor_cores = precision == 'single' and n >= 9
        if tensor_cores and (precision != 'single' or n < P.TC_AXES):
            raise BasicAerError('tensor-core template sweeps need FP32 and >= %d qubits' % P.TC_AXES)
        self.tc = False
        if tensor_cores:
            try:
                self._plan_tc(rec.ops, n)
                self.tc = True
            except P.TcPlanError:       # a pass with more rounds than a table holds: the CUDA-core plan
                pass
        if not self.tc:
            self._plan(rec.ops, n, min((kmax or {}).get(n, 7 if precision == 'single' else 6), n), width)

    def _plan_tc(self, ops, n):
        """Tensor-core passes: 7 resident axes, rounds in their layouts' digit order; op o of a pass
        reads the o-th 16-value slot of the coefficients the kernel composes per pass."""
        from .batch import fill_tc_tables
        passes, slots, chain = [], [], []
        for p in P.plan_passes(ops, n, P.TC_AXES, 2):
            pp = P.pad_pass(p, n)
            rounds = P.plan_rounds(pp, 3, pad='neighbors')
            if len(rounds) > N.DM_MAX_ROUNDS:
                raise P.TcPlanError('pass needs %d rounds (> %d)' % (len(rounds), N.DM_MAX_ROUNDS))
            direct = P.direct_last_eligible([axes for axes, _ in rounds])
            layouts = P._choose_layouts([axes for axes, _ in rounds], direct=direct)
            bp = N.DmBatchTcPass()
            o = bp.ops
            o.k = len(pp.axes)
            for r, q in enumerate(pp.axes):
                o.axes[r] = q
            o.nrounds = len(rounds)
            idx = 0
            for ri, ((_, rops), L) in enumerate(zip(rounds, layouts)):
                digits = list(L.digits)
                for i, a in enumerate(digits):
                    o.round_axes[ri][i] = a
                o.round_axes[ri][3] = -1
                for op in rops:
                    d = o.ops[idx]
                    d.a = op.axes[0]
                    d.moff = idx * 16
                    flags = digits.index(op.axes[0]) << 8
                    if op.kind == 'map1':
                        d.kind = N.DM_OP_MAP1
                        d.b = 0
                    else:
                        d.kind = N.DM_OP_CX if op.kind == 'cx' else N.DM_OP_DIAG2
                        d.b = op.axes[1]
                        flags |= digits.index(op.axes[1]) << 12
                    d.flags = flags
                    slots.append((len(chain), len(op.src)))
                    chain.extend(op.src)
                    idx += 1
                o.round_end[ri] = idx
            o.nops = idx
            fill_tc_tables(bp.tables, pp, layouts, direct)
            passes.append(bp)
        self.passes = (N.DmBatchTcPass * len(passes))(*passes)
        self.npasses = len(passes)
        self.slots = (N.DmParamSlot * len(slots))(*[N.DmParamSlot(b, l) for b, l in slots])
        self.nslots = len(slots)
        self.chain = np.asarray(chain, dtype=np.int32)

    def _plan(self, ops, n, k, width):
        passes, slots, chain = [], [], []
        for p in P.plan_passes(ops, n, k, 2):
            pp = p if len(p.axes) >= width else P.pad_pass(p, n, width)
            rounds = P.plan_rounds(pp, width)
            if len(rounds) > N.DM_MAX_ROUNDS:
                raise BasicAerError('pass needs too many rounds')
            bp = N.DmBatchPass()
            bp.k = len(pp.axes)
            for r, q in enumerate(pp.axes):
                bp.axes[r] = q
            bp.nrounds = len(rounds)
            o = 0
            for ri, (axes, rops) in enumerate(rounds):
                for i, a in enumerate(axes):
                    bp.round_axes[ri][i] = a
                for i in range(len(axes), 4):
                    bp.round_axes[ri][i] = -1
                for op in rops:
                    d = bp.ops[o]
                    d.a = op.axes[0]
                    d.moff = 0
                    flags = axes.index(op.axes[0]) << 8
                    if op.kind == 'map1':
                        d.kind = N.DM_OP_MAP1
                        d.b = 0
                        if all(self._trace_preserving(i) for i in op.src):
                            flags |= N.DM_MAP1_ROW0_IDENTITY
                    else:
                        d.kind = N.DM_OP_CX if op.kind == 'cx' else N.DM_OP_DIAG2
                        d.b = op.axes[1]
                        flags |= axes.index(op.axes[1]) << 12
                    d.flags = flags
                    slots.append((len(chain), len(op.src)))
                    chain.extend(op.src)
                    o += 1
                bp.round_end[ri] = o
            bp.nops = o
            passes.append(bp)
        self.passes = (N.DmBatchPass * len(passes))(*passes)
        self.npasses = len(passes)
        self.slots = (N.DmParamSlot * len(slots))(*[N.DmParamSlot(b, l) for b, l in slots])
        self.nslots = len(slots)
        self.chain = np.asarray(chain, dtype=np.int32)

    def _trace_preserving(self, i):
        r = self.recipes[i]
        if r.kind in (N.DM_RECIPE_ROT, N.DM_RECIPE_NOISE):
            return True
        m = self.consts[r.const_off:r.const_off + 16]
        return m[0] == 1.0 and not m[1:4].any()

    def host_struct(self):
        """dm_param_program pointing at the host copies (kept alive by this object)."""
        P_ = N.DmParamProgram()
        P_.n, P_.npasses, P_.nslots = self.n, self.npasses, self.nslots
        P_.nchain, P_.nrecipes, P_.nconsts = self.chain.size, self.nrecipes, self.nconsts
        P_.passes = None if self.tc else ctypes.cast(self.passes, ctypes.c_void_p)
        P_.slots = ctypes.cast(self.slots, ctypes.c_void_p)
        P_.chain = self.chain.ctypes.data_as(ctypes.c_void_p)
        P_.recipes = ctypes.cast(self.recipes, ctypes.c_void_p)
        P_.consts = self.consts.ctypes.data_as(ctypes.c_void_p)
        return P_


class TemplateRunner:
    """A template program on the device: runs parameter vectors in chunks of resident states."""

    def __init__(self, program, device=None, max_states_bytes=32 << 30):
        import torch
        if not torch.cuda.is_available():
            raise BasicAerError('template sweeps need a CUDA device')
        N.lib()
        self.p = program
        self.device = torch.device(device or 'cuda')
        dev = self.device

        def up(buf):
            return torch.from_numpy(np.frombuffer(bytes(buf), dtype=np.uint8).copy()).to(dev)

        self._bufs = [up(program.passes), up(program.slots), torch.from_numpy(program.chain.copy()).to(dev),
                      up(program.recipes), torch.from_numpy(program.consts.copy()).to(dev)]
        d = program.host_struct()
        d.passes, d.slots, d.chain, d.recipes, d.consts = [b.data_ptr() for b in self._bufs]
        if program.tc:
            d.passes = None
            self.tc_passes_dev = self._bufs[0]
            self.scratch = torch.empty(N.lib().dm_batch_tc_scratch_bytes(), dtype=torch.uint8, device=dev)
            self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        self.dev_struct = d
        self.host = program.host_struct()
        esize = 4 if program.dtype == N.DM_F32 else 8
        self.state_elems = 4 ** program.n
        self.chunk = max(1, min(65536, int(max_states_bytes // (self.state_elems * esize))))
        self.states = None
        self.counter = torch.zeros(1, dtype=torch.int32, device=dev)
        self.tdt = torch.float32 if program.dtype == N.DM_F32 else torch.float64

    def run(self, params, out=None):
        """Z-outcome probabilities [S, 2**n] (FP64, on the device) for parameter vectors [S, PARAM_STRIDE]."""
        import torch
        prm = torch.as_tensor(params, dtype=torch.float64).to(self.device).contiguous()
        S = prm.shape[0]
        if prm.dim() != 2 or prm.shape[1] < N.DM_PARAMS_MIN_STRIDE:
            raise BasicAerError('parameters must be [instances, %d]' % PARAM_STRIDE)
        npr = 2 ** self.p.n
        if out is None:
            out = torch.empty((S, npr), dtype=torch.float64, device=self.device)
        c = min(self.chunk, S)
        if self.states is None or self.states.numel() < c * self.state_elems:
            self.states = torch.empty(c * self.state_elems, dtype=self.tdt, device=self.device)
        stream = torch.cuda.current_stream(self.device)
        for s0 in range(0, S, c):
            k = min(c, S - s0)
            if self.p.tc:
                N.call('dm_batch_run_params_tc', ctypes.byref(self.host), ctypes.byref(self.dev_struct),
                       self.p.passes, ctypes.c_void_p(self.tc_passes_dev.data_ptr()),
                       ctypes.c_void_p(prm[s0].data_ptr()), prm.shape[1], k, ctypes.c_void_p(self.states.data_ptr()),
                       ctypes.c_size_t(self.states.numel()), ctypes.c_void_p(out[s0].data_ptr()),
                       ctypes.c_size_t(k * npr), ctypes.c_void_p(self.counter.data_ptr()),
                       ctypes.c_void_p(self.scratch.data_ptr()), ctypes.c_size_t(self.scratch.numel()),
                       ctypes.c_void_p(self.status.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
                continue
            N.call('dm_batch_run_params', self.p.dtype, ctypes.byref(self.host), ctypes.byref(self.dev_struct),
                   ctypes.c_void_p(prm[s0].data_ptr()), prm.shape[1], k, ctypes.c_void_p(self.states.data_ptr()),
                   ctypes.c_size_t(self.states.numel()), ctypes.c_void_p(out[s0].data_ptr()),
                   ctypes.c_size_t(k * npr), ctypes.c_void_p(self.counter.data_ptr()),
                   ctypes.c_void_p(stream.cuda_stream))
        if self.p.tc and int(self.status.item()) != 0:
            raise BasicAerError('a tensor-core template pass abandoned a bounded wait')
        return out
