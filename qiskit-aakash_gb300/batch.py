"""Batched noise sweeps: thousands of independent circuit instances, one persistent launch.

Each instance is an ordinary dm_simulator experiment (same merge, levels,
per-level memory noise and final Z ensemble measurement as
``DmSimulatorGPU.run_experiment``); the batch runs them all in one
``dm_batch_run`` launch, where every CTA takes the next instance from a
work counter and runs it start to finish (state preparation, fused passes,
read-out).  The launch can be captured in a CUDA graph and replayed.

Host work is kept small by sharing plans: instances with the same
structure (qubit count and depth of the layered template) share one pass /
round plan; per instance only the coefficients of the plan's operations are
rebuilt from the instance's own gate and noise matrices (``Op.src``).  The
resident-axis count per qubit count is picked by ``autotune``, which times
each candidate on the device.
"""
import ctypes
import time

import numpy as np

from . import _native as N
from . import program as P
from .circuit import noise_options, random_layer_circuit
from .exceptions import BasicAerError

MAX_QUBITS = 12


class HostRecorder:
    """DeviceState's interface without a device: records one experiment's op stream and read-outs."""

    def __init__(self, n, **_):
        self.n = n
        self.init = None
        self.ops = []
        self.readouts = []
        self.passes_run = 0
        self.h2d_bytes = 0
        self.d2h_bytes = 0

    def init_product(self, vectors, scale):
        self.init = (np.asarray(vectors, dtype=float), float(scale))
        self.ops = []

    def load(self, coeffs):
        raise BasicAerError('batched programs start from product states')

    def map1(self, q, m, tag=None):
        self.ops.append(P.Op('map1', (q,), np.asarray(m, dtype=float), tag=tag))

    def cx(self, ctl, tgt, tsp):
        coef, ideal = P.cx_coefficients(tsp)
        self.ops.append(P.Op('cx', (ctl, tgt), np.array(coef), ideal, tag=('cx',)))

    def diag2(self, qa, qb, d):
        self.ops.append(P.Op('diag2', (qa, qb), np.asarray(d, dtype=float)))

    def axis_probs(self, mode, err):
        self.readouts.append(('axis', len(self.ops), list(mode), float(err)))
        return np.zeros(2 ** sum(1 for m in mode if m))

    def nbasis_probs(self, nvec, err):
        raise BasicAerError('batched programs read out Z ensemble probabilities only')

    def sample_counts(self, shots, seed):
        raise BasicAerError('batched programs report probabilities, not counts')

    def gather(self, indices):
        raise BasicAerError('batched programs read out Z ensemble probabilities only')

    def coefficients(self, chop_threshold):
        return None

    def raw_coefficients(self):
        return None

    def density_matrix(self):
        return None

    def overlap(self, other):
        raise BasicAerError('batched programs do not compare states')

    def trace_error(self):
        return 0.0

    def synchronize(self):
        pass


def compile_experiment(experiment, options):
    """Op stream and final Z read-out of one experiment, through the backend's own run loop."""
    from .dm_simulator import DmSimulatorGPU
    # the backend mirrors the reference's class-level rotation_error leak; an
    # instance compile starts from the pristine default and leaves the class as it was
    saved = DmSimulatorGPU.DEFAULT_OPTIONS['rotation_error']
    DmSimulatorGPU.DEFAULT_OPTIONS['rotation_error'] = {'rx': [1., 0.], 'ry': [1., 0.], 'rz': [1., 0.]}
    try:
        b = DmSimulatorGPU()
        opts = dict(options)
        opts['compute_densitymatrix'] = False
        b._set_options(backend_options=opts)
        rec = b.compile_experiment(experiment)
    finally:
        DmSimulatorGPU.DEFAULT_OPTIONS['rotation_error'] = saved
    if len(rec.readouts) != 1 or any(m != 3 for m in rec.readouts[0][2]):
        raise BasicAerError('a batched instance must end with one Z ensemble measurement of every qubit')
    # the level's memory noise after the read-out does not change the probabilities
    del rec.ops[rec.readouts[0][1]:]
    if rec.init is None or not np.array_equal(rec.init[0], np.tile([1.0, 0.0, 0.0, 1.0], (rec.n, 1))):
        raise BasicAerError('batched instances start in |0...0>')
    return rec


def _error_params(options):
    """The backend's error parameters for ``options`` (pristine class defaults, as compile_experiment)."""
    from .dm_simulator import DmSimulatorGPU
    saved = DmSimulatorGPU.DEFAULT_OPTIONS['rotation_error']
    DmSimulatorGPU.DEFAULT_OPTIONS['rotation_error'] = {'rx': [1., 0.], 'ry': [1., 0.], 'rz': [1., 0.]}
    try:
        b = DmSimulatorGPU()
        opts = dict(options)
        opts['compute_densitymatrix'] = False
        b._set_options(backend_options=opts)
        b._initialize_errors()
    finally:
        DmSimulatorGPU.DEFAULT_OPTIONS['rotation_error'] = saved
    return b._error_params, b.MERGE


def derive_recording(ref, spec):
    """The recording of sweep instance ``spec`` from ``ref``, the backend's recording of another
    instance of the same structure (qubits, depth): the same operations in the same order, with
    this instance's matrices built by the functions the run loop uses (its merged gates'
    rotations in program order per qubit, its memory noise, its CX error, its read-out
    polarisation).  None when the instance does not line up with ``ref`` (qubit count,
    rotation axes per qubit, the (control, target) sequence of its CX gates, or a read-out
    other than one Ensemble Z measurement of every qubit); the caller then records it
    through the run loop."""
    from .dm_simulator import _u_decomposition
    from .scheduler import merge_single_gates
    exp, opts = instance_experiment(spec)
    n = ref.n
    if exp.config.n_qubits != n:
        return None
    err, merge = _error_params(opts)
    gates = [[] for _ in range(n)]
    cxs = []
    measured = set()
    for inst in merge_single_gates(exp.instructions, n, merge):
        if inst.name in ('u1', 'u3'):
            gates[inst.qubits[0]].append(_u_decomposition(inst.name, inst.params))
        elif inst.name in ('cx', 'CX'):
            cxs.append(tuple(int(q) for q in inst.qubits))
        elif inst.name == 'measure':
            params = getattr(inst, 'params', None) or []
            if len(params) != 2 or str(params[0]) != 'Ensemble' or str(params[1]) != 'Z':
                return None
            measured.update(int(q) for q in inst.qubits)
    if measured != set(range(n)) or len(ref.readouts) != 1 or list(ref.readouts[0][2]) != [3] * n:
        return None
    mem = err['memory']
    noise = P.noise_ptm(mem['decoherence'], mem['thermalization'], mem['amplitude_decay'])
    if np.array_equal(noise, P.IDENTITY4):
        return None                    # the run loop records no memory noise then
    coef, ideal = P.cx_coefficients(err['two_qubit_gates'])
    rot_err = err['one_qubit_gates']
    used = [0] * n
    used_cx = 0
    ops = []
    for op in ref.ops:
        if op.kind == 'map1' and op.tag and op.tag[0] == 'rot':
            q = op.axes[0]
            if used[q] >= len(gates[q]):
                return None
            gate = gates[q][used[q]]
            used[q] += 1
            if [a for a, _ in gate] != [a for a, _ in op.tag[1]]:
                return None
            ops.append(P.Op('map1', op.axes, P.rotations_ptm(gate, rot_err),
                            tag=('rot', tuple((a, float(t)) for a, t in gate))))
        elif op.kind == 'map1' and op.tag == ('noise',):
            ops.append(P.Op('map1', op.axes, noise, tag=('noise',)))
        elif op.kind == 'cx':
            if used_cx >= len(cxs) or tuple(op.axes) != cxs[used_cx]:
                return None
            used_cx += 1
            ops.append(P.Op('cx', op.axes, np.array(coef), ideal, tag=('cx',)))
        else:
            return None
    if used != [len(g) for g in gates] or used_cx != len(cxs):
        return None
    rec = HostRecorder(n)
    rec.init = ref.init
    rec.ops = ops
    kind, pos, mode, _ = ref.readouts[0]
    rec.readouts = [(kind, pos, list(mode), float(err['measurement']))]
    return rec


def record_group(specs):
    """Recordings of sweep instances of one structure: the first through the backend's run
    loop, the others derived from it (``derive_recording``) where they line up."""
    recs, ref = [], None
    for spec in specs:
        rec = derive_recording(ref, spec) if ref is not None else None
        if rec is None:
            rec = compile_experiment(*instance_experiment(spec))
            if ref is None:
                ref = rec
        recs.append(rec)
    return recs


def _signature(ops):
    return tuple((op.kind, op.axes, op.ideal) for op in ops)


class _Plan:
    """A pass / round plan shared by instances of one structure (CUDA-core register rounds)."""

    kind = 'cuda'

    def __init__(self, ops, n, kmax, dtype):
        self.n = n
        width = N.DM_ROUND_AXES[N.DM_F64 if dtype == np.float64 else N.DM_F32]
        self.passes = []     # dm_batch_pass
        self.slots = []      # (kind, src, ideal, flags) per coefficient block entry, in mats order
        self.mats_len = 0
        for p in P.plan_passes(ops, n, kmax, 2):
            pp = p if len(p.axes) >= width else P.pad_pass(p, n, width)
            rounds = P.plan_rounds(pp, width)
            bp = N.DmBatchPass()
            self._fill(bp, pp, rounds, [axes for axes, _ in rounds])
            self.passes.append(bp)

    def _fill(self, bp, pp, rounds, digit_orders):
        """Pass header, round axes (in ``digit_orders``) and ops of one dm_batch_pass."""
        def place(op, flags, size):
            if op.kind not in ('map1', 'cx', 'diag2'):
                raise BasicAerError('batched programs hold 4x4 maps, CX and diagonal pair maps only')
            self.slots.append((op.kind, list(op.src), op.ideal,
                               (flags & (N.DM_MAP1_ROW0_IDENTITY | N.DM_MAP1_XY_UNITAL))
                               if op.kind == 'map1' else 0))
            self.mats_len += size
            return self.mats_len - size

        P.fill_round_ops(bp, pp, rounds, digit_orders, place)

    def table_bytes(self):
        return bytes((N.DmBatchPass * len(self.passes))(*self.passes))

    def coefficients(self, ops, dtype):
        """The coefficient block of one instance (its own op matrices, composed along the plan)."""
        out = np.empty(self.mats_len, dtype=np.float64)
        pos = 0
        for kind, src, ideal, row0 in self.slots:
            if kind == 'map1':
                m = ops[src[0]].data
                for i in src[1:]:
                    m = ops[i].data @ m
                m = m.reshape(16)
                if (row0 & N.DM_MAP1_ROW0_IDENTITY) and not (m[0] == 1.0 and not m[1:4].any()):
                    raise BasicAerError('instance does not share the plan (I row)')
                if (row0 & N.DM_MAP1_XY_UNITAL) and (m[4] != 0.0 or m[8] != 0.0):
                    raise BasicAerError('instance does not share the plan (I column)')
                out[pos:pos + 16] = m
                pos += 16
            elif kind == 'cx':
                out[pos:pos + 5] = ops[src[0]].data
                pos += 5
            else:
                out[pos:pos + 16] = np.asarray(ops[src[0]].data).reshape(16)
                pos += 16
        return out.astype(dtype)


def fill_tc_tables(t, pp, layouts, direct=False):
    """The conversion and epilogue tables of a 7-axis pass (dm_tc_pass; umoff left 0)."""
    conv, rtables = P.tc_tables(layouts, 'xor', direct)
    t.direct_last = 1 if direct else 0
    for r, q in enumerate(pp.axes):
        t.axes[r] = q
    t.nrounds = len(layouts)
    t.vec0 = conv['vec0']
    for i in range(8):
        t.natrow[i] = conv['natrow'][i]
    for i in range(6):
        t.natk[i] = conv['natk'][i]
    for r, rt in enumerate(rtables):
        for i in range(3):
            t.rounds[r].digits[i] = rt['digits'][i]
        t.rounds[r].vec = rt['vec']
        t.rounds[r].umoff = 0
        for i in range(8):
            t.rounds[r].rowc[i] = rt['rowc'][i]
        for i in range(6):
            t.rounds[r].kc[i] = rt['kc'][i]


class _TcPlan(_Plan):
    """A tensor-core plan shared by instances of one structure: passes of 7
    resident axes, rounds of 3 axes in the digit order their layouts chose;
    the device composes each round's 64x64 matrix from the instance's block."""

    kind = 'tc'

    def __init__(self, ops, n):
        self.n = n
        self.passes = []     # dm_batch_tc_pass
        self.slots = []
        self.mats_len = 0
        for p in P.plan_passes(ops, n, P.TC_AXES, 2):
            pp = P.pad_pass(p, n)
            rounds = P.plan_rounds(pp, 3, pad='neighbors')
            if len(rounds) > N.DM_MAX_ROUNDS:
                raise P.TcPlanError('pass needs %d rounds (> %d)' % (len(rounds), N.DM_MAX_ROUNDS))
            direct = P.direct_last_eligible([axes for axes, _ in rounds])
            layouts = P._choose_layouts([axes for axes, _ in rounds], direct=direct)
            bp = N.DmBatchTcPass()
            self._fill(bp.ops, pp, rounds, [L.digits for L in layouts])
            fill_tc_tables(bp.tables, pp, layouts, direct)
            self.passes.append(bp)

    def table_bytes(self):
        return bytes((N.DmBatchTcPass * len(self.passes))(*self.passes))


TC = 'tc'    # resident-axes choice of a qubit count whose instances run on the tensor cores


def _make_plan(ops, n, k, np_dtype):
    if k == TC:
        if np_dtype != np.float32 or n < P.TC_AXES:
            raise BasicAerError('tensor-core batched passes need FP32 instances of >= %d qubits' % P.TC_AXES)
        try:
            return _TcPlan(ops, n)
        except P.TcPlanError:       # more rounds than a pass table holds: the CUDA-core plan
            return _Plan(ops, n, P.TC_AXES, np_dtype)
    return _Plan(ops, n, min(k, n), np_dtype)


def sweep_specs(count, seed=0, n_range=(6, 12), depth_range=(10, 50), noise_range=(1e-4, 1e-2)):
    """The seeded batched noise sweep: qubits, depth, circuit seed and log-uniform noise per instance."""
    rng = np.random.default_rng(seed)
    lo, hi = np.log(noise_range[0]), np.log(noise_range[1])
    specs = []
    for i in range(count):
        specs.append({
            'n': int(rng.integers(n_range[0], n_range[1] + 1)),
            'depth': int(rng.integers(depth_range[0], depth_range[1] + 1)),
            'seed': seed * 1000003 + i,
            'depolarisation': float(np.exp(rng.uniform(lo, hi))),
            'decoherence': 1.0 - float(np.exp(rng.uniform(lo, hi))),
            'decay': 1.0 - float(np.exp(rng.uniform(lo, hi))),
        })
    return specs


def instance_experiment(spec):
    qc = random_layer_circuit(spec['n'], spec['depth'], spec['seed'])
    opts = noise_options(depolarisation=spec['depolarisation'], decoherence=spec['decoherence'],
                         decay=spec['decay'])
    return qc.to_experiment(copy=False), opts


def _structure(spec):
    """Instances with the same key run the same template structure (gate angles and noise aside)."""
    return (spec['n'], spec['depth'])


def compile_group(specs, variants):
    """Op streams of one structure group, planned for each (precision, resident axes) variant.

    Returns, per variant, the distinct plans (their dm_batch_pass tables as
    bytes, pass count, coefficient count) and per instance (plan index,
    FP64 coefficient block, measurement polarisation).
    """
    recs = record_group(specs)
    out = []
    for precision, k in variants:
        np_dtype = np.float32 if precision == 'single' else np.float64
        by_sig, plans, insts = {}, [], []
        for spec, rec in zip(specs, recs):
            sig = _signature(rec.ops)
            if sig not in by_sig:
                by_sig[sig] = len(plans)
                plans.append(_make_plan(rec.ops, spec['n'], k, np_dtype))
            pi = by_sig[sig]
            insts.append((pi, plans[pi].coefficients(rec.ops, np.float64), rec.readouts[0][3]))
        out.append(([(pl.table_bytes(), len(pl.passes), pl.mats_len, pl.kind) for pl in plans], insts))
    return out


_WORKER = r"""
import importlib.util, os, pickle, sys
pkg_dir, task_path, out_path = sys.argv[1:4]
spec = importlib.util.spec_from_file_location('qiskit_aakash_gb300', os.path.join(pkg_dir, '__init__.py'),
                                              submodule_search_locations=[pkg_dir])
mod = importlib.util.module_from_spec(spec)
sys.modules['qiskit_aakash_gb300'] = mod
spec.loader.exec_module(mod)
from qiskit_aakash_gb300 import batch
with open(task_path, 'rb') as f:
    groups, variants = pickle.load(f)
res = [batch.compile_group(g, variants) for g in groups]
with open(out_path + '.tmp', 'wb') as f:
    pickle.dump(res, f, protocol=pickle.HIGHEST_PROTOCOL)
os.replace(out_path + '.tmp', out_path)
"""


def _compile_groups(groups, variants, workers):
    """compile_group over every group, in ``workers`` host processes (fresh interpreters)."""
    if workers <= 1 or len(groups) <= 1:
        return [compile_group(g, variants) for g in groups]
    import os
    import pickle
    import subprocess
    import sys
    import tempfile
    cost = [sum(s['n'] * s['depth'] for s in g) for g in groups]
    bins = [[] for _ in range(min(workers, len(groups)))]
    load = [0] * len(bins)
    for gi in sorted(range(len(groups)), key=lambda g: -cost[g]):     # longest first onto the lightest bin
        b = load.index(min(load))
        bins[b].append(gi)
        load[b] += cost[gi]
    pkg_dir = os.path.dirname(os.path.abspath(__file__))
    results = [None] * len(groups)
    with tempfile.TemporaryDirectory(prefix='dm_batch_') as tmp:
        procs = []
        for b, members in enumerate(bins):
            task = os.path.join(tmp, 'task%d' % b)
            out = os.path.join(tmp, 'out%d' % b)
            with open(task, 'wb') as f:
                pickle.dump(([groups[g] for g in members], variants), f, protocol=pickle.HIGHEST_PROTOCOL)
            env = dict(os.environ, OMP_NUM_THREADS='1', OPENBLAS_NUM_THREADS='1')
            procs.append((members, out, subprocess.Popen([sys.executable, '-c', _WORKER, pkg_dir, task, out],
                                                         env=env, stderr=subprocess.PIPE)))
        for members, out, proc in procs:
            _, err = proc.communicate()
            if proc.returncode != 0:
                raise BasicAerError('batch compile worker failed:\n' + err.decode(errors='replace')[-2000:])
            with open(out, 'rb') as f:
                for g, r in zip(members, pickle.load(f)):
                    results[g] = r
    return results


def compile_sweep(specs, variants, workers=None, kmax=None):
    """BatchTables for each variant ('single' or 'double') of one sweep, compiled once.

    ``kmax`` maps a qubit count to resident axes (default 7 for FP32, 6
    for FP64), or a precision name to such a map; ``workers`` host
    processes share the host-side compile (default: every core for large
    sweeps, in-process for small ones).
    """
    import os
    kmax = dict(kmax or {})
    if not any(p in kmax for p in ('single', 'double')):
        kmax = {p: kmax for p in variants}
    t0 = time.perf_counter()
    for spec in specs:
        for precision in variants:
            lo = N.DM_ROUND_AXES[N.DM_F32 if precision == 'single' else N.DM_F64]
            if not lo <= spec['n'] <= MAX_QUBITS:
                raise BasicAerError('batched instances hold %d..%d qubits' % (lo, MAX_QUBITS))
    for per_n in kmax.values():
        for n, k in per_n.items():
            if k == TC:
                if n < P.TC_AXES:
                    raise BasicAerError('tensor-core batched passes need >= %d qubits' % P.TC_AXES)
                continue
            if k < min(4, n):
                # the two lowest qubits are always resident: a CX elsewhere needs two more axes
                raise BasicAerError('a pass of %d-qubit instances needs at least %d resident axes' % (n, min(4, n)))
    if workers is None:
        workers = (os.cpu_count() or 1) if len(specs) >= 64 else 1
    keys = {}
    for i, spec in enumerate(specs):
        keys.setdefault(_structure(spec), []).append(i)
    order = list(keys)
    groups = [[specs[i] for i in keys[key]] for key in order]
    # one variant list per structure: the resident axes depend on the qubit count
    by_group = {}
    for key in order:
        n = key[0]
        by_group[key] = [(p, kmax.get(p, {}).get(n, 7 if p == 'single' else 6)) for p in variants]
    # compile_group takes one variant list; groups with equal lists are compiled together
    results = [None] * len(groups)
    for vlist in {tuple(v) for v in by_group.values()}:
        idx = [g for g, key in enumerate(order) if tuple(by_group[key]) == vlist]
        for g, r in zip(idx, _compile_groups([groups[g] for g in idx], list(vlist), workers)):
            results[g] = r
    seconds = time.perf_counter() - t0
    tables = {}
    for vi, precision in enumerate(variants):
        per_instance = [None] * len(specs)
        plans = []
        for g, key in enumerate(order):
            gplans, ginsts = results[g][vi]
            base = len(plans)
            plans.extend(gplans)
            for i, (pi, block, err) in zip(keys[key], ginsts):
                per_instance[i] = (base + pi, block, err)
        tables[precision] = BatchTables(specs, precision, plans, per_instance, seconds)
    return tables


class _Part:
    """The instances of a batch that one kernel runs: their table entries, passes and coefficients."""

    def __init__(self, pass_type, np_dtype):
        self.pass_type = pass_type
        self.np_dtype = np_dtype
        self.insts, self.blobs, self.blocks = [], [], []
        self.pass_begin = {}
        self.npasses = 0
        self.mats_off = 0

    def add(self, pi, raw, npasses, mats_len, block, I):
        if pi not in self.pass_begin:
            self.pass_begin[pi] = self.npasses
            self.blobs.append(raw)
            self.npasses += npasses
        I.npasses = npasses
        I.pass_begin = self.pass_begin[pi]
        I.mats_off, I.mats_len = self.mats_off, mats_len
        self.mats_off += mats_len
        self.insts.append(I)
        self.blocks.append(block)

    def finish(self):
        self.ninst = len(self.insts)
        self.insts = (N.DmBatchInstance * self.ninst)(*self.insts)
        blob = b''.join(self.blobs)
        self.passes = (self.pass_type * self.npasses).from_buffer_copy(blob) if blob else (self.pass_type * 0)()
        self.mats = (np.concatenate(self.blocks) if self.blocks else np.zeros(0)).astype(self.np_dtype)
        del self.blobs, self.blocks


class BatchTables:
    """Host tables of a batch: instance table, shared pass plans and coefficient blocks.

    Instances are laid out largest first (4**n x depth), the order the
    device's work counter hands them out; ``index[i]`` is the slot of input
    instance i.  States and outcome probabilities are packed back to back in
    slot order.  Instances whose plan runs on the CUDA-core rounds form the
    main part (``insts``, ``passes``, ``mats``, ``ninst``, ``npasses``);
    those planned for the tensor cores form ``tc`` (same fields), each part
    with its own coefficient array.  Built by ``compile_sweep``; the
    constructor with ``specs`` only compiles one variant.
    """

    def __init__(self, specs, precision='single', plans=None, per_instance=None, compile_seconds=None,
                 kmax=None, workers=None):
        if plans is None:
            t = compile_sweep(specs, [precision], workers=workers, kmax=kmax)[precision]
            self.__dict__.update(t.__dict__)
            return
        t0 = time.perf_counter()
        self.precision = precision
        self.dtype = N.DM_F32 if precision == 'single' else N.DM_F64
        self.np_dtype = np.float32 if precision == 'single' else np.float64
        self.specs = specs
        order = sorted(range(len(specs)), key=lambda i: -(4 ** specs[i]['n'] * specs[i]['depth']))
        # the tensor-core part keeps FP64 coefficients: its round matrices are composed in FP64
        main, tc = _Part(N.DmBatchPass, self.np_dtype), _Part(N.DmBatchTcPass, np.float64)
        state_off = prob_off = 0
        self.index = []
        for i in order:
            pi, block, err = per_instance[i]
            raw, npasses, mats_len = plans[pi][:3]
            kind = plans[pi][3] if len(plans[pi]) > 3 else 'cuda'
            n = specs[i]['n']
            I = N.DmBatchInstance()
            I.n = n
            I.state_off, I.prob_off = state_off, prob_off
            I.meas_err = err
            part = tc if kind == 'tc' else main
            self.index.append((part, len(part.insts)))
            part.add(pi, raw, npasses, mats_len, block, I)
            state_off += 4 ** n
            prob_off += 2 ** n
        main.finish()
        tc.finish()
        slots = [None] * len(specs)
        for i, ref in zip(order, self.index):
            slots[i] = ref
        self.index = slots
        self.nplans = len(main.pass_begin) + len(tc.pass_begin)
        self.insts, self.passes, self.mats = main.insts, main.passes, main.mats
        self.ninst, self.npasses = main.ninst, main.npasses
        self.tc = tc
        self.ninst_total = main.ninst + tc.ninst
        self.states_count = state_off
        self.probs_count = prob_off
        self.compile_seconds = compile_seconds
        self.layout_seconds = time.perf_counter() - t0

    def instance(self, i):
        """The instance table entry of input instance i."""
        part, slot = self.index[i]
        return part.insts[slot]

    def all_instances(self):
        """Every instance table entry (main part, then tensor-core part)."""
        return list(self.insts) + list(self.tc.insts)

    def swept_bytes(self, esize):
        """State bytes read and written by all passes of all instances (one pass = one sweep of 4**n)."""
        return sum(2 * 4 ** I.n * esize * I.npasses for I in self.all_instances())

    def split(self, probs):
        """Per-instance outcome probabilities (input order) from the packed output."""
        out = []
        for i in range(len(self.specs)):
            I = self.instance(i)
            out.append(np.asarray(probs[I.prob_off:I.prob_off + 2 ** I.n]))
        return out


class BatchProgram:
    """A batch on the device: uploaded tables, resident states and outputs, optional CUDA graph."""

    def __init__(self, tables, device=None):
        import torch
        if not torch.cuda.is_available():
            raise BasicAerError('batched sweeps need a CUDA device')
        L = N.lib()
        self.t = tables
        self.dtype = tables.dtype
        self.device = torch.device(device or 'cuda')
        dev = self.device

        def to_dev(buf):
            raw = np.frombuffer(bytes(buf), dtype=np.uint8)
            return torch.from_numpy(raw.copy() if raw.size else np.zeros(16, dtype=np.uint8)).to(dev)

        self.insts_dev = to_dev(tables.insts)
        self.passes_dev = to_dev(tables.passes)
        self.mats_dev = torch.from_numpy(tables.mats if tables.mats.size else np.zeros(1, tables.mats.dtype)).to(dev)
        tc = tables.tc
        self.h2d_bytes = ctypes.sizeof(tables.insts) + ctypes.sizeof(tables.passes) + tables.mats.nbytes
        if tc.ninst:
            if self.dtype != N.DM_F32:
                raise BasicAerError('tensor-core batched passes run FP32 states only')
            self.tc_insts_dev = to_dev(tc.insts)
            self.tc_passes_dev = to_dev(tc.passes)
            self.tc_mats_dev = torch.from_numpy(tc.mats).to(dev)
            self.tc_scratch = torch.empty(L.dm_batch_tc_scratch_bytes(), dtype=torch.uint8, device=dev)
            self.h2d_bytes += ctypes.sizeof(tc.insts) + ctypes.sizeof(tc.passes) + tc.mats.nbytes
        tdt = torch.float32 if self.dtype == N.DM_F32 else torch.float64
        self.states = torch.empty(tables.states_count, dtype=tdt, device=dev)
        self.probs = torch.zeros(tables.probs_count, dtype=torch.float64, device=dev)
        self.counter = torch.zeros(2, dtype=torch.int32, device=dev)
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        self.graph = None

    def launch(self, stream=None):
        """The tensor-core part (the largest instances) first, then the CUDA-core part, on one stream."""
        import torch
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        vp = ctypes.c_void_p
        t = self.t
        tc = t.tc
        if tc.ninst:
            N.call('dm_batch_run_tc', vp(self.states.data_ptr()), ctypes.c_size_t(t.states_count),
                   vp(self.probs.data_ptr()), ctypes.c_size_t(t.probs_count), vp(self.tc_mats_dev.data_ptr()),
                   ctypes.c_size_t(tc.mats.size), tc.insts, vp(self.tc_insts_dev.data_ptr()), tc.ninst,
                   tc.passes, vp(self.tc_passes_dev.data_ptr()), tc.npasses, vp(self.counter.data_ptr() + 4),
                   vp(self.tc_scratch.data_ptr()), ctypes.c_size_t(self.tc_scratch.numel()),
                   vp(self.status.data_ptr()), vp(s.cuda_stream))
        if t.ninst:
            N.call('dm_batch_run', self.dtype, vp(self.states.data_ptr()), ctypes.c_size_t(t.states_count),
                   vp(self.probs.data_ptr()), ctypes.c_size_t(t.probs_count), vp(self.mats_dev.data_ptr()),
                   ctypes.c_size_t(t.mats.size), t.insts, vp(self.insts_dev.data_ptr()), t.ninst,
                   t.passes, vp(self.passes_dev.data_ptr()), t.npasses, vp(self.counter.data_ptr()),
                   vp(self.status.data_ptr()), vp(s.cuda_stream))

    def capture(self):
        """Capture one launch in a CUDA graph (after a first, uncaptured launch)."""
        import torch
        self.launch()
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.launch(torch.cuda.current_stream(self.device))
        self.graph = g
        return g

    def run(self):
        if self.graph is not None:
            self.graph.replay()
        else:
            self.launch()

    def results(self):
        """Outcome probabilities per instance (input order; qubit 0 is the most significant bit)."""
        if int(self.status.item()) != 0:
            raise BasicAerError('a tensor-core batched pass abandoned a bounded wait')
        return self.t.split(self.probs.cpu().numpy())


def autotune(specs, precision='single', candidates=None, sample=8, fill=None, reps=2):
    """Pick the resident axes (pass width k) per qubit count by timing each candidate on the device.

    For every qubit count in ``specs``, up to ``sample`` of its instances are
    recorded once and planned for every candidate k; each plan runs as a
    batch of ``fill`` instances (the sample repeated; default one per SM, so
    the timing sees a full GPU's memory traffic) and the fastest k wins.
    FP32 instances of >= 7 qubits also try ``TC`` (every pass on the
    tensor cores).  Returns ({n: k}, {(n, k): ms per launch}).
    """
    import torch
    lo = N.DM_ROUND_AXES[N.DM_F32 if precision == 'single' else N.DM_F64]
    hi = 7 if precision == 'single' else 6
    candidates = candidates or (([TC] if precision == 'single' else []) + list(range(hi, max(lo, hi - 2) - 1, -1)))
    if fill is None:
        fill = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    by_n = {}
    for s in specs:
        by_n.setdefault(s['n'], []).append(s)
    choice, timings = {}, {}
    for n, group in sorted(by_n.items()):
        ks = [k for k in candidates if (k == TC and n >= P.TC_AXES and precision == 'single') or
              (k != TC and lo <= k <= min(n, hi))]
        if len(ks) <= 1:
            choice[n] = ks[0] if ks else min(n, hi)
            continue
        # a short prefix of each sampled instance is enough to rank pass widths
        smp = [dict(sp, depth=min(sp['depth'], 12)) for sp in group[:sample]]
        # one recording per instance, one plan per candidate (instances may differ in depth)
        per_spec = [compile_group([sp], [(precision, k) for k in ks]) for sp in smp]
        reps_specs = [smp[j % len(smp)] for j in range(max(fill, len(smp)))]
        best = None
        for vi, k in enumerate(ks):    # in candidate order: the usually fastest first
            plans, per_instance = [], []
            for j in range(len(reps_specs)):
                gplans, ginsts = per_spec[j % len(smp)][vi]
                if j < len(smp):
                    plans.extend(gplans)
                _, block, err = ginsts[0]
                per_instance.append((j % len(smp), block, err))    # plan j % len(smp): one per sample
            prog = BatchProgram(BatchTables(reps_specs, precision, plans, per_instance, 0.0))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            prog.launch()
            b.record()
            torch.cuda.synchronize()
            ms = a.elapsed_time(b)
            if best is None or ms < 1.5 * best[0]:     # a clear loser is not timed again
                a.record()
                for _ in range(reps):
                    prog.launch()
                b.record()
                torch.cuda.synchronize()
                ms = a.elapsed_time(b) / reps
            timings[(n, k)] = ms
            if best is None or ms < best[0]:
                best = (ms, k)
            del prog
        choice[n] = best[1]
    return choice, timings
