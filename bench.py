"""Benchmark: gate-layers/s of the 16-qubit noisy random-layer workload on one GB300.

Workload (one "step"): the seeded random brick-layer circuit at n = 16
qubits (4**16 = 4.3e9 Pauli coefficients), 60 layers of U3 on every qubit
then CX on the brick pairs, with the full noise model after every gate
(depolarisation 1e-3 at measurement, decoherence 0.995, amplitude decay
0.998, rotation error sigma 1e-3 rad; a barrier after each gate so that the
reference's per-level memory noise follows every gate), ending with a
Z-basis ensemble measurement of all qubits (65,536 probabilities).

Reported (one JSON line on rank 0):
* value       -- gate-layers/s of the fused FP32 form, device path with
                 the circuit's program resident in HBM (CUDA events);
* plain_fp64  -- the same for the FP64 form (reference parity form);
* accuracy    -- FP32 vs FP64: max-abs error of the Pauli expectations
                 2**n a_s and L1 error of the outcome probabilities;
* e2e         -- the same metric through the public API
                 (``backend.run(qobj).result()``): host planning, program
                 upload, device work, results copied to host;
* roofline    -- the fused pass kernel: algorithmic bytes per launch
                 (read + write of every coefficient) / mean launch time;
* cpu_baseline-- the CPU oracle (a numpy restatement of the reference's
                 algorithm) timed on a bounded sample and scaled.

``--impl reference`` times the reference's CPU algorithm (the oracle port)
instead and prints its line.  Under torchrun every rank runs an independent
replica (the path does not shard across GPUs); value sums the replicas.
"""
import argparse
import copy
import gc
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import __graft_entry__  # noqa: E402

METRIC = 'gate-layers/s at n=16 (random U3+CX brick layers, full noise after every gate): fused FP32 vs plain FP64'
NOISE = dict(depolarisation=1e-3, decoherence=0.995, decay=0.998, rotation_sigma=1e-3)
CPU_SAMPLE_N = 11      # one noisy layer at 11 qubits: about 7 s of single-core reference work on the host


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=3)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', choices=['ours', 'reference'], default='ours')
    ap.add_argument('--n', type=int, default=16)
    ap.add_argument('--layers', type=int, default=60)
    ap.add_argument('--seed', type=int, default=0)
    ap.add_argument('--fp64-steps', type=int, default=1)
    ap.add_argument('--e2e-steps', type=int, default=2)
    ap.add_argument('--no-cpu', action='store_true', help='skip the CPU baseline sample')
    ap.add_argument('--no-gate-kinds', action='store_true', help='skip the per-gate-kind bandwidth table')
    ap.add_argument('--batch', type=int, default=4096,
                    help='instances of the batched noise sweep (0 skips the sweep leg)')
    ap.add_argument('--surrogate-train', type=int, default=1048576,
                    help='training points of the noise surrogate (0 skips the surrogate leg)')
    ap.add_argument('--surrogate-test', type=int, default=65536, help='held-out points of the noise surrogate')
    ap.add_argument('--surrogate-epochs', type=int, default=20)
    ap.add_argument('--c2-layers', type=int, default=40, help='random layers after the QFT in the n=14 leg')
    ap.add_argument('--legs', default='headline,c2,batch,surrogate',
                    help='comma list of legs to run (the JSON line keeps only what ran)')
    ap.add_argument('--no-autotune', action='store_true',
                    help='batched sweep without timing candidates: tensor cores from 9 qubits, 7 resident axes below')
    return ap.parse_args()


def workload(pkg, n, layers, seed):
    qc = pkg.random_layer_circuit(n, layers, seed, barrier_after_gate=True)
    opts = pkg.noise_options(**NOISE)
    opts['compute_densitymatrix'] = False
    return qc, opts


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ('uuid,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
              'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
              'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, uuid):
        self.uuid = uuid
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(['nvidia-smi', '--query-gpu=' + self.FIELDS, '--format=csv,noheader,nounits',
                                          '-lms', '200'], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(',')]
            if len(parts) < 9:
                continue
            if self.uuid and self.uuid not in parts[0]:
                continue
            rows.append(parts)
        if not rows:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['no nvidia-smi samples'], 'samples': 0}
        sm = [float(r[1]) for r in rows if r[1].replace('.', '', 1).isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace('.', '', 1).isdigit()]
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == 'active'})
        pw = [float(r[3]) for r in rows if r[3].replace('.', '', 1).isdigit()]
        return {'sm_mhz': statistics.median(sm) if sm else None, 'sm_max_mhz': max(smax) if smax else None,
                'reasons': reasons, 'samples': len(rows), 'power_w_max': max(pw) if pw else None}


def gpu_uuid(torch):
    try:
        u = str(torch.cuda.get_device_properties(0).uuid)
        return u.replace('GPU-', '')
    except Exception:  # noqa: BLE001
        return None


def measured_peaks():
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            d = json.load(f)
        return float(d['hbm_gbs']), 'measured'
    except Exception:  # noqa: BLE001
        return 6800.0, 'fallback'


def profiled_value(key):
    """A figure of the pass kernel's committed ncu summary ('key: value' line), if any."""
    path = os.path.join(ROOT, 'profiles', 'pass_tma_kernel_fp16_split_fp32_n14.md')
    try:
        for line in open(path):
            if line.startswith(key + ':'):
                return float(line.split(':', 1)[1])
    except OSError:
        pass
    return None


def profiled_traffic():
    """Per-launch DRAM bytes of the pass kernel from the committed ncu summary, if any."""
    return profiled_value('traffic_bytes_per_launch')


# ---------------------------------------------------------------------------
# CPU baseline (the oracle, a numpy restatement of the reference's algorithm)
# ---------------------------------------------------------------------------

def cpu_simulator():
    """(kind, factory) of the CPU implementation timed: the reference's own DmSimulatorPy (unmodified,
    loaded by oracle/refload.py from the reference tree or its byte-compiled copy in oracle/_ref), else
    the oracle port (a numpy restatement of the same algorithm)."""
    from oracle import refload
    if refload.available():
        dm = refload.load()

        def make(opts):
            dm.DmSimulatorPy.DEFAULT_OPTIONS['rotation_error'] = {'rx': [1., 0.], 'ry': [1., 0.], 'rz': [1., 0.]}
            b = dm.DmSimulatorPy()
            b._set_options(qobj_config=None, backend_options=copy.deepcopy(opts))
            return b
        return 'reference', make
    from oracle import dm_oracle
    return 'port', lambda opts: dm_oracle.OracleDmSimulator(copy.deepcopy(opts))


def cpu_sample(pkg, n_full, seed):
    """Time one noisy random layer of the reference at CPU_SAMPLE_N qubits; scale to n_full.

    The reference's work per level is n full-state sweeps of 4**n
    coefficients and a layer has n U3 levels plus the CX levels, so the
    per-layer time scales by levels(n) * n * 4**n.  The n = 16 workload
    itself does not fit the reference on the host (a 34 GB state plus a
    full copy per rotation).
    """
    kind, make = cpu_simulator()
    n = CPU_SAMPLE_N
    qc = pkg.random_layer_circuit(n, 1, seed, barrier_after_gate=True, measure=False)
    opts = pkg.noise_options(**NOISE)
    opts['compute_densitymatrix'] = False
    sim = make(opts)
    t0 = time.perf_counter()
    res = sim.run_experiment(qc.to_experiment())
    dt = time.perf_counter() - t0
    lv_small = res['number_of_clock_cycles']
    # levels per layer at n_full: n U3 levels + CX levels (n//2 in even, (n-1)//2 in odd layers)
    lv_full = n_full + ((n_full // 2) + ((n_full - 1) // 2)) / 2.0
    scale = (lv_full * n_full * 4.0 ** n_full) / (lv_small * n * 4.0 ** n)
    sec_per_layer_full = dt * scale
    what = ('the reference DmSimulatorPy.run_experiment (dm_simulator.py:950-1196, unmodified)' if kind == 'reference'
            else 'the oracle port')
    return {'value': 1.0 / sec_per_layer_full, 'unit': 'gate-layers/s', 'cores': 1, 'kind': kind,
            'sample': ('1 noisy random layer at n=%d through %s (%d levels, %.2f s, numpy FP64, 1 thread), '
                       'scaled to n=%d by levels*n*4^n (x%.0f); n=%d itself does not fit the reference on the host'
                       % (n, what, lv_small, dt, n_full, scale, n_full)),
            'sample_seconds': dt}


# ---------------------------------------------------------------------------
# the GPU arm
# ---------------------------------------------------------------------------

def dist_setup(args):
    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    return world, rank, local


def barrier(torch, world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(torch, world, x, device='cuda'):
    """Max of x over the ranks (the slowest replica's time defines the job's time)."""
    if world <= 1:
        return x
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(torch, world, units_local, ms_local, device='cuda'):
    """Whole-job throughput of independent replicas: all units / the slowest rank's time."""
    ms = allmax(torch, world, ms_local, device)
    units = units_local
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([units_local], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        units = float(t.item())
    return units / (ms / 1e3), ms


def time_replays(torch, state, steps):
    stream = torch.cuda.current_stream()
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    start.record(stream)
    for _ in range(steps):
        state.replay()
    end.record(stream)
    torch.cuda.synchronize()
    return start.elapsed_time(end) / steps


PASS_KERNELS = {'dm_apply_pass': 'pass_pipe_kernel', 'dm_apply_pass_tc': 'pass_tc_kernel',
                'dm_apply_pass_tma': 'pass_tma_kernel', 'dm_compose_rounds': 'compose_pass_kernel'}


def pass_kernel_profile(torch, state):
    """Durations (ms) of the pass-kernel launches of one replay, by kernel (events on the launching stream)."""
    stream = torch.cuda.current_stream()
    marks = []

    def on_call(name, before):
        if name in PASS_KERNELS:
            ev = torch.cuda.Event(enable_timing=True)
            ev.record(stream)
            marks.append((name, ev))

    torch.cuda.synchronize()
    state.replay(on_call)
    torch.cuda.synchronize()
    out = {}
    for i in range(0, len(marks) - 1, 2):
        name = PASS_KERNELS[marks[i][0]]
        out.setdefault(name, []).append(marks[i][1].elapsed_time(marks[i + 1][1]))
    return out


def tile_pattern_ceiling(torch, N, state, entry):
    """DRAM rate of the tiles that the recorded step's `entry` passes stream: dm_tile_copy_probe (an
    in-place read and write of every tile, 16-byte accesses, values unchanged) over each such pass's
    resident qubits, CUDA events on the current stream; algorithmic bytes / probe time."""
    import ctypes
    shapes = {}
    for name, args in state.tape:
        if name == entry:
            ax = tuple(int(a) for a in args[2]._obj.axes)
            shapes[ax] = shapes.get(ax, 0) + 1
    if not shapes:
        return None
    L = N.lib()
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    ptr = ctypes.c_void_p(state.state.data_ptr())
    total_ms, count = 0.0, 0
    for ax, k in shapes.items():
        a = (ctypes.c_int32 * 7)(*ax)
        N.call('dm_tile_copy_probe', ptr, state.n, a, sp)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(2):
            N.call('dm_tile_copy_probe', ptr, state.n, a, sp)
        e1.record(stream)
        torch.cuda.synchronize()
        total_ms += k * e0.elapsed_time(e1) / 2
        count += k
    gbs = count * 2 * 4.0 ** state.n * 4 / (total_ms / 1e3) / 1e9
    return {'gbs': gbs, 'passes': count, 'tile_shapes': len(shapes),
            'probe': 'dm_tile_copy_probe over the same passes\' tiles (in-place read + write, 16-byte accesses)'}


def all_durations(by_kernel):
    """Durations of the pass launches (the round-matrix composition launches are listed apart)."""
    return [d for k, v in by_kernel.items() if k != 'compose_pass_kernel' for d in v]


def fp64_peak(torch, N, seconds=0.5):
    """Measured FP64 FMA throughput of this GPU (dm_fp64_fma_probe, CUDA events, clocks sampled)."""
    import ctypes
    L = N.lib()
    threads = L.dm_fp64_fma_probe_threads()
    out = torch.empty(threads, dtype=torch.float64, device='cuda')
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)

    def run(iters):
        N.call('dm_fp64_fma_probe', ctypes.c_void_p(out.data_ptr()), ctypes.c_int64(iters), sp)

    run(1000)
    iters = 1000
    while True:     # grow the launch to about `seconds`
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(stream)
        run(iters)
        b.record(stream)
        torch.cuda.synchronize()
        ms = a.elapsed_time(b)
        if ms > 1e3 * seconds / 4 or iters > 1 << 30:
            break
        iters *= 4
    with ClockSampler(gpu_uuid(torch)) as clocks:
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(4):
            run(iters)
        b.record(stream)
        torch.cuda.synchronize()
    ms = a.elapsed_time(b) / 4
    flops = 2.0 * 8 * iters * threads
    return {'tflops': flops / (ms / 1e3) / 1e12, 'ms': ms, 'fmas_per_launch': flops / 2,
            'kernel': 'fp64_fma_probe: 8 independent FMA chains per thread, %d threads' % threads,
            'clocks': clocks.summary()}


def fp64_flops(pkg, qc, opts, tile_axes=6, low=2):
    """FP64 FLOPs of one run of the circuit as the fused FP64 passes apply it: the circuit's operations
    planned into passes (consecutive maps on one axis of a pass composed into one), and per planned
    operation 2 * its matrix's nonzeros / its dimension per coefficient (a dense 4x4 map: 8; an ideal
    CX: 0, a signed permutation), times 4**n."""
    from qiskit_aakash_gb300 import batch as B
    from qiskit_aakash_gb300 import program as P
    rec = B.compile_experiment(qc.to_experiment(), opts)
    per = 0.0
    for op in (o for p in P.plan_passes(rec.ops, rec.n, tile_axes, low) for o in p.ops):
        if op.kind == 'map1':
            per += 2.0 * np.count_nonzero(np.asarray(op.data)) / 4
        elif op.kind == 'cx':
            per += 0.0 if op.ideal else 2.0 * np.count_nonzero(P.cx_matrix16(op.data, op.ideal)) / 16
        elif op.kind == 'diag2':
            per += np.count_nonzero(np.asarray(op.data) != 1.0) / 16
        else:
            per += 2.0 * np.count_nonzero(np.asarray(op.data)) / 16
    return per * 4.0 ** rec.n


def per_gate_kind(torch, N, n=14, reps=3, dtype=None):
    """HBM GB/s of each single-operation sweep at n qubits (2 * 4**n * s bytes per sweep, s = 8 FP64 / 4 FP32)."""
    import ctypes
    L = N.lib()
    dtype = N.DM_F64 if dtype is None else dtype
    esize = 8 if dtype == N.DM_F64 else 4
    st = torch.empty(4 ** n, dtype=torch.float64 if dtype == N.DM_F64 else torch.float32, device='cuda')
    v = np.tile(np.array([1.0, 0.0, 0.0, 1.0]), n)
    N.call('dm_init_product', ctypes.c_void_p(st.data_ptr()), n, dtype,
           v.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 0.5 ** n, None)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ptr = ctypes.c_void_p(st.data_ptr())
    rng = np.random.default_rng(0)
    u3 = np.eye(4)
    u3[1:, 1:] = np.linalg.qr(rng.normal(size=(3, 3)))[0]
    noise = np.diag([1.0, 0.99, 0.99, 0.998])
    noise[3, 0] = 0.001
    out = torch.empty(2 ** n, dtype=torch.float64, device='cuda')
    scratch = torch.empty(max(8, L.dm_nbasis_probs_scratch_bytes(n)), dtype=torch.uint8, device='cuda')
    mode = (ctypes.c_int * n)(*([3] * n))
    nvec = N.f64_array([0.6, 0.0, 0.8])
    keep = []

    def arr(a):
        a = np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
        keep.append(a)
        return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))

    kinds = {
        'u3 (4x4 map, one qubit)': (lambda: N.call('dm_apply_map1', ptr, n, dtype, n // 2, arr(u3), s), 1),
        'memory noise (one qubit)': (lambda: N.call('dm_apply_map1', ptr, n, dtype, 0, arr(noise), s), 1),
        'cx ideal (signed permutation)': (lambda: N.call('dm_apply_cx', ptr, n, dtype, 3, 4, arr([1.0, 0.0]), s), 1),
        'cx with tsp error': (lambda: N.call('dm_apply_cx', ptr, n, dtype, 3, 4, arr([0.98, 0.02]), s), 1),
        'memory noise, every qubit (n sweeps)': (
            lambda: N.call('dm_apply_memory_noise', ptr, n, dtype, 0.995, 1.0, 0.998, s), n),
        'ensemble Z probabilities (2^n gather + WHT)': (
            lambda: N.call('dm_axis_probs', ptr, n, dtype, mode, 0.999, ctypes.c_void_p(out.data_ptr()), s), None),
        'ensemble N probabilities (full contraction)': (
            lambda: N.call('dm_nbasis_probs', ptr, n, dtype, nvec, 0.999, ctypes.c_void_p(out.data_ptr()),
                           ctypes.c_void_p(scratch.data_ptr()), s), 0.5),
    }
    hbm, _ = measured_peaks()
    res = {}
    for name, (fn, sweeps) in kinds.items():
        fn()
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            fn()
        b.record()
        torch.cuda.synchronize()
        ms = a.elapsed_time(b) / reps
        ent = {'ms': ms}
        if sweeps:
            gbs = sweeps * 2 * 4 ** n * esize / (ms / 1e3) / 1e9
            ent.update(gbs=gbs, frac_of_hbm=gbs / hbm)
        res[name] = ent
    del st, out, scratch
    torch.cuda.empty_cache()
    return {'n_qubits': n, 'dtype': 'f64' if esize == 8 else 'f32', 'bytes_per_sweep': 2 * 4 ** n * esize,
            'kinds': res}


def batch_cpu_sample(pkg, specs, budget_s=8.0):
    """Oracle seconds per instance cost unit (4**n x n x depth) on a few small instances of the sweep."""
    from oracle import dm_oracle as O
    from qiskit_aakash_gb300 import batch as B
    units = secs = 0.0
    used = []
    t_all = time.perf_counter()
    for spec in sorted((s for s in specs if s['n'] <= 9), key=lambda s: -s['n']):
        exp, opts = B.instance_experiment(spec)
        t0 = time.perf_counter()
        O.OracleDmSimulator(dict(opts, compute_densitymatrix=False)).run_experiment(exp)
        secs += time.perf_counter() - t0
        units += 4.0 ** spec['n'] * spec['n'] * spec['depth']
        used.append((spec['n'], spec['depth']))
        if time.perf_counter() - t_all > budget_s:
            break
    total_units = sum(4.0 ** s['n'] * s['n'] * s['depth'] for s in specs)
    est = secs / units * total_units
    return {'value': len(specs) / est, 'unit': 'instances/s', 'cores': 1, 'kind': 'port',
            'sample': '%d sweep instances (n, depth) %s through the oracle (%.1f s), extrapolated to the whole '
                      'sweep by 4**n * n * depth' % (len(used), used, secs)}


def batch_leg(args, pkg, torch, N):
    """Batched noise sweep: all instances in one persistent launch, replayed from a CUDA graph."""
    from qiskit_aakash_gb300 import batch as B
    specs = B.sweep_specs(args.batch, seed=args.seed)
    t0 = time.perf_counter()
    if args.no_autotune:
        choice, tune_ms = {n: (B.TC if n >= 9 else min(7, n)) for n in range(6, 13)}, {}
    else:
        choice, tune_ms = B.autotune(specs, 'single')
    tune_s = time.perf_counter() - t0
    tables = B.compile_sweep(specs, ['single', 'double'], kmax={'single': choice})
    t32, t64 = tables['single'], tables['double']

    prog = B.BatchProgram(t32)
    prog.capture()
    for _ in range(args.warmup):
        prog.run()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(args.steps):
        prog.run()
    b.record()
    torch.cuda.synchronize()
    ms32 = a.elapsed_time(b) / args.steps
    p32 = prog.results()
    del prog
    torch.cuda.empty_cache()
    prog = B.BatchProgram(t64)
    prog.launch()
    torch.cuda.synchronize()
    a.record()
    prog.launch()
    b.record()
    torch.cuda.synchronize()
    ms64 = a.elapsed_time(b)
    p64 = prog.results()
    del prog
    torch.cuda.empty_cache()
    tv = np.array([0.5 * np.abs(x - y).sum() for x, y in zip(p32, p64)])
    mx = max(float(np.max(np.abs(x - y))) for x, y in zip(p32, p64))
    # end to end: host compile of the sweep, upload, one launch, outcome distributions back
    torch.cuda.synchronize()
    e0 = time.perf_counter()
    te = B.compile_sweep(specs, ['single'], kmax={'single': choice})['single']
    pe = B.BatchProgram(te)
    pe.launch()
    res = pe.results()
    e2e_s = time.perf_counter() - e0
    h2d, d2h = pe.h2d_bytes, int(te.probs_count * 8)
    del pe, res
    torch.cuda.empty_cache()
    hbm, peak_kind = measured_peaks()
    by32 = t32.swept_bytes(4)
    kernels = (['batch_tc_kernel (tcgen05, %d instances)' % t32.tc.ninst] if t32.tc.ninst else []) + \
        (['batch_kernel<float,3> (%d instances)' % t32.ninst] if t32.ninst else [])
    out = {
        'metric': 'instances/s, batched noise sweep (4096 random-layer instances, n~U{6..12}, depth~U{10..50})',
        'value': t32.ninst_total / (ms32 / 1e3), 'unit': 'instances/s', 'ms_per_step': ms32, 'steps': args.steps,
        'dtype': 'f32', 'gpu_launches_per_step': len(kernels),
        'config': {'instances': t32.ninst_total, 'seed': args.seed, 'n_range': [6, 12], 'depth_range': [10, 50],
                   'noise': 'log-uniform depolarisation, 1-decoherence, 1-decay in [1e-4, 1e-2]',
                   'state_bytes_fp32': int(t32.states_count * 4), 'passes': t32.npasses + t32.tc.npasses,
                   'plans': t32.nplans,
                   'l2': 'inputs larger than L2: %.1f GB of states' % (t32.states_count * 4 / 1e9),
                   'launch': 'persistent launches per step (dm_batch_run_tc for the instances autotune put on '
                             'the tensor cores, dm_batch_run for the rest), CUDA graph replay'},
        'autotune': {'k_by_n': {str(k): v for k, v in choice.items()},
                     'ms': {'%s/%s' % nk: v for nk, v in tune_ms.items()}, 'seconds': tune_s},
        'accuracy_vs_fp64': {'max_tv': float(tv.max()), 'median_tv': float(np.median(tv)), 'max_abs_prob': mx,
                             'against': 'the same sweep in the batched FP64 form'},
        'fp64': {'value': t64.ninst_total / (ms64 / 1e3), 'unit': 'instances/s', 'ms_per_step': ms64,
                 'passes': t64.npasses},
        'roofline': {'bound': 'hbm', 'achieved': by32 / (ms32 / 1e3) / 1e9, 'peak': hbm, 'unit': 'GB/s',
                     'frac': by32 / (ms32 / 1e3) / 1e9 / hbm, 'kernel': ' + '.join(kernels),
                     'algorithmic_bytes_per_launch': by32, 'peak_kind': peak_kind},
        'host_compile_s': t32.compile_seconds,
        'e2e': {'value': t32.ninst_total / e2e_s, 'unit': 'instances/s', 'seconds_per_step': e2e_s,
                'h2d_bytes_per_step': int(h2d), 'd2h_bytes_per_step': d2h,
                'api': 'batch.compile_sweep + BatchProgram.launch + results (host compile included)'},
    }
    if not args.no_cpu:
        out['cpu_baseline'] = batch_cpu_sample(pkg, specs)
    return out


def surrogate_leg(args, torch):
    """Noise surrogate on a fixed 10-qubit, 30-layer template: data generation, training, held-out TV."""
    from qiskit_aakash_gb300 import surrogate as S
    tmpl = S.Template(n=10, layers=30, seed=args.seed)
    raw_tr = S.sample_noise(args.surrogate_train, seed=args.seed + 101)
    raw_te = S.sample_noise(args.surrogate_test, seed=args.seed + 202)
    tmpl.simulate(raw_te[:256])       # warm-up (tables, states)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    y_tr = tmpl.simulate(raw_tr).float()
    torch.cuda.synchronize()
    gen_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    y_te = tmpl.simulate(raw_te).float()
    torch.cuda.synchronize()
    sim_te_s = time.perf_counter() - t0
    f_tr = torch.from_numpy(S.features(raw_tr)).cuda()
    f_te = torch.from_numpy(S.features(raw_te)).cuda()
    ens = S.MLPEnsemble(members=5, batch=1024, seed=args.seed)
    fit = ens.fit(f_tr, y_tr, epochs=args.surrogate_epochs)
    ens.predict(f_te[:1024])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    qs = ens.predict(f_te)
    mean, spread, tv = ens.ensemble(qs, y_te)
    torch.cuda.synchronize()
    inf_s = time.perf_counter() - t0
    tv_np, spread_np = tv.cpu().numpy(), spread.cpu().numpy()
    blind = y_tr.mean(dim=0, keepdim=True)
    tv_blind = (0.5 * (y_te - blind).abs().sum(dim=1)).cpu().numpy()
    sim_rate = len(raw_te) / sim_te_s
    fallback = {}
    for tau in (0.0005, 0.001, 0.002):
        fb = spread_np > tau
        hybrid_tv = np.where(fb, 0.0, tv_np)
        t_h = inf_s + fb.sum() / sim_rate
        fallback['%g' % tau] = {'fallback_fraction': float(fb.mean()), 'hybrid_mean_tv': float(hybrid_tv.mean()),
                                'hybrid_max_tv': float(hybrid_tv.max()), 'points_per_s': len(raw_te) / t_h}
    return {
        'template': 'random brick layers n=10, 30 layers, Z ensemble; 6 noise inputs',
        'train_points': len(raw_tr), 'test_points': len(raw_te), 'members': 5, 'epochs': args.surrogate_epochs,
        'data_generation': {'instances_per_s': len(raw_tr) / gen_s, 'seconds': gen_s,
                            'kernel': ('batch_param_tc_kernel (tcgen05; FP64 recipe and round-matrix composition '
                                       'per pass)' if tmpl.program.tc else
                                       'batch_param_kernel<float,3> (FP64 recipe composition per pass)')},
        'training': {'steps': fit['steps'], 'seconds': fit['seconds'],
                     'samples_per_s': fit['steps'] * 1024 * 5 / fit['seconds']},
        'inference': {'points_per_s': len(raw_te) / inf_s, 'seconds': inf_s},
        'plain_simulation_points_per_s': sim_rate,
        'held_out_tv': {'mean': float(tv_np.mean()), 'median': float(np.median(tv_np)),
                        'p99': float(np.quantile(tv_np, 0.99)), 'max': float(tv_np.max())},
        'parameter_blind_baseline_tv': {'mean': float(tv_blind.mean()), 'max': float(tv_blind.max())},
        'spread': {'mean': float(spread_np.mean()), 'corr_with_tv': float(np.corrcoef(spread_np, tv_np)[0, 1])},
        'fallback_by_spread_threshold': fallback,
    }


def headline_leg(args, pkg, torch, N, DmSimulatorGPU, world, rank):
    """The n=16 layered workload: TC FP32 (value), CUDA-core FP32, FP64, e2e; None on ranks != 0."""
    n, layers = args.n, args.layers
    seed = args.seed + rank
    qc, opts = workload(pkg, n, layers, seed)

    def backend_for(precision, tensor_cores=True, tma=True):
        DmSimulatorGPU.DEFAULT_OPTIONS['rotation_error'] = {'rx': [1., 0.], 'ry': [1., 0.], 'rz': [1., 0.]}
        b = DmSimulatorGPU()
        o = copy.deepcopy(opts)
        o['precision'] = precision
        o['tensor_cores'] = tensor_cores
        o['tma'] = tma
        o['coefficients_to_host'] = False      # compared on the device below
        b._set_options(backend_options=o)
        return b

    # --- FP32 on the CUDA cores (the register-round kernel), for comparison ----
    bcc = backend_for('single', tensor_cores=False)
    bcc.record_experiment(qc.to_experiment())
    stcc = bcc.recorded_state
    stcc.replay()
    ms_cc = time_replays(torch, stcc, 1)
    by_cc = pass_kernel_profile(torch, stcc)
    durs_cc = all_durations(by_cc)
    kernels_cc = {k: {'launches': len(v), 'mean_ms': float(np.mean(v)),
                      'achieved_gbs': 2 * 4.0 ** n * 4 / (float(np.mean(v)) / 1e3) / 1e9} for k, v in by_cc.items()}
    del stcc, bcc
    torch.cuda.empty_cache()

    # --- FP32 tensor cores with cp.async-fed tiles only (the previous form), for comparison ----
    bca = backend_for('single', tma=False)
    bca.record_experiment(qc.to_experiment())
    stca = bca.recorded_state
    stca.replay()
    ms_ca = time_replays(torch, stca, 1)
    durs_ca = all_durations(pass_kernel_profile(torch, stca))
    del stca, bca
    torch.cuda.empty_cache()

    # --- fused FP32: record once, then time replays ---------------------------
    b32 = backend_for('single')
    r32 = b32.record_experiment(qc.to_experiment())
    st32 = b32.recorded_state
    stats32 = dict(b32.last_run_stats)
    for _ in range(args.warmup):
        st32.replay()
    uuid = gpu_uuid(torch)
    l0 = N.lib().dm_kernel_launch_count()
    barrier(torch, world)
    with ClockSampler(uuid) as clocks:
        ms32 = time_replays(torch, st32, args.steps)
    launches = (N.lib().dm_kernel_launch_count() - l0)
    barrier(torch, world)
    value32, ms32 = replica_throughput(torch, world, float(layers), ms32)
    by_kernel = pass_kernel_profile(torch, st32)     # a full replay: leaves the final FP32 state
    passes_by_kernel = dict(st32.passes_by_kernel)
    top_kernel = max(by_kernel, key=lambda k: sum(by_kernel[k]))
    pattern = tile_pattern_ceiling(torch, N, st32, {v: k for k, v in PASS_KERNELS.items()}[top_kernel])
    prob32 = np.array(list(r32['data']['ensemble_probability'].values()))

    # --- plain FP64 (the parity form) ---------------------------------------
    b64 = backend_for('double')
    r64 = b64.record_experiment(qc.to_experiment())
    st64 = b64.recorded_state
    stats64 = dict(b64.last_run_stats)
    st64.replay()
    ms64 = time_replays(torch, st64, args.fp64_steps)
    durs64 = all_durations(pass_kernel_profile(torch, st64))
    prob64 = np.array(list(r64['data']['ensemble_probability'].values()))
    max_abs = st32.max_abs_diff(st64) * 2.0 ** n
    peak64 = fp64_peak(torch, N)
    flops64 = fp64_flops(pkg, qc, opts)
    prob_l1 = float(np.abs(prob32 - prob64).sum())
    del st64, b64, r64, st32, b32, r32
    torch.cuda.empty_cache()

    # --- e2e through the public API (FP32 form) ------------------------------
    backend = pkg.BasicAer.get_backend('dm_simulator')
    e2e_opts = copy.deepcopy(opts)
    e2e_opts['precision'] = 'single'
    DmSimulatorGPU.DEFAULT_OPTIONS['rotation_error'] = {'rx': [1., 0.], 'ry': [1., 0.], 'rz': [1., 0.]}
    # warm-up in the timed loop's own pattern (each step holds the previous result while it runs, so
    # the copy-out alternates between two page-locked result blocks): planning caches, pinned staging
    # buffers, both result blocks made and each used again once
    res = None
    for _ in range(4):
        DmSimulatorGPU.DEFAULT_OPTIONS['rotation_error'] = {'rx': [1., 0.], 'ry': [1., 0.], 'rz': [1., 0.]}
        res = pkg.execute(qc, backend, **copy.deepcopy(e2e_opts)).result()
    gc.collect()       # the earlier legs' garbage is not the timed steps' work
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    each, copies = [], []
    for _ in range(args.e2e_steps):
        DmSimulatorGPU.DEFAULT_OPTIONS['rotation_error'] = {'rx': [1., 0.], 'ry': [1., 0.], 'rz': [1., 0.]}
        res = pkg.execute(qc, backend, **copy.deepcopy(e2e_opts)).result()
        each.append(time.perf_counter() - t0 - sum(each))
        copies.append(backend.last_run_stats.get('copy_out'))
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / args.e2e_steps
    e2e_s = allmax(torch, world, e2e_s)
    st = backend.last_run_stats
    del res

    if rank != 0:
        return None
    hbm, peak_kind = measured_peaks()
    N4 = 4.0 ** n
    # the dominant kernel: the most device time of the step's pass launches
    top = max(by_kernel, key=lambda k: sum(by_kernel[k]))
    durs = by_kernel[top]
    mean_pass_ms = float(np.mean(durs)) if durs else float('nan')
    achieved = 2 * N4 * 4 / (mean_pass_ms / 1e3) / 1e9
    kernels = {k: {'launches': len(v), 'total_ms': float(np.sum(v)), 'mean_ms': float(np.mean(v)),
                   'achieved_gbs': 2 * N4 * 4 / (float(np.mean(v)) / 1e3) / 1e9} for k, v in by_kernel.items()}
    mean_pass64 = float(np.mean(durs64)) if durs64 else float('nan')
    achieved64 = 2 * N4 * 8 / (mean_pass64 / 1e3) / 1e9
    traffic = profiled_traffic()
    line = {
        'metric': METRIC,
        'value': value32,
        'unit': 'gate-layers/s',
        'n_gpus': world,
        'steps': args.steps,
        'warmup': args.warmup,
        'ms_per_step': ms32,
        'higher_is_better': True,
        'scaling': 'weak',
        'vs_baseline': None,
        'dtype': 'f32',
        'data': 'synthetic: seeded random circuits (numpy default_rng), no dataset',
        'config': {'workload': 'random brick layers n=%d, %d layers, noise after every gate, Ensemble Z' % (n, layers),
                   'n_qubits': n, 'layers': layers, 'seed': args.seed, 'noise': NOISE,
                   'levels': stats32['levels'], 'fused_passes': stats32['passes'],
                   'passes_per_layer': stats32['passes'] / layers,
                   'state_bytes_fp32': int(N4 * 4),
                   'l2': 'inputs larger than L2: the %.1f GB state >> 129 MB L2' % (N4 * 4 / 1e9),
                   'parallelism': 'replicas' if world > 1 else 'single GPU'},
        'plain_fp64': {'value': world * layers / (ms64 / 1e3), 'unit': 'gate-layers/s', 'ms_per_step': ms64,
                       'fused_passes': stats64['passes'], 'mean_pass_ms': mean_pass64,
                       'pass_achieved_gbs': achieved64, 'pass_frac_of_hbm': achieved64 / hbm,
                       'fp64_flops_per_step': flops64,
                       'achieved_fp64_tflops': flops64 / (ms64 / 1e3) / 1e12,
                       'frac_of_fp64_peak': flops64 / (ms64 / 1e3) / 1e12 / peak64['tflops'],
                       'fp64_peak': peak64},
        'fp32_over_fp64': ms64 / ms32,
        'fp32_cuda_cores': {'value': world * layers / (ms_cc / 1e3), 'unit': 'gate-layers/s', 'ms_per_step': ms_cc,
                            'kernel': 'pass_pipe_kernel<float,3>',
                            'pass_kernels': kernels_cc,
                            'mean_pass_ms': float(np.mean(durs_cc)) if durs_cc else None,
                            'pass_achieved_gbs': (2 * N4 * 4 / (float(np.mean(durs_cc)) / 1e3) / 1e9) if durs_cc else None,
                            'pass_frac_of_hbm': (2 * N4 * 4 / (float(np.mean(durs_cc)) / 1e3) / 1e9 / hbm)
                            if durs_cc else None},
        'fp32_tc_cp_async': {'value': world * layers / (ms_ca / 1e3), 'unit': 'gate-layers/s', 'ms_per_step': ms_ca,
                             'kernel': 'pass_tc_kernel only (tiles by cp.async, two CTAs per SM)',
                             'mean_pass_ms': float(np.mean(durs_ca)) if durs_ca else None},
        'accuracy': {'max_abs_coeff_err': max_abs, 'prob_l1_err': prob_l1,
                     'against': 'FP64 GPU plain form (itself parity-checked against the reference at n<=14)',
                     'coeff_scale': 'Pauli expectations 2^n * a_s'},
        'roofline': {'bound': 'hbm', 'achieved': achieved, 'peak': hbm, 'unit': 'GB/s', 'frac': achieved / hbm,
                     'traffic': traffic, 'kernel': top + ' (tcgen05 kind::f16, 3-way FP16 split)',
                     'launches_per_step': len(durs), 'pass_kernels': kernels, 'passes_by_form': passes_by_kernel,
                     'mean_launch_ms': mean_pass_ms,
                     'tensor_pipe_active': profiled_value('tensor_pipe_active'),
                     'tensor_pipe_source': 'sm__pipe_tensor_cycles_active of the committed ncu capture at n = 14',
                     'algorithmic_bytes_per_launch': 2 * N4 * 4, 'peak_kind': peak_kind,
                     'tile_pattern': dict(pattern, frac=achieved / pattern['gbs']) if pattern else None},
        'e2e': {'value': world * layers / e2e_s, 'unit': 'gate-layers/s', 'seconds_per_step': e2e_s,
                'seconds_each': each, 'copy_out_each': copies,
                'h2d_bytes_per_step': int(st['h2d_bytes']), 'd2h_bytes_per_step': int(st['d2h_bytes']),
                'api': "BasicAer.get_backend('dm_simulator') + execute(...).result()"},
        'gpu_launches': int(launches),
        'clocks': clocks.summary(),
    }
    return line


def c2_leg(args, pkg, torch, N, DmSimulatorGPU):
    """The 14-qubit workload: QFT on all qubits, then random layers, full noise after every gate.

    FP64 (the parity form) and FP32 (tensor cores), each recorded once and
    then replayed with its program resident on the device (CUDA events);
    per-pass bandwidth against the algorithmic bytes 2 * 4**14 * s per pass,
    and the FP32 result against the FP64 one on the device."""
    n, layers = 14, args.c2_layers
    qc = pkg.random_layer_circuit(n, layers, args.seed, barrier_after_gate=True, qft=True)
    opts = pkg.noise_options(**NOISE)
    opts['compute_densitymatrix'] = False
    hbm, peak_kind = measured_peaks()
    out = {'workload': 'QFT on 14 qubits + %d random brick layers, noise after every gate, Ensemble Z' % layers,
           'noise': NOISE}
    states, probs = {}, {}
    for precision, s in (('double', 8), ('single', 4)):
        DmSimulatorGPU.DEFAULT_OPTIONS['rotation_error'] = {'rx': [1., 0.], 'ry': [1., 0.], 'rz': [1., 0.]}
        b = DmSimulatorGPU()
        o = copy.deepcopy(opts)
        o['precision'] = precision
        o['coefficients_to_host'] = False
        b._set_options(backend_options=o)
        res = b.record_experiment(qc.to_experiment())
        st = b.recorded_state
        st.replay()
        steps = max(1, min(args.steps, 3))
        ms = time_replays(torch, st, steps)
        by_kernel = pass_kernel_profile(torch, st)
        durs = all_durations(by_kernel)
        mean = float(np.mean(durs))
        gbs = 2 * 4.0 ** n * s / (mean / 1e3) / 1e9
        out['fp64' if precision == 'double' else 'fp32'] = {
            'ms_per_circuit': ms, 'levels': b.last_run_stats['levels'], 'passes': len(durs),
            'pass_kernels': {k: len(v) for k, v in by_kernel.items()}, 'mean_pass_ms': mean,
            'pass_achieved_gbs': gbs, 'pass_frac_of_hbm': gbs / hbm, 'gate_layers_per_s': layers / (ms / 1e3)}
        states[precision] = st
        probs[precision] = np.array(list(res['data']['ensemble_probability'].values()))
        del b
    out['fp32_over_fp64'] = out['fp64']['ms_per_circuit'] / out['fp32']['ms_per_circuit']
    out['accuracy_fp32'] = {
        'max_abs_coeff_err': states['single'].max_abs_diff(states['double']) * 2.0 ** n,
        'prob_l1_err': float(np.abs(probs['single'] - probs['double']).sum()),
        'against': 'the same circuit in FP64 on the GPU'}
    out['peak_gbs'] = hbm
    out['peak_kind'] = peak_kind
    del states
    torch.cuda.empty_cache()
    return out


def run_ours(args):
    import torch
    world, rank, local = dist_setup(args)
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group('nccl')
    pkg = __graft_entry__.build()
    from qiskit_aakash_gb300 import _native as N
    from qiskit_aakash_gb300.dm_simulator import DmSimulatorGPU
    legs = set(args.legs.split(','))
    line = headline_leg(args, pkg, torch, N, DmSimulatorGPU, world, rank) if 'headline' in legs else None
    if rank != 0:
        return None
    if line is None:
        line = {'metric': METRIC, 'legs': sorted(legs), 'note': 'headline leg not run'}
    if 'headline' in legs and not args.no_gate_kinds:
        line['per_gate_kind_fp64'] = per_gate_kind(torch, N)
        line['per_gate_kind_fp32'] = per_gate_kind(torch, N, dtype=N.DM_F32)
    if 'c2' in legs:
        line['qft14_workload'] = c2_leg(args, pkg, torch, N, DmSimulatorGPU)
    if 'batch' in legs and args.batch > 0:
        line['batched_sweep'] = batch_leg(args, pkg, torch, N)
    if 'surrogate' in legs and args.surrogate_train > 0:
        line['noise_surrogate'] = surrogate_leg(args, torch)
    if 'headline' in legs and not args.no_cpu:
        line['cpu_baseline'] = cpu_sample(pkg, args.n, args.seed)
    return line


def _reference_worker(job):
    """One oracle layer sample in a worker process (fresh interpreter)."""
    n_full, seed = job
    return cpu_sample(__graft_entry__.load_package(), n_full, seed)


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def run_reference(args):
    """The reference's own CPU implementation on every host core: each step runs one layer sample
    per core in parallel worker processes and reports their total work over the wall time."""
    import multiprocessing
    from concurrent.futures import ProcessPoolExecutor
    world, rank, _ = dist_setup(args)
    if rank != 0:
        return None
    workers = host_threads()
    for var in ('OMP_NUM_THREADS', 'OPENBLAS_NUM_THREADS', 'MKL_NUM_THREADS'):
        os.environ[var] = '1'           # one thread per worker process: the workers fill the cores
    samples = []
    with ProcessPoolExecutor(max_workers=workers, mp_context=multiprocessing.get_context('spawn')) as pool:
        for i in range(args.warmup + args.steps):
            jobs = [(args.n, args.seed + i * workers + w) for w in range(workers)]
            t0 = time.perf_counter()
            res = list(pool.map(_reference_worker, jobs))
            wall = time.perf_counter() - t0
            # every sample is one layer at the sample size; 1 / value is its full-size time
            full_seconds = sum(1.0 / r['value'] for r in res)
            scale = full_seconds / sum(r['sample_seconds'] for r in res)
            if i >= args.warmup:
                samples.append({'value': workers / (wall * scale), 'wall': wall, 'first': res[0]})
    value = float(np.mean([s['value'] for s in samples]))
    last = samples[-1]
    cb = {'value': value, 'unit': 'gate-layers/s', 'cores': workers, 'kind': last['first']['kind'],
          'sample': ('%d noisy random layers at n=%d, one per worker process on %d host threads in parallel '
                     '(numpy FP64, 1 thread each, %.2f s wall per step), scaled to n=%d like the single-core '
                     'sample: %s' % (workers, CPU_SAMPLE_N, workers, last['wall'], args.n, last['first']['sample'])),
          'sample_seconds': last['wall']}
    return {
        'impl': 'reference',
        'metric': METRIC,
        'value': value,
        'unit': 'gate-layers/s',
        'n_gpus': world,
        'steps': args.steps,
        'warmup': args.warmup,
        'ms_per_step': float(np.mean([s['wall'] for s in samples])) * 1e3,
        'higher_is_better': True,
        'scaling': 'weak',
        'vs_baseline': None,
        'dtype': 'f64',
        'data': 'synthetic: seeded random circuits (numpy default_rng), no dataset',
        'config': {'workload': 'random brick layers n=%d, %d layers, noise after every gate, Ensemble Z'
                               % (args.n, args.layers), 'n_qubits': args.n, 'layers': args.layers},
        'cpu_baseline': cb,
        'e2e': {'value': value, 'unit': 'gate-layers/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0},
    }


def main():
    args = parse()
    line = run_reference(args) if args.impl == 'reference' else run_ours(args)
    if line is not None:
        print(json.dumps(line))


if __name__ == '__main__':
    main()
