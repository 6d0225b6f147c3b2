"""The device-resident Pauli-coefficient state and its operation queue.

``DeviceState`` owns the 4**n coefficient vector in GPU memory (a torch
tensor used only as a buffer) and queues gates / noise / measurement updates
as small Pauli transfer matrices.  Queued operations are executed when a
read-out needs the state (``flush``): the planner groups them into fused
passes and each pass is one launch of the library's pass kernel.  Every
numerical step runs in libdmgb300.so; there is no host fallback.
"""
import ctypes
import time

import numpy as np

from . import _native as N
from .exceptions import BasicAerError
from .program import (TC_AXES, Op, OpTableError, TcPlanError, cx_coefficients, encode_pass, encode_pass_tc,
                      encode_pass_tc_ops, encode_pass_tma,
                      plan_passes)

# Tile sizes of the fused pass: 4**6 FP64 = 32 KB and 4**7 FP32 = 64 KB of
# shared memory per tile; the two lowest qubit axes (16 contiguous
# coefficients, one 128-byte line in FP64) are always resident.
DEFAULT_TILE_AXES = {'double': 6, 'single': 7}
DEFAULT_LOW_AXES = 2
# Queued operations at which the passes they already fix are planned and
# launched (the rest of the queue waits for later operations or a read-out).
STREAM_OPS = 4096

# Copy-out of large states: 32 Mi coefficients (256 MB FP64) per chunk, two
# device and two pinned host buffers per device, host copies in 16 MB slices.
_COPY_CHUNK = 1 << 25
_HOST_SLICE = 1 << 21
_COPY_BUFFERS = {}
_POOL = []
# Host result memory of large copy-outs, up to two blocks per size (a loop
# that keeps the previous result while it runs the next alternates between
# them): page-locked (pinned) allocations, so copy-outs go straight from the
# device into them.  A block is handed out as one numpy array and reused only
# after that array and every view of it have been released.  Blocks are made
# only while the host has room for them.
_RESULT_BLOCKS = {}
_BLOCKS_PER_SIZE = 2


class _ResultBlock:
    """Page-locked host memory of exactly nbytes, mapped into the device's address space
    (dm_host_alloc): the chop kernel writes a result into it directly over the CPU-GPU link."""

    def __init__(self, nbytes, ptr):
        self.nbytes = nbytes
        self.ptr = ptr
        self.dev = N.lib().dm_host_device_pointer(ctypes.c_void_p(ptr))
        self.free = True

    def array(self):
        return np.ctypeslib.as_array((ctypes.c_double * (self.nbytes // 8)).from_address(self.ptr))


def _pinned_host(nbytes):
    """Address of nbytes of mapped page-locked host memory, or None if it cannot be had."""
    ptr = N.lib().dm_host_alloc(ctypes.c_size_t(nbytes))
    return ptr or None


def _free_blocks():
    for blocks in _RESULT_BLOCKS.values():
        for b in blocks:
            try:
                N.lib().dm_host_free(ctypes.c_void_p(b.ptr))
            except Exception:  # noqa: BLE001 - interpreter shutdown: the process frees it anyway
                pass
    _RESULT_BLOCKS.clear()


def _release_block(blk):
    blk.free = True


def _host_bytes_available():
    """Bytes the host can still hand out: MemAvailable, capped by the cgroup's free allowance."""
    avail = 0
    try:
        with open('/proc/meminfo') as f:
            for line in f:
                if line.startswith('MemAvailable:'):
                    avail = int(line.split()[1]) * 1024
    except OSError:
        return 0
    for lim_file, cur_file in (('/sys/fs/cgroup/memory.max', '/sys/fs/cgroup/memory.current'),
                               ('/sys/fs/cgroup/memory/memory.limit_in_bytes',
                                '/sys/fs/cgroup/memory/memory.usage_in_bytes')):
        try:
            with open(lim_file) as f:
                lim = f.read().strip()
            with open(cur_file) as f:
                cur = int(f.read().strip())
        except (OSError, ValueError):
            continue
        if lim != 'max' and int(lim) < (1 << 60):
            avail = min(avail, int(lim) - cur)
    return avail


def _result_array(total):
    """(float64 array of ``total`` values, its result block or None) for one copy-out."""
    import atexit
    import weakref
    nbytes = total * 8
    if not _RESULT_BLOCKS:
        atexit.register(_free_blocks)
    blocks = _RESULT_BLOCKS.setdefault(nbytes, [])
    blk = next((b for b in blocks if b.free), None)
    if blk is None and blocks:
        # a released result may still sit in an unreachable reference cycle (job, future, result)
        import gc
        gc.collect()
        blk = next((b for b in blocks if b.free), None)
    if blk is None:
        buf = None
        if len(blocks) < _BLOCKS_PER_SIZE and _host_bytes_available() >= 2 * nbytes:
            buf = _pinned_host(nbytes)
        if buf is None:          # earlier results still held, or no room: plain memory
            return np.empty(total, dtype=np.float64), None
        blk = _ResultBlock(nbytes, buf)
        blocks.append(blk)
    arr = blk.array()
    blk.free = False
    weakref.finalize(arr, _release_block, blk)
    return arr, blk


def _copy_buffers(device):
    torch = _torch()
    key = (str(device), _COPY_CHUNK)
    if key not in _COPY_BUFFERS:
        dev = [torch.empty(_COPY_CHUNK, dtype=torch.float64, device=device) for _ in range(2)]
        pinned = [torch.empty(_COPY_CHUNK, dtype=torch.float64).pin_memory() for _ in range(2)]
        _COPY_BUFFERS[key] = (dev, pinned)
    return _COPY_BUFFERS[key]


def _host_pool():
    if not _POOL:
        import os
        from concurrent.futures import ThreadPoolExecutor
        _POOL.append(ThreadPoolExecutor(max_workers=max(1, min(16, os.cpu_count() or 1))))
    return _POOL[0]


def _torch():
    import torch
    return torch


class DeviceState:
    """An n-qubit Pauli-coefficient vector on a CUDA device."""

    def __init__(self, n, precision='double', fusion=True, tile_axes=None, low_axes=DEFAULT_LOW_AXES,
                 device=None, rounds=True, tensor_cores=True, tma=True, compose='device'):
        torch = _torch()
        if not torch.cuda.is_available():
            raise BasicAerError('dm_simulator (GB300) needs a CUDA device; none is visible')
        N.lib()
        if not 1 <= n <= N.DM_MAX_QUBITS:
            raise BasicAerError('Number of qubits %d is outside 1..%d' % (n, N.DM_MAX_QUBITS))
        if precision not in ('double', 'single'):
            raise BasicAerError("precision must be 'double' or 'single'")
        self.n = n
        self.precision = precision
        self.dtype = N.DM_F64 if precision == 'double' else N.DM_F32
        self.np_dtype = np.float64 if precision == 'double' else np.float32
        self.device = torch.device(device if device is not None else 'cuda')
        self.torch_dtype = torch.float64 if precision == 'double' else torch.float32
        self.state = torch.empty(4 ** n, dtype=self.torch_dtype, device=self.device)
        self.fusion = fusion
        self.rounds = rounds
        # FP32 passes of 7 resident axes run on the tensor cores (3-way FP16 split)
        self.tensor_cores = bool(tensor_cores) and precision == 'single' and n >= TC_AXES
        self.tma = bool(tma)      # TMA-fed tensor-core passes where a pass fits them
        if compose not in ('device', 'host'):
            raise BasicAerError("compose must be 'device' or 'host'")
        # where the tensor-core rounds' 64x64 matrices are composed in FP64:
        # 'device' (dm_compose_rounds from the ops' coefficients) or 'host' (numpy, FP16 images uploaded)
        self.compose = compose
        self.passes_by_kernel = {'tma': 0, 'tc': 0, 'cuda_cores': 0}
        self.composed_on = {'device': 0, 'host': 0}
        self._images = None       # device round images of the pass in flight (DM_MAX_ROUNDS x 12288 FP16)
        self.status = torch.zeros(1, dtype=torch.int32, device=self.device) if self.tensor_cores else None
        self.kmax = min(tile_axes or DEFAULT_TILE_AXES[precision], N.DM_MAX_TILE_AXES)
        self.low = low_axes
        self.pending = []
        self._stream_at = STREAM_OPS
        self.passes_run = 0
        self.h2d_bytes = 0
        self.d2h_bytes = 0
        self.tape = None          # list of recorded C-ABI calls (see record())
        self.copy_stats = {}      # the last large copy-out: seconds, whether it went into a result block
        self._keep_alive = []

    # -- recording -----------------------------------------------------------
    def record(self):
        """Start recording every C-ABI call (with its argument buffers).

        The calls issued from now on still run; ``replay()`` issues the same
        device work again on the same buffers, with no host planning and no
        host<->device copies.  A circuit's device work does not depend on
        measurement outcomes, so the replay is the whole experiment.
        """
        self.tape = []

    def replay(self, on_call=None):
        for name, args in self.tape:
            if on_call is not None:
                on_call(name, True)
            N.call(name, *args)
            if on_call is not None:
                on_call(name, False)

    def _call(self, name, *args, keep=()):
        if self.tape is not None:
            self.tape.append((name, args))
            self._keep_alive.append((args, keep))
        N.call(name, *args)

    # -- plumbing ------------------------------------------------------------
    @property
    def stream(self):
        return ctypes.c_void_p(_torch().cuda.current_stream(self.device).cuda_stream)

    @property
    def ptr(self):
        return ctypes.c_void_p(self.state.data_ptr())

    def _to_host(self, t):
        self.d2h_bytes += t.numel() * t.element_size()
        return t.cpu().numpy()

    # -- set-up --------------------------------------------------------------
    def init_product(self, vectors, scale):
        v = np.ascontiguousarray(np.asarray(vectors, dtype=np.float64).reshape(self.n, 4))
        self.pending = []
        self._stream_at = STREAM_OPS
        self._call('dm_init_product', self.ptr, self.n, self.dtype,
                   v.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), float(scale), self.stream, keep=(v,))

    def load(self, coeffs):
        a = np.ascontiguousarray(np.asarray(coeffs, dtype=np.float64).reshape(-1))
        if a.size != 4 ** self.n:
            raise BasicAerError('initial densitymatrix is incorrect length: %d != %d' % (a.size, 4 ** self.n))
        self.pending = []
        self.h2d_bytes += a.size * (8 if self.dtype == N.DM_F64 else 4)
        N.call('dm_load_state', self.ptr, self.n, self.dtype,
               a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), self.stream)

    # -- queued operations ---------------------------------------------------
    def map1(self, q, m, tag=None):
        self._queue(Op('map1', (q,), np.asarray(m, dtype=np.float64)))

    def cx(self, ctl, tgt, tsp):
        coef, ideal = cx_coefficients(tsp)
        self._queue(Op('cx', (ctl, tgt), np.array(coef), ideal))

    def diag2(self, qa, qb, d):
        self._queue(Op('diag2', (qa, qb), np.asarray(d, dtype=np.float64)))

    def _queue(self, op):
        self.pending.append(op)
        if self.fusion and len(self.pending) >= self._stream_at:
            self._flush_closed()

    def _flush_closed(self):
        """Launch the passes that the queued ops already fix; later ops cannot change them.

        The device starts on the first passes while the host is still
        producing the rest of the circuit's operations.
        """
        passes, self.pending = plan_passes(self.pending, self.n, self.kmax, self.low, partial=True)
        if passes:
            self._launch(passes)
        self._stream_at = len(self.pending) + STREAM_OPS

    def flush(self):
        """Run every queued operation (fused passes, or one sweep per operation)."""
        self._stream_at = STREAM_OPS
        if not self.pending:
            return
        ops, self.pending = self.pending, []
        if not self.fusion:
            self._run_unfused(ops)
            return
        self._launch(plan_passes(ops, self.n, self.kmax, self.low))
        if self.tensor_cores and int(self.status.item()) != 0:
            raise BasicAerError('a tensor-core pass abandoned a bounded wait (status %d)' % int(self.status.item()))

    def _launch(self, passes):
        if self.tensor_cores:
            self._run_passes_tc(passes)
        else:
            self._run_passes(passes)

    def _encode_tc(self, p):
        """(entry point, descriptor, ops table or None, coefficients or FP16 images) of a tensor-core pass, or None.

        The TMA-fed kernel takes passes of up to 16 rounds whose resident axes
        fit a 5-dimensional tensor map; other passes run on the cp.async-fed
        kernel; a pass with more rounds than a descriptor holds, on neither.
        With compose='device' the round matrices are composed by
        dm_compose_rounds from the ops' FP64 coefficients; a pass with more
        ops than its table holds is composed on the host."""
        kernels = (('tma', 'dm_apply_pass_tma', encode_pass_tma),) if self.tma else ()
        kernels += (('tc', 'dm_apply_pass_tc', encode_pass_tc),)
        for kernel, name, host_encoder in kernels:
            if self.compose == 'device':
                coefs = []
                try:
                    d, bp = encode_pass_tc_ops(p, self.n, coefs, kernel)
                    return name, d, bp, coefs
                except OpTableError:
                    pass
                except TcPlanError:
                    continue
            umats = []
            try:
                return name, host_encoder(p, self.n, umats), None, umats
            except TcPlanError:
                continue
        return None

    def _image_buffer(self):
        if self._images is None:
            torch = _torch()
            self._images = torch.empty(N.DM_MAX_ROUNDS * 3 * 4096, dtype=torch.int16, device=self.device)
        return self._images

    def _run_passes_tc(self, passes):
        """Encode and launch pass by pass: the host plans pass i+1 while the GPU runs pass i.

        Device composition: the ops' coefficients go up (a few KB), one
        dm_compose_rounds launch writes the round images into one device
        buffer, and the pass reads them; the stream orders each pass's
        composition after the previous pass's reads."""
        torch = _torch()
        sp = ctypes.c_void_p(self.status.data_ptr())
        keep = []
        for p in passes:
            enc = self._encode_tc(p)
            if enc is None:
                self._run_passes([p])     # more rounds than a descriptor holds: the CUDA-core pass
                self.passes_by_kernel['cuda_cores'] += 1
                continue
            name, d, bp, data = enc
            self.passes_by_kernel['tma' if name == 'dm_apply_pass_tma' else 'tc'] += 1
            if bp is not None:
                host = np.concatenate(data) if data else np.zeros(1)
                h = torch.from_numpy(host).pin_memory()
                dev = h.to(self.device, non_blocking=True)
                self.h2d_bytes += host.nbytes
                img = self._image_buffer()
                fmt = N.DM_IMAGE_TMA if name == 'dm_apply_pass_tma' else N.DM_IMAGE_TC
                ip, isz = ctypes.c_void_p(img.data_ptr()), ctypes.c_size_t(img.numel())
                self._call('dm_compose_rounds', fmt, ctypes.byref(bp), ctypes.c_void_p(dev.data_ptr()),
                           ctypes.c_size_t(host.size), ip, isz, self.stream, keep=(bp, dev))
                self._call(name, self.ptr, self.n, ctypes.byref(d), ip, isz, sp, self.stream, keep=(d,))
                self.composed_on['device'] += 1
                keep.append((h, dev, d, bp))
                continue
            host = np.concatenate(data).view(np.int16)      # FP16 bit patterns
            h = torch.from_numpy(host).pin_memory()
            dev = h.to(self.device, non_blocking=True)
            self.h2d_bytes += host.nbytes
            self._call(name, self.ptr, self.n, ctypes.byref(d), ctypes.c_void_p(dev.data_ptr()),
                       ctypes.c_size_t(host.size), sp, self.stream, keep=(d, dev))
            self.composed_on['host'] += 1
            keep.append((h, dev, d))
        self.passes_run += len(keep)
        self._keep = keep

    def _run_passes(self, passes):
        torch = _torch()
        mats = []
        width = N.DM_ROUND_AXES[self.dtype] if self.rounds else None
        descs = [encode_pass(p, mats, self.np_dtype, width, self.n) for p in passes]
        host = np.concatenate(mats) if mats else np.zeros(1, dtype=self.np_dtype)
        h = torch.from_numpy(host)
        if self.device.type == 'cuda':
            h = h.pin_memory()
        dev = h.to(self.device, non_blocking=True)
        self.h2d_bytes += host.nbytes
        mp = ctypes.c_void_p(dev.data_ptr())
        for d in descs:
            self._call('dm_apply_pass', self.ptr, self.n, self.dtype, ctypes.byref(d), mp,
                       ctypes.c_size_t(host.size), self.stream, keep=(d, dev))
        self.passes_run += len(descs)
        self._keep = (h, dev)    # keep both alive until the next flush

    def _run_unfused(self, ops):
        for op in ops:
            if op.kind == 'map1':
                m = np.ascontiguousarray(op.data, dtype=np.float64).reshape(16)
                self._call('dm_apply_map1', self.ptr, self.n, self.dtype, op.axes[0],
                           m.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), self.stream, keep=(m,))
            else:
                # pair operations: a pass holding only this operation
                self._run_passes(plan_passes([op], self.n, self.kmax, self.low))

    # -- read-outs (each flushes first) --------------------------------------
    def axis_probs(self, mode, err):
        """Probabilities for per-qubit measurement axes mode[q] in {0 (unmeasured), 1, 2, 3}."""
        self.flush()
        torch = _torch()
        m = sum(1 for x in mode if x)
        out = torch.empty(2 ** m, dtype=torch.float64, device=self.device)
        md = (ctypes.c_int * self.n)(*[int(x) for x in mode])
        self._call('dm_axis_probs', self.ptr, self.n, self.dtype, md, float(err),
                   ctypes.c_void_p(out.data_ptr()), self.stream, keep=(out,))
        self.last_readout = out
        return self._to_host(out)

    def nbasis_probs(self, nvec, err):
        self.flush()
        torch = _torch()
        L = N.lib()
        nbytes = L.dm_nbasis_probs_scratch_bytes(self.n)
        scratch = torch.empty(max(nbytes, 8), dtype=torch.uint8, device=self.device)
        out = torch.empty(2 ** self.n, dtype=torch.float64, device=self.device)
        v = N.f64_array(nvec)
        self._call('dm_nbasis_probs', self.ptr, self.n, self.dtype, v, float(err),
                   ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(scratch.data_ptr()), self.stream,
                   keep=(out, scratch))
        self.last_readout = out
        return self._to_host(out)

    def sample_counts(self, shots, seed):
        """Shot counts (numpy int64, 2**m) drawn on the device from the last probability read-out."""
        torch = _torch()
        probs = self.last_readout
        m = int(probs.numel()).bit_length() - 1
        L = N.lib()
        scratch = torch.empty(max(L.dm_sample_counts_scratch_bytes(m), 8), dtype=torch.uint8, device=self.device)
        counts = torch.empty(2 ** m, dtype=torch.int64, device=self.device)
        self._call('dm_sample_counts', ctypes.c_void_p(probs.data_ptr()), m, ctypes.c_int64(int(shots)),
                   ctypes.c_uint64(int(seed) & (2 ** 64 - 1)), ctypes.c_void_p(counts.data_ptr()),
                   ctypes.c_void_p(scratch.data_ptr()), self.stream, keep=(counts, scratch))
        out = self._to_host(counts)
        if shots > 0 and int(out.sum()) != int(shots):
            raise BasicAerError('cannot draw counts: no outcome has a positive probability')
        return out

    def gather(self, indices):
        self.flush()
        torch = _torch()
        out = []
        idx = [int(i) for i in indices]
        for s in range(0, len(idx), 64):
            chunk = idx[s:s + 64]
            o = torch.empty(len(chunk), dtype=torch.float64, device=self.device)
            arr = (ctypes.c_int64 * len(chunk))(*chunk)
            self._call('dm_gather', self.ptr, self.n, self.dtype, arr, len(chunk),
                       ctypes.c_void_p(o.data_ptr()), self.stream, keep=(o,))
            out.append(self._to_host(o))
        return np.concatenate(out)

    def coefficients(self, chop_threshold):
        """FP64 copy of the coefficients with |a| < chop_threshold set to 0.

        Large states stream out in chunks: the chop kernel fills one of two
        device buffers and an async copy moves it into the page-locked
        result block.  When that block is still held by an earlier result,
        the chunks go to one of two pinned staging buffers instead and host
        threads copy the previous chunk into a fresh array while the GPU
        works on the next one.
        """
        self.flush()
        torch = _torch()
        total = 4 ** self.n
        if total <= _COPY_CHUNK:
            out = torch.empty(total, dtype=torch.float64, device=self.device)
            N.call('dm_chop_copy', self.ptr, self.n, self.dtype, float(chop_threshold),
                   ctypes.c_void_p(out.data_ptr()), self.stream)
            return self._to_host(out)
        t0 = time.perf_counter()
        result, blk = _result_array(total)
        self.copy_stats = {'result_block': blk is not None, 'block_seconds': time.perf_counter() - t0}
        stream = torch.cuda.current_stream(self.device)
        if blk is not None:
            # mapped page-locked result block: the chop kernel writes it directly, one pass
            N.call('dm_chop_copy', self.ptr, self.n, self.dtype, float(chop_threshold), ctypes.c_void_p(blk.dev),
                   self.stream)
            stream.synchronize()
            self.d2h_bytes += total * 8
            self.copy_stats['seconds'] = time.perf_counter() - t0
            return result
        dev, pinned = _copy_buffers(self.device)
        events = [None, None]
        pending = None
        pool = _host_pool()

        def drain(item):
            b, off, cnt = item
            events[b].synchronize()
            src = pinned[b].numpy()
            parts = [(s0, min(cnt, s0 + _HOST_SLICE)) for s0 in range(0, cnt, _HOST_SLICE)]
            list(pool.map(lambda r: np.copyto(result[off + r[0]:off + r[1]], src[r[0]:r[1]]), parts))

        for i, off in enumerate(range(0, total, _COPY_CHUNK)):
            b = i % 2
            cnt = min(_COPY_CHUNK, total - off)
            N.call('dm_chop_copy_range', self.ptr, self.n, self.dtype, ctypes.c_int64(off), ctypes.c_int64(cnt),
                   float(chop_threshold), ctypes.c_void_p(dev[b].data_ptr()), self.stream)
            pinned[b][:cnt].copy_(dev[b][:cnt], non_blocking=True)
            events[b] = torch.cuda.Event()
            events[b].record(stream)
            if pending is not None:
                drain(pending)      # the other buffer pair: its host copy overlaps this chunk's GPU work
            pending = (b, off, cnt)
        drain(pending)
        self.d2h_bytes += total * 8
        self.copy_stats['seconds'] = time.perf_counter() - t0
        return result

    def raw_coefficients(self):
        """FP64 copy of the unchopped coefficients."""
        return self.coefficients(0.0)

    def density_matrix(self):
        """2**n x 2**n complex matrix in the computational basis."""
        self.flush()
        torch = _torch()
        L = N.lib()
        scratch = torch.empty(L.dm_pauli_to_matrix_scratch_bytes(self.n), dtype=torch.uint8, device=self.device)
        out = torch.empty((2 ** self.n, 2 ** self.n), dtype=torch.complex128, device=self.device)
        N.call('dm_pauli_to_matrix', self.ptr, self.n, self.dtype, ctypes.c_void_p(out.data_ptr()),
               ctypes.c_void_p(scratch.data_ptr()), self.stream)
        return self._to_host(out)

    def overlap(self, other_coeffs):
        """2**n * <a, b> against a host coefficient vector."""
        self.flush()
        torch = _torch()
        b = torch.from_numpy(np.asarray(other_coeffs, dtype=self.np_dtype).reshape(-1)).to(self.device)
        self.h2d_bytes += b.numel() * b.element_size()
        L = N.lib()
        scratch = torch.empty(L.dm_overlap_scratch_bytes(self.n), dtype=torch.uint8, device=self.device)
        out = torch.empty(1, dtype=torch.float64, device=self.device)
        N.call('dm_overlap', self.ptr, ctypes.c_void_p(b.data_ptr()), self.n, self.dtype,
               ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(scratch.data_ptr()), self.stream)
        return float(self._to_host(out)[0])

    def max_abs_diff(self, other):
        """max |a_s - b_s| against another device state of the same size (FP64, on the device)."""
        self.flush()
        other.flush()
        if other.n != self.n:
            raise BasicAerError('states of %d and %d qubits cannot be compared' % (self.n, other.n))
        out = _torch().empty(1, dtype=_torch().float64, device=self.device)
        N.call('dm_max_abs_diff', self.ptr, self.dtype, other.ptr, other.dtype, self.n,
               ctypes.c_void_p(out.data_ptr()), self.stream)
        return float(self._to_host(out)[0])

    def trace_error(self):
        """|2**n a_0 - 1| of the current state, a_0 read from the device in FP64 (not recorded)."""
        self.flush()
        o = _torch().empty(1, dtype=_torch().float64, device=self.device)
        idx = (ctypes.c_int64 * 1)(0)
        N.call('dm_gather', self.ptr, self.n, self.dtype, idx, 1, ctypes.c_void_p(o.data_ptr()), self.stream)
        return abs(float(self._to_host(o)[0]) * 2.0 ** self.n - 1.0)

    def synchronize(self):
        _torch().cuda.synchronize(self.device)
