"""The C-ABI library builds for sm_103a, loads, and exports what include/dm_gb300.h declares.

No kernel runs here: only calls that the library rejects on the host
(invalid arguments) are made.
"""
import ctypes
import os
import re
import subprocess

import pytest

from qiskit_aakash_gb300 import _native as N

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), 'include', 'dm_gb300.h')


@pytest.fixture(scope='module')
def lib():
    N.build()
    return N.lib()


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r'/\*.*?\*/', '', text, flags=re.S)
    return sorted(set(re.findall(r'\b(dm_[a-z0-9_]+)\s*\(', text)))


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 18
    for name in names:
        assert hasattr(lib, name), name
        assert name in N.SIGNATURES, name


def test_struct_layout_matches_header(tmp_path):
    """ctypes mirrors of dm_op / dm_pass have the C compiler's sizes and offsets."""
    src = tmp_path / 'layout.c'
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "dm_gb300.h"\n'
        'int main(void) { printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n", '
        'sizeof(dm_op), sizeof(dm_pass), '
        'offsetof(dm_pass, nops), offsetof(dm_pass, nrounds), offsetof(dm_pass, round_axes), '
        'offsetof(dm_pass, round_end), offsetof(dm_pass, ops), sizeof(dm_tc_pass), '
        'sizeof(dm_batch_pass), offsetof(dm_batch_pass, axes), offsetof(dm_batch_pass, round_axes), '
        'offsetof(dm_batch_pass, round_end), offsetof(dm_batch_pass, ops), sizeof(dm_batch_instance), '
        'offsetof(dm_batch_instance, meas_err)); printf("%zu %zu %zu\\n", sizeof(dm_mlp_gemm), '
        'offsetof(dm_mlp_gemm, A), offsetof(dm_mlp_gemm, t_ms)); printf("%zu %zu %zu %zu\\n", sizeof(dm_recipe), '
        'offsetof(dm_recipe, angle), sizeof(dm_param_program), offsetof(dm_param_program, consts)); '
        'printf("%zu %zu\\n", sizeof(dm_batch_tc_pass), offsetof(dm_batch_tc_pass, tables)); return 0; }\n')
    exe = tmp_path / 'layout'
    subprocess.run(['gcc', '-I', os.path.dirname(HEADER), str(src), '-o', str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    want = [ctypes.sizeof(N.DmOp), ctypes.sizeof(N.DmPass), N.DmPass.nops.offset, N.DmPass.nrounds.offset,
            N.DmPass.round_axes.offset, N.DmPass.round_end.offset, N.DmPass.ops.offset, ctypes.sizeof(N.DmTcPass),
            ctypes.sizeof(N.DmBatchPass), N.DmBatchPass.axes.offset, N.DmBatchPass.round_axes.offset,
            N.DmBatchPass.round_end.offset, N.DmBatchPass.ops.offset, ctypes.sizeof(N.DmBatchInstance),
            N.DmBatchInstance.meas_err.offset, ctypes.sizeof(N.DmMlpGemm), N.DmMlpGemm.A.offset,
            N.DmMlpGemm.t_ms.offset, ctypes.sizeof(N.DmRecipe), N.DmRecipe.angle.offset,
            ctypes.sizeof(N.DmParamProgram), N.DmParamProgram.consts.offset,
            ctypes.sizeof(N.DmBatchTcPass), N.DmBatchTcPass.tables.offset]
    assert got == want
    text = open(HEADER).read()
    assert int(re.search(r'#define DM_MAX_TILE_AXES (\d+)', text).group(1)) == N.DM_MAX_TILE_AXES
    assert int(re.search(r'#define DM_MAX_PASS_OPS (\d+)', text).group(1)) == N.DM_MAX_PASS_OPS
    assert int(re.search(r'#define DM_MAX_QUBITS (\d+)', text).group(1)) == N.DM_MAX_QUBITS
    assert int(re.search(r'#define DM_MAX_ROUNDS (\d+)', text).group(1)) == N.DM_MAX_ROUNDS


def test_error_strings_and_version(lib):
    assert lib.dm_error_string(0) == b'ok'
    assert b'invalid' in lib.dm_error_string(-1)
    assert lib.dm_version().startswith(b'dm_gb300')


def test_invalid_arguments_are_rejected_on_host(lib):
    m = N.f64_array([0.0] * 16)
    # null state, bad qubit, bad dtype, bad n: all rejected before any CUDA call
    assert lib.dm_apply_map1(None, 4, 0, 0, m, None) == N.DM_ERR_ARG
    assert lib.dm_apply_map1(ctypes.c_void_p(16), 4, 0, 7, m, None) == N.DM_ERR_ARG
    assert lib.dm_apply_map1(ctypes.c_void_p(16), 4, 5, 0, m, None) == N.DM_ERR_ARG
    assert lib.dm_apply_map1(ctypes.c_void_p(16), 0, 0, 0, m, None) == N.DM_ERR_ARG
    assert lib.dm_apply_map1(ctypes.c_void_p(16), 18, 0, 0, m, None) == N.DM_ERR_ARG
    tsp = N.f64_array([1.0, 0.0])
    assert lib.dm_apply_cx(ctypes.c_void_p(16), 4, 0, 2, 2, tsp, None) == N.DM_ERR_ARG
    assert lib.dm_apply_cx(ctypes.c_void_p(16), 1, 0, 0, 1, tsp, None) == N.DM_ERR_ARG
    idx = (ctypes.c_int64 * 1)(4 ** 4)
    assert lib.dm_gather(ctypes.c_void_p(16), 4, 0, idx, 1, ctypes.c_void_p(16), None) == N.DM_ERR_ARG
    mode = (ctypes.c_int * 4)(0, 4, 0, 0)
    assert lib.dm_axis_probs(ctypes.c_void_p(16), 4, 0, mode, 1.0, ctypes.c_void_p(16), None) == N.DM_ERR_ARG


def test_malformed_pass_is_rejected_on_host(lib):
    p = N.DmPass()
    p.k = 3
    p.axes[0], p.axes[1], p.axes[2] = 3, 4, 2          # not strictly decreasing
    p.nops = 0
    rc = lib.dm_apply_pass(ctypes.c_void_p(16), 5, 0, ctypes.byref(p), ctypes.c_void_p(16), 16, None)
    assert rc == N.DM_ERR_PROGRAM
    p.axes[0], p.axes[1], p.axes[2] = 4, 3, 2
    p.nops = 1
    p.ops[0].kind = N.DM_OP_MAP1
    p.ops[0].a = 0
    p.ops[0].moff = 8                                  # 8 + 16 > 16 coefficients
    rc = lib.dm_apply_pass(ctypes.c_void_p(16), 5, 0, ctypes.byref(p), ctypes.c_void_p(16), 16, None)
    assert rc == N.DM_ERR_PROGRAM
    p.ops[0].moff = 0
    p.ops[0].a = 3                                     # local axis beyond k
    rc = lib.dm_apply_pass(ctypes.c_void_p(16), 5, 0, ctypes.byref(p), ctypes.c_void_p(16), 16, None)
    assert rc == N.DM_ERR_PROGRAM
    p.k = 8                                            # beyond DM_MAX_TILE_AXES
    rc = lib.dm_apply_pass(ctypes.c_void_p(16), 9, 0, ctypes.byref(p), ctypes.c_void_p(16), 16, None)
    assert rc == N.DM_ERR_PROGRAM


def test_malformed_tma_pass_is_rejected_on_host(lib):
    """dm_apply_pass_tma checks its descriptor before any CUDA call (here there is no GPU)."""
    import numpy as np
    from qiskit_aakash_gb300 import program as P
    n = 10
    ops = [P.Op('map1', (q,), np.eye(4)) for q in range(n - 2)]     # off the two lowest-stride qubits
    passes = P.plan_passes(ops, n, 7, 2)
    umats = []
    good = P.encode_pass_tma(passes[0], n, umats)
    count = sum(m.size for m in umats)
    dev = ctypes.c_void_p(1 << 20)

    def run(d, cnt=count, state=dev):
        return lib.dm_apply_pass_tma(state, n, ctypes.byref(d), dev, ctypes.c_size_t(cnt), dev, None)

    def copy():
        return N.DmTcPass.from_buffer_copy(bytes(good))

    assert run(copy(), state=ctypes.c_void_p(None)) == N.DM_ERR_ARG
    assert run(copy(), state=ctypes.c_void_p((1 << 20) + 4)) == N.DM_ERR_ARG     # unaligned state
    assert run(copy(), cnt=count - 8) == N.DM_ERR_PROGRAM                         # images beyond the buffer
    bad = copy()
    bad.nrounds = P.TMA_MAX_ROUNDS + 1
    assert run(bad) == N.DM_ERR_PROGRAM
    bad = copy()
    bad.axes[0] = n - 2                                                           # lowest axis not resident
    assert run(bad) == N.DM_ERR_PROGRAM
    bad = copy()
    bad.natrow[0] = 3                                                             # not a power of two
    assert run(bad) == N.DM_ERR_PROGRAM
    bad = copy()
    bad.rounds[bad.nrounds - 1].kc[0] = 1 << 14                                   # beyond the natural tile
    assert run(bad) == N.DM_ERR_PROGRAM
    bad = copy()
    bad.rounds[0].umoff = 4                                                       # images not 16-byte aligned
    assert run(bad) == N.DM_ERR_PROGRAM
    # seven isolated resident qubits need seven tensor-map dimensions
    bad = copy()
    for r, q in enumerate([16, 14, 12, 10, 8, 6, 4]):
        bad.axes[r] = q
    assert lib.dm_apply_pass_tma(dev, 17, ctypes.byref(bad), dev, ctypes.c_size_t(count), dev, None) \
        == N.DM_ERR_PROGRAM


def test_malformed_tensor_core_batch_tables_are_rejected_on_host(lib):
    """dm_batch_run_tc / dm_batch_run_params_tc validate every table before any CUDA call."""
    from qiskit_aakash_gb300 import batch as B
    from qiskit_aakash_gb300 import template as TP
    from qiskit_aakash_gb300.circuit import noise_options, random_layer_circuit
    specs = B.sweep_specs(2, seed=4, n_range=(8, 8), depth_range=(2, 3))
    t = B.BatchTables(specs, 'single', kmax={8: B.TC}, workers=1)
    tc = t.tc
    dev = ctypes.c_void_p(1 << 20)                     # never dereferenced: validation fails first

    def run(insts, passes):
        return lib.dm_batch_run_tc(dev, t.states_count, dev, t.probs_count, dev, tc.mats.size, insts, dev,
                                   tc.ninst, passes, dev, tc.npasses, dev, dev, 1 << 40, dev, None)

    def fresh():
        return (N.DmBatchTcPass * tc.npasses).from_buffer_copy(bytes(tc.passes))

    bad = fresh()
    bad[0].ops.round_axes[0][1] = bad[0].ops.round_axes[0][0]          # a digit twice
    assert run(tc.insts, bad) == N.DM_ERR_PROGRAM
    bad = fresh()
    bad[0].ops.ops[0].moff = 10 ** 6                                    # beyond the coefficient block
    assert run(tc.insts, bad) == N.DM_ERR_PROGRAM
    bad = fresh()
    bad[0].tables.natrow[0] = 0
    assert run(tc.insts, bad) == N.DM_ERR_PROGRAM
    insts = (N.DmBatchInstance * tc.ninst).from_buffer_copy(bytes(tc.insts))
    insts[0].n = 13
    assert run(insts, tc.passes) == N.DM_ERR_RANGE
    insts = (N.DmBatchInstance * tc.ninst).from_buffer_copy(bytes(tc.insts))
    insts[0].state_off = t.states_count
    assert run(insts, tc.passes) == N.DM_ERR_ARG

    qc = random_layer_circuit(9, 2, seed=1)
    opts = noise_options(depolarisation=1e-3, decoherence=0.99, decay=0.99, rotation_sigma=1e-2)
    prog = TP.TemplateProgram(qc.to_experiment(), opts, 'single')
    assert prog.tc
    host = prog.host_struct()

    def run_params(passes):
        return lib.dm_batch_run_params_tc(ctypes.byref(host), ctypes.byref(host), passes, dev, dev, 16, 1, dev,
                                          4 ** 9, dev, 2 ** 9, dev, dev, 1 << 40, dev, None)

    bad = (N.DmBatchTcPass * prog.npasses).from_buffer_copy(bytes(prog.passes))
    bad[0].ops.ops[0].moff = 16                                         # op 0 must read slot 0
    assert run_params(bad) == N.DM_ERR_PROGRAM
    bad = (N.DmBatchTcPass * prog.npasses).from_buffer_copy(bytes(prog.passes))
    bad[0].ops.ops[0].kind = N.DM_OP_CX if bad[0].ops.ops[0].kind == N.DM_OP_MAP1 else N.DM_OP_MAP1
    assert run_params(bad) == N.DM_ERR_PROGRAM                          # slot recipe no longer fits the op


def test_malformed_compose_table_is_rejected_on_host(lib):
    """dm_compose_rounds checks its op table before any CUDA call (here there is no GPU)."""
    import numpy as np
    from qiskit_aakash_gb300 import program as P
    n = 9
    rng = np.random.default_rng(3)
    ops = [P.Op('map1', (q,), rng.normal(size=(4, 4))) for q in range(n)]
    ops += [P.Op('cx', (n - 1, n - 2), (1.0, 0.0, 1.0, 0.0, 0.0), True),
            P.Op('map2', (n - 3, n - 4), rng.normal(size=(16, 16)))]
    coefs = []
    _, good = P.encode_pass_tc_ops(P.plan_passes(ops, n, 7, 2)[0], n, coefs, 'tc')
    count = sum(c.size for c in coefs)
    halves = good.nrounds * P.TC_IMAGE_HALVES
    dev = ctypes.c_void_p(1 << 20)

    def run(bp, fmt=N.DM_IMAGE_TC, cnt=count, images=dev, nimg=halves):
        return lib.dm_compose_rounds(fmt, ctypes.byref(bp), dev, ctypes.c_size_t(cnt), images,
                                     ctypes.c_size_t(nimg), None)

    def copy():
        return N.DmBatchPass.from_buffer_copy(bytes(good))

    assert run(copy(), fmt=7) == N.DM_ERR_ARG                                    # unknown image format
    assert run(copy(), images=ctypes.c_void_p(None)) == N.DM_ERR_ARG
    assert run(copy(), images=ctypes.c_void_p((1 << 20) + 8)) == N.DM_ERR_ARG    # images not 16-byte aligned
    assert run(copy(), nimg=halves - 1) == N.DM_ERR_ARG                          # images beyond the buffer
    assert run(copy(), nimg=good.nrounds * P.TMA_IMAGE_HALVES) == N.DM_ERR_ARG  # 12288 values per round
    assert run(copy(), cnt=count - 1) == N.DM_ERR_PROGRAM                        # coefficients beyond mats
    bad = copy()
    bad.nrounds = 0
    assert run(bad) == N.DM_ERR_PROGRAM
    bad = copy()
    bad.round_end[bad.nrounds - 1] -= 1                                          # an op left outside every round
    assert run(bad) == N.DM_ERR_PROGRAM
    bad = copy()
    bad.ops[0].kind = 9
    assert run(bad) == N.DM_ERR_PROGRAM
    bad = copy()
    bad.ops[0].flags |= 3 << 8                                                   # digit position 3 of a 3-digit round
    assert run(bad) == N.DM_ERR_PROGRAM
    bad = copy()
    bad.round_axes[0][1] = bad.round_axes[0][0]                                  # repeated round axis
    assert run(bad) == N.DM_ERR_PROGRAM
    pair = next(i for i in range(good.nops) if good.ops[i].kind != N.DM_OP_MAP1)
    bad = copy()
    bad.ops[pair].flags = (bad.ops[pair].flags & ~(3 << 12)) | (((bad.ops[pair].flags >> 8) & 3) << 12)
    assert run(bad) == N.DM_ERR_PROGRAM                                          # both axes on one digit


def test_direct_last_round_tables_are_checked_on_host(lib):
    """dm_apply_pass_tc checks a direct last round's tables (linear offsets of 14 distinct tile bits,
    rows 0-3 on tile bits 0-3) before any CUDA call (here there is no GPU)."""
    import numpy as np
    from qiskit_aakash_gb300 import program as P
    from test_planner import random_ops
    n = 10
    ops = [op for op in random_ops(np.random.default_rng(21), n, 120) if all(q < n - 2 for q in op.axes)]
    good = None
    for p in P.plan_passes(ops, n, 7, 2):
        d, _ = P.encode_pass_tc_ops(p, n, [], 'tc')
        if d.direct_last:
            good = d
            break
    assert good is not None
    dev = ctypes.c_void_p(1 << 20)

    def run(d):
        return lib.dm_apply_pass_tc(dev, n, ctypes.byref(d), dev, ctypes.c_size_t(1 << 20), dev, None)

    def copy():
        return N.DmTcPass.from_buffer_copy(bytes(good))

    last = good.nrounds - 1
    assert sorted(good.rounds[last].rowc[:4]) == [1, 2, 4, 8]
    bad = copy()
    bad.direct_last = 2
    assert run(bad) == N.DM_ERR_PROGRAM
    bad = copy()
    bad.rounds[last].rowc[0], bad.rounds[last].rowc[4] = bad.rounds[last].rowc[4], bad.rounds[last].rowc[0]
    assert run(bad) == N.DM_ERR_PROGRAM                                  # rows 0-3 not the contiguous bits
    bad = copy()
    bad.rounds[last].kc[0] = bad.rounds[last].kc[1]                      # a tile bit twice
    assert run(bad) == N.DM_ERR_PROGRAM
    bad = copy()
    bad.rounds[last].kc[0] = 3                                           # not a power of two
    assert run(bad) == N.DM_ERR_PROGRAM


def test_tile_copy_probe_rejects_bad_tiles_on_host(lib):
    """dm_tile_copy_probe checks its arguments before any CUDA call (here there is no GPU)."""
    dev = ctypes.c_void_p(1 << 20)

    def run(axes, n=10, state=dev):
        a = (ctypes.c_int32 * 7)(*axes)
        return lib.dm_tile_copy_probe(state, n, a, None)

    good = [9, 8, 6, 5, 3, 2, 0]
    assert run(good, state=ctypes.c_void_p(None)) == N.DM_ERR_ARG
    assert run(good, state=ctypes.c_void_p((1 << 20) + 4)) == N.DM_ERR_ARG      # unaligned state
    assert run(good, n=6) == N.DM_ERR_ARG                                       # fewer than 7 qubits
    assert run([8, 7, 6, 5, 3, 2, 0]) == N.DM_ERR_ARG                           # lowest qubit not resident
    assert run([9, 8, 8, 5, 3, 2, 0]) == N.DM_ERR_ARG                           # not strictly decreasing
    assert run([9, 8, 6, 5, 3, 2, -1]) == N.DM_ERR_ARG                          # qubit out of range
