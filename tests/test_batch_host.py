"""Host side of the batched noise sweep (no GPU).

The instance table, shared pass plans and per-instance coefficient blocks
are replayed with numpy, exactly as the batch kernel reads them (local axis
digits, coefficient offsets, CX flags), and the resulting Z ensemble
probabilities must equal the oracle's for every instance.
"""
import numpy as np
import pytest

from oracle import dm_oracle as O
from qiskit_aakash_gb300 import _native as N
from qiskit_aakash_gb300 import batch as B

from test_planner import apply_map1, apply_pair, cx_matrix


def emulate_instance(T, i):
    I = T.instance(i)
    n = I.n
    st = np.zeros(4 ** n)
    # |0...0>: 2**-n on every string of I and Z
    for m in range(2 ** n):
        idx = sum((3 if (m >> (n - 1 - q)) & 1 else 0) * 4 ** (n - 1 - q) for q in range(n))
        st[idx] = 2.0 ** -n
    part = T.index[i][0]
    mats = part.mats[I.mats_off:I.mats_off + I.mats_len].astype(np.float64)
    for p in range(I.pass_begin, I.pass_begin + I.npasses):
        bp = part.passes[p]
        if isinstance(bp, N.DmBatchTcPass):
            bp = bp.ops
        axes = [bp.axes[r] for r in range(bp.k)]
        assert axes[0] == n - 1 and axes == sorted(axes, reverse=True)
        o = 0
        for r in range(bp.nrounds):
            rax = [bp.round_axes[r][j] for j in range(4)]
            for o in range(o, bp.round_end[r]):
                d = bp.ops[o]
                da, db = (d.flags >> 8) & 3, (d.flags >> 12) & 3
                assert rax[da] == d.a
                qa = axes[d.a]
                if d.kind == N.DM_OP_MAP1:
                    st = apply_map1(st, n, qa, mats[d.moff:d.moff + 16].reshape(4, 4))
                    continue
                assert rax[db] == d.b
                qb = axes[d.b]
                if d.kind == N.DM_OP_CX:
                    st = apply_pair(st, n, qa, qb, cx_matrix(mats[d.moff:d.moff + 5], d.flags & N.DM_CX_IDEAL))
                elif d.kind == N.DM_OP_DIAG2:
                    st = apply_pair(st, n, qa, qb, np.diag(mats[d.moff:d.moff + 16]))
                else:
                    raise AssertionError(d.kind)
            o = bp.round_end[r]
        assert o == bp.nops
    return O.ensemble_probabilities(st, n, 'Z', None, I.meas_err)


def oracle_probs(spec):
    exp, opts = B.instance_experiment(spec)
    res = O.OracleDmSimulator(dict(opts, compute_densitymatrix=False)).run_experiment(exp)
    p = res['data']['ensemble_probability']
    return np.array([p[k] for k in O.bitstring_keys(spec['n'])])


@pytest.mark.parametrize('precision', ['double', 'single'])
def test_batch_tables_replay_equals_oracle(precision):
    specs = B.sweep_specs(12, seed=3, n_range=(3, 6), depth_range=(2, 9))
    T = B.BatchTables(specs, precision)
    tol = 1e-12 if precision == 'double' else 1e-6
    for i, spec in enumerate(specs):
        got = emulate_instance(T, i)
        assert np.max(np.abs(got - oracle_probs(spec))) < tol, (i, spec)


def test_batch_layout_is_largest_first_and_packed():
    specs = B.sweep_specs(30, seed=5, n_range=(3, 7), depth_range=(1, 6))
    T = B.BatchTables(specs, 'single', kmax={7: 5, 6: 4})
    work = [4 ** T.insts[s].n for s in range(T.ninst)]
    sizes = [4 ** specs[i]['n'] * specs[i]['depth'] for i in sorted(range(30), key=lambda i: T.index[i])]
    assert sizes == sorted(sizes, reverse=True)
    s_off = p_off = m_off = 0
    for s in range(T.ninst):
        I = T.insts[s]
        assert (I.state_off, I.prob_off, I.mats_off) == (s_off, p_off, m_off)
        s_off += 4 ** I.n
        p_off += 2 ** I.n
        m_off += I.mats_len
        for p in range(I.pass_begin, I.pass_begin + I.npasses):
            assert T.passes[p].k <= {7: 5, 6: 4}.get(I.n, 7)
    assert (s_off, p_off, m_off) == (T.states_count, T.probs_count, T.mats.size) and sum(work) == s_off


def test_plans_are_shared_by_instances_of_one_structure():
    base = B.sweep_specs(1, seed=9, n_range=(5, 5), depth_range=(6, 6))[0]
    specs = [dict(base, seed=base['seed'] + j, depolarisation=d, decoherence=1 - d, decay=1 - 2 * d)
             for j, d in enumerate((1e-4, 1e-3, 1e-2))]
    T = B.BatchTables(specs, 'double')
    assert T.nplans == 1 and T.npasses == T.insts[0].npasses
    assert len({T.insts[s].pass_begin for s in range(3)}) == 1
    blocks = [T.mats[T.insts[s].mats_off:T.insts[s].mats_off + T.insts[s].mats_len] for s in range(3)]
    assert not np.array_equal(blocks[0], blocks[1])
    for i, spec in enumerate(specs):
        assert np.max(np.abs(emulate_instance(T, i) - oracle_probs(spec))) < 1e-12


def test_batch_rejects_unsupported_instances():
    with pytest.raises(Exception):
        B.BatchTables([dict(B.sweep_specs(1, seed=1)[0], n=13)])
    with pytest.raises(Exception):
        B.BatchTables([dict(B.sweep_specs(1, seed=1)[0], n=2)], 'single')
    with pytest.raises(Exception):
        B.BatchTables(B.sweep_specs(2, seed=1, n_range=(6, 6)), 'single', kmax={6: 3})


def test_sweep_specs_ranges():
    specs = B.sweep_specs(500, seed=0)
    ns = [s['n'] for s in specs]
    ds = [s['depth'] for s in specs]
    assert min(ns) == 6 and max(ns) == 12 and min(ds) >= 10 and max(ds) <= 50
    for s in specs:
        assert 1e-4 <= s['depolarisation'] <= 1e-2
        assert 1e-4 <= 1 - s['decoherence'] <= 1e-2 and 1e-4 <= 1 - s['decay'] <= 1e-2


def test_worker_processes_compile_the_same_tables():
    specs = B.sweep_specs(24, seed=11, n_range=(3, 6), depth_range=(2, 6))
    a = B.compile_sweep(specs, ['single', 'double'], workers=1)
    b = B.compile_sweep(specs, ['single', 'double'], workers=3)
    for prec in ('single', 'double'):
        assert bytes(a[prec].insts) == bytes(b[prec].insts)
        assert bytes(a[prec].passes) == bytes(b[prec].passes)
        assert np.array_equal(a[prec].mats, b[prec].mats)


def test_tensor_core_batch_tables_replay_equals_oracle():
    """Instances planned for the tensor cores (7 resident axes, rounds in their layouts' digit order)."""
    specs = B.sweep_specs(5, seed=11, n_range=(7, 9), depth_range=(2, 5))
    T = B.BatchTables(specs, 'single', kmax={7: B.TC, 8: B.TC, 9: B.TC})
    assert T.tc.ninst == len(specs) and T.ninst == 0
    for i, spec in enumerate(specs):
        np.testing.assert_allclose(emulate_instance(T, i), oracle_probs(spec), atol=2e-6)


def _op_from_table(d, rax, mats):
    from qiskit_aakash_gb300 import program as P
    da, db = (d.flags >> 8) & 3, (d.flags >> 12) & 3
    if d.kind == N.DM_OP_MAP1:
        return P.Op('map1', (rax[da],), mats[d.moff:d.moff + 16].reshape(4, 4))
    if d.kind == N.DM_OP_CX:
        return P.Op('cx', (rax[da], rax[db]), mats[d.moff:d.moff + 5], bool(d.flags & N.DM_CX_IDEAL))
    return P.Op('diag2', (rax[da], rax[db]), mats[d.moff:d.moff + 16])


def test_tensor_core_round_matrices_from_the_table_equal_the_single_state_plan():
    """The device composes round r's U from the table (ops on the 64 unit vectors, K digits in the
    round's order); that U equals the one the single-state tensor-core path composes on the host."""
    from qiskit_aakash_gb300 import program as P
    spec = B.sweep_specs(1, seed=5, n_range=(9, 9), depth_range=(6, 6))[0]
    rec = B.compile_experiment(*B.instance_experiment(spec))
    plan = B._TcPlan(rec.ops, spec['n'])
    mats = plan.coefficients(rec.ops, np.float64)
    host_passes = P.plan_passes(rec.ops, spec['n'], P.TC_AXES, 2)
    assert len(host_passes) == len(plan.passes)
    for hp, bp in zip(host_passes, plan.passes):
        _, layouts, want = P.plan_tc_pass(hp, spec['n'])
        o = bp.ops
        assert o.nrounds == len(want)
        begin = 0
        for r in range(o.nrounds):
            rax = [o.round_axes[r][j] for j in range(3)]
            assert rax == list(layouts[r].digits) == [bp.tables.rounds[r].digits[j] for j in range(3)]
            U = np.eye(64)
            for idx in range(begin, o.round_end[r]):
                U = P.op_matrix64(_op_from_table(o.ops[idx], rax, mats), rax) @ U
            np.testing.assert_allclose(U, want[r], atol=1e-14)
            begin = o.round_end[r]


def test_mixed_batch_packs_both_parts():
    specs = B.sweep_specs(12, seed=3, n_range=(6, 8), depth_range=(2, 4))
    T = B.BatchTables(specs, 'single', kmax={7: B.TC, 8: B.TC})
    n_small = sum(1 for s in specs if s['n'] == 6)
    assert T.ninst == n_small and T.tc.ninst == len(specs) - n_small
    seen_states, seen_probs = [], []
    for i, spec in enumerate(specs):
        I = T.instance(i)
        assert I.n == spec['n']
        seen_states.append((I.state_off, 4 ** I.n))
        seen_probs.append((I.prob_off, 2 ** I.n))
        part = T.index[i][0]
        assert (part is T.tc) == (spec['n'] >= 7)
        assert I.mats_off + I.mats_len <= part.mats.size
    for seen, total in ((seen_states, T.states_count), (seen_probs, T.probs_count)):
        seen.sort()
        pos = 0
        for off, size in seen:
            assert off == pos
            pos += size
        assert pos == total
    assert T.swept_bytes(4) == sum(2 * 4 ** I.n * 4 * I.npasses for I in T.all_instances())


def test_tensor_core_choice_is_rejected_where_it_cannot_run():
    specs = B.sweep_specs(2, seed=1, n_range=(6, 6), depth_range=(2, 3))
    with pytest.raises(Exception):
        B.BatchTables(specs, 'single', kmax={6: B.TC}, workers=1)       # fewer than 7 qubits
    specs = B.sweep_specs(2, seed=1, n_range=(8, 8), depth_range=(2, 3))
    with pytest.raises(Exception):
        B.BatchTables(specs, 'double', kmax={8: B.TC}, workers=1)       # FP64 runs on the CUDA cores


def test_derived_recordings_equal_the_run_loop():
    """Instances of one structure after the first are derived from its recording; every op (kind,
    axes, matrix bit for bit) and the read-out equal the backend's own run loop."""
    specs = B.sweep_specs(400, seed=5)
    groups = {}
    for s in specs:
        groups.setdefault(B._structure(s), []).append(s)
    checked = 0
    for key, gs in list(groups.items())[:12]:
        if len(gs) < 2:
            continue
        ref = B.compile_experiment(*B.instance_experiment(gs[0]))
        for s in gs[1:4]:
            d = B.derive_recording(ref, s)
            f = B.compile_experiment(*B.instance_experiment(s))
            assert d is not None
            assert d.readouts == f.readouts and len(d.ops) == len(f.ops)
            for a, b in zip(d.ops, f.ops):
                assert (a.kind, tuple(a.axes), a.ideal) == (b.kind, tuple(b.axes), b.ideal)
                assert np.array_equal(np.asarray(a.data), np.asarray(b.data))
            checked += 1
    assert checked >= 10


def test_derived_recording_refuses_a_different_structure():
    a, b = B.sweep_specs(2, seed=6, n_range=(7, 7), depth_range=(4, 4))
    ref = B.compile_experiment(*B.instance_experiment(a))
    assert B.derive_recording(ref, dict(b, depth=5)) is None          # one more layer of gates
    assert B.derive_recording(ref, dict(b, n=8)) is None
    assert B.derive_recording(ref, dict(b, decoherence=1.0, decay=1.0, depolarisation=0.0)) is None


def test_derived_recording_refuses_other_cx_pairs_or_read_out():
    """The CX (control, target) sequence and the Z read-out of every qubit are compared with the
    reference recording, not copied from it."""
    import copy
    a, b = B.sweep_specs(2, seed=6, n_range=(7, 7), depth_range=(4, 4))
    ref = B.compile_experiment(*B.instance_experiment(a))
    assert B.derive_recording(ref, b) is not None
    swapped = copy.deepcopy(ref)
    i = next(k for k, op in enumerate(swapped.ops) if op.kind == 'cx')
    swapped.ops[i].axes = tuple(reversed(swapped.ops[i].axes))        # control and target exchanged
    assert B.derive_recording(swapped, b) is None
    other = copy.deepcopy(ref)
    kind, pos, mode, err = other.readouts[0]
    other.readouts = [(kind, pos, [1] * len(mode), err)]                # an X read-out
    assert B.derive_recording(other, b) is None
