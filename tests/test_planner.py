"""Host-side checks of the transfer matrices and the fused-pass planner (no GPU).

The passes the planner emits are replayed with numpy (each op applied to the
whole state, which is what applying it to every tile does) and must equal
the operations applied one by one in program order.
"""
import numpy as np
import pytest

from oracle import dm_oracle as O
from qiskit_aakash_gb300 import _native as N
from qiskit_aakash_gb300 import program as P


def apply_map1(st, n, q, m):
    v = st.reshape(4 ** q, 4, 4 ** (n - q - 1))
    return np.einsum('ij,ajb->aib', m, v).reshape(-1)


def apply_pair(st, n, qa, qb, m16):
    """16x16 map on (qa, qb), index 4*p_a + p_b."""
    t = st.reshape([4] * n)
    t = np.moveaxis(t, (qa, qb), (0, 1)).reshape(16, -1)
    t = (m16 @ t).reshape([4, 4] + [4] * (n - 2))
    return np.moveaxis(t, (0, 1), (qa, qb)).reshape(-1)


def cx_matrix(coef, ideal):
    """The CX map (control, target) as a dense 16x16 matrix, from the kernel's formulas."""
    if ideal:
        coef = (1.0, 0.0, 1.0, 0.0, 0.0)
    c, s, c2, s2, cs = coef
    M = np.eye(16)
    rows = {
        2: {2: s2, 14: c2, 3: -cs, 15: cs},
        14: {2: c2, 14: s2, 3: cs, 15: -cs},
        3: {3: s2, 15: c2, 2: cs, 14: -cs},
        15: {3: c2, 15: s2, 2: -cs, 14: cs},
        4: {5: c, 8: -s}, 5: {4: c, 9: -s},
        6: {10: -s, 11: c}, 7: {10: -c, 11: -s},
        8: {4: s, 9: c}, 9: {5: s, 8: c},
        10: {6: s, 7: -c}, 11: {6: c, 7: s},
    }
    for r, entries in rows.items():
        M[r, :] = 0
        for col, v in entries.items():
            M[r, col] = v
    return M


def apply_op(st, n, op):
    if op.kind == 'map1':
        return apply_map1(st, n, op.axes[0], op.data)
    if op.kind == 'cx':
        return apply_pair(st, n, op.axes[0], op.axes[1], cx_matrix(op.data, op.ideal))
    if op.kind == 'diag2':
        return apply_pair(st, n, op.axes[0], op.axes[1], np.diag(op.data))
    if op.kind == 'map2':
        return apply_pair(st, n, op.axes[0], op.axes[1], op.data)
    raise ValueError(op.kind)


def random_ops(rng, n, count):
    ops = []
    for _ in range(count):
        r = rng.random()
        if r < 0.6 or n < 2:
            q = int(rng.integers(n))
            ops.append(P.Op('map1', (q,), rng.normal(size=(4, 4))))
        elif r < 0.85:
            a, b = (int(x) for x in rng.choice(n, 2, replace=False))
            coef, ideal = P.cx_coefficients([rng.uniform(0.9, 1.0), rng.uniform(-0.2, 0.2)]
                                            if rng.random() < 0.5 else [1.0, 0.0])
            ops.append(P.Op('cx', (a, b), np.array(coef), ideal))
        elif r < 0.95:
            a, b = (int(x) for x in rng.choice(n, 2, replace=False))
            ops.append(P.Op('diag2', (a, b), rng.normal(size=16)))
        else:
            a, b = (int(x) for x in rng.choice(n, 2, replace=False))
            ops.append(P.Op('map2', (a, b), rng.normal(size=(16, 16)) / 4))
    return ops


def test_cx_formula_matches_oracle():
    rng = np.random.default_rng(0)
    n = 4
    for tsp in ([1.0, 0.0], [0.97, 0.05], [0.9, -0.3]):
        for (c, t) in ((0, 1), (1, 0), (0, 3), (3, 1), (2, 3)):
            st = rng.normal(size=4 ** n)
            ref = O.cx_apply(st.copy(), n, c, t, tsp)
            coef, ideal = P.cx_coefficients(tsp)
            got = apply_pair(st, n, c, t, cx_matrix(coef, ideal))
            np.testing.assert_allclose(got, ref, atol=1e-13)


def test_u_gate_ptm_matches_oracle_rotations():
    rng = np.random.default_rng(1)
    n = 3
    err = {'rx': [0.98, 0.01], 'ry': [0.97, -0.02], 'rz': [0.99, 0.03]}
    for _ in range(20):
        st = rng.normal(size=4 ** n)
        q = int(rng.integers(n))
        params = rng.uniform(0, 2 * np.pi, 3)
        ref = st.copy()
        v = ref.reshape(4 ** q, 4, 4 ** (n - q - 1))
        for name, ang in O.u_decomposition('u3', params):
            O.rotate(v, name, ang, err[name])
        got = apply_map1(st, n, q, P.u_gate_ptm('u3', params, err))
        np.testing.assert_allclose(got, ref, atol=1e-13)


def test_noise_ptm_matches_oracle():
    rng = np.random.default_rng(2)
    n = 3
    st = rng.normal(size=4 ** n)
    ref = O.memory_noise(st.copy(), n, 0.93, 0.3, 0.91)
    got = st
    for q in range(n):
        got = apply_map1(got, n, q, P.noise_ptm(0.93, 0.3, 0.91))
    np.testing.assert_allclose(got, ref, atol=1e-14)


@pytest.mark.parametrize('n,kmax,low', [(1, 6, 2), (2, 6, 2), (3, 3, 1), (5, 4, 2), (6, 6, 2),
                                        (7, 5, 2), (8, 6, 2), (8, 7, 3), (9, 4, 0)])
def test_passes_equal_program_order(n, kmax, low):
    rng = np.random.default_rng(100 + n * 10 + kmax)
    for trial in range(6):
        ops = random_ops(rng, n, int(rng.integers(1, 60)))
        st0 = rng.normal(size=4 ** n)
        ref = st0.copy()
        for op in ops:
            ref = apply_op(ref, n, op)
        passes = P.plan_passes(ops, n, kmax, low)
        got = st0.copy()
        k = min(kmax, n)
        lowset = set(range(n - 1, n - 1 - min(low, k), -1))
        for p in passes:
            assert len(p.axes) <= k
            assert lowset.issubset(p.axes)
            assert list(p.axes) == sorted(p.axes, reverse=True)
            assert len(p.ops) <= 128
            for op in p.ops:
                assert set(op.axes).issubset(p.axes)
                got = apply_op(got, n, op)
        np.testing.assert_allclose(got, ref, rtol=1e-10, atol=1e-10 * np.abs(ref).max())


def test_brick_layers_fuse_into_few_passes():
    """n=16 random brick layers with noise after every level: passes per layer stay small."""
    n = 16
    rng = np.random.default_rng(3)
    ops = []
    noise = P.noise_ptm(0.995, 1.0, 0.998)
    for L in range(6):
        for q in range(n):
            ops.append(P.Op('map1', (q,), rng.normal(size=(4, 4))))
        for q in range(n):
            ops.append(P.Op('map1', (q,), noise))
        for a in range(L % 2, n - 1, 2):
            coef, ideal = P.cx_coefficients([1.0, 0.0])
            ops.append(P.Op('cx', (a, a + 1), np.array(coef), ideal))
        for q in range(n):
            ops.append(P.Op('map1', (q,), noise))
    passes = P.plan_passes(ops, n, 7, 2)
    assert len(passes) / 6 <= 4.0


def _same_passes(a, b):
    assert len(a) == len(b)
    for p, q in zip(a, b):
        assert list(p.axes) == list(q.axes)
        assert len(p.ops) == len(q.ops)
        for x, y in zip(p.ops, q.ops):
            assert x.kind == y.kind and tuple(x.axes) == tuple(y.axes)
            np.testing.assert_array_equal(np.asarray(x.data), np.asarray(y.data))


@pytest.mark.parametrize('n,kmax,low,chunk', [(6, 4, 2, 7), (9, 6, 2, 40), (12, 7, 2, 150), (16, 7, 2, 500)])
def test_streamed_planning_gives_the_passes_of_the_whole_stream(n, kmax, low, chunk):
    """Planning a growing prefix and launching only its closed passes (the engine's
    streaming flush) yields exactly the passes of planning the whole op list at once."""
    rng = np.random.default_rng(7 * n + chunk)
    ops = []
    noise = P.noise_ptm(0.995, 1.0, 0.998)
    for L in range(8):
        for q in range(n):
            ops.append(P.Op('map1', (q,), rng.normal(size=(4, 4))))
            ops.append(P.Op('map1', (q,), noise))
        for a in range(L % 2, n - 1, 2):
            coef, ideal = P.cx_coefficients([1.0, 0.0])
            ops.append(P.Op('cx', (a, a + 1), np.array(coef), ideal))
            for q in range(n):
                ops.append(P.Op('map1', (q,), noise))
    ops += random_ops(rng, n, 80)
    whole = P.plan_passes(ops, n, kmax, low)
    streamed, pending, launched_early = [], [], 0
    for i in range(0, len(ops), chunk):
        pending = pending + ops[i:i + chunk]
        done, pending = P.plan_passes(pending, n, kmax, low, partial=True)
        launched_early += len(done)
        streamed += done
    streamed += P.plan_passes(pending, n, kmax, low)
    _same_passes(streamed, whole)
    assert launched_early > len(whole) // 2     # most passes start before the stream ends


def test_streamed_planning_edge_cases():
    """No ops: nothing launched, nothing left; ops that fit one open pass: all of them stay queued."""
    assert P.plan_passes([], 6, 4, 2, partial=True) == ([], [])
    ops = [P.Op('map1', (5,), np.eye(4)), P.Op('map1', (4,), np.eye(4))]
    done, rest = P.plan_passes(ops, 6, 4, 2, partial=True)
    assert done == [] and rest == ops
    # a full pass whose resident axes are all blocked by later ops closes before the end of the queue
    n = 6
    ops = [P.Op('map1', (q,), np.eye(4)) for q in (5, 4, 3, 2)]
    ops += [P.Op('map1', (q,), np.eye(4)) for q in (1, 0)]                     # outside the full pass
    ops += [P.Op('cx', (1, q), np.array(P.cx_coefficients([1.0, 0.0])[0]), True) for q in (5, 4, 3, 2)]
    done, rest = P.plan_passes(ops, n, 4, 2, partial=True)
    assert len(done) == 1 and sorted(done[0].axes) == [2, 3, 4, 5]
    assert rest == ops[4:]


@pytest.mark.parametrize('width', [2, 3])
@pytest.mark.parametrize('n,kmax,low', [(5, 4, 2), (7, 6, 2), (8, 7, 2), (9, 7, 3)])
def test_register_rounds_equal_program_order(n, kmax, low, width):
    """Rounds regroup a pass's ops; replaying them in round order equals program order."""
    rng = np.random.default_rng(7 * n + kmax + width)
    for trial in range(4):
        ops = [op for op in random_ops(rng, n, int(rng.integers(5, 60))) if op.kind != 'map2']
        st0 = rng.normal(size=4 ** n)
        ref = st0.copy()
        for op in ops:
            ref = apply_op(ref, n, op)
        got = st0.copy()
        for p in P.plan_passes(ops, n, kmax, low):
            rounds = P.plan_rounds(p, width)
            for axes, rops in rounds:
                assert len(axes) == min(width, len(p.axes)) and axes == sorted(axes)
                for op in rops:
                    assert set(op.axes).issubset(axes)
                    glob = P.Op(op.kind, tuple(p.axes[a] for a in op.axes), op.data, op.ideal)
                    got = apply_op(got, n, glob)
            dp = P.encode_pass(p, [], np.float32, width, n)
            if width <= len(p.axes) <= 7 and p.axes[0] == n - 1:
                assert dp.nrounds == len(rounds)
                assert dp.round_end[dp.nrounds - 1] == dp.nops
        np.testing.assert_allclose(got, ref, rtol=1e-10, atol=1e-10 * np.abs(ref).max())


def _emulate_tc_pass(st, n, p):
    """numpy model of dm_apply_pass_tc's data movement (exact arithmetic, no FP16 split)."""
    pp, layouts, mats = P.plan_tc_pass(p, n)
    direct = P.direct_last_eligible([L.digits for L in layouts])
    conv, rounds = P.tc_tables(layouts, 'xor', direct)
    if direct:   # the last round's rows 0-3: the 16 contiguous coefficients of the tile
        assert sorted(rounds[-1]['rowc'][:4]) == [1, 2, 4, 8]
    k = 7
    non = [q for q in range(n - 1, -1, -1) if q not in pp.axes]
    out = st.copy()
    for t in range(4 ** (n - k)):
        base = sum(((t >> (2 * u)) & 3) * 4 ** (n - 1 - q) for u, q in enumerate(non))
        idx = np.array([base + sum(((e >> (2 * r)) & 3) * 4 ** (n - 1 - q) for r, q in enumerate(pp.axes))
                        for e in range(4 ** k)])
        nat = np.zeros(4 ** k)
        nat[[P.nat_swz(e) for e in range(4 ** k)]] = st[idx]          # cp.async landing
        A = np.zeros(16384)                                            # operand, FP16 index = byte / 2

        def xor_bits(x, c):
            o = 0
            for i, ci in enumerate(c):
                if (x >> i) & 1:
                    o ^= ci
            return o

        for row in range(256):                                         # conversion
            nb = xor_bits(row, conv['natrow'])
            for j in range(64):
                A[(P._row_off(row) + P._k_off(j)) // 2] = nat[nb ^ xor_bits(j, conv['natk'])]
        for r, (rd, U) in enumerate(zip(rounds, mats)):
            X = np.array([[A[(P._row_off(row) + P._k_off(j)) // 2] for j in range(64)] for row in range(256)])
            D = X @ U.T
            last = r + 1 == len(rounds)
            newA = np.zeros(16384) if not last else None
            natout = np.zeros(4 ** k) if last else None
            for row in range(256):
                b = xor_bits(row, rd['rowc'])
                for j in range(64):
                    o = b ^ xor_bits(j, rd['kc'])
                    if last:
                        natout[o] = D[row, j]
                    else:
                        newA[o // 2] = D[row, j]
            if not last:
                A = newA
        # a direct last round writes linear natural positions straight to global memory
        out[idx] = natout if direct else natout[[P.nat_swz(e) for e in range(4 ** k)]]
    return out


@pytest.mark.parametrize('kind', ['random', 'off_low'])
def test_tensor_core_tables_emulated(kind):
    """The tensor-core pass's layouts and tables, replayed in numpy, equal program order.  'off_low':
    ops off the two lowest-stride qubits, so last rounds leave local axes 0 and 1 alone and store
    straight to global memory (direct last rounds)."""
    n = 8 if kind == 'random' else 9
    rng = np.random.default_rng(21)
    ops = random_ops(rng, n, 40 if kind == 'random' else 90)
    if kind == 'off_low':
        ops = [op for op in ops if all(q < n - 2 for q in op.axes)]
    st0 = rng.normal(size=4 ** n)
    ref = st0.copy()
    for op in ops:
        ref = apply_op(ref, n, op)
    got = st0.copy()
    direct = 0
    for p in P.plan_passes(ops, n, 7, 2):
        _, layouts, _ = P.plan_tc_pass(p, n)
        direct += P.direct_last_eligible([L.digits for L in layouts])
        got = _emulate_tc_pass(got, n, p)
    if kind == 'off_low':
        assert direct > 0
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-10 * np.abs(ref).max())


def _tma_tile_index(n, dims, t):
    """Global element of each shared-memory position of tile t, as the TMA box delivers it.

    Dimension i: stride 4**start, box 4**len, coordinate ((t >> 2 g) & (4**gap - 1)) * 4**len
    with g the non-resident digits below its gap (tile_coords in csrc/dm_tma.cu); the box
    lands densely in dimension order."""
    idx = np.zeros(1, dtype=np.int64)
    g = 0
    for start, length, gap in dims:
        c = ((t >> (2 * g)) & ((1 << (2 * gap)) - 1)) << (2 * length)
        x = np.arange(4 ** length, dtype=np.int64)
        idx = (idx[None, :] + ((c + x) * 4 ** start)[:, None]).reshape(-1)
        g += gap
    return idx


def _emulate_tma_pass(st, n, p):
    """numpy model of dm_apply_pass_tma: TMA box addressing, linear natural tables (the last round's
    written to the tile's global positions), exact arithmetic."""
    pp, layouts, mats = P.plan_tc_pass(p, n, nat='tma')
    conv, rounds = P.tc_tables(layouts, 'linear')
    dims = P.tma_box_dims(n, pp.axes)
    out = st.copy()
    seen = np.zeros(4 ** n, dtype=np.int64)

    def xor_bits(x, c):
        o = 0
        for i, ci in enumerate(c):
            if (x >> i) & 1:
                o ^= ci
        return o

    for t in range(4 ** (n - 7)):
        idx = _tma_tile_index(n, dims, t)
        seen[idx] += 1
        nat = st[idx]
        A = np.zeros(16384)
        for row in range(256):
            nb = xor_bits(row, conv['natrow'])
            for j in range(64):
                A[(P._row_off(row) + P._k_off(j)) // 2] = nat[nb ^ xor_bits(j, conv['natk'])]
        for r, (rd, U) in enumerate(zip(rounds, mats)):
            X = np.array([[A[(P._row_off(row) + P._k_off(j)) // 2] for j in range(64)] for row in range(256)])
            D = X @ U.T
            last = r + 1 == len(rounds)
            newA = np.zeros(16384)
            natout = np.zeros(4 ** 7)
            for row in range(256):
                b = xor_bits(row, rd['rowc'])
                for j in range(64):
                    o = b ^ xor_bits(j, rd['kc'])
                    if last:
                        natout[o] = D[row, j]
                    else:
                        newA[o // 2] = D[row, j]
            A = newA
        out[idx] = natout
    assert np.all(seen == 1)          # the tiles' boxes cover the state exactly once
    return out


def test_tma_tables_emulated():
    """The TMA-fed pass's tensor-map boxes and linear tables, replayed in numpy, equal program order."""
    n = 9
    rng = np.random.default_rng(23)
    ops = random_ops(rng, n, 50)
    st0 = rng.normal(size=4 ** n)
    ref = st0.copy()
    for op in ops:
        ref = apply_op(ref, n, op)
    got = st0.copy()
    used = 0
    for p in P.plan_passes(ops, n, 7, 2):
        pp, layouts, _ = P.plan_tc_pass(p, n, nat='tma')
        if P.tma_eligible(pp, n, layouts):
            got = _emulate_tma_pass(got, n, p)
            used += 1
        else:
            got = _emulate_tc_pass(got, n, p)
    assert used > 0
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-10 * np.abs(ref).max())


@pytest.mark.parametrize('axes_pos', [(0, 1, 2, 3, 4, 5, 6), (0, 1, 4, 5, 6, 9, 10), (0, 3, 5, 7, 9, 11, 13),
                                      (0, 2, 3, 4, 5, 6, 7), (0, 1, 2, 3, 4, 5, 13)])
def test_tma_box_dims(axes_pos):
    """Box dimensions: chunks of <= 4 resident digits, the gaps above them, every tile covered once."""
    n = 14
    axes = sorted((n - 1 - x for x in axes_pos), reverse=True)
    dims = P.tma_box_dims(n, axes)
    assert sum(length for _, length, _ in dims) == 7
    assert sum(gap for _, _, gap in dims) == n - 7
    assert all(1 <= length <= 4 for _, length, _ in dims)
    if len(dims) <= P.TMA_MAX_DIMS and n <= 10:
        seen = np.zeros(4 ** n, dtype=np.int64)
        for t in range(4 ** (n - 7)):
            seen[_tma_tile_index(n, dims, t)] += 1
        assert np.all(seen == 1)
    # shared-memory position e holds the tile's natural element e (local axis r = r-th lowest resident digit)
    idx = _tma_tile_index(n, dims, 0) if len(dims) <= P.TMA_MAX_DIMS else None
    if idx is not None:
        pos = sorted(axes_pos)
        want = np.array([sum(((e >> (2 * r)) & 3) * 4 ** pos[r] for r in range(7)) for e in range(4 ** 7)])
        assert np.array_equal(idx, want)


def test_tma_tables_are_valid():
    """TMA-pass tables obey dm_apply_pass_tma's checks (linear natural offsets, operand alignment)."""
    n = 16
    rng = np.random.default_rng(5)
    ops = random_ops(rng, n, 300)
    checked = 0
    for p in P.plan_passes(ops, n, 7, 2):
        pp, layouts, _ = P.plan_tc_pass(p, n, nat='tma')
        if not P.tma_eligible(pp, n, layouts):
            continue
        checked += 1
        conv, rounds = P.tc_tables(layouts, 'linear')
        assert all(x > 0 and x & (x - 1) == 0 and x < 16384 for x in conv['natrow'] + conv['natk'])
        if not {0, 1} & set(layouts[0].digits):
            assert {1, 2, 4, 8} <= set(conv['natrow'][:5])      # lanes: the 16 contiguous coefficients
        last = layouts[-1]
        assert not {0, 1} <= set(last.digits)                   # such passes run on pass_tc_kernel
        if 0 in last.digits:
            assert last.digits[0] == 0 and rounds[-1]['kc'][:2] == [1, 2]    # 16-byte stores
        elif 1 not in last.digits:
            assert sorted(rounds[-1]['rowc'][:4]) == [1, 2, 4, 8]   # lanes 0-15 contiguous
        else:
            assert sorted(rounds[-1]['rowc'][:2]) == [1, 2]
        for r, rd in enumerate(rounds):
            c = rd['rowc'] + rd['kc']
            assert len(set(c)) == 14
            if r + 1 < len(rounds):
                assert all(x > 0 and x & (x - 1) == 0 and x < P.TC_A_BYTES for x in c)
            else:
                assert all(x > 0 and x & (x - 1) == 0 and x < 16384 for x in c)
    assert checked > 0


def test_tma_image_layout_and_split():
    U = np.random.default_rng(3).normal(size=(64, 64)) / 8
    img = P.tc_round_image_tma(U)
    assert img.dtype == np.uint16 and img.size == P.TMA_IMAGE_HALVES
    uh, ul = (img[4096 * i + P._KMAJOR].view(np.float16).astype(np.float64).reshape(64, 64) for i in range(2))
    assert np.array_equal(uh, U.astype(np.float16).astype(np.float64))
    np.testing.assert_allclose(uh + ul / P.TC_LO_SCALE, U, rtol=0, atol=2.0 ** -21 * np.abs(U).max())
    # the TMA form's first two products equal the cp.async form's up to the power-of-two scale of Uh
    old = P.tc_round_image(U)
    assert np.array_equal(old[4096:8192], img[4096:8192])
    assert np.array_equal(old[8192:], img[:4096])


def test_tensor_core_tables_are_valid():
    """Every table entry obeys the kernel's checks (distinct power-of-two operand offsets, alignment)."""
    n = 16
    rng = np.random.default_rng(4)
    ops = random_ops(rng, n, 300)
    for p in P.plan_passes(ops, n, 7, 2):
        _, layouts, _ = P.plan_tc_pass(p, n)
        conv, rounds = P.tc_tables(layouts)
        for r, rd in enumerate(rounds):
            c = rd['rowc'] + rd['kc']
            if r + 1 < len(rounds):
                assert all(x > 0 and x & (x - 1) == 0 and x < P.TC_A_BYTES for x in c)
                assert len(set(c)) == 14
                if rd['vec'] >= 0:
                    v = rd['vec']
                    assert rd['kc'][2 * v] == 2 and rd['kc'][2 * v + 1] == 4
                    assert all(x % 8 == 0 for i, x in enumerate(c) if i < 8 or (i - 8) // 2 != v)
            else:
                assert all(0 < x < 16384 for x in c)


def test_tc_image_layout_and_split():
    U = np.random.default_rng(2).normal(size=(64, 64)) / 8
    img = P.tc_round_image(U)
    assert img.dtype == np.uint16 and img.size == P.TC_IMAGE_HALVES
    assert len(set(P._KMAJOR.tolist())) == 4096
    parts = [np.zeros((64, 64)) for _ in range(3)]
    for i in range(3):
        parts[i].reshape(-1)[:] = img[4096 * i + P._KMAJOR].view(np.float16).astype(np.float64)
    big, ul, uh = parts
    assert np.array_equal(big, uh * P.TC_LO_SCALE)                  # 2**11 Uh is exact in FP16
    assert np.array_equal(uh, U.astype(np.float16).astype(np.float64))
    # Uh + 2**-11 Ul carries U to about 2**-22 relative
    np.testing.assert_allclose(uh + ul / P.TC_LO_SCALE, U, rtol=0, atol=2.0 ** -21 * np.abs(U).max())


def test_fp16_three_way_split_accuracy():
    """h (2**11 Uh)^T + l Uh^T + h Ul^T, with FP16 operands and exact products, reproduces 2**11 x U^T."""
    rng = np.random.default_rng(8)
    U = rng.normal(size=(64, 64)) / 8
    x = rng.normal(size=(256, 64)) * np.exp(rng.uniform(-12, 0, size=(256, 64)))   # |x| <= ~1, many tiny
    h = x.astype(np.float16).astype(np.float64)
    lo = ((x - h) * P.TC_LO_SCALE).astype(np.float16).astype(np.float64)
    uh = U.astype(np.float16).astype(np.float64)
    ul = ((U - uh) * P.TC_LO_SCALE).astype(np.float16).astype(np.float64)
    D = (h @ (uh * P.TC_LO_SCALE).T + lo @ uh.T + h @ ul.T) / P.TC_LO_SCALE
    assert np.max(np.abs(D - x @ U.T)) < 2e-6 * np.abs(x @ U.T).max()


def _tc_split_round(st, n, qubits, U):
    """One tensor-core round in numpy: the state (units of 2**-n, FP32 between rounds) split into
    FP16 h / l, U into Uh / Ul, products exact, FP32 rounding of the sum."""
    perm = [q for q in range(n) if q not in qubits] + [qubits[2], qubits[1], qubits[0]]
    X = np.transpose(st, perm).reshape(-1, 64).astype(np.float32).astype(np.float64)
    h = X.astype(np.float16).astype(np.float64)
    lo = ((X - h) * P.TC_LO_SCALE).astype(np.float16).astype(np.float64)
    uh = U.astype(np.float16).astype(np.float64)
    ul = ((U - uh) * P.TC_LO_SCALE).astype(np.float16).astype(np.float64)
    D = ((h @ (P.TC_LO_SCALE * uh).T + (h @ ul.T + lo @ uh.T)) / P.TC_LO_SCALE).astype(np.float32)
    return np.transpose(D.astype(np.float64).reshape([4] * n), np.argsort(perm))


def test_tensor_core_split_model_stays_at_fp32_accuracy_over_a_deep_noisy_circuit():
    """The 3-way FP16 split with exactly rounded FP32 sums, applied round by round (the planner's
    rounds, digit orders and composed matrices) to a low-noise 40-layer 8-qubit circuit, stays
    within 1e-6 TV of exact FP64 application: the split itself is not the accuracy limit."""
    import copy
    from qiskit_aakash_gb300 import batch as B
    spec = dict(B.sweep_specs(1, seed=12, n_range=(8, 8), depth_range=(40, 40))[0],
                depolarisation=1e-4, decoherence=1 - 1e-4, decay=1 - 1e-4)
    rec = B.compile_experiment(*B.instance_experiment(spec))
    n = rec.n
    exact = np.zeros([4] * n)
    for m in range(2 ** n):
        exact[tuple(3 if (m >> (n - 1 - q)) & 1 else 0 for q in range(n))] = 1.0   # |0..0> in units of 2**-n
    split = exact.copy()
    for p in P.plan_passes(rec.ops, n, P.TC_AXES, 2):
        pp, layouts, mats = P.plan_tc_pass(p, n)
        for L, U in zip(layouts, mats):
            qubits = [pp.axes[a] for a in L.digits]
            perm = [q for q in range(n) if q not in qubits] + [qubits[2], qubits[1], qubits[0]]
            X = np.transpose(exact, perm).reshape(-1, 64)
            exact = np.transpose((X @ U.T).reshape([4] * n), np.argsort(perm))
            split = _tc_split_round(split, n, qubits, U)
    err = rec.readouts[0][3]
    pe = O.ensemble_probabilities(exact.reshape(-1) * 2.0 ** -n, n, 'Z', None, err)
    ps = O.ensemble_probabilities(split.reshape(-1) * 2.0 ** -n, n, 'Z', None, err)
    assert 0.5 * np.abs(pe - ps).sum() < 1e-6
    assert abs(ps.sum() - 1.0) < 1e-6


def test_xy_unital_flag_marks_exactly_the_maps_without_i_in_x_and_y():
    """DM_MAP1_XY_UNITAL is set from the composed matrix itself (a product of such maps need not be one)."""
    n = 6
    rot = P.u_gate_ptm('u3', [0.3, 0.2, 0.1], {'rx': [1, 0], 'ry': [1, 0], 'rz': [1, 0]})
    noise = P.noise_ptm(0.99, 0.9, 0.98)
    assert rot[1, 0] == 0 and rot[2, 0] == 0 and noise[1, 0] == 0 and noise[2, 0] == 0
    both = rot @ noise                      # noise first, then the rotation: X picks up I
    assert both[1, 0] != 0 or both[2, 0] != 0
    ops = [P.Op('map1', (5,), noise), P.Op('map1', (4,), rot), P.Op('map1', (3,), rot @ noise)]
    mats = []
    p = P.plan_passes(ops, n, 6, 2)[0]
    dp = P.encode_pass(p, mats, np.float64, 2, n)
    for i in range(dp.nops):
        m = mats[i].reshape(16)
        xy = m[4] == 0 and m[8] == 0
        assert bool(dp.ops[i].flags & N.DM_MAP1_XY_UNITAL) == xy


def test_too_many_tensor_core_rounds_raise_a_plan_error():
    """A pass whose rounds overflow the descriptor raises TcPlanError (the engine runs it on the CUDA cores)."""
    n = 7
    coef = np.array(P.cx_coefficients([0.99, 0.01])[0])
    ops = []
    for i in range(120):           # a CX chain around all 7 qubits: two CX per 3-axis round at most
        ops.append(P.Op('cx', (i % 7, (i + 1) % 7), coef, False))
    passes = P.plan_passes(ops, n, 7, 2)
    counts = [len(P.plan_tc_pass(p, n)[1]) for p in passes]
    assert max(counts) > N.DM_MAX_ROUNDS
    with pytest.raises(P.TcPlanError):
        for p in passes:
            P.encode_pass_tc(p, n, [])


def _compose_from_table(bp, coefs):
    """Each round's 64x64 U rebuilt from a DmBatchPass and its coefficients alone (what
    dm_compose_rounds reads): ops act on digit positions taken from their flags."""
    mats = np.concatenate(coefs)
    out = []
    kinds = {N.DM_OP_MAP1: 'map1', N.DM_OP_CX: 'cx', N.DM_OP_DIAG2: 'diag2', N.DM_OP_MAP2: 'map2'}
    o = 0
    for r in range(bp.nrounds):
        U = np.eye(64)
        for i in range(o, bp.round_end[r]):
            d = bp.ops[i]
            da, db = (d.flags >> 8) & 3, (d.flags >> 12) & 3
            kind = kinds[d.kind]
            size = {'map1': 16, 'cx': 5, 'diag2': 16, 'map2': 256}[kind]
            c = mats[d.moff:d.moff + size]
            if kind == 'map1':
                op = P.Op(kind, (da,), c.reshape(4, 4))
            elif kind == 'map2':
                op = P.Op(kind, (da, db), c.reshape(16, 16))
            else:
                op = P.Op(kind, (da, db), c if kind == 'diag2' else tuple(c), bool(d.flags & N.DM_CX_IDEAL))
            U = P.op_matrix64(op, (0, 1, 2)) @ U
        o = bp.round_end[r]
        out.append(U)
    return out


@pytest.mark.parametrize('kernel', ['tc', 'tma'])
def test_device_composition_table_restates_the_rounds(kernel):
    """The op table of a device-composed pass gives the host-composed round matrices, and its
    conversion / epilogue tables are the host encoder's with round r's images at r * image size."""
    rng = np.random.default_rng(11)
    n = 10
    ops = []
    for layer in range(6):
        for q in range(n - 2):
            ops.append(P.Op('map1', (q,), rng.uniform(-0.6, 0.6, size=(4, 4))))
        for q in range(layer % 2, n - 3, 2):
            ops.append(P.Op('cx', (q, q + 1), P.cx_coefficients((0.99, 0.01))[0]))
        ops.append(P.Op('diag2', (2, 5), rng.uniform(-1, 1, size=16)))
        ops.append(P.Op('map2', (4, 1), rng.uniform(-0.25, 0.25, size=(16, 16))))
    checked = 0
    for p in P.plan_passes(ops, n, 7, 2):
        coefs = []
        try:
            dp, bp = P.encode_pass_tc_ops(p, n, coefs, kernel)
        except P.TcPlanError:
            continue
        nat = 'tma' if kernel == 'tma' else 'xor'
        pp, rounds, layouts = P.plan_tc_rounds(p, n, nat)
        want = P.compose_round_matrices(rounds, layouts)
        got = _compose_from_table(bp, coefs)
        assert len(got) == len(want) == dp.nrounds == bp.nrounds
        for g, w in zip(got, want):
            np.testing.assert_allclose(g, w, rtol=0, atol=1e-12 * max(1.0, np.abs(w).max()))
        umats = []
        host = (P.encode_pass_tma if kernel == 'tma' else P.encode_pass_tc)(p, n, umats)
        halves = P.TMA_IMAGE_HALVES if kernel == 'tma' else P.TC_IMAGE_HALVES
        for r in range(dp.nrounds):
            assert dp.rounds[r].umoff == host.rounds[r].umoff == r * halves
            assert list(dp.rounds[r].rowc) == list(host.rounds[r].rowc)
            assert list(dp.rounds[r].kc) == list(host.rounds[r].kc)
        assert list(dp.natrow) == list(host.natrow) and list(dp.natk) == list(host.natk)
        checked += 1
    assert checked > 0
