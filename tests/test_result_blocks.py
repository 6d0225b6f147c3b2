"""Host result blocks of large copy-outs: handed out once, reused only after release."""
import gc

import numpy as np
import torch

from qiskit_aakash_gb300 import engine


_KEEP = []


def _host_memory(nbytes):
    buf = torch.empty(nbytes, dtype=torch.uint8)     # stands in for dm_host_alloc's page-locked memory
    _KEEP.append(buf)
    return buf.data_ptr()


def _fake_pinned(monkeypatch, room=1 << 40, blocks_per_size=None):
    monkeypatch.setattr(engine, '_RESULT_BLOCKS', {})
    monkeypatch.setattr(engine, '_pinned_host', _host_memory)
    monkeypatch.setattr(engine, '_host_bytes_available', lambda: room)
    if blocks_per_size is not None:
        monkeypatch.setattr(engine, '_BLOCKS_PER_SIZE', blocks_per_size)


def test_result_blocks_are_reused_only_after_every_view_is_released(monkeypatch):
    _fake_pinned(monkeypatch)
    total = 1 << 16
    a, ha = engine._result_array(total)
    assert ha is not None and a.shape == (total,) and a.dtype == np.float64
    assert a.ctypes.data == ha.ptr                 # the array is the page-locked block
    a[:] = 1.0
    view = a.reshape(256, 256)[3:]
    del a, ha
    gc.collect()
    b, hb = engine._result_array(total)            # the first block is still viewed: the second block
    assert hb is not None and len(engine._RESULT_BLOCKS[total * 8]) == 2
    c, hc = engine._result_array(total)            # both held: a plain array
    assert hc is None
    assert float(view[0, 0]) == 1.0                # the held view was not handed out again
    b_ptr = b.ctypes.data
    del b, hb
    gc.collect()
    d, hd = engine._result_array(total)            # the released block comes back
    assert hd is not None and d.ctypes.data == b_ptr
    del view
    gc.collect()
    e, he = engine._result_array(total)
    assert he is not None and e.ctypes.data != d.ctypes.data


def test_no_result_block_without_host_room(monkeypatch):
    _fake_pinned(monkeypatch, room=1 << 10)
    a, h = engine._result_array(1 << 12)
    assert h is None and a.shape == (1 << 12,)
    assert engine._RESULT_BLOCKS[(1 << 12) * 8] == []


def test_result_held_only_by_a_dead_reference_cycle_is_reclaimed(monkeypatch):
    _fake_pinned(monkeypatch, blocks_per_size=1)
    total = 1 << 12
    a, _ = engine._result_array(total)
    cycle = {'coeffmatrix': a}
    cycle['self'] = cycle                 # released only by the cyclic collector
    ptr = a.ctypes.data
    del a, cycle
    b, hb = engine._result_array(total)
    assert hb is not None and b.ctypes.data == ptr
