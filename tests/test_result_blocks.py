"""Host result blocks of large copy-outs: handed out once, reused only after release."""
import gc

import numpy as np

from qiskit_aakash_gb300 import engine


def test_result_blocks_are_reused_only_after_every_view_is_released(monkeypatch):
    monkeypatch.setattr(engine, '_RESULT_BLOCKS', {})
    monkeypatch.setattr(engine, '_page_lock', lambda ptr, nbytes: True)
    monkeypatch.setattr(engine, '_page_unlock', lambda ptr: None)
    monkeypatch.setattr(engine, '_host_bytes_available', lambda: 1 << 40)
    total = 1 << 16
    a, pa = engine._result_array(total)
    assert pa and a.shape == (total,) and a.dtype == np.float64
    a[:] = 1.0
    view = a.reshape(256, 256)[3:]
    del a
    gc.collect()
    b, pb = engine._result_array(total)           # the first block is still viewed: the second block
    assert pb and len(engine._RESULT_BLOCKS[total * 8]) == 2
    c, pc = engine._result_array(total)           # both held: a plain array, not page-locked
    assert not pc
    assert float(view[0, 0]) == 1.0               # the held view was not handed out again
    b_ptr = b.ctypes.data
    del b
    gc.collect()
    d, pd = engine._result_array(total)           # the released block comes back
    assert pd and d.ctypes.data == b_ptr
    del view
    gc.collect()
    e, pe = engine._result_array(total)
    assert pe and e.ctypes.data != d.ctypes.data


def test_no_result_block_without_host_room(monkeypatch):
    monkeypatch.setattr(engine, '_RESULT_BLOCKS', {})
    monkeypatch.setattr(engine, '_page_lock', lambda ptr, nbytes: True)
    monkeypatch.setattr(engine, '_page_unlock', lambda ptr: None)
    monkeypatch.setattr(engine, '_host_bytes_available', lambda: 1 << 10)
    a, pa = engine._result_array(1 << 12)
    assert not pa and a.shape == (1 << 12,)
    assert engine._RESULT_BLOCKS[(1 << 12) * 8] == []


def test_result_held_only_by_a_dead_reference_cycle_is_reclaimed(monkeypatch):
    monkeypatch.setattr(engine, '_RESULT_BLOCKS', {})
    monkeypatch.setattr(engine, '_page_lock', lambda ptr, nbytes: True)
    monkeypatch.setattr(engine, '_page_unlock', lambda ptr: None)
    monkeypatch.setattr(engine, '_host_bytes_available', lambda: 1 << 40)
    monkeypatch.setattr(engine, '_BLOCKS_PER_SIZE', 1)
    total = 1 << 12
    a, _ = engine._result_array(total)
    cycle = {'coeffmatrix': a}
    cycle['self'] = cycle                 # released only by the cyclic collector
    ptr = a.ctypes.data
    del a, cycle
    b, pb = engine._result_array(total)
    assert pb and b.ctypes.data == ptr
