"""Host-side logic of the Python Vector's array access (python/ceed_vector.py:73-270), on CPU.

Vector keeps its array in a torch tensor on its context's device; these tests give it a stand-in context on the CPU,
so the get/restore, context-manager and take semantics are checked without a GPU (no kernel is called).
"""
import types

import numpy as np
import pytest
import torch

import libceed_gb300 as lc
from libceed_gb300.ceed import Vector


@pytest.fixture
def host_ceed():
    return types.SimpleNamespace(device=torch.device("cpu"))


def _vec(ceed, values):
    v = Vector(ceed, len(values))
    v.set_array(np.asarray(values, dtype=np.float64))
    return v


def test_get_array_writes_back_on_restore(host_ceed):
    v = _vec(host_ceed, [1.0, 2.0, 3.0])
    a = v.get_array()
    a[1] = 20.0
    assert v.get_array_read()[1] == 2.0  # not yet published
    v.restore_array()
    assert v.get_array_read().tolist() == [1.0, 20.0, 3.0]
    v.restore_array()  # a second restore has nothing to publish
    assert v.get_array_read().tolist() == [1.0, 20.0, 3.0]


def test_context_managers(host_ceed):
    v = _vec(host_ceed, [1.0, 2.0, 3.0])
    with v.array() as a:
        a *= 2.0
    assert v.get_array_read().tolist() == [2.0, 4.0, 6.0]
    with v.array_write() as a:
        a[:] = 7.0
    assert v.get_array_read().tolist() == [7.0, 7.0, 7.0]
    with v.array_read() as a:
        b = a.copy()
        a[:] = -1.0  # read access: nothing is published
    assert v.get_array_read().tolist() == b.tolist() == [7.0, 7.0, 7.0]
    with pytest.raises(RuntimeError):
        with v.array() as a:
            a[0] = 99.0
            raise RuntimeError("the block failed")
    assert v.get_array_read()[0] == 99.0  # restored even when the block raises, as the reference's try/finally


def test_take_array_returns_the_borrowed_host_array_with_current_values(host_ceed):
    h = np.array([1.0, 2.0, 3.0, 4.0])
    v = Vector(host_ceed, 4)
    v.set_array(h, lc.MEM_HOST, lc.USE_POINTER)
    with v.array() as a:
        a += 10.0
    got = v.take_array()
    assert got is h and h.tolist() == [11.0, 12.0, 13.0, 14.0]
    with pytest.raises(lc.B200Error):
        v.take_array()  # nothing is borrowed any more


def test_take_array_after_copy_values_is_refused(host_ceed):
    v = Vector(host_ceed, 2)
    v.set_array(np.zeros(2), lc.MEM_HOST, lc.COPY_VALUES)
    with pytest.raises(lc.B200Error, match="USE_POINTER"):
        v.take_array()


def test_take_array_copies_back_into_a_tensor_that_was_copied(host_ceed):
    t = torch.arange(3, dtype=torch.float32)  # another scalar type: copied at set_array, not borrowed
    v = Vector(host_ceed, 3)
    v.set_array(t, lc.MEM_DEVICE, lc.USE_POINTER)
    with v.array() as a:
        a[:] = 5.0
    assert v.take_array() is t and t.tolist() == [5.0, 5.0, 5.0]


def test_repr_and_str(host_ceed):
    v = _vec(host_ceed, [0.5, 0.25])
    assert "length 2" in repr(v)
    assert str(v).splitlines() == ["CeedVector length 2", "  0.5", "  0.25"]
