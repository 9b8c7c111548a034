"""Host logic of the autotuner (libceed_gb300/tune.py) on CPU: the sweep over staging and elements per block, the
choice of the fastest tile, and the JSON cache.  The C ABI is replaced by a stand-in that reports per-stage tile
limits and synthetic timings, so no kernel runs."""
import json
import types

import pytest

from libceed_gb300 import tune
from libceed_gb300.ceed import F32, QF_POISSON


class _Fused:
    h = "fused-handle"

    def __init__(self):
        self.tile = None

    def set_tile(self, epb, stage=0):
        self.tile = (epb, stage)


def _fake_op(deterministic=False):
    ptr = types.SimpleNamespace(ptr=lambda: None)
    field = types.SimpleNamespace(basis=types.SimpleNamespace(dim=3, P1d=5, Q1d=6), rstr=types.SimpleNamespace(ncomp=1))
    fused = _Fused()
    op = types.SimpleNamespace(
        ceed=types.SimpleNamespace(deterministic=deterministic), qf=types.SimpleNamespace(name="Poisson3DApply", kind=QF_POISSON),
        _fused={}, elems_per_block=0, staging=0)
    op._kernel_prec = lambda prec: prec
    op.fused = lambda prec: fused
    op._active_input = lambda: field
    op._passive = lambda name, prec: ptr
    return op, fused


@pytest.fixture
def fake_abi(monkeypatch, tmp_path):
    monkeypatch.setenv("CEED_B200_TUNE_CACHE", str(tmp_path / "tune.json"))
    state = types.SimpleNamespace(limits={1: 8, 2: 4, 3: 4, 4: 2, 5: 6, 6: 12, 7: 7}, timed=[], fused=None)

    def call(name, *args):
        if name == "b200_op_tile_limits":
            _, stage, out = args
            out._obj.value = state.limits[stage]
        elif name == "b200_op_time":
            epb, stage = state.fused.tile
            state.timed.append((epb, stage))
            args[-1]._obj.value = 1.0 + abs(epb - 6) * 0.01 + (0.0 if stage == 7 else 0.05)  # best: 6 per block, staging 7
        else:
            raise AssertionError(name)

    monkeypatch.setattr(tune, "call", call)
    return state


def test_sweep_picks_fastest_and_caches(fake_abi):
    op, fused = _fake_op()
    fake_abi.fused = fused
    u = types.SimpleNamespace(prec=F32, ptr=lambda: None)
    res = tune.autotune(op, u, u, reps=2)
    assert (res["epb"], res["staging"]) == (6, "persistent")
    assert fused.tile == (6, 7) and (op.elems_per_block, op.staging) == (6, 7)
    # every stage swept up to its limit, over the candidate list
    for stage, m in fake_abi.limits.items():
        swept = sorted(e for e, s in fake_abi.timed if s == stage)
        assert swept == [e for e in (1, 2, 3, 4, 5, 6, 7, 8, 10, 12) if e <= m]
    cache = json.load(open(tune.cache_path()))
    assert cache[res["key"]] == {"epb": 6, "staging": "persistent", "ms": res["ms"]}
    assert res["key"] == "dim3_P5_Q6_nc1_f32_Poisson3DApply_atomic"
    fresh, _ = _fake_op()
    assert tune.apply_cached(fresh, F32)["epb"] == 6 and (fresh.elems_per_block, fresh.staging) == (6, 7)
    other, _ = _fake_op(deterministic=True)
    assert tune.apply_cached(other, F32) is None  # the deterministic scatter is tuned separately


def test_unreadable_cache_is_empty(fake_abi, tmp_path):
    (tmp_path / "tune.json").write_text("{not json")
    assert tune.load_cache() == {}
