"""Host-side measurement policy of bench.py, on CPU.

* The round engine's window radius per workload: 3 for the small system,
  4 for the large ones.
* The L2 flush between timed calls: a state of less than twice the L2 size
  gets a device write of twice the L2 size before every timed call, a larger
  one none, and `config.l2` says which.  A stand-in for torch's CUDA calls
  gives the flusher a device here.
"""
import os
import sys
import types

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402

L2 = 136 * 2 ** 20


class _Buf:
    def __init__(self, n):
        self.n, self.fills = n, []
        self.device = "cuda:0"

    def fill_(self, v):
        self.fills.append(v)

    def numel(self):
        return self.n


def _fake_torch(made):
    cuda = types.SimpleNamespace(
        is_available=lambda: True,
        get_device_properties=lambda dev: types.SimpleNamespace(L2_cache_size=L2),
        synchronize=lambda dev=None: None)

    def empty(n, dtype=None, device=None):
        b = _Buf(n)
        made.append(b)
        return b

    return types.SimpleNamespace(cuda=cuda, empty=empty, uint8="uint8")


def test_round_radius_per_workload():
    assert bench.DEFAULT_RADIUS["plain_small"] == 3
    for w in ("batched", "single_large", "single_4m"):
        assert bench.DEFAULT_RADIUS[w] == 4
    assert set(bench.DEFAULT_RADIUS) == set(bench.DEFAULT_ENGINE)


def test_small_state_is_flushed_before_every_timed_call(monkeypatch):
    made = []
    monkeypatch.setitem(sys.modules, "torch", _fake_torch(made))
    f = bench.L2Flusher(0, 1980 * 160)
    assert len(made) == 1 and made[0].n == 2 * L2
    for _ in range(3):
        f()
    assert made[0].fills == [1, 2, 3]          # a different byte each time: every write reaches memory
    assert "L2 flushed before every timed call" in f.describe()


def test_large_state_is_not_flushed(monkeypatch):
    made = []
    monkeypatch.setitem(sys.modules, "torch", _fake_torch(made))
    f = bench.L2Flusher(0, 4096 * 2176 * 160)    # the batched workload, ~1.4 GB
    f()
    assert made == []
    assert "larger than twice L2" in f.describe() and "no flush" in f.describe()


def test_flusher_without_a_device_says_so(monkeypatch):
    torch = types.SimpleNamespace(cuda=types.SimpleNamespace(is_available=lambda: False))
    monkeypatch.setitem(sys.modules, "torch", torch)
    f = bench.L2Flusher(0, 1980 * 160)
    f()
    assert "no flush" in f.describe()


def test_failed_flush_buffer_is_reported(monkeypatch):
    made = []
    fake = _fake_torch(made)

    def no_memory(n, dtype=None, device=None):
        raise RuntimeError("CUDA out of memory")

    fake.empty = no_memory
    monkeypatch.setitem(sys.modules, "torch", fake)
    f = bench.L2Flusher(0, 1980 * 160)
    f()
    d = f.describe()
    assert "no flush" in d and "out of memory" in d
