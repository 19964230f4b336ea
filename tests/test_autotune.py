"""Host logic of the per-class autotuner (openqp_gb300/autotune.py), on CPU.

A fake builder stands in for FockBuilder: its per-class "event times" follow a
cost model whose optimum is known class by class, so the coordinate search must
find it exactly: the kernel family first (only where a class has both), then
the primitive-count split, the grab chunk and the grid cap; the two
thread-per-quartet parameters are left alone for classes that run warp per
quartet; idle classes are untouched; and a cached table is reapplied without
a search.
"""
import json

import pytest

torch = pytest.importorskip("torch")

from openqp_gb300 import autotune, fock  # noqa: E402
from openqp_gb300.fock import NCLASS  # noqa: E402

IDLE = NCLASS - 1   # a class with no quartets (time 0)


def avail_of(c):
    return (3, 1, 2)[c % 3]   # both families / thread only / warp only


def split_opt(c):
    return 6 + c % 5          # 6..10, all among the candidates


def chunk_opt(c):
    return 64 if c % 3 == 0 else 32


def ctas_opt(c):
    return 1 if c % 4 == 0 else 0


def warp_better(c):
    return avail_of(c) == 3 and c % 2 == 0


class FakeBuilder:
    def __init__(self):
        self.family = [0] * NCLASS
        self.tune = dict(split_log2=[-1] * NCLASS, chunk=[32] * NCLASS, ctas_per_sm=[0] * NCLASS)
        self.builds = 0

    # the FockBuilder surface the tuner uses
    def get_kernel_family(self):
        return list(self.family), [avail_of(c) for c in range(NCLASS)]

    def set_kernel_family(self, family):
        self.family = list(family)

    def get_tuning(self):
        return {k: list(v) for k, v in self.tune.items()}

    def set_tuning(self, split_log2=None, chunk=None, ctas_per_sm=None):
        for k, v in (("split_log2", split_log2), ("chunk", chunk), ("ctas_per_sm", ctas_per_sm)):
            if v is not None:
                self.tune[k] = list(v)

    def fock_jk_device(self, d):
        self.builds += 1

    def stats(self):
        return {"ms_per_class": [self.ms(c) for c in range(NCLASS)]}

    # cost model: each knob adds a penalty away from its class optimum
    def runs_warp(self, c):
        a = avail_of(c)
        return a == 2 or (a == 3 and self.family[c] == 2)

    def ms(self, c):
        if c == IDLE:
            return 0.0
        t = 10.0 + c
        if avail_of(c) == 3 and self.family[c] == 2:
            t *= 0.5 if warp_better(c) else 1.5
        if not self.runs_warp(c):
            s = self.tune["split_log2"][c]
            s = 8 if s < 0 else s
            t += 0.1 * abs(s - split_opt(c))
            t += 0.05 * (self.tune["chunk"][c] != chunk_opt(c))
        t += 0.2 * (self.tune["ctas_per_sm"][c] != ctas_opt(c))
        return t


@pytest.fixture
def fake_env(monkeypatch):
    monkeypatch.setattr(autotune, "_device_name", lambda: "fake-gpu")
    monkeypatch.setattr(fock, "class_labels", lambda: ["class%d" % c for c in range(NCLASS)])


def test_coordinate_search_finds_every_class_optimum(fake_env):
    b = FakeBuilder()
    d = torch.zeros(1, 3, dtype=torch.float64)
    default = [b.ms(c) for c in range(NCLASS)]
    tab = autotune.autotune(b, d, "fake", reps=1)
    assert tab["cached"] is False
    for c in range(NCLASS):
        if c == IDLE:
            assert tab["family"][c] == 0 and tab["split_log2"][c] == -1 and tab["chunk"][c] == 32
            assert tab["ctas_per_sm"][c] == 0
            continue
        assert tab["family"][c] == (2 if warp_better(c) else 0), c
        if b.runs_warp(c):
            # thread-per-quartet parameters stay at their defaults for warp-per-quartet classes
            assert tab["split_log2"][c] == -1 and tab["chunk"][c] == 32, c
        else:
            # a candidate equal to the default's time (2^8) leaves the default (-1) in place
            assert tab["split_log2"][c] == (-1 if split_opt(c) == 8 else split_opt(c)), c
            assert tab["chunk"][c] == chunk_opt(c), c
        assert tab["ctas_per_sm"][c] == ctas_opt(c), c
    # the builder is left with the chosen table, and no class got slower
    assert b.family == tab["family"]
    assert b.get_tuning() == {k: tab[k] for k in ("split_log2", "chunk", "ctas_per_sm")}
    assert all(t <= d0 + 1e-12 for t, d0 in zip(tab["class_ms"], default))
    assert sum(tab["class_ms"]) < sum(default)


def test_cached_table_is_reapplied_without_search(fake_env, tmp_path):
    cache = str(tmp_path / "tuning.json")
    b1 = FakeBuilder()
    d = torch.zeros(1, 3, dtype=torch.float64)
    t1 = autotune.autotune(b1, d, "fake", cache=cache, reps=1)
    stored = json.load(open(cache))
    assert list(stored) == ["fake-gpu|fake|nfocks=1|fp64"]
    b2 = FakeBuilder()
    t2 = autotune.autotune(b2, d, "fake", cache=cache, reps=1)
    assert t2["cached"] is True and b2.builds == 0
    assert b2.family == t1["family"]
    assert b2.get_tuning() == {k: t1[k] for k in ("split_log2", "chunk", "ctas_per_sm")}
    # another workload key or precision is searched afresh
    b3 = FakeBuilder()
    t3 = autotune.autotune(b3, d, "fake", cache=cache, reps=1, precision="mixed")
    assert t3["cached"] is False and b3.builds > 0
    assert len(json.load(open(cache))) == 2
