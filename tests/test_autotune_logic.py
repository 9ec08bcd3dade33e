"""The autotuner's search on the host, with a fake batch and a deterministic cost model in
place of CUDA-event timing: shape search, per-model lanes by coordinate descent (largest tree
first), the refinement pass over the best candidates, and the cache (no GPU needed)."""
import json

import numpy as np
import pytest

from sapien_gb300 import autotune


class FakeModel:
    def __init__(self, nv, nj):
        self.nv, self.njoints = nv, nj


class FakeBatch:
    """Records the configuration; step() is a no-op, the cost model reads the state."""

    def __init__(self, models, counts):
        self.models = models
        self.model_of_env = np.repeat(np.arange(len(models)), counts)
        self.device = "cpu"
        self.shape, self.lanes = None, [1] * len(models)

    def set_launch(self, c, w, o):
        self.shape = (c, w, o)

    def set_lanes(self, lanes):
        self.lanes = list(lanes)

    def alloc_outputs(self, ops):
        return {}

    def step(self, *args):
        pass


def cost(batch, best_shape=(2, 2, 0), best_lanes=(1, 2, 4)):
    """Separable bowl: distance of each choice from the optimum, plus a tiny shape term."""
    c = sum(abs(np.log2(a) - np.log2(b)) for a, b in zip(batch.lanes, best_lanes))
    c += 0.1 * sum(abs(a - b) for a, b in zip(batch.shape, best_shape))
    return 1.0 + c


@pytest.fixture
def fake(monkeypatch, tmp_path):
    batch = FakeBatch([FakeModel(6, 7), FakeModel(18, 14), FakeModel(35, 31)], [10, 6, 4])
    calls = []

    def fake_time(fn, reps=5):
        fn()
        calls.append(reps)
        return cost(batch)

    monkeypatch.setattr(autotune, "_time", fake_time)
    monkeypatch.setenv("SGDYN_AUTOTUNE_CACHE", str(tmp_path))
    monkeypatch.setattr(autotune.torch.cuda, "get_device_name", lambda dev=None: "fake-gpu")
    return batch, calls, tmp_path


def test_search_finds_the_optimum_and_caches_it(fake):
    batch, calls, tmp_path = fake
    shape, table = autotune.tune_batch(batch, None, None, None, None, ops=28)
    assert tuple(shape) == (2, 2, 0) and batch.shape == (2, 2, 0)
    assert batch.lanes == [1, 2, 4]
    nshapes = len(autotune.CANDIDATES)
    # shape sweep with one lane, then 3 other lane counts x every shape for each model
    assert len(table) == nshapes + 3 * 3 * nshapes
    # largest tree first: the first lane trials change the humanoid (model 2)
    first = table[nshapes]["lanes"]
    assert first[2] != 1 and first[:2] == [1, 1]
    # refinement: the five best pairs again with 20 launches each
    assert calls.count(20) == 5
    cache = json.load(open(tmp_path / "autotune.json"))
    (entry,) = cache.values()
    assert entry["shape"] == [2, 2, 0] and entry["lanes"] == [1, 2, 4]
    # second call: from the cache, no timing
    n = len(calls)
    batch.set_launch(1, 1, 1)
    batch.set_lanes([8, 8, 8])
    shape2, _ = autotune.tune_batch(batch, None, None, None, None, ops=28)
    assert len(calls) == n and tuple(shape2) == (2, 2, 0) and batch.lanes == [1, 2, 4]


def test_signature_depends_on_mix_and_ops():
    b1 = FakeBatch([FakeModel(6, 7), FakeModel(35, 31)], [10, 4])
    b2 = FakeBatch([FakeModel(6, 7), FakeModel(35, 31)], [10, 5])
    s = autotune.batch_signature
    assert s(b1, 28) != s(b2, 28) and s(b1, 28) != s(b1, 16) and s(b1, 28) == s(b1, 28)
