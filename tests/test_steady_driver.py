"""The host logic of the steady-state batch driver (surrogate.run_batch_to_steady)
on a scripted stand-in for mantiis_gb300.Batch: when images settle, which leave
the batch, what the new batches hold and carry over, and the lattice updates
counted.  No GPU."""
import numpy as np
import pytest

from mantiis_gb300 import native, surrogate


class FakeSolver:
    def __init__(self, name, lu, settle_at, k_final):
        self.name, self.info = name, {"lu_per_step": lu}
        self.settle_at, self.k_final = settle_at, k_final
        self.steps = 0

    def permeability(self):
        # swings by 2 % per 1000 steps until settle_at, then drifts by 1e-9 per 1000
        if self.steps >= self.settle_at:
            return self.k_final * (1.0 + 1e-9 * (self.steps - self.settle_at) / 1000.0)
        return self.k_final * (1.0 + 0.01 * (-1) ** (self.steps // 1000))


class FakeBatch:
    made = []

    def __init__(self, solvers):
        self.solvers = list(solvers)
        self.stream, self.engine, self.closed = None, None, False
        FakeBatch.made.append(self)

    def set_stream(self, s):
        self.stream = s

    def set_engine(self, engine, group=0):
        self.engine = (engine, group)

    def advance(self, n):
        assert not self.closed
        for s in self.solvers:
            s.steps += n

    def sync(self):
        pass

    def observables(self):
        return [dict(permeability=s.permeability()) for s in self.solvers]

    def close(self):
        self.closed = True


@pytest.fixture
def fake_batches(monkeypatch):
    FakeBatch.made = []
    monkeypatch.setattr(native, "Batch", FakeBatch)
    return FakeBatch


@pytest.mark.parametrize("drop", [True, False])
def test_settling_and_dropping(fake_batches, drop):
    sols = [FakeSolver("a", 10.0, 3000, 2.0), FakeSolver("b", 20.0, 5000, 3.0), FakeSolver("c", 5.0, 3000, 1.0),
            FakeSolver("d", 40.0, 10 ** 9, 4.0)]
    b = FakeBatch(sols)
    b.set_stream(7)
    b.set_engine(1, 2)
    stats = {}
    steps, k = surrogate.run_batch_to_steady(b, chunk=1000, tol=1e-6, max_steps=8000, drop_settled=drop, stats=stats)
    # settled at the first chunk whose change is below tol: one chunk past settle_at
    assert list(steps) == [4000, 6000, 4000, 8000]
    assert np.allclose(k[:3], [2.0, 3.0, 1.0], rtol=1e-8)
    if drop:
        # a and c leave at 4000 steps, b at 6000; d runs to the end
        assert [s.steps for s in sols] == [4000, 6000, 4000, 8000]
        assert stats["lu"] == 1000 * (4 * (10 + 20 + 5 + 40) + 2 * (20 + 40) + 2 * 40)
        assert stats["batches"] == 3
        later = fake_batches.made[1:]
        assert [[s.name for s in x.solvers] for x in later] == [["b", "d"], ["d"]]
        assert all(x.stream == 7 and x.engine == (1, 2) for x in later)
        assert all(x.closed for x in later) and not b.closed  # the caller's batch is the caller's to close
    else:
        assert [s.steps for s in sols] == [8000] * 4
        assert stats["lu"] == 8000 * (10 + 20 + 5 + 40) and stats["batches"] == 1
        assert len(fake_batches.made) == 1


def test_nothing_settles(fake_batches):
    sols = [FakeSolver("x", 1.0, 10 ** 9, 1.0)]
    steps, _ = surrogate.run_batch_to_steady(FakeBatch(sols), chunk=1000, tol=1e-6, max_steps=3000)
    assert list(steps) == [3000] and sols[0].steps == 3000
