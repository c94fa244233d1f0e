"""The queue-size autotuner (lightmetrica/autotune.py) on the CPU: a fake wavefront whose render
time depends on the queue size; the tuner warms each candidate once, keeps the best of its
repeats and returns the fastest size."""


class _Clock:
    t = 0.0

    @classmethod
    def perf_counter(cls):
        return cls.t


def test_tune_queue_picks_the_fastest(monkeypatch):
    from lightmetrica import autotune
    cost = {1 << 22: 3.0, 1 << 23: 2.0, 1 << 24: 1.5, 1 << 25: 1.7}
    made, closed = [], []

    class FakeBatch:
        def __init__(self, queue_paths=0):
            self.q = queue_paths
            self.calls = 0
            made.append(queue_paths)

        def submit(self, *a, **k):
            return 0

        def run(self, chunks=0):
            return 0

        def reset(self):
            pass

        def render(self, jobs):
            self.calls += 1
            _Clock.t += cost[self.q] + (0.5 if self.calls == 1 else 0.0)   # the first repeat is slower
            return list(range(len(jobs)))

        def close(self):
            closed.append(self.q)

    monkeypatch.setattr(autotune, "BatchRenderer", FakeBatch)
    monkeypatch.setattr(autotune, "time", _Clock)
    jobs = [{"scene": None, "film": None, "max_verts": 5}]
    best, times = autotune.tune_queue(jobs, repeats=2)
    assert best == 1 << 24
    import pytest
    assert times == pytest.approx(cost)          # the best of two repeats
    assert made == closed == list(autotune.DEFAULT_CANDIDATES)
