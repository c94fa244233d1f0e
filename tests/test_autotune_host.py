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


def test_tune_searches_every_parameter(monkeypatch):
    """tune(): queue size first, then each launch-shape key and the node width (rebuilding the
    probe scenes per width and once more when the last width built is not the choice), keeping
    the fastest candidate of each; the process-wide tuning is left at the choices."""
    from lightmetrica import autotune
    state = {"trace_refill": 24, "shade_minblocks": 4, "shade_specialize": 1, "node_width": 8}
    best = {"trace_refill": 28, "shade_minblocks": 3, "shade_specialize": 1, "node_width": 4}
    rebuilt = []

    def render_time(jobs, queue, repeats):
        t = {1 << 22: 2.0, 1 << 23: 1.5, 1 << 24: 1.0, 1 << 25: 1.2}[queue]
        t += sum(0.1 for k, v in state.items() if v != best[k])
        return t

    monkeypatch.setattr(autotune, "_render_time", render_time)
    monkeypatch.setattr(autotune, "_tune_set", lambda k, v: state.__setitem__(k, v))
    monkeypatch.setattr(autotune, "_tune_get", lambda k: state[k])
    chosen, times = autotune.tune([{}], rebuild=lambda: rebuilt.append(state["node_width"]))
    assert chosen == {"queue_paths": 1 << 24, **best}
    assert state == best
    assert rebuilt == [4, 8, 4]                      # each width, then back to the winner
    assert set(times) == {"queue_paths", "trace_refill", "shade_minblocks", "shade_specialize", "node_width"}
    assert times["trace_refill"][28] < times["trace_refill"][24]
