"""Autotuning of the shared wavefront's launch shape.

The only free parameter of the shared wavefront that changes its speed but not its images is the
number of paths in flight (the queue size): too small and the trace kernels do not fill the
device's 152 SMs once paths start to die; too large and the queues fall out of L2 and each
CUDA-graph chunk takes longer to react to new jobs. `tune_queue` renders a probe set of jobs at
each candidate size and keeps the fastest (wall clock, host overhead included).
"""
from __future__ import annotations

import time

from .serving import BatchRenderer

DEFAULT_CANDIDATES = (1 << 22, 1 << 23, 1 << 24, 1 << 25)


def tune_queue(jobs: list[dict], candidates=DEFAULT_CANDIDATES, repeats: int = 1) -> tuple[int, dict]:
    """jobs: BatchRenderer.render() job dicts (their films are overwritten). Returns the fastest
    queue size and {size: seconds}."""
    times = {}
    for q in candidates:
        b = BatchRenderer(queue_paths=q)
        try:
            j0 = jobs[0]
            b.submit(j0["scene"], j0["film"], max_verts=j0["max_verts"], spp=1, seed=0)  # graph capture, warm caches
            b.run(0)
            best = float("inf")
            for _ in range(repeats):
                b.reset()
                t = time.perf_counter()
                b.render(jobs)
                best = min(best, time.perf_counter() - t)
            times[q] = best
        finally:
            b.close()
    return min(times, key=times.get), times
