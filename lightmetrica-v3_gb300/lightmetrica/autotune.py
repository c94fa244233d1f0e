"""Autotuning of the shared wavefront's launch shape, node width and shade-kernel split.

Everything tuned here changes speed, never images:

* queue_paths -- paths in flight: too few and the trace kernels do not fill the device's 152
  SMs once paths start to die; too many and the queues fall out of L2 and each CUDA-graph chunk
  takes longer to react to new jobs (`tune_queue`);
* trace_refill -- how few busy lanes a persistent trace warp tolerates before its idle lanes
  fetch new rays;
* shade_minblocks -- the register budget of the shade kernels (resident blocks per SM);
* shade_specialize -- the shade-kernel split: kernels specialised for the features present
  (without the code of absent materials and lights) or the one full-feature kernel;
* node_width -- children per BVH node the collapse may use (the 80-byte node keeps 8 slots).

`tune` times each candidate on a probe set of jobs, one parameter at a time in that order, keeps
the fastest (wall clock, host overhead included) and returns the choices with every candidate's
time, which the batched benchmark records.
"""
from __future__ import annotations

import time

from . import _native as N
from .serving import BatchRenderer

DEFAULT_CANDIDATES = (1 << 22, 1 << 23, 1 << 24, 1 << 25)
KEY_CANDIDATES = (("trace_refill", (16, 24, 28)), ("shade_minblocks", (3, 4)), ("shade_specialize", (0, 1)))
WIDTH_CANDIDATES = (4, 8)


def _tune_set(key: str, value: int) -> None:
    N.check(N.lib().lmgpu_tune_set(key.encode(), int(value)))


def _tune_get(key: str) -> int:
    import ctypes as C
    v = C.c_int64()
    N.check(N.lib().lmgpu_tune_get(key.encode(), C.byref(v)))
    return int(v.value)


def _render_time(jobs: list[dict], queue: int, repeats: int) -> float:
    """Best wall-clock seconds of rendering `jobs` on a fresh shared wavefront of `queue` paths
    (one warm-up render of one pass of the first job captures the graph and warms the caches)."""
    b = BatchRenderer(queue_paths=queue)
    try:
        j0 = jobs[0]
        b.submit(j0["scene"], j0["film"], max_verts=j0["max_verts"], spp=1, seed=0)
        b.run(0)
        best = float("inf")
        for _ in range(repeats):
            b.reset()
            t = time.perf_counter()
            b.render(jobs)
            best = min(best, time.perf_counter() - t)
        return best
    finally:
        b.close()


def tune_queue(jobs: list[dict], candidates=DEFAULT_CANDIDATES, repeats: int = 1) -> tuple[int, dict]:
    """jobs: BatchRenderer.render() job dicts (their films are overwritten). Returns the fastest
    queue size and {size: seconds}."""
    times = {q: _render_time(jobs, q, repeats) for q in candidates}
    return min(times, key=times.get), times


def tune(jobs: list[dict], queue_candidates=DEFAULT_CANDIDATES, key_candidates=KEY_CANDIDATES,
         width_candidates=WIDTH_CANDIDATES, rebuild=None, repeats: int = 1) -> tuple[dict, dict]:
    """Coordinate search over queue size, the launch-shape keys and (with `rebuild`, a callable
    that rebuilds the probe jobs' scenes under the current "node_width") the node width. Each
    parameter keeps its fastest candidate before the next one is tried. Leaves the process-wide
    tuning at the choices (the caller rebuilds its other scenes when node_width changed). Returns
    (choices, {parameter: {candidate: seconds}})."""
    queue, tq = tune_queue(jobs, queue_candidates, repeats)
    chosen: dict = {"queue_paths": queue}
    times: dict = {"queue_paths": tq}
    for key, cands in key_candidates:
        res = {}
        for v in cands:
            _tune_set(key, v)
            res[v] = _render_time(jobs, queue, repeats)
        best = min(res, key=res.get)
        _tune_set(key, best)
        chosen[key], times[key] = best, res
    if rebuild is not None and width_candidates:
        res = {}
        built = None
        for w in width_candidates:
            _tune_set("node_width", w)
            rebuild()
            built = w
            res[w] = _render_time(jobs, queue, repeats)
        best = min(res, key=res.get)
        _tune_set("node_width", best)
        if built != best:
            rebuild()
        chosen["node_width"], times["node_width"] = best, res
    return chosen, times
