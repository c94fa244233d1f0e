"""Batched and served rendering on top of the shared GPU wavefront (lmgpu_batch_* in include/lmgpu.h).

The reference renders one job at a time (renderer_pt.cpp:80-315 under scheduler::spp::sample).
Two serving-side patterns come on top of it here; they change only how work is scheduled, never
the estimator or the intersection arithmetic:

* BatchRenderer -- many uneven jobs (scene, film, spp, path length) share one persistent
  wavefront: every path carries its job id, and finished paths are replaced by new ones from the
  same or the next job, so the GPU stays full even when each job alone would not fill it. Each
  job's film equals what renderer::pt gives for it alone (same random streams).
* RenderServer -- a resident request loop: requests arrive over time and are admitted as slots and
  HBM allow (each scene's measured device footprint counts against a budget; idle scenes are
  evicted least-recently-used), their paths join the wavefront already in flight (continuous
  batching), scenes stay resident so progressive refinements (+spp on an existing film) reuse the
  BVH and the film accumulator, and per-request time-to-first-image and time-to-completion are
  recorded for p50/p99 reporting.
"""
from __future__ import annotations

import ctypes as C
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass
from typing import Any

import numpy as np

from . import _native as N

_MODES = {"naive": 0, "nee": 1, "mis": 2}
_PRIMARY = {"pixel": 0, "image": 1}


def _params(spp: int, max_verts: int, seed: int, sampling_mode: str = "mis", primary: str = "pixel",
            accumulate: bool = False, split: bool = False) -> N.PTParams:
    p = N.PTParams()
    p.spp = int(spp)
    p.max_verts = int(max_verts)
    p.seed = int(seed) & 0xFFFFFFFF
    p.sampling_mode = _MODES[sampling_mode]
    p.primary_mode = _PRIMARY[primary]
    p.accumulate = int(bool(accumulate))
    p.split_passes = int(bool(split))
    return p


class BatchRenderer:
    """Many path-tracing jobs in one shared wavefront (see module docstring)."""

    def __init__(self, queue_paths: int = 0):
        h = C.c_void_p()
        N.check(N.lib().lmgpu_batch_create(C.byref(h), int(queue_paths)))
        self._h = h
        self._keep: list[Any] = []

    def close(self) -> None:
        if getattr(self, "_h", None):
            N.lib().lmgpu_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, scene, film, *, max_verts: int, spp: int, seed: int = 0, sampling_mode: str = "mis",
               primary_ray_sampling_mode: str = "pixel", accumulate: bool = False, split: bool = False) -> int:
        """Queues a renderer::pt job (`scene` built, `film` a film::bitmap); returns its job id.
        split: even and odd sample passes accumulate apart, for film.rel_mse()."""
        scene._require_built()
        job = C.c_int32()
        p = _params(spp, max_verts, seed, sampling_mode, primary_ray_sampling_mode, accumulate, split)
        N.check(N.lib().lmgpu_batch_submit(self._h, scene._h, film._h, C.byref(p), C.byref(job)))
        self._keep.append((scene, film))
        return job.value

    def run(self, max_chunks: int = 0) -> int:
        """Advances the wavefront (max_chunks chunks of 8 bounce iterations; 0 = until every
        submitted path is done). Returns the paths still in flight or waiting."""
        left = C.c_int64()
        N.check(N.lib().lmgpu_batch_run(self._h, int(max_chunks), None, C.byref(left)))
        return left.value

    def status(self, job: int) -> tuple[int, bool]:
        """(complete spp passes, done) as of the last run()."""
        passes, done = C.c_int32(), C.c_int32()
        N.check(N.lib().lmgpu_batch_job_status(self._h, int(job), C.byref(passes), C.byref(done)))
        return passes.value, bool(done.value)

    def resolve(self, job: int) -> None:
        """Rescales a finished job's film so film.buffer() reads the estimate."""
        N.check(N.lib().lmgpu_batch_resolve(self._h, int(job), None))

    def stats(self) -> dict:
        st = N.RenderStats()
        N.check(N.lib().lmgpu_batch_get_stats(self._h, C.byref(st)))
        return {"paths": st.paths, "rays": st.rays, "extension_rays": st.extension_rays, "shadow_rays": st.shadow_rays,
                "device_ms": st.elapsed_ms}

    def reset(self) -> None:
        N.check(N.lib().lmgpu_batch_reset(self._h))
        self._keep.clear()

    def render(self, jobs: list[dict]) -> list[int]:
        """Submits every job ({scene, film, max_verts, spp, seed, ...}), runs to completion and
        resolves the films. Returns the job ids."""
        ids = [self.submit(j["scene"], j["film"], **{k: v for k, v in j.items() if k not in ("scene", "film")})
               for j in jobs]
        self.run(0)
        for i in ids:
            self.resolve(i)
        return ids


def scene_footprint(scene) -> int:
    """Device bytes a built scene holds: accel nodes + triangles, shading data and tables."""
    acc = scene.accel().stats()
    b = C.c_int64()
    N.check(N.lib().lmgpu_scene_device_bytes(scene._h, C.byref(b)))
    return int(acc["device_bytes"]) + int(b.value)


def _release_scene(scene) -> None:
    """Frees a scene's device tables and its accel's BVH."""
    acc = scene.accel()
    scene._release()
    if acc is not None and hasattr(acc, "_release"):
        acc._release()


@dataclass
class Request:
    """A render request: `scene_key` names a resident scene (or one `make_scene` builds on
    admission); `refine` names an earlier request whose film receives `spp` more samples."""
    rid: int
    arrival: float
    scene_key: Any
    w: int
    h: int
    spp: int
    max_verts: int
    seed: int
    refine: int | None = None
    # filled by the server
    admitted: float | None = None
    first_image: float | None = None
    done: float | None = None
    job: int | None = None
    film: Any = None
    pass_times: list = None      # completion time of each of its sample passes
    base_passes: int = 0         # passes the film held before this request (refinements)
    rel_mse: float | None = None  # estimated relative MSE of the finished image


class RenderServer:
    """Resident request loop with continuous batching and HBM-budget admission.

    make_scene(scene_key) -> a built `lightmetrica` scene whose asset names are unique to the key
    (loading an existing asset name replaces that asset). With build_threads > 0 it runs on worker
    threads, so the wavefront keeps serving admitted requests while a scene builds (the native
    build releases the GIL). Scenes are cached by key; their
    measured device footprint plus the films of admitted requests count against hbm_budget.
    A request waits when admitting it would exceed the budget or the in-flight request limit; idle
    scenes (no admitted request uses them) are evicted least-recently-used to make room.
    """

    def __init__(self, make_scene, hbm_budget: int, queue_paths: int = 0, max_inflight: int = 256,
                 chunks_per_step: int = 1, clock=time.perf_counter, build_threads: int = 1):
        self.make_scene = make_scene
        self.budget = int(hbm_budget)
        self.max_inflight = max_inflight
        self.chunks = chunks_per_step
        self.clock = clock
        self.batch = BatchRenderer(queue_paths)
        self.scenes: dict[Any, tuple[Any, int]] = {}    # key -> (scene, bytes)
        self.scene_users: dict[Any, int] = {}
        self.scene_last_use: dict[Any, float] = {}
        self.pending: list[Request] = []
        self.inflight: list[Request] = []
        self.finished: list[Request] = []
        self.by_id: dict[int, Request] = {}
        self.resident_bytes = 0
        self.peak_resident_bytes = 0
        self.evictions = 0
        self.owns_scenes = True  # False: make_scene hands out scenes the caller keeps; eviction only forgets them
        self.scene_builds = 0
        self.scene_build_seconds = 0.0
        self.footprints: dict[Any, int] = {}  # measured device bytes per scene key
        self.track_error = True               # split passes: each finished image's rel-MSE estimate
        self.rel_mse_eps = 1e-2
        self._pool = ThreadPoolExecutor(build_threads) if build_threads > 0 else None
        self._building: dict[Any, Any] = {}  # scene key -> future of (scene, build seconds)
        self._film_seq = 0

    # -- admission -------------------------------------------------------------------------------
    def submit(self, req: Request) -> None:
        self.by_id[req.rid] = req
        self.pending.append(req)

    def _film_bytes(self, req: Request) -> int:
        return 0 if req.refine is not None else req.w * req.h * 3 * 4 * 2

    def _evictable(self, keep=None) -> int:
        return sum(nb for k, (_, nb) in self.scenes.items() if self.scene_users.get(k, 0) == 0 and k != keep)

    def _evict_for(self, need: int, keep=None) -> bool:
        """Makes `need` more bytes fit by evicting idle scenes (least recently used first, never
        `keep`). Evicts nothing and returns False when even evicting every idle scene would not do."""
        if self.resident_bytes + need <= self.budget:
            return True
        if self.resident_bytes - self._evictable(keep) + need > self.budget:
            return False
        idle = sorted(((t, k) for k, t in self.scene_last_use.items() if self.scene_users.get(k, 0) == 0 and k != keep),
                      key=lambda e: e[0])
        for _, k in idle:
            if self.resident_bytes + need <= self.budget:
                break
            scene, nbytes = self.scenes.pop(k)
            if self.owns_scenes:
                _release_scene(scene)
            self.resident_bytes -= nbytes
            del self.scene_last_use[k]
            self.scene_users.pop(k, None)
            self.evictions += 1
        return self.resident_bytes + need <= self.budget

    def _try_admit(self, req: Request) -> bool:
        if len(self.inflight) >= self.max_inflight:
            return False
        if req.refine is not None:
            base = self.by_id[req.refine]
            if base.done is None:
                return False  # refine a finished image only
            if base.film is None:
                raise ValueError(f"request {req.rid} refines request {req.refine}, whose film was released")
        need = self._film_bytes(req)
        if req.scene_key not in self.scenes:
            # a scene measured before is not rebuilt until its footprint fits
            known = self.footprints.get(req.scene_key)
            if known is not None and req.scene_key not in self._building and not self._evict_for(need + known):
                return False
            built = self._scene_ready(req.scene_key)
            if built is None:
                return False
            scene, secs = built
            self.scene_builds += 1
            self.scene_build_seconds += secs
            nbytes = scene_footprint(scene)
            self.footprints[req.scene_key] = nbytes
            if not self._evict_for(need + nbytes):
                if self.owns_scenes:
                    _release_scene(scene)
                return False
            self.scenes[req.scene_key] = (scene, nbytes)
            self.resident_bytes += nbytes
        else:
            if not self._evict_for(need, keep=req.scene_key):
                return False
        scene, _ = self.scenes[req.scene_key]
        import lightmetrica as lm
        if req.refine is not None:
            req.film = self.by_id[req.refine].film
            accumulate = True
        else:
            self._film_seq += 1
            req.film = lm.load_film(f"__served_film_{self._film_seq}", "bitmap", w=req.w, h=req.h)
            accumulate = False
        self.resident_bytes += need
        self.peak_resident_bytes = max(self.peak_resident_bytes, self.resident_bytes)
        if req.refine is not None:
            base = self.by_id[req.refine]
            req.base_passes = base.base_passes + base.spp
        req.pass_times = []
        req.job = self.batch.submit(scene, req.film, max_verts=req.max_verts, spp=req.spp, seed=req.seed,
                                    accumulate=accumulate, split=self.track_error)
        req.admitted = self.clock()
        self.scene_users[req.scene_key] = self.scene_users.get(req.scene_key, 0) + 1
        self.scene_last_use[req.scene_key] = req.admitted
        self.inflight.append(req)
        return True

    def _build(self, key):
        t0 = time.perf_counter()
        scene = self.make_scene(key)
        return scene, time.perf_counter() - t0

    def _scene_ready(self, key):
        """(scene, build seconds) once the scene for `key` is built, else None (a build is started
        on the worker threads, or runs here when there are none)."""
        if self._pool is None:
            return self._build(key)
        fut = self._building.get(key)
        if fut is None:
            self._building[key] = self._pool.submit(self._build, key)
            return None
        if not fut.done():
            return None
        del self._building[key]
        return fut.result()

    def close(self) -> None:
        if self._pool is not None:
            self._pool.shutdown(wait=True)
            self._pool = None
        self.batch.close()

    # -- loop ------------------------------------------------------------------------------------
    def step(self) -> None:
        """Admits what fits, advances the wavefront one step, and records progress."""
        still = []
        for req in self.pending:
            if not self._try_admit(req):
                still.append(req)
        self.pending = still
        if not self.inflight:
            if self._building:
                time.sleep(2e-4)  # waiting for a scene build only: let the worker run
            return
        self.batch.run(self.chunks)
        now = self.clock()
        remaining = []
        for req in self.inflight:
            passes, done = self.batch.status(req.job)
            if req.first_image is None and passes >= 1:
                req.first_image = now
            if passes > len(req.pass_times):
                req.pass_times.extend([now] * (passes - len(req.pass_times)))
            if done:
                self.batch.resolve(req.job)
                req.done = now
                if self.track_error and req.base_passes + req.spp >= 2:
                    req.rel_mse = req.film.rel_mse(self.rel_mse_eps)
                if req.first_image is None:
                    req.first_image = now
                self.scene_users[req.scene_key] -= 1
                self.scene_last_use[req.scene_key] = now
                self.finished.append(req)
            else:
                remaining.append(req)
        self.inflight = remaining

    def release(self, rid: int) -> None:
        """Frees a finished request's film (no later request may refine it)."""
        req = self.by_id[rid]
        if req.done is None:
            raise ValueError(f"request {rid} is not finished")
        if any(r.refine == rid for r in self.pending + self.inflight):
            raise ValueError(f"request {rid} has a refinement waiting")
        if req.film is not None and req.refine is None:
            req.film._release()
            self.resident_bytes -= self._film_bytes(req)
        req.film = None

    def idle(self) -> bool:
        return not self.pending and not self.inflight

    @staticmethod
    def time_to_rel_mse(req: Request, target: float) -> float | None:
        """Seconds from arrival until the request's image reached relative MSE `target`, or None if
        its passes never did. The error of an N-pass estimate falls as 1/N, so with the finished
        image's estimate e over N passes, pass k = ceil(N * e / target) of the film is the first
        at or below target (0 for a refinement whose base image was already there)."""
        if req.rel_mse is None or not req.pass_times:
            return None
        total = req.base_passes + req.spp
        k = int(np.ceil(total * req.rel_mse / target - 1e-9))
        if k > total:
            return None
        own = k - req.base_passes
        if own <= 0:
            return 0.0
        return req.pass_times[own - 1] - req.arrival

    def latencies(self, rel_mse_targets=(1e-3, 1e-2)) -> dict:
        """p50/p99 of time-to-first-image and time-to-done (from arrival, seconds); with error
        tracking also the finished images' relative MSE and, per target, the time to reach it over
        the requests that did and the fraction that did."""
        tfi = np.array([r.first_image - r.arrival for r in self.finished])
        ttd = np.array([r.done - r.arrival for r in self.finished])
        if len(ttd) == 0:
            return {}
        out = {"requests": len(ttd), "ttfi_p50": float(np.percentile(tfi, 50)), "ttfi_p99": float(np.percentile(tfi, 99)),
               "done_p50": float(np.percentile(ttd, 50)), "done_p99": float(np.percentile(ttd, 99)),
               "evictions": self.evictions}
        errs = [r.rel_mse for r in self.finished if r.rel_mse is not None]
        if errs:
            out["rel_mse_p50"] = float(np.percentile(errs, 50))
            out["rel_mse_p99"] = float(np.percentile(errs, 99))
            for t in rel_mse_targets:
                ts = [x for x in (self.time_to_rel_mse(r, t) for r in self.finished) if x is not None]
                key = f"{t:g}"
                out[f"time_to_rel_mse_{key}_p50"] = float(np.percentile(ts, 50)) if ts else None
                out[f"time_to_rel_mse_{key}_p99"] = float(np.percentile(ts, 99)) if ts else None
                out[f"reached_rel_mse_{key}"] = len(ts) / len(self.finished)
        return out
