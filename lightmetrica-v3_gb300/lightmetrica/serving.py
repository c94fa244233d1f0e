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

    def set_spp(self, job: int, spp: int) -> int:
        """Moves a job's sample count between runs (down to stop early, up to at most the spp it
        was submitted with); passes already started stay. Returns the count now in effect."""
        out = C.c_int32()
        N.check(N.lib().lmgpu_batch_job_set_spp(self._h, int(job), int(spp), C.byref(out)))
        return out.value

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

    def render_to_error(self, jobs: list[dict], target: float, spp_first: int = 8, eps: float = 1e-2,
                        chunks: int = 2) -> list[dict]:
        """Renders every job ({scene, film, max_verts, spp, seed, ...}; spp is the most it may
        render) progressively until its film's relative-MSE estimate is at or below `target`, all
        in the one shared wavefront: each job starts with spp_first passes; whenever a job is done
        at its current count the host reads its estimate (lmgpu_film_rel_mse over even / odd
        passes) and either finishes it or raises its count to what the 1/N fall-off predicts
        (lmgpu_batch_job_set_spp); the other jobs keep the queue full meanwhile. Returns per job
        {job, spp, rel_mse, rounds}."""
        from . import next_spp_for_error
        info = []
        for j in jobs:
            budget = int(j["spp"])
            jid = self.submit(j["scene"], j["film"], split=True,
                              **{k: v for k, v in j.items() if k not in ("scene", "film", "split")})
            cur = self.set_spp(jid, min(budget, max(2, spp_first)))
            info.append({"job": jid, "film": j["film"], "budget": budget, "spp": cur, "rel_mse": None, "rounds": 1})
        pending = list(range(len(info)))
        while pending:
            left = self.run(chunks)
            still = []
            moved = 0
            for k in pending:
                r = info[k]
                _, done = self.status(r["job"])
                if not done:
                    still.append(k)
                    continue
                moved += 1
                err = r["film"].rel_mse(eps)
                r["rel_mse"] = err
                if err <= target or r["spp"] >= r["budget"]:
                    self.resolve(r["job"])
                    continue
                want = min(r["budget"], max(next_spp_for_error(r["spp"], err, target), r["spp"] + 1))
                r["spp"] = self.set_spp(r["job"], want)
                r["rounds"] += 1
                still.append(k)
            if left == 0 and moved == 0 and still:
                raise RuntimeError("render_to_error: the wavefront drained with jobs unfinished")
            pending = still
        return [{k: r[k] for k in ("job", "spp", "rel_mse", "rounds")} for r in info]

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
    target: float | None = None  # render until the film's rel-MSE estimate <= target (spp: the most it may take)
    # filled by the server
    admitted: float | None = None
    first_image: float | None = None
    done: float | None = None
    job: int | None = None
    film: Any = None
    pass_times: list = None      # completion time of each of its sample passes
    base_passes: int = 0         # passes the film held before this request (refinements)
    rel_mse: float | None = None  # estimated relative MSE of the finished image
    spp_run: int = 0             # samples per pixel rendered (target requests stop early)
    target_time: float | None = None  # when the server read an estimate at or below `target`
    rounds: int = 0              # error checks of a target request
    cancelled: bool = False      # RenderServer.cancel: stopped at the passes it had started
    error: str | None = None     # why the request failed (its scene build raised or timed out)


class RequestFailed(RuntimeError):
    """A request the server cannot serve; it is recorded in RenderServer.failed with the reason."""


class SceneBuildError(RequestFailed):
    """A scene build for a request failed (make_scene raised, e.g. out of device memory) or did
    not finish within the server's build_timeout."""


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
        self.spp_first = 8                    # first error check of a target request
        self._pool = ThreadPoolExecutor(build_threads) if build_threads > 0 else None
        self._building: dict[Any, Any] = {}  # scene key -> future of (scene, build seconds)
        self._build_started: dict[Any, float] = {}
        self.build_timeout: float | None = None  # seconds a scene build may take before its requests fail
        self.failed: list[Request] = []           # requests whose scene build failed
        self.cancelled: list[Request] = []
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
            if base.error is not None or base.cancelled:
                raise RequestFailed(f"request {req.rid} refines request {base.rid}, which "
                                    + ("failed" if base.error is not None else "was cancelled"))
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
            req.base_passes = base.base_passes + base.spp_run
        req.pass_times = []
        if req.target is not None and not self.track_error:
            raise ValueError("target requests need track_error (split passes)")
        req.job = self.batch.submit(scene, req.film, max_verts=req.max_verts, spp=req.spp, seed=req.seed,
                                    accumulate=accumulate, split=self.track_error)
        req.spp_run = req.spp
        if req.target is not None:
            req.spp_run = self.batch.set_spp(req.job, min(req.spp, max(2, self.spp_first)))
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
        on the worker threads, or runs here when there are none). Raises SceneBuildError when the
        build raised, or ran longer than build_timeout (the worker is then abandoned: a Python
        thread cannot be stopped, its late result is dropped)."""
        if self._pool is None:
            try:
                return self._build(key)
            except Exception as e:
                raise SceneBuildError(f"scene {key!r}: {e}") from e
        fut = self._building.get(key)
        if fut is None:
            self._building[key] = self._pool.submit(self._build, key)
            self._build_started[key] = self.clock()
            return None
        if not fut.done():
            if self.build_timeout is not None and self.clock() - self._build_started[key] > self.build_timeout:
                del self._building[key]
                raise SceneBuildError(f"scene {key!r}: build did not finish within {self.build_timeout} s")
            return None
        del self._building[key]
        try:
            return fut.result()
        except Exception as e:
            raise SceneBuildError(f"scene {key!r}: {e}") from e

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
            try:
                admitted = self._try_admit(req)
            except RequestFailed as e:
                # the request fails; the others go on, and a later request for the key builds again
                req.error = str(e)
                req.done = self.clock()
                self.failed.append(req)
                continue
            if not admitted:
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
            if done and req.target is not None:
                # progressive to a target error: finish, or raise the count the estimate asks for
                req.rounds += 1
                req.rel_mse = req.film.rel_mse(self.rel_mse_eps)
                if req.rel_mse <= req.target:
                    req.target_time = now
                elif req.spp_run < req.spp:
                    from . import next_spp_for_error
                    want = min(req.spp, max(next_spp_for_error(req.spp_run, req.rel_mse, req.target), req.spp_run + 1))
                    req.spp_run = self.batch.set_spp(req.job, want)
                    remaining.append(req)
                    continue
            if done:
                self.batch.resolve(req.job)
                req.done = now
                if self.track_error and req.target is None and req.base_passes + req.spp_run >= 2:
                    req.rel_mse = req.film.rel_mse(self.rel_mse_eps)
                if req.first_image is None:
                    req.first_image = now
                self.scene_users[req.scene_key] -= 1
                self.scene_last_use[req.scene_key] = now
                (self.cancelled if req.cancelled else self.finished).append(req)
            else:
                remaining.append(req)
        self.inflight = remaining

    def cancel(self, rid: int) -> bool:
        """Cancels a request. Waiting: it is dropped. In flight: its job stops at the sample passes
        it has already started (lmgpu_batch_job_set_spp; paths on the device are not aborted), and
        it leaves the loop when those are done, apart from the finished requests. Returns False
        for a request that has already finished or failed."""
        req = self.by_id[rid]
        if req.done is not None or req.cancelled:
            return False
        req.cancelled = True
        if req in self.pending:
            self.pending.remove(req)
            req.done = self.clock()
            self.cancelled.append(req)
            return True
        req.target = None
        req.spp_run = self.batch.set_spp(req.job, 1)
        return True

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
    def time_to_target(req: Request) -> float | None:
        """Seconds from arrival until the server read an error estimate at or below the request's
        target (measured at the error check, not extrapolated), or None if it never did."""
        if req.target is None or req.target_time is None:
            return None
        return req.target_time - req.arrival

    def latencies(self) -> dict:
        """p50/p99 over every finished request of time-to-first-image and time-to-done (from
        arrival, seconds); with error tracking the finished images' relative-MSE estimates; for
        target requests the measured time-to-target over those that reached it, the fraction that
        did, and the samples per pixel they took."""
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
        tgt = [r for r in self.finished if r.target is not None]
        if tgt:
            ts = [self.time_to_target(r) for r in tgt]
            reached = [t for t in ts if t is not None]
            spp = [r.spp_run for r in tgt]
            out["target_requests"] = len(tgt)
            out["reached_target"] = len(reached) / len(tgt)
            out["time_to_target_p50"] = float(np.percentile(reached, 50)) if reached else None
            out["time_to_target_p99"] = float(np.percentile(reached, 99)) if reached else None
            out["target_spp_p50"] = float(np.percentile(spp, 50))
            out["target_spp_p99"] = float(np.percentile(spp, 99))
            out["target_rounds_mean"] = float(np.mean([r.rounds for r in tgt]))
        return out
