"""RenderServer's host logic (admission by measured HBM footprint, least-recently-used eviction of
idle scenes, the in-flight limit, refinements on a finished film, film release) on the CPU: the
shared wavefront is replaced by a fake that finishes one sample pass per step, and scenes and
films by objects with a byte size. The GPU tests run the same server on the real wavefront."""
import pytest


class FakeBatch:
    def __init__(self, queue_paths=0):
        self.jobs = {}

    def submit(self, scene, film, *, max_verts, spp, seed=0, accumulate=False, split=False, **kw):
        j = len(self.jobs)
        self.jobs[j] = {"spp": spp, "budget": spp, "passes": 0, "film": film, "accumulate": accumulate}
        film.job = self.jobs[j]
        return j

    def set_spp(self, job, spp):
        j = self.jobs[job]
        j["spp"] = max(min(spp, j["budget"]), j["passes"])
        return j["spp"]

    def run(self, chunks=0):
        for j in self.jobs.values():
            j["passes"] = min(j["spp"], j["passes"] + 1)

    def status(self, job):
        j = self.jobs[job]
        return j["passes"], j["passes"] >= j["spp"]

    def resolve(self, job):
        pass

    def close(self):
        pass


class FakeScene:
    def __init__(self, key, nbytes):
        self.key, self.nbytes, self.released = key, nbytes, False


class FakeFilm:
    """err0: the relative MSE of one pass; an N-pass image reads err0 / N."""

    def __init__(self, err0=0.08):
        self.released = False
        self.err0 = err0

    def rel_mse(self, eps=1e-2):
        return self.err0 / max(1, self.job["passes"])

    def _release(self):
        self.released = True


@pytest.fixture
def server(monkeypatch):
    from lightmetrica import serving
    import lightmetrica as lm
    monkeypatch.setattr(serving, "BatchRenderer", FakeBatch)
    monkeypatch.setattr(serving, "scene_footprint", lambda s: s.nbytes)
    released = []
    monkeypatch.setattr(serving, "_release_scene", lambda s: released.append(s.key))
    monkeypatch.setattr(lm, "load_film", lambda *a, **k: FakeFilm())
    sizes = {"A": 400, "B": 400, "C": 400, "huge": 5000}
    t = [0.0]

    def clock():
        t[0] += 1.0
        return t[0]
    srv = serving.RenderServer(lambda key: FakeScene(key, sizes[key]), hbm_budget=1000, max_inflight=3, clock=clock,
                               build_threads=0)
    srv.track_error = False
    srv.released = released
    yield srv
    srv.close()


def _req(rid, key, spp=2, w=2, h=2, refine=None):
    from lightmetrica.serving import Request
    return Request(rid=rid, arrival=0.0, scene_key=key, w=w, h=h, spp=spp, max_verts=5, seed=rid, refine=refine)


FILM = 2 * 2 * 3 * 4 * 2   # a 2x2 film: sum and split-pass buffers, fp32


def test_admission_waits_for_budget_then_evicts_lru(server):
    server.submit(_req(0, "A", spp=1))
    server.submit(_req(1, "B", spp=3))
    server.step()                       # both admitted; A finishes its one pass in this step
    assert [r.rid for r in server.inflight] == [1] and server.by_id[0].done is not None
    assert set(server.scenes) == {"A", "B"} and server.resident_bytes == 800 + 2 * FILM
    server.submit(_req(2, "C"))
    server.step()                       # C does not fit while A and B render
    assert [r.rid for r in server.pending] == [2]
    while server.inflight:
        server.step()
    server.release(0)
    server.release(1)
    server.step()                       # A and B idle: C evicts the least recently used (A)
    assert [r.rid for r in server.inflight] == [2]
    # C was built once to measure it and released (no room); then A, idle longest, was evicted
    assert server.released == ["C", "A"] and server.evictions == 1 and server.scene_builds == 4
    assert set(server.scenes) == {"B", "C"}
    assert server.peak_resident_bytes <= server.budget


def test_scene_larger_than_budget_is_never_admitted(server):
    server.submit(_req(0, "huge"))
    for _ in range(3):
        server.step()
    assert [r.rid for r in server.pending] == [0] and not server.scenes
    assert server.released == ["huge"] * 3 or server.released[:1] == ["huge"]
    assert server.footprints["huge"] == 5000


def test_inflight_limit(server):
    for i in range(5):
        server.submit(_req(i, "A", spp=4))
    server.step()
    assert len(server.inflight) == 3 and len(server.pending) == 2
    assert server.scene_users["A"] == 3


def test_refinement_reuses_the_finished_film(server):
    server.submit(_req(0, "A", spp=2))
    server.submit(_req(1, "A", spp=3, refine=0))
    server.step()
    assert [r.rid for r in server.pending] == [1]      # waits for its base to finish
    while not server.idle():
        server.step()
    base, ref = server.by_id[0], server.by_id[1]
    assert ref.film is base.film and ref.base_passes == 2
    assert server.batch.jobs[ref.job]["accumulate"]
    assert server.resident_bytes == 400 + FILM          # the refinement adds no film
    assert ref.first_image is not None and ref.done >= ref.first_image >= ref.admitted


def test_release_frees_film_and_guards_refinements(server):
    server.submit(_req(0, "A"))
    while not server.idle():
        server.step()
    film = server.by_id[0].film
    server.submit(_req(1, "A", refine=0))
    with pytest.raises(ValueError):
        server.release(0)                              # a refinement still waits for this film
    while not server.idle():
        server.step()
    server.release(0)
    assert film.released and server.resident_bytes == 400
    server.submit(_req(2, "A", refine=0))
    with pytest.raises(ValueError):
        server.step()                                  # refining a released film


def test_target_requests_stop_at_the_error_and_report_measured_latency(server):
    """A request with a target renders spp_first passes, reads the estimate, raises its count to
    what the 1/N fall-off predicts and finishes once the estimate is at or below the target; its
    time-to-target is the clock at that check, not an extrapolation. A target its budget cannot
    reach ends at the budget and counts as not reached."""
    from lightmetrica.serving import Request
    server.track_error = True
    server.spp_first = 4
    ok = Request(rid=0, arrival=0.0, scene_key="A", w=2, h=2, spp=64, max_verts=5, seed=0, target=0.005)
    short = Request(rid=1, arrival=0.0, scene_key="A", w=2, h=2, spp=8, max_verts=5, seed=1, target=0.005)
    server.submit(ok)
    server.submit(short)
    for _ in range(200):
        if server.idle():
            break
        server.step()
    assert server.idle()
    # err0 / N <= 0.005 needs N >= 16: 4 passes (0.02), then ceil(4 * 0.02 / 0.005 * 1.05) = 17
    assert ok.spp_run == 17 and ok.rel_mse <= 0.005 and ok.rounds == 2
    assert ok.target_time is not None and server.time_to_target(ok) == ok.target_time - ok.arrival
    assert short.spp_run == 8 and short.target_time is None and short.rel_mse > 0.005
    lat = server.latencies()
    assert lat["target_requests"] == 2 and lat["reached_target"] == 0.5
    assert lat["time_to_target_p50"] == server.time_to_target(ok)


def test_cancel_waiting_and_in_flight_requests(server):
    """A waiting request is dropped; one in flight stops at the passes it has started and leaves
    the loop apart from the finished requests (the reference's parallel loop stops on an
    exception and rethrows it, parallel_openmp.cpp:41-99; here one request stops, the rest go on)."""
    server.submit(_req(0, "A", spp=6))
    server.submit(_req(1, "A", spp=6))
    server.step()                      # both admitted, one pass each
    server.submit(_req(2, "B", spp=3))
    assert server.cancel(2)            # still waiting: dropped
    assert server.cancel(0)            # in flight: stops at the started pass
    while not server.idle():
        server.step()
    r0, r1, r2 = (server.by_id[i] for i in range(3))
    assert r0.cancelled and r0.spp_run == 1 and r0 in server.cancelled
    assert r2.cancelled and r2.job is None and r2 in server.cancelled
    assert [r.rid for r in server.finished] == [1] and r1.spp_run == 6
    assert server.latencies()["requests"] == 1
    assert not server.cancel(1)        # already finished
    assert server.scene_users["A"] == 0


def test_failed_scene_build_fails_its_request_only(server, monkeypatch):
    """A scene build that raises (here the fake allocator's out-of-memory on the second build)
    fails the requests that needed it; the others are served, a refinement of a failed request
    fails too, and a later request for the same scene builds it again."""
    from lightmetrica import _native as N
    calls = []
    make = server.make_scene

    def flaky(key):
        calls.append(key)
        if len(calls) == 2:
            raise N.LmGpuError(5, "cudaMalloc: out of memory")
        return make(key)
    server.make_scene = flaky
    server.submit(_req(0, "A", spp=2))
    server.submit(_req(1, "B", spp=2))
    server.submit(_req(2, "A", spp=1))
    for _ in range(20):
        server.step()
    assert server.by_id[1].error and "out of memory" in server.by_id[1].error
    assert [r.rid for r in server.failed] == [1]
    assert sorted(r.rid for r in server.finished) == [0, 2]
    server.submit(_req(3, "B", spp=2, refine=1))
    server.submit(_req(4, "B", spp=2))
    for _ in range(20):
        server.step()
    assert "refines request 1" in server.by_id[3].error
    assert server.by_id[4].done is not None and server.by_id[4].error is None and calls.count("B") == 2


def test_stuck_scene_build_times_out(monkeypatch):
    """A build worker that never returns: its request fails after build_timeout seconds and the
    server keeps serving; the worker's late result is dropped."""
    import threading
    from lightmetrica import serving
    import lightmetrica as lm
    monkeypatch.setattr(serving, "BatchRenderer", FakeBatch)
    monkeypatch.setattr(serving, "scene_footprint", lambda s: s.nbytes)
    monkeypatch.setattr(serving, "_release_scene", lambda s: None)
    monkeypatch.setattr(lm, "load_film", lambda *a, **k: FakeFilm())
    gate = threading.Event()
    t = [0.0]

    def clock():
        t[0] += 0.05
        return t[0]

    def make(key):
        if key == "stuck":
            gate.wait(10.0)
        return FakeScene(key, 100)
    srv = serving.RenderServer(make, hbm_budget=10**6, clock=clock, build_threads=2)
    srv.track_error = False
    srv.build_timeout = 1.0
    srv.submit(_req(0, "stuck", spp=2))
    srv.submit(_req(1, "ok", spp=2))
    for _ in range(400):
        if srv.idle():
            break
        srv.step()
        import time
        time.sleep(0.001)
    assert srv.idle()
    assert "did not finish within 1.0 s" in srv.by_id[0].error
    assert srv.by_id[1].done is not None and srv.by_id[1].error is None
    gate.set()
    srv.close()
