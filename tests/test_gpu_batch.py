"""The shared wavefront (lmgpu_batch_*): every job's image is the same alone and in the mix, jobs
admitted while others are in flight, progressive refinement, and the served request loop."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = dict(rtol=1e-5, atol=1e-6)  # the order of fp32 film additions is all that differs


@pytest.fixture(scope="module", autouse=True)
def _device(native_lib):
    from lightmetrica import _native as N
    N.check(native_lib.lmgpu_set_device(0))


def _alone(lm, scene, film, **kw):
    r = lm.load_renderer(f"pt_{id(film)}", "pt", scene=scene, output=film, scheduler="sample", **kw)
    r.render()
    return film.buffer_f32().copy()


def _scenes(lm):
    """Three unlike jobs: the box, the spheres (glossy/glass/env) and the box in image mode."""
    from lightmetrica import synthetic as syn
    out = []
    s1, f1 = syn.box_scene(w=24, h=20, prefix="mixbox_")
    s1.build()
    out.append((s1, f1, dict(max_verts=9, spp=8, seed=3)))
    s2, lm_film2, _ = syn.spheres_scene(n_spheres=5, subdiv=3, ground_quads=16, w=32, h=18, prefix="mixsph_")
    s2.build()
    out.append((s2, lm_film2, dict(max_verts=11, spp=4, seed=7)))
    lm_film3 = lm.load_film("film3", "bitmap", w=24, h=20)
    out.append((s1, lm_film3, dict(max_verts=6, spp=5, seed=11, primary_ray_sampling_mode="image")))
    return out


@pytest.mark.parametrize("queue", [1000, 1 << 25])
def test_each_job_same_alone_and_in_mix(lm, queue):
    """A small queue (paths of several jobs share it) and the largest size the autotuner tries."""
    from lightmetrica.serving import BatchRenderer
    jobs = _scenes(lm)
    alone = [_alone(lm, s, f, **kw) for s, f, kw in jobs]
    b = BatchRenderer(queue_paths=queue)
    ids = b.render([dict(scene=s, film=f, **kw) for s, f, kw in jobs])
    for (s, f, kw), a, j in zip(jobs, alone, ids):
        np.testing.assert_allclose(f.buffer_f32(), a, **TOL)
        assert b.status(j) == (kw["spp"], True)
    st = b.stats()
    assert st["rays"] > 0 and st["paths"] == sum(f.w * f.h * kw["spp"] for _, f, kw in jobs)
    b.close()


def test_continuous_batching_admits_while_in_flight(lm):
    """A job submitted after the wavefront started runs alongside the first and still matches its
    standalone render."""
    from lightmetrica.serving import BatchRenderer
    jobs = _scenes(lm)
    alone = [_alone(lm, s, f, **kw) for s, f, kw in jobs[:2]]
    b = BatchRenderer(queue_paths=512)
    j0 = b.submit(jobs[0][0], jobs[0][1], **jobs[0][2])
    left = b.run(max_chunks=1)
    assert left > 0
    j1 = b.submit(jobs[1][0], jobs[1][1], **jobs[1][2])
    b.run(0)
    for j, (s, f, kw), a in zip((j0, j1), jobs[:2], alone):
        assert b.status(j)[1]
        b.resolve(j)
        np.testing.assert_allclose(f.buffer_f32(), a, **TOL)
    b.close()


def test_progressive_refinement_accumulates(lm):
    """+spp on a resident film: two passes equal one render with both passes' samples averaged."""
    from lightmetrica import synthetic as syn
    from lightmetrica.serving import BatchRenderer
    s, f = syn.box_scene(w=16, h=16, prefix="refine_")
    s.build()
    a = _alone(lm, s, f, max_verts=9, spp=8, seed=1)
    g = lm.load_film("g", "bitmap", w=16, h=16)
    c = _alone(lm, s, g, max_verts=9, spp=8, seed=2)
    b = BatchRenderer(queue_paths=2048)
    h = lm.load_film("h", "bitmap", w=16, h=16)
    j0 = b.submit(s, h, max_verts=9, spp=8, seed=1)
    b.run(0)
    b.resolve(j0)
    j1 = b.submit(s, h, max_verts=9, spp=8, seed=2, accumulate=True)
    b.run(0)
    b.resolve(j1)
    np.testing.assert_allclose(h.buffer_f32(), 0.5 * (a + c), rtol=1e-5, atol=2e-6)
    b.close()


def test_render_server_admission_and_latency(lm):
    """Requests arriving over time under a small HBM budget: every request completes, scenes are
    evicted when the budget demands, and refinements reuse the resident film."""
    from lightmetrica import synthetic as syn
    from lightmetrica.serving import RenderServer, Request

    def make_scene(key):
        s, _ = syn.box_scene(seed=key, w=8, h=8, prefix=f"served{key}_")
        s.build()
        return s
    from lightmetrica.serving import scene_footprint
    fps = []
    for key in range(4):
        probe, _ = syn.box_scene(seed=key, w=8, h=8, prefix=f"probe{key}_")
        probe.build()
        fps.append(scene_footprint(probe))
    film = 16 * 12 * 3 * 4 * 2
    # room for every film (ten; the refinement reuses one) and two and a half scenes: the four
    # scenes cannot all stay resident, so some idle scene is evicted
    budget = 2 * max(fps) + 10 * film + min(fps) // 2
    assert 4 * min(fps) + 10 * film > budget
    srv = RenderServer(make_scene, hbm_budget=budget, queue_paths=4096)
    t0 = srv.clock()
    reqs = []
    for i in range(10):
        reqs.append(Request(rid=i, arrival=t0, scene_key=i % 4, w=16, h=12, spp=4, max_verts=7, seed=i))
    reqs.append(Request(rid=10, arrival=t0, scene_key=0, w=16, h=12, spp=4, max_verts=7, seed=99, refine=0))
    for r in reqs:
        srv.submit(r)
    import time
    t_end = time.time() + 120
    while not srv.idle() and time.time() < t_end:
        srv.step()
    assert srv.idle()
    assert len(srv.finished) == 11
    lat = srv.latencies()
    assert lat["ttfi_p50"] <= lat["done_p50"] and lat["done_p99"] >= lat["done_p50"]
    assert srv.evictions > 0
    assert srv.resident_bytes <= srv.budget
    assert reqs[10].film is reqs[0].film
    # a released film leaves the budget
    before = srv.resident_bytes
    srv.release(1)
    assert srv.resident_bytes == before - film and reqs[1].film is None
    srv.close()


def test_first_pass_priority(lm, native_lib):
    """With batch_first_pass on (the default), a small job submitted while a large one is in
    flight shows its first complete sample pass before the large job finishes; every image is
    still the standalone one."""
    from lightmetrica import synthetic as syn
    from lightmetrica.serving import BatchRenderer
    big_s, big_f = syn.box_scene(w=64, h=64, prefix="fpbig_")
    big_s.build()
    small_s, small_f = syn.box_scene(seed=9, w=8, h=8, prefix="fpsmall_")
    small_s.build()
    a_big = _alone(lm, big_s, big_f, max_verts=8, spp=48, seed=4)
    a_small = _alone(lm, small_s, small_f, max_verts=8, spp=4, seed=6)
    b = BatchRenderer(queue_paths=4096)
    jb = b.submit(big_s, big_f, max_verts=8, spp=48, seed=4)
    b.run(max_chunks=1)
    js = b.submit(small_s, small_f, max_verts=8, spp=4, seed=6)
    chunks_to_first, chunks = None, 0
    while b.run(max_chunks=1) > 0:
        chunks += 1
        if chunks_to_first is None and b.status(js)[0] >= 1:
            chunks_to_first = chunks
            assert not b.status(jb)[1]
    assert chunks_to_first is not None and chunks_to_first <= 2
    for j in (jb, js):
        b.resolve(j)
    np.testing.assert_allclose(big_f.buffer_f32(), a_big, **TOL)
    np.testing.assert_allclose(small_f.buffer_f32(), a_small, **TOL)
    b.close()


def test_split_passes_estimate_relative_mse(lm):
    """Even / odd pass accumulators: the image is unchanged, and the relative-MSE estimate agrees
    with the error against the committed 16k-spp reference and falls as 1/spp."""
    import json
    import os
    from lightmetrica import synthetic as syn
    from lightmetrica.serving import BatchRenderer
    gdir = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    ref = np.load(os.path.join(gdir, "box_ref_16k.npy")).astype(np.float64)
    meta = json.load(open(os.path.join(gdir, "box_ref_16k.json")))
    s, f = syn.box_scene(seed=1234, w=meta["w"], h=meta["h"], prefix="split_")
    s.build()
    plain = _alone(lm, s, f, max_verts=meta["max_verts"], spp=64, seed=5)
    b = BatchRenderer(queue_paths=1 << 16)
    est = {}
    for spp in (16, 64):
        j = b.submit(s, f, max_verts=meta["max_verts"], spp=spp, seed=5, split=True)
        b.run(0)
        b.resolve(j)
        est[spp] = f.rel_mse(1e-2)
        if spp == 64:
            img = f.buffer_f32().astype(np.float64)
            np.testing.assert_allclose(img, plain, **TOL)
            true = float(np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2)))
            assert 0.7 < est[64] / true < 1.4, (est[64], true)
    assert 2.8 < est[16] / est[64] < 5.7, est      # about 4: error falls as 1/spp
    # refinement keeps splitting: 64 + 64 passes halve the estimate again
    j = b.submit(s, f, max_verts=meta["max_verts"], spp=64, seed=6, accumulate=True)
    b.run(0)
    b.resolve(j)
    assert 1.4 < est[64] / f.rel_mse(1e-2) < 2.9
    b.close()


def test_set_spp_stops_and_resumes(lm):
    """lmgpu_batch_job_set_spp: a job stopped after N passes holds exactly the first N passes of
    its submitted render (streams stay keyed by the submitted spp), whether stopped before it
    starts or while it is in flight, and raising the count back completes the submitted render."""
    from lightmetrica.serving import BatchRenderer
    from lightmetrica import synthetic as syn
    s, f = syn.box_scene(w=24, h=20, prefix="sppbox_")
    s.build()
    kw = dict(max_verts=9, spp=16, seed=5)
    full = _alone(lm, s, f, **kw)
    # stopped before the first run, then resumed: the film adds up to the full render
    b = BatchRenderer(queue_paths=1000)
    j = b.submit(s, f, **kw)
    assert b.set_spp(j, 6) == 6
    b.run(0)
    assert b.status(j) == (6, True)
    assert b.set_spp(j, 16) == 16
    assert b.status(j)[1] is False
    b.run(0)
    assert b.status(j) == (16, True)
    b.resolve(j)
    np.testing.assert_allclose(f.buffer_f32(), full, **TOL)
    with pytest.raises(lm.LmGpuError):
        b.set_spp(j, 4)  # resolved
    b.close()
    # stopped in flight: the count becomes at least the passes already started, and the image
    # is the same as that many passes stopped before the start, alone or beside another job
    b = BatchRenderer(queue_paths=2000)
    j = b.submit(s, f, **kw)
    b.run(1)
    n = b.set_spp(j, 3)
    assert 3 <= n <= 16
    b.run(0)
    assert b.status(j) == (n, True)
    b.resolve(j)
    stopped = f.buffer_f32().copy()
    b.close()
    f2 = lm.load_film("spp_f2", "bitmap", w=24, h=20)
    s2, fo, _ = syn.spheres_scene(n_spheres=3, subdiv=2, ground_quads=4, w=16, h=12, prefix="sppsph_")
    s2.build()
    b = BatchRenderer(queue_paths=700)
    other = b.submit(s2, fo, max_verts=8, spp=6, seed=2)
    j2 = b.submit(s, f2, **kw)
    assert b.set_spp(j2, n) == n
    b.run(0)
    assert b.status(j2) == (n, True) and b.status(other) == (6, True)
    b.resolve(j2)
    np.testing.assert_allclose(f2.buffer_f32(), stopped, **TOL)
    with pytest.raises(lm.LmGpuError):
        b.set_spp(other, 7)  # above the submitted spp
    b.close()


def test_render_to_error_reaches_target(lm):
    """Progressive rendering to a target relative MSE: every job of a mix ends at or below the
    target (or at its spp budget), the batched loop and the renderer::pt 'error' scheduler agree on
    the spp each job needs within the estimate's noise, and jobs that are stopped at a count hold
    that many passes."""
    from lightmetrica.serving import BatchRenderer
    from lightmetrica import synthetic as syn
    jobs = []
    for k, (w, h) in enumerate([(32, 32), (48, 40), (24, 24)]):
        s, f = syn.box_scene(seed=100 + k, w=w, h=h, prefix=f"errbox{k}_")
        s.build()
        jobs.append(dict(scene=s, film=f, max_verts=9, spp=4096, seed=20 + k))
    target = 3e-3
    b = BatchRenderer(queue_paths=1 << 16)
    res = b.render_to_error(jobs, target, spp_first=8)
    b.close()
    for r in res:
        assert r["rel_mse"] <= target and 8 <= r["spp"] < 4096, r
    # the same jobs one at a time through renderer::pt's 'error' scheduler
    for j, r in zip(jobs, res):
        f = lm.load_film(f"err_plain_{id(j)}", "bitmap", w=j["film"].w, h=j["film"].h)
        rp = lm.load_renderer(f"err_pt_{id(j)}", "pt", scene=j["scene"], output=f, max_verts=9, seed=j["seed"],
                              scheduler="error", target_rel_mse=target, spp=4096)
        rp.render()
        assert rp.last_rel_mse <= target
        assert 0.5 < rp.last_spp / r["spp"] < 2.0, (rp.last_spp, r)
