"""Batch render (rc_batch_render): several scenes, one context each, rendered as one
launch set per iteration (one light pass and one camera pass over all scenes, the
per-scene KD builds and gathers as branches of one CUDA graph).  Each scene's image
must be the one its own context renders alone: the same samples, photons and merges,
with FP64 pixel sums taken in another order."""
import numpy as np
import pytest

from realcausticsengine_gb300 import _native, abi, scenes
from realcausticsengine_gb300.session import Context, Renderer, batch_render


RC_E_NO_SCENE, RC_E_INVALID = -1, -2


def _handles(ctxs):
    import ctypes as C
    return (C.c_void_p * len(ctxs))(*[c.handle for c in ctxs])


def test_batch_rejects_bad_arguments():
    """Null or empty context lists, a repeated context, a context without a scene and a
    scene set up for a Metropolis sampler are refused before any device work."""
    lib = _native.lib()
    assert lib.rc_batch_render(None, 1, 1, None) == RC_E_INVALID
    a, b = Context(), Context()
    try:
        assert lib.rc_batch_render(_handles([a]), 0, 1, None) == RC_E_INVALID
        assert lib.rc_batch_render(_handles([a]), 1, -1, None) == RC_E_INVALID
        assert lib.rc_batch_render(_handles([a, a]), 2, 1, None) == RC_E_INVALID
        assert b"repeated" in lib.rc_last_error()
        assert lib.rc_batch_render(_handles([a, b]), 2, 1, None) == RC_E_NO_SCENE
        assert b"scene 0" in lib.rc_last_error()
        with b:
            Renderer(scenes.test_scene(), sampler=abi.SAMPLER_PSSMLT)
        with a:
            Renderer(scenes.test_scene())
        assert lib.rc_batch_render(_handles([a, b]), 2, 1, None) == RC_E_INVALID
        assert b"Metropolis" in lib.rc_last_error()
    finally:
        for c in (a, b):
            with c:
                lib.rc_release()
            c.destroy()


# (scene, light paths per iteration, max path length, iterations rendered alone before
# the batch, graph_replay setting)
def _specs():
    s3, p3 = scenes.batch_scene(3, 96, 96)      # 3.9k triangles, point/area lights
    s9, _ = scenes.batch_scene(9, 80, 64)       # 1.6k triangles
    return [
        (scenes.test_scene(64, 48), 65536, 6, 0, 1),
        (scenes.glass_sphere_point(96, 64, subdiv=3, light="area"), 100000, 8, 2, 1),
        (s3, min(p3, 300000), 8, 0, 1),
        # tight capacities: iterations that store more photons or queries than the first
        # overflow and are rendered again alone after the batch
        (s9, 150000, 8, 1, 2),
    ]


def _render_alone(sc, paths, depth, seed, iterations, replay):
    ctx = Context()
    with ctx:
        r = Renderer(sc, max_path_length=depth, photons_per_iter=paths, seed=seed, graph_replay=replay)
        r.render(iterations)
        img = r.image()
        r.release()
    ctx.destroy()
    return img


@pytest.mark.gpu
def test_batch_render_equals_per_scene_renders():
    """Scenes with iterations rendered before go straight into the batch; fresh ones
    render their first iteration alone, so the batch's active set shrinks in its last
    iteration (the graph is instantiated again).  Each scene ends with `before` +
    `iterations` iterations and the image its context renders alone for that many."""
    specs = _specs()
    iterations = 4
    ctxs, rs = [], []
    try:
        for k, (sc, p, d, before, rp) in enumerate(specs):
            c = Context()
            ctxs.append(c)
            with c:
                r = Renderer(sc, max_path_length=d, photons_per_iter=p, seed=10 + k, graph_replay=rp)
                rs.append(r)
                if before:
                    r.render(before)
        out = batch_render(ctxs, iterations)
        assert out[1] == iterations and out[2] > 0
        got = []
        for c, r, spec in zip(ctxs, rs, specs):
            with c:
                got.append(r.image())
                assert r.stats()["iterations"] == spec[3] + iterations
        for k, ((sc, p, d, before, rp), g) in enumerate(zip(specs, got)):
            w = _render_alone(sc, p, d, 10 + k, before + iterations, rp)
            assert w.sum() > 0, k
            np.testing.assert_allclose(g, w, rtol=1e-5, atol=1e-7, err_msg=f"scene {k}")
    finally:
        for c in ctxs:
            with c:
                _native.lib().rc_release()
            c.destroy()


@pytest.mark.gpu
def test_batch_calls_continue_each_scenes_iterations():
    """Two batch calls of two iterations each continue every scene's iteration count
    (and radius schedule); a third scene added in the second call starts at its own
    first iteration."""
    specs = _specs()[:3]
    ctxs = []
    for k, (sc, p, d, _, _) in enumerate(specs):
        c = Context()
        with c:
            Renderer(sc, max_path_length=d, photons_per_iter=p, seed=20 + k)
        ctxs.append(c)
    try:
        batch_render(ctxs[:2], 2)
        batch_render(ctxs, 2)
        for k, (c, (sc, p, d, _, _)) in enumerate(zip(ctxs, specs)):
            st = np.zeros(16)
            with c:
                _native.check(_native.lib().rc_get_stats(st.ctypes.data, 16), "rc_get_stats")
                img = np.zeros((sc.camera.height, sc.camera.width, 3), np.float32)
                _native.check(_native.lib().rc_read_image(img.ctypes.data, sc.camera.width, sc.camera.height),
                              "rc_read_image")
            assert st[10] == (4 if k < 2 else 2), (k, st[10])
            n = 4 if k < 2 else 2
            want = _render_alone(sc, p, d, 20 + k, n, 1)
            np.testing.assert_allclose(img, want, rtol=1e-5, atol=1e-7, err_msg=f"scene {k}")
    finally:
        for c in ctxs:
            with c:
                _native.lib().rc_release()
            c.destroy()
