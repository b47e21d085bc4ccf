"""Library contexts: a thread that binds its own context holds its own scene, settings
and last error; threads that bind none share the default context (the reference's one
global scene)."""
import threading

import numpy as np
import pytest

from realcausticsengine_gb300 import _native, scenes
from realcausticsengine_gb300.session import Context, Renderer


def _host_info(sc):
    r = Renderer(sc)
    info = r.prepare_host()
    r.release()
    return info


def test_contexts_hold_separate_scenes_and_errors():
    lib = _native.lib()
    a, b = scenes.test_scene(), scenes.glass_sphere_point(32, 32, subdiv=2)
    want = [_host_info(a), _host_info(b)]          # default context, one after the other
    got, errs = [None, None], [None, None]
    start = threading.Barrier(2)

    def worker(k, sc):
        ctx = Context()
        with ctx:
            r = Renderer(sc)
            start.wait()                            # both scenes loaded before either prepares
            got[k] = r.prepare_host()
            assert lib.rc_render(-1) != 0           # an error in this context only
            errs[k] = lib.rc_last_error()
            r.release()
        ctx.destroy()

    ts = [threading.Thread(target=worker, args=(k, sc)) for k, sc in enumerate((a, b))]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    for k in range(2):
        assert (got[k].view(np.uint32) == want[k].view(np.uint32)).all()
        assert b"iterations < 0" in errs[k]
    # the default context saw neither scene nor error
    assert lib.rc_prepare_host(None) != 0 and b"no scene" in lib.rc_last_error()


def test_destroy_rejects_null():
    lib = _native.lib()
    assert lib.rc_context_destroy(None) != 0


@pytest.mark.gpu
def test_concurrent_contexts_render_like_sequential():
    """Two scenes rendered at the same time from two threads, each in its own context,
    give the images the default context renders for them one after the other (up to the
    FP64 summation order of the merges)."""
    scs = [scenes.test_scene(64, 48), scenes.glass_sphere_point(64, 64, subdiv=3, light="area")]
    kw = dict(max_path_length=6, photons_per_iter=65536, seed=3)

    def render(sc):
        r = Renderer(sc, **kw)
        r.render(4)
        img = r.image()
        r.release()
        return img

    want = [render(sc) for sc in scs]
    got = [None, None]

    def worker(k):
        ctx = Context()
        with ctx:
            got[k] = render(scs[k])
        ctx.destroy()

    ts = [threading.Thread(target=worker, args=(k,)) for k in range(2)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    for g, w in zip(got, want):
        assert w.sum() > 0
        np.testing.assert_allclose(g, w, rtol=1e-5, atol=1e-7)


def test_new_entry_points_validate_arguments():
    """gpu_bvh is 0 or 1; the scene dump needs a prepared scene and a known selector;
    the prepare statistics copy at most what they hold."""
    import ctypes as C
    from realcausticsengine_gb300 import abi
    lib = _native.lib()
    lib.rc_release()
    cfg = abi.RcConfig()
    lib.rc_default_config(C.byref(cfg))
    assert cfg.gpu_bvh == 1
    cfg.gpu_bvh = 2
    assert lib.rc_set_config(C.byref(cfg)) != 0 and b"gpu_bvh" in lib.rc_last_error()
    cfg.gpu_bvh = 0
    assert lib.rc_set_config(C.byref(cfg)) == 0
    n = C.c_longlong(-1)
    assert lib.rc_scene_dump(0, None, 0, C.byref(n)) != 0 and b"not prepared" in lib.rc_last_error()
    out = np.full(8, -1.0)
    assert lib.rc_prepare_stats(out.ctypes.data, 2) == 2 and (out[2:] == -1.0).all()
    lib.rc_default_config(C.byref(cfg))
    assert lib.rc_set_config(C.byref(cfg)) == 0


def test_unbound_threads_share_the_default_context():
    """A thread that never binds (and one that binds and unbinds) sees the default
    context: a scene loaded there on one thread is visible from another, as with the
    reference's single global scene."""
    lib = _native.lib()
    sc = scenes.test_scene()
    r = Renderer(sc)                        # default context, main thread
    seen = []

    def worker():
        ctx = Context()
        ctx.bind()
        ctx.unbind()                        # back to the default context
        info = (np.zeros(9, np.float32))
        seen.append(lib.rc_prepare_host(info.ctypes.data_as(_ctypes_float_p())))
        ctx.destroy()

    t = threading.Thread(target=worker)
    t.start()
    t.join()
    assert seen == [0]
    r.release()


def _ctypes_float_p():
    import ctypes as C
    return C.POINTER(C.c_float)


def test_parity_hooks_validate_shapes_before_device_work():
    """The traversal and Metropolis parity hooks refuse an unknown shape, and the
    Metropolis hook a configuration without a Metropolis sampler, before any device work."""
    import ctypes as C
    from realcausticsengine_gb300 import abi
    lib = _native.lib()
    r = Renderer(scenes.test_scene())
    o = np.zeros((1, 3), np.float32)
    out = np.zeros((1, 16), np.float32)
    assert lib.rc_trace_rays_shape(1, o.ctypes.data, o.ctypes.data, C.c_float(0.001), out.ctypes.data, 3) != 0
    assert b"shape" in lib.rc_last_error()
    n = C.c_longlong()
    assert lib.rc_mlt_photons(0, 0, None, 0, C.byref(n), None) != 0       # uniform sampler
    assert b"Metropolis" in lib.rc_last_error()
    cfg = abi.RcConfig()
    lib.rc_default_config(C.byref(cfg))
    cfg.sampler, cfg.write_exr = abi.SAMPLER_PSSMLT, 0
    assert lib.rc_set_config(C.byref(cfg)) == 0
    assert lib.rc_mlt_photons(2, 0, None, 0, C.byref(n), None) != 0       # variants 0 and 1 only
    assert b"shape" in lib.rc_last_error()
    lib.rc_default_config(C.byref(cfg))
    assert lib.rc_set_config(C.byref(cfg)) == 0
    r.release()
