"""Checkpoint / resume of a progressive render (rc_save_state / rc_load_state)."""
import ctypes as C

import numpy as np
import pytest

from realcausticsengine_gb300 import _native, abi, scenes
from realcausticsengine_gb300.scene import InitArgs


def _config(L, **kw):
    cfg = abi.RcConfig()
    L.rc_default_config(C.byref(cfg))
    cfg.write_exr = 0
    cfg.max_path_length = 8
    cfg.photons_per_iter = 200000
    cfg.seed = 5
    for k, v in kw.items():
        setattr(cfg, k, v)
    assert L.rc_set_config(C.byref(cfg)) == 0, L.rc_last_error()


def _image(L, w, h):
    img = np.zeros((h, w, 3), np.float32)
    _native.check(L.rc_read_image(img.ctypes.data, w, h), "rc_read_image")
    return img.astype(np.float64)


def test_save_without_scene_is_an_error(tmp_path):
    L = _native.lib()
    L.rc_release()
    assert L.rc_save_state(str(tmp_path / "s.bin").encode()) != 0


@pytest.mark.gpu
def test_resume_equals_uninterrupted(tmp_path):
    """4 iterations, save, re-init, load, 4 more == 8 uninterrupted iterations (the
    counter RNG continues from the saved iteration; FP64 sums agree to summation order)."""
    L = _native.lib()
    sc = scenes.water_pool(96, 64, grid=64, samples=8)
    _config(L)
    args = InitArgs(sc)
    args.call(L.init)
    _native.check(L.rc_render(8), "rc_render")
    full = _image(L, 96, 64)
    L.rc_release()

    _config(L)
    InitArgs(sc).call(L.init)
    _native.check(L.rc_render(4), "rc_render")
    path = str(tmp_path / "state.bin").encode()
    _native.check(L.rc_save_state(path), "rc_save_state")
    L.rc_release()

    _config(L, seed=99)                    # the saved seed wins on load
    InitArgs(sc).call(L.init)
    _native.check(L.rc_load_state(path), "rc_load_state")
    _native.check(L.rc_render(4), "rc_render")
    resumed = _image(L, 96, 64)
    L.rc_release()
    assert full.max() > 0
    assert np.abs(resumed - full).max() <= 1e-5 * full.max()

    # a state of another scene is refused
    other = scenes.water_pool(96, 64, grid=32, samples=8)
    _config(L)
    InitArgs(other).call(L.init)
    assert L.rc_load_state(path) == -2      # RC_E_INVALID
    assert b"another scene" in L.rc_last_error()
    L.rc_release()


@pytest.mark.gpu
def test_resume_keeps_learned_proposal(tmp_path):
    """The network and Adam state travel with the checkpoint: a resumed learned render
    guides emission from its first iteration (no fresh training round)."""
    L = _native.lib()
    sc = scenes.water_pool(96, 64, grid=64, samples=8)
    _config(L, learned_proposal=1, train_iterations=2, train_steps=16)
    InitArgs(sc).call(L.init)
    _native.check(L.rc_render(3), "rc_render")
    path = str(tmp_path / "learned.bin").encode()
    _native.check(L.rc_save_state(path), "rc_save_state")
    L.rc_release()
    _config(L, learned_proposal=1, train_iterations=2, train_steps=16)
    InitArgs(sc).call(L.init)
    _native.check(L.rc_load_state(path), "rc_load_state")
    _native.check(L.rc_render(1), "rc_render")
    n = 200000
    prop = np.zeros((n, 4), np.float32)
    _native.check(L.rc_proposal_state(n, prop.ctypes.data, None), "rc_proposal_state")
    st = np.zeros(16)
    L.rc_get_stats(st.ctypes.data, 16)
    L.rc_release()
    assert st[10] == 4                      # iterations counted across the resume
    assert st[8] > 0                        # proposal inference ran
    w = prop[:, 3]
    # E_q[p_light / q] = 1 (the defensive component keeps q > 0 wherever p_light > 0)
    assert (w > 0).mean() > 0.5 and abs(w.mean() - 1.0) < 0.05
