"""Learned emission proposal inside the renderer, on a reduced water-pool scene (2x2
area light over a refracting height field, camera looking at the floor through the
water): only part of the light's emission reaches the part of the floor the camera
sees.

The vertex-merging estimate with a fixed radius schedule has the same expectation for
any number of light paths per iteration, so a plain render with 8x the light paths is
the reference image for both estimators at the same iteration count.  The reference
uses another light seed but the same camera seed: all three renders share their
camera paths (merge queries), and the differences are photon noise alone.

* unbiased: the learned render's mean stays within 1.5% of the reference mean;
* gain: at equal light paths per iteration its per-pixel RMSE against the reference
  is below 0.85x the plain render's.
"""
import numpy as np
import pytest

from realcausticsengine_gb300 import scenes
from realcausticsengine_gb300.session import Renderer

pytestmark = pytest.mark.gpu

ITERS, PATHS = 12, 1 << 20


def _render(sc, paths, seed, learned):
    r = Renderer(sc, max_path_length=8, photons_per_iter=paths, seed=seed, camera_seed=7, learned_proposal=learned,
                 train_iterations=6, train_steps=64, learning_rate=1e-3)
    r.render(ITERS)
    img, st = r.image(), r.stats()
    r.release()
    return img.astype(np.float64), st


@pytest.fixture(scope="module")
def renders():
    sc = scenes.water_pool(240, 135, grid=256, samples=ITERS)
    ref, _ = _render(sc, PATHS * 8, 101, False)
    plain, st_plain = _render(sc, PATHS, 7, False)
    learned, st_learned = _render(sc, PATHS, 7, True)
    return ref, plain, learned, st_plain, st_learned


def test_learned_proposal_is_unbiased(renders):
    ref, plain, learned, _, st = renders
    assert st["accum_ms"] > 0.0          # proposal inference ran in the last iteration
    assert np.isfinite(learned).all() and (learned >= 0).all()
    m_ref, m_plain, m_learned = ref.mean(), plain.mean(), learned.mean()
    print(f"mean ref {m_ref:.5g} plain {m_plain:.5g} learned {m_learned:.5g}")
    assert abs(m_learned / m_ref - 1.0) < 0.015, (m_learned, m_ref)
    assert abs(m_plain / m_ref - 1.0) < 0.015, (m_plain, m_ref)


def test_learned_proposal_reduces_error(renders):
    ref, plain, learned, st_plain, st_learned = renders
    e_plain = np.sqrt(((plain - ref) ** 2).mean())
    e_learned = np.sqrt(((learned - ref) ** 2).mean())
    print(f"rmse plain {e_plain:.4g} learned {e_learned:.4g} ratio {e_learned / e_plain:.3f}; "
          f"photons/iter plain {st_plain['photons']:.0f} learned {st_learned['photons']:.0f}")
    assert e_learned < 0.85 * e_plain, (e_learned, e_plain)
