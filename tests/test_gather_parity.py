"""Photon sets of the render's own gather kernel against the oracle's KD-tree query.

rc_gather_query runs the kernel the render launches (`k_gather`: chunk boxes, KD-cell
query order, the group traversal, the pending-pair lists and their flushes), in every
launch shape the autotuner can pick, with a sink that records photon ids where the
render evaluates merges.  Every query's photon set must equal, id for id, the set the
oracle's restatement of KD_Tree::find_closest_in_radius (src/KD_Tree.cpp:217-280)
returns; the oracle is itself pinned to the compiled reference (test_oracle_golden.py).
"""
import ctypes as C

import numpy as np
import pytest

from realcausticsengine_gb300 import scenes
from realcausticsengine_gb300.session import Renderer, gather_variants, kd_query

pytestmark = pytest.mark.gpu


def _oracle_sets(orc, pos, q, r2, per_query=4096):
    cnt = np.zeros(len(q), np.int32)
    cap = int(len(q) * per_query)
    idx = np.zeros(cap, np.int32)
    tot = orc.oracle_kd_query(len(pos), pos.ctypes.data, len(q), q.ctypes.data, C.c_float(r2), cnt.ctypes.data,
                              idx.ctypes.data, cap)
    assert tot <= cap
    offs = np.concatenate([[0], np.cumsum(cnt)])
    return cnt, idx[:offs[-1]], offs


def _assert_same_sets(counts, sets, ocnt, oidx, offs):
    assert (counts == ocnt).all(), f"{int((counts != ocnt).sum())} queries differ in count"
    for j in range(len(counts)):
        a = np.sort(sets[j])
        b = np.sort(oidx[offs[j]:offs[j + 1]])
        assert (a == b).all(), f"query {j}: sets differ"


def _hard_photons(n, seed):
    """Uniform photons with tied coordinates, duplicated photons and a flat sheet."""
    rng = np.random.default_rng(seed)
    pos = rng.uniform(-1, 1, (n, 3)).astype(np.float32)
    if n > 100:
        pos[: n // 8] = np.round(pos[: n // 8] * 16) / 16
        pos[n // 8: n // 6] = pos[0]
        pos[n // 6: n // 5, 2] = 0.25
    q = rng.uniform(-1.05, 1.05, (3000, 3)).astype(np.float32)
    if n >= 100:
        q[:100] = pos[:100]
    return pos, q


def test_variants_are_listed():
    assert gather_variants() >= 2


@pytest.mark.parametrize("n", [0, 1, 2, 3, 31, 32, 33, 63, 64, 2047, 2048, 2049, 4097, 65537, 1000003])
def test_every_shape_vs_oracle(orc, n):
    pos, q = _hard_photons(n, n + 5)
    r = 0.04 if n < 100000 else 0.012
    r2 = float(np.float32(r * r))
    ocnt, oidx, offs = _oracle_sets(orc, pos, q, r2)
    for v in range(gather_variants()):
        counts, sets = kd_query(pos, q, r2, variant=v)
        _assert_same_sets(counts, sets, ocnt, oidx, offs)


def test_padded_capacity_vs_oracle(orc):
    """Graph-replayed iterations build the tree over a fixed photon capacity whose unused
    slots sit one scene extent beyond the scene; the padded tree answers the same sets."""
    pos, q = _hard_photons(200003, 11)
    pad = np.tile(np.float32([4.0, 0.0, 0.0]), (40961, 1))
    r2 = float(np.float32(0.02 * 0.02))
    ocnt, oidx, offs = _oracle_sets(orc, pos, q, r2)
    for v in range(gather_variants()):
        counts, sets = kd_query(np.concatenate([pos, pad]), q, r2, variant=v)
        _assert_same_sets(counts, sets, ocnt, oidx, offs)


def test_dense_queries_overflow_pending_lists(orc):
    """Many accepted photons per query (a radius holding hundreds of photons): the
    pending-pair lists flush many times per chunk and queries span many flushes."""
    rng = np.random.default_rng(8)
    pos = rng.uniform(-1, 1, (50000, 3)).astype(np.float32)
    pos[:, 2] *= 0.01                                   # a thin slab: dense in 2D
    q = rng.uniform(-1, 1, (2000, 3)).astype(np.float32)
    q[:, 2] = 0.0
    r2 = float(np.float32(0.08 * 0.08))
    ocnt, oidx, offs = _oracle_sets(orc, pos, q, r2, per_query=8192)
    assert ocnt.mean() > 100
    for v in range(gather_variants()):
        counts, sets = kd_query(pos, q, r2, variant=v)
        _assert_same_sets(counts, sets, ocnt, oidx, offs)


def test_kd_sets_at_8m_photons(orc):
    """A photon count above 2^23 (more global KD levels than the smaller cases)."""
    n = 8_400_007
    pos, q = _hard_photons(n, 21)
    r2 = float(np.float32(0.004 * 0.004))
    ocnt, oidx, offs = _oracle_sets(orc, pos, q, r2)
    counts, sets = kd_query(pos, q, r2)
    _assert_same_sets(counts, sets, ocnt, oidx, offs)


def test_water_pool_iteration_vs_oracle(orc):
    """The photon map and merge queries of one iteration of the 1920x1080 water-pool
    workload (16.7M light paths, ~7.6M stored photons, ~3.6M queries) at the render's
    merge radius: every shape's counts agree over all queries, and a seeded subset of
    50,000 queries matches the oracle set for set."""
    sc = scenes.water_pool(1920, 1080, grid=512, samples=1)
    r = Renderer(sc, max_path_length=8, photons_per_iter=16 << 20, seed=0)
    r.prepare()
    ph = r.light_photons(0)
    qs = r.camera_queries(0)
    r.render(1)
    st = r.stats()
    r.release()
    pos = np.ascontiguousarray(ph[:, :3])
    qpos = np.ascontiguousarray(qs[:, :3])
    assert len(pos) > 5_000_000 and len(qpos) > 2_000_000
    assert int(st["photons"]) == len(pos) and int(st["queries"]) == len(qpos)
    # the reported radius is the double square root of the render's FP32 r^2: squaring it
    # in double and rounding to FP32 gives that r^2 back exactly
    r2 = float(np.float32(st["radius"] ** 2))
    base, _ = kd_query(pos, qpos, r2, with_indices=False)
    assert base.mean() > 2.0                        # the workload merges several photons per query
    # the render's own gather (merge evaluation sink) accepted exactly these pairs
    assert int(base.sum()) == int(st["merged"])
    for v in range(gather_variants()):
        counts, _ = kd_query(pos, qpos, r2, with_indices=False, variant=v)
        assert (counts == base).all(), f"shape {v} differs from the default on {int((counts != base).sum())} queries"
    sub = np.random.default_rng(0).choice(len(qpos), 50000, replace=False)
    q = np.ascontiguousarray(qpos[sub])
    ocnt, oidx, offs = _oracle_sets(orc, pos, q, r2)
    counts, sets = kd_query(pos, q, r2)
    assert (counts == base[sub]).all()
    _assert_same_sets(counts, sets, ocnt, oidx, offs)
