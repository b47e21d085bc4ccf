"""rc_kd_build_noalloc: the KD-tree build for callers that cannot allocate GPU memory
(hosts that pass this library only pre-allocated device buffers).  It must build the
same tree as the allocating entry point, from its fixed in-library scratch, on
repeated calls (the scratch keeps the previous call's contents), and reject photon
counts beyond its fixed maximum.  Collected last so that a run stopping at the first
failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from realcausticsengine_gb300 import _native
from realcausticsengine_gb300.session import kd_build_nodes

pytestmark = pytest.mark.gpu

MAX_PHOTONS = 1 << 19


def _call_noalloc(torch, pos: np.ndarray):
    lib = _native.lib()
    n = len(pos)
    p4 = np.zeros((max(n, 1), 4), np.float32)
    p4[:n, :3] = pos
    d_pos = torch.from_numpy(p4).cuda()
    node_len = int(2 ** (int(np.log2(n)) + 1)) if n else 2
    node_len = max(node_len, len(kd_build_nodes(pos)) if n else 2)
    d_nodes = torch.full((node_len, 2), -1, dtype=torch.int32, device="cuda")
    d_x = torch.empty(max(n, 1), dtype=torch.float32, device="cuda")
    d_y = torch.empty_like(d_x)
    d_z = torch.empty_like(d_x)
    d_ids = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.rc_kd_build_noalloc(d_pos.data_ptr(), n, d_nodes.data_ptr(), node_len, d_x.data_ptr(), d_y.data_ptr(),
                                 d_z.data_ptr(), d_ids.data_ptr(), stream)
    assert rc == 0, lib.rc_kd_noalloc_last_error()
    return (d_nodes.cpu().numpy().view(np.uint32), d_x.cpu().numpy()[:n], d_y.cpu().numpy()[:n],
            d_z.cpu().numpy()[:n], d_ids.cpu().numpy().view(np.uint32)[:n])


def test_noalloc_kd_build_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    rng = np.random.default_rng(2024)
    # two calls in a row with different sizes and data: the second must not see the
    # first call's leftovers in the shared scratch
    for n in (300001, 70003, MAX_PHOTONS):
        # distinct coordinates on every axis, so the median photon of every node is
        # unique and both builds must produce identical node words
        pos = np.stack([rng.permutation(np.linspace(-1, 1, n, dtype=np.float32)) for _ in range(3)], 1)
        assert all(len(np.unique(pos[:, k])) == n for k in range(3))
        want = kd_build_nodes(pos)                       # allocating entry point
        nodes, x, y, z, ids = _call_noalloc(torch, pos)
        assert (nodes[: len(want)] == want).all(), f"node arrays differ for n={n}"
        # photons come back in tree order: a permutation with matching coordinates
        assert (np.sort(ids) == np.arange(n, dtype=np.uint32)).all()
        assert (x == pos[ids, 0]).all() and (y == pos[ids, 1]).all() and (z == pos[ids, 2]).all()


def test_noalloc_small_counts_match_allocating_entry_point():
    """The early returns and the smallest scratch layouts: no photons, one, two, three,
    and a count just above one on-chip subtree (1025)."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    rng = np.random.default_rng(7)
    for n in (0, 1, 2, 1025, 3):
        pos = np.stack([rng.permutation(np.linspace(-1, 1, max(n, 1), dtype=np.float32))[:n] for _ in range(3)], 1)
        pos = pos.reshape(n, 3)
        nodes, x, y, z, ids = _call_noalloc(torch, pos)
        if n == 0:
            continue
        want = kd_build_nodes(pos)
        assert (nodes[: len(want)] == want).all(), f"node arrays differ for n={n}"
        assert (np.sort(ids) == np.arange(n, dtype=np.uint32)).all()
        assert (x == pos[ids, 0]).all() and (y == pos[ids, 1]).all() and (z == pos[ids, 2]).all()


def test_noalloc_rejects_counts_beyond_fixed_scratch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = _native.lib()
    d = torch.zeros(16, dtype=torch.float32, device="cuda")
    rc = lib.rc_kd_build_noalloc(d.data_ptr(), MAX_PHOTONS + 1, d.data_ptr(), 1 << 21, d.data_ptr(), d.data_ptr(),
                                 d.data_ptr(), d.data_ptr(), None)
    assert rc == -5
    assert b"524288" in lib.rc_kd_noalloc_last_error()
