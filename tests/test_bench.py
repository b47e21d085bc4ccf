"""bench.py's host logic without a GPU: the JSON line's contract (driven through a fake
library and renderer), the rank coordination of multi-process runs (two gloo ranks on
the CPU), the GPU each rank pins, and the reference arm's other ranks."""
import ctypes as C
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]

import bench  # noqa: E402  (repo root on sys.path via conftest)


class _Fn:
    """A library entry point: callable, and it takes ctypes attributes (argtypes...)."""

    def __init__(self, body):
        self.body = body

    def __call__(self, *a):
        return self.body(*a)


class FakeLib:
    """The C ABI calls bench.run_ours makes, returning success; rc_render_timed reports
    a fixed device time, gather time, gather bytes and launch count."""

    DEVICE_MS, GATHER_MS, GATHER_BYTES, LAUNCHES = 200.0, 6.5, 7.7e8, 1496.0

    def __init__(self):
        self.calls = []

        def record(name, rc=0):
            def body(*a):
                self.calls.append(name)
                return rc
            return _Fn(body)

        def timed(steps, ptr):
            self.calls.append("rc_render_timed")
            out = (C.c_double * 4).from_address(ptr)
            out[0], out[1], out[2], out[3] = self.DEVICE_MS, self.GATHER_MS, self.GATHER_BYTES, self.LAUNCHES
            return 0

        def bus_id(buf, n):
            C.memmove(buf, b"0000:1b:00.0\0", 13)
            return 0

        self.rc_render_timed = _Fn(timed)
        self.rc_device_bus_id = _Fn(bus_id)
        for name in ("rc_default_config", "rc_set_config", "rc_prepare", "rc_render", "rc_read_image",
                     "rc_release"):
            setattr(self, name, record(name))
        self.init = record("init", None)
        self.rc_last_error = _Fn(lambda: b"")


class FakeRenderer:
    def __init__(self, sc, **kw):
        self.kw = kw

    def prepare(self):
        pass

    def render(self, k):
        pass

    def stats(self):
        return {"queries": 3.6e6, "photons": 7.6e6, "merged": 2.5e7, "light_ms": 13.7, "kd_ms": 6.2,
                "camera_ms": 15.4, "gather_ms": 6.6, "light_rays": 6.0e7}

    def release(self):
        pass


def test_bench_line_contract(monkeypatch, capsys):
    from realcausticsengine_gb300 import _native, session
    fake = FakeLib()
    monkeypatch.setattr(_native, "lib", lambda: fake)
    monkeypatch.setattr(session, "Renderer", FakeRenderer)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    args = bench.parse_args(["--steps", "4", "--warmup", "3", "--width", "64", "--height", "36", "--grid", "16",
                             "--photons", "65536", "--no-learned", "--no-cpu-baseline"])
    bench.run_ours(args)
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    # the keys every bench line carries, with their meaning
    assert line["metric"] == "photons/s" and line["unit"] == "photons/s" and line["higher_is_better"] is True
    assert line["n_gpus"] == 1 and line["steps"] == 4 and line["warmup"] == 3
    assert line["scaling"] == "weak" and line["vs_baseline"] is None and line["data"] == "synthetic"
    assert line["value"] == pytest.approx(65536 * 4 / (FakeLib.DEVICE_MS / 1000.0))
    assert line["ms_per_step"] == pytest.approx(FakeLib.DEVICE_MS / 4)
    assert "water_pool 64x36" in line["config"]["workload"] and "l2" in line["config"]
    e2e = line["e2e"]
    assert e2e["unit"] == "photons/s" and e2e["value"] > 0
    assert e2e["d2h_bytes_per_step"] == 64 * 36 * 3 * 4 and e2e["h2d_bytes_per_step"] > 0
    roof = line["roofline"]
    assert roof["bound"] == "hbm" and roof["unit"] == "GB/s"
    assert roof["achieved"] == pytest.approx(FakeLib.GATHER_BYTES / (FakeLib.GATHER_MS / 1000.0) / 1e9)
    assert roof["frac"] == pytest.approx(roof["achieved"] / roof["peak"])
    assert roof["traffic"] == pytest.approx(bench.GATHER_TRAFFIC_OVER_ALGORITHMIC * FakeLib.GATHER_BYTES)
    assert line["gpu_launches"] == int(FakeLib.LAUNCHES)
    assert "sm_mhz" in line["clocks"] and "reasons" in line["clocks"]
    # the end-to-end part goes through the public ABI: init, prepare, render + read per step
    e2e_calls = fake.calls[fake.calls.index("init"):]
    assert e2e_calls[:2] == ["init", "rc_prepare"]
    assert e2e_calls[2:10] == ["rc_render", "rc_read_image"] * 4 and e2e_calls[10] == "rc_release"


def test_visible_device(monkeypatch):
    monkeypatch.delenv("CUDA_VISIBLE_DEVICES", raising=False)
    assert bench.visible_device(3) == "3"
    monkeypatch.setenv("CUDA_VISIBLE_DEVICES", "4,5,6,7")
    assert bench.visible_device(0) == "4" and bench.visible_device(3) == "7"
    monkeypatch.setenv("CUDA_VISIBLE_DEVICES", "GPU-1234")          # one GPU given per rank
    assert bench.visible_device(2) == "GPU-1234"
    monkeypatch.setenv("CUDA_VISIBLE_DEVICES", "0,1")
    with pytest.raises(SystemExit):
        bench.visible_device(2)


def test_single_rank_is_a_no_op(monkeypatch):
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    r = bench.Ranks()
    r.barrier()
    assert r.max(2.0, 5.0) == [2.0, 5.0]
    r.close()


_RANK_SCRIPT = """
import json, sys, time
sys.path.insert(0, {root!r})
import bench
r = bench.Ranks()
if r.rank == 1:
    time.sleep(0.5)        # the other rank waits at the barrier
t0 = time.perf_counter()
r.barrier()
waited = time.perf_counter() - t0
out = r.max(10.0 + r.rank, 100.0 - r.rank)
r.close()
print(json.dumps({{"rank": r.rank, "world": r.world, "max": out, "waited": waited}}))
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_barrier_and_max():
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", _RANK_SCRIPT.format(root=str(ROOT))], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=120)
        assert p.returncode == 0, err[-2000:]
        outs.append(json.loads(out.strip().splitlines()[-1]))
    for o in outs:
        assert o["world"] == 2 and o["max"] == [11.0, 100.0]   # max over ranks of each value
    assert outs[0]["waited"] > 0.3                             # rank 0 waited for rank 1 at the barrier


def test_reference_arm_other_ranks_do_no_work(monkeypatch, capsys):
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setattr(bench, "cpu_baseline", lambda **kw: pytest.fail("rank 1 ran the CPU baseline"))
    bench.run_reference(bench.parse_args(["--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0"]))
    assert capsys.readouterr().out == ""


def test_clock_sampler_names_the_gpu_by_bus_id():
    """nvidia-smi numbers GPUs physically: the sampler must name the CUDA device the
    process runs on by its PCI bus id, in nvidia-smi's 8-digit-domain form."""
    import bench
    assert bench.nvsmi_id(FakeLib()) == "00000000:1B:00.0"


def test_kd_roofline_bytes():
    """The KD build's algorithmic bytes: 12 P + 32 P ceil(log2 P) + 8 x 2^(floor(log2 P) + 1)."""
    import bench
    r = bench.kd_roofline(1 << 20, 2.0, 6000.0, "measured")
    want = 12 * 2 ** 20 + 32 * 2 ** 20 * 20 + 8 * 2 ** 21
    assert r["algorithmic_bytes"] == want
    assert abs(r["achieved"] - want / 2e-3 / 1e9) < 1e-6 and abs(r["frac"] - r["achieved"] / 6000.0) < 1e-12
    assert bench.kd_roofline(1, 1.0, 6000.0, "measured") is None
