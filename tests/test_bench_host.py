"""Host-side logic of bench.py: the max-over-ranks reduction across two
gloo ranks on CPU, the clock-log summary and the sampler's bounded padding,
the byte model, and the reference arm (CPU restatement on a process pool)
end to end on a small workload."""
import json
import os
import subprocess
import sys
import time

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)
import bench  # noqa: E402


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        q.put((rank, bench.reduce_max(10.0 + 5.0 * rank, dist, "cpu")))
    finally:
        dist.destroy_process_group()


def test_reduce_max_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 1000)
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == {0: 15.0, 1: 15.0}
    assert bench.reduce_max(3.5, None, "cpu") == 3.5


def test_clock_summary_flags_throttle_reasons():
    lines = ["2070, 2070, 900.1, Not Active, Not Active, Not Active, Not Active",
             "1980, 2070, 1390.5, Not Active, Not Active, Not Active, Active",
             "2070, 2070, 1200.0, Not Active, Not Active, Not Active, Not Active", "garbage"]
    c = bench.summarize_clocks(lines)
    assert c["sm_mhz"] == 2070 and c["sm_max_mhz"] == 2070 and c["reasons"] == ["sw_power_cap"] and c["samples"] == 3


def test_clock_sampler_padding_is_bounded(tmp_path):
    fake = tmp_path / "fake_smi.py"
    fake.write_text("import sys, time\n"
                    "for _ in range(200):\n"
                    "    print('2070, 2070, 1000.0, Not Active, Not Active, Not Active, Not Active', flush=True)\n"
                    "    time.sleep(0.05)\n")
    calls = []

    def busy():
        calls.append(1)
        time.sleep(0.01)

    c = bench.ClockSampler(0, cmd=[sys.executable, str(fake)])
    c.start()
    c.wait_samples(2, busy)
    n0 = len(c.lines)
    c.wait_samples(1, busy)
    out = c.stop()
    assert n0 >= 2 and len(c.lines) >= n0 + 1 and calls
    assert out["samples"] >= 3 and out["sm_mhz"] == 2070 and out["reasons"] == []
    # no sampler (missing tool or one that exits at once): the padding returns without waiting
    for cmd in (["/nonexistent/nvidia-smi"], [sys.executable, "-c", "pass"]):
        c = bench.ClockSampler(0, cmd=cmd)
        c.start()
        time.sleep(0.2)
        t0 = time.perf_counter()
        c.wait_samples(2, busy)
        assert time.perf_counter() - t0 < 0.5
        assert c.stop()["samples"] == 0


def test_byte_model():
    b = bench.algorithmic_bytes([100, 200, 300], [10, 20], 3)
    wh = 752 * 480
    assert b["pyramid_per_frame"] == wh + 4 * (1047287 - wh)
    assert b["describe_total"] == 48 * 600
    assert b["match_total"] == 32 * (600 + 300) + 8 * 30
    assert b["total_per_step"] == 3 * b["pyramid_per_frame"] + b["describe_total"] + b["match_total"]


def test_reference_arm_prints_one_line():
    env = dict(os.environ)
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--frames", "3"], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "frames/s" and line["value"] > 0
    # the matcher leg is the reference's own compiled matcher wherever its source is at hand
    import oracle

    assert line["cpu_baseline"]["kind"] == ("reference" if oracle.ref_matcher_expected() else "port")
    assert line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["config"]["pairs"] == 2 and "l2" in line["config"] and "parallelism" in line["config"]


def test_reference_arm_nonzero_rank_exits_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2")
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--frames", "2"], capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == ""


def test_served_streams_walk_their_trajectory_back_and_forth():
    """A served stream's frames follow its trajectory forwards, then
    backwards: every step moves to a neighbouring frame, every frame is used."""
    import bench

    n = 64
    idx = [bench._walk(c, n) for c in range(5 * n)]
    assert idx[:n] == list(range(n)) and idx[n] == n - 2
    assert all(abs(a - b) == 1 for a, b in zip(idx, idx[1:]))
    assert set(idx) == set(range(n))
    assert bench._walk(7, 1) == 0


def test_profile_lines_cover_every_stage():
    """The roofline's traffic and SM-side figures are machine-read from the
    committed ncu summaries: every stage of the step has both."""
    traffic = bench.measured_traffic()
    pipes = bench.measured_pipes()
    for k in ("k_pyramid", "k_detect", "k_blur_border", "compaction", "k_describe", "k_match"):
        assert traffic.get(k, 0) > 0, k
    for k in ("k_pyramid", "k_detect", "k_blur_border", "k_describe", "k_match"):
        assert 0 < pipes[k]["issue"] <= 100, k


def test_native_server_client_compiles(tmp_path):
    """The served form's native closed-loop client (bench served.saturation_native)
    builds against the C header and the library built here."""
    import shutil

    lib = os.path.join(REPO, "uni_slam_gb300")
    if not shutil.which("g++") or not os.path.exists(os.path.join(lib, "libuslam.so")):
        pytest.skip("g++ or the built library is missing")
    exe = tmp_path / "server_load"
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(REPO, "include"),
                        os.path.join(REPO, "tests", "adapter", "server_load.cpp"), "-o", str(exe), "-L", lib,
                        "-luslam", f"-Wl,-rpath,{lib}", "-lpthread"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    # wrong argument count: usage and exit code 2, no device touched
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr
