"""The bench's host-side bookkeeping (no GPU): the byte and launch counts of one vesicle
step, the roofline traffic read from the committed ncu summary, and the whole-job
throughput."""
import importlib
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
bench = importlib.import_module("bench")


def test_step_counts():
    # 30 extension + 1 advection + 20 reinitialization pseudo-steps
    assert (bench.EXT, bench.ADV, bench.RE) == (30, 1, 20)
    w = 4
    assert bench.BYTES_PER_NODE_STEP == 30 * 56 * w + 17 * w + 20 * (29 * w + 3) + 38 * w
    # toolbox, sum, classify, velocity (2), crossing, 90 x (tiled + band), band max, time
    # step, 3 advection stages, setDistance (2), classify, 60 x (tiled + band)
    assert bench.LAUNCHES_PER_STEP == 314


def test_profiled_traffic_matches_summary():
    t = bench.profiled_traffic()
    assert t is not None and 2.5e8 < t < 5e8  # about 20 bytes per node at 256^3
    with open(os.path.join(ROOT, "profiles", "extend_stage_f32_256.md")) as f:
        assert any(line.startswith("dram_bytes_per_launch_256:") for line in f)


def test_whole_job_throughput():
    assert bench.whole_job_gpt_s(1, 2e9, 0.5) == 4.0
    assert bench.whole_job_gpt_s(4, 2e9, 0.5) == 16.0


def test_peaks_fall_back_without_file(monkeypatch, tmp_path):
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    assert bench.peaks() == (6800.0, "fallback")
