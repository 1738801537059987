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
    # toolbox, sum, classify, velocity (2), crossing, shadow, 90 tiled (band blocks inside), band max,
    # time step, 3 advection stages, setDistance (2), classify, 60 x (tiled + band)
    assert bench.LAUNCHES_PER_STEP == 225


def test_profiled_figures_match_summaries():
    """The per-launch DRAM bytes of both dominant kernels come from their committed ncu
    summaries (about 20 and 7 bytes per node at 256^3)."""
    t = bench.profiled("extend_stage_f32_256.md", "dram_bytes_per_launch_256")
    assert t is not None and 2.5e8 < t < 5e8
    r = bench.profiled("reinit_stage_f32_256.md", "dram_bytes_per_launch_256")
    assert r is not None and 5e7 < r < 3e8
    assert bench.profiled("extend_stage_f32_256.md", "no_such_key") is None
    assert bench.profiled("no_such_summary.md", "dram_bytes_per_launch_256") is None


def test_stage_roofline_fractions():
    """Effective, DRAM and issue fractions of a stage from its time, its algorithmic bytes,
    the summary's per-launch figures and the sampled clock."""
    e = bench.stage_roofline("extension", "k", 0.2, 1.0e9, "extend_stage_f32_256.md", 5000.0, "measured", 2000.0, 100)
    assert abs(e["achieved"] - 5000.0) < 1e-9 and abs(e["frac"] - 1.0) < 1e-12
    assert abs(e["dram_gbs"] - e["traffic"] / 0.2e-3 / 1e9) < 1e-6
    if "warp_instructions_per_launch" in e:
        slots = 100 * 4 * 2000.0e6 * 0.2e-3
        assert abs(e["issue_frac"] - e["warp_instructions_per_launch"] / slots) < 1e-12


def test_whole_job_throughput():
    assert bench.whole_job_gpt_s(1, 2e9, 0.5) == 4.0
    assert bench.whole_job_gpt_s(4, 2e9, 0.5) == 16.0


def test_peaks_fall_back_without_file(monkeypatch, tmp_path):
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    assert bench.peaks() == (6800.0, "fallback")
