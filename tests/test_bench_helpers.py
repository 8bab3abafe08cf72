"""The bench's host-side arithmetic on the CPU: the mandatory bytes of a
frame, the issue roofline from instruction counts and CUDA-event times, the
clock record's throttle reasons, and the config both arms print."""
import os
import sys
import types

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def frame(w, h, bd, true_w=None, true_h=None):
    return types.SimpleNamespace(w=w, h=h, bd=bd, true_w=true_w or w, true_h=true_h or h,
                                 luma_px=(true_w or w) * (true_h or h))


def test_stage_bytes_counts_planes_and_geometry():
    # recon in, source in, recon out at 1.5 planes each, plus 4 bytes per 4x4
    assert bench.stage_bytes(frame(3840, 2160, 8)) == 3 * 1.5 * 3840 * 2160 + 4 * 960 * 540
    assert bench.stage_bytes(frame(64, 64, 10)) == 3 * 2 * 1.5 * 64 * 64 + 4 * 16 * 16


def test_issue_roofline_takes_the_three_longest_counted_kernels():
    frames = [frame(3840, 2160, 8)] * 4
    px = 4 * 3840 * 2160
    prof = {"k_deblock_sse": (6, 0.70), "k_cdef_search": (4, 0.50), "k_lr_stats5": (4, 0.30),
            "k_lr_trial_tiles": (4, 0.29), "k_unknown": (1, 9.0)}
    r = bench.issue_roofline(prof, frames, 152, 2070.0)
    names = [k["kernel"] for k in r["kernels"]]
    assert names == ["k_deblock_sse", "k_cdef_search", "k_lr_stats5"]  # no count for k_unknown
    peak = 4.0 * 152 * 2070e6
    k0 = r["kernels"][0]
    want = bench.KERNEL_WARP_INST_PER_PX["k_deblock_sse"] * px / 0.70e-3
    assert k0["achieved_winst_per_s"] == pytest.approx(want, rel=1e-6)
    assert k0["int_frac"] == pytest.approx(want / peak, abs=1e-4)
    assert 0 < k0["int_frac"] < 1.5
    assert bench.issue_roofline(prof, frames, 152, None) is None  # no clock sample, no roofline


def test_clock_record_reports_throttle_reasons(tmp_path):
    cs = bench.ClockSampler(0)
    lines = ["0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active",
             "0, 1980, 2070, 1390.5, 0x4, Not Active, Not Active, Not Active, Active",
             "0, 2070, 2070, 1100.0, 0x0, Not Active, Not Active, Not Active, Not Active"]
    cs.tmp.write("\n".join(lines) + "\n")
    cs.tmp.flush()

    class Done:
        def terminate(self):
            pass

        def wait(self, timeout=None):
            return 0

    cs.proc = Done()
    out = cs.stop()
    assert out["sm_mhz"] == 2070.0 and out["sm_max_mhz"] == 2070.0 and out["samples"] == 3
    assert out["reasons"] == ["sw_power_cap"]


def test_clock_record_without_nvidia_smi():
    cs = bench.ClockSampler(0)
    out = cs.stop()
    assert out["sm_mhz"] is None and out["reasons"] == ["nvidia-smi unavailable"]
    os.unlink(cs.tmp.name)


def test_config_is_shared_by_both_arms():
    c = bench.ours_config(4)
    assert c["frames_per_step"] == 4 and c["parallelism"] == "single"
    assert "3840x2160" in c["workload"] and "presets {4,6}" in c["workload"]
    assert "one context (one stream) per frame" in c["concurrency"]
    assert bench.ours_config(4, world=8)["parallelism"] == "replicas"


def test_reference_arm_line(monkeypatch, capsys):
    """The reference arm's JSON line on small frames: the oracle on the host
    cores with the GPU arm's config, its own cpu_baseline and an e2e with no
    device copies."""
    import json
    from zenav1_svt_gb300 import synth
    small = [synth.make_frame(synth.frame_seed(2, 900 + k), 96, 64, 8, qp, preset, "power")
             for k, (preset, qp) in enumerate(bench.WORKLOAD)]
    monkeypatch.setattr(bench, "make_workload", lambda *a, **k: small)
    monkeypatch.setattr(bench, "env_rank", lambda: (0, 1, 0))
    args = types.SimpleNamespace(steps=1, warmup=0)
    assert bench.run_reference(args) == 0
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "MPix/s" and line["value"] > 0
    assert line["config"] == bench.ours_config(len(small))
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "MPix/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
