"""The plan autotuner's candidates, choice and cache logic (CPU; timings injected)."""

import json

from dlux_gb300.autotune import PlanTuner, candidate_configs, config_label


def test_candidates():
    labels = [config_label(c) for c in candidate_configs(256, 128)]
    # 256 columns are two 128-column tiles: the paired (256 x 128) tile is a candidate
    assert labels == ["split_bf16/op0", "split_bf16/op0/pair", "split_bf16/op1", "fp32/op0"]
    # 128 -> 64: every GEMM has one column tile, so pairing never applies
    assert [config_label(c) for c in candidate_configs(128, 64)] == \
        ["split_bf16/op0", "split_bf16/op1", "fp32/op0"]
    # plans with their own workspace also try keeping every GEMM whole (no K split)
    assert "split_bf16/op0/nosplit" in [config_label(c) for c in
                                         candidate_configs(512, 512, own_workspace=True)]
    # every side has the split form (rows padded to 8); no tensor cores: FP32 only
    assert [config_label(c) for c in candidate_configs(100, 64)] == \
        ["split_bf16/op0", "split_bf16/op1", "fp32/op0"]
    assert [config_label(c) for c in candidate_configs(256, 128, tensor_cores=False)] == \
        ["fp32/op0"]


def _timer(calls):
    def timer(n, m, cfg):
        calls.append((n, m, config_label(cfg)))
        t = {"split_bf16/op0": 3.0, "split_bf16/op0/pair": 2.5, "split_bf16/op1": 2.0,
             "fp32/op0": 5.0}
        if n == 128:   # a tiny transform: the CUDA-core form wins
            t["fp32/op0"] = 1.0
        if n == 1024:  # a large one: the paired tile wins
            t["split_bf16/op0/pair"] = 1.5
        return t[config_label(cfg)]
    return timer


def test_chooses_fastest_and_caches(tmp_path):
    calls = []
    timer = _timer(calls)
    path = tmp_path / "tune.json"
    tuner = PlanTuner(cache_path=str(path), timer=timer, device_name="GB300-test")
    assert tuner.choose(512, 256)["operand_mode"] == 1
    assert tuner.choose(128, 64)["variant"] == "fp32"
    big = tuner.choose(1024, 512)
    assert big["variant"] == "split_bf16" and big["pair"] == 1 and big["operand_mode"] == 0
    assert len(calls) == 4 + 3 + 4               # each shape timed once
    assert tuner.choose(512, 256)["operand_mode"] == 1
    assert len(calls) == 11                     # served from memory
    data = json.loads(path.read_text())
    assert data["GB300-test|shared|512|256"]["operand_mode"] == 1
    assert data["GB300-test|shared|1024|512"]["pair"] == 1
    # a new tuner reads the file instead of timing again
    other = PlanTuner(cache_path=str(path), timer=timer, device_name="GB300-test")
    assert other.choose(128, 64)["variant"] == "fp32"
    assert len(calls) == 11
    # another device name, or plans with their own workspace, are different keys
    third = PlanTuner(cache_path=str(path), timer=timer, device_name="other-gpu")
    third.choose(128, 64)
    assert len(calls) == 14
    own = PlanTuner(cache_path=str(path), timer=timer, device_name="GB300-test",
                    own_workspace=True)
    own.choose(128, 64)
    assert len(calls) == 18


def test_failing_candidates_are_skipped(tmp_path):
    def timer(n, m, cfg):
        if cfg["variant"] == "split_bf16":
            raise RuntimeError("not on this device")
        return 1.0
    tuner = PlanTuner(cache_path=str(tmp_path / "t.json"), timer=timer, device_name="x")
    assert tuner.choose(256, 128) == {"variant": "fp32", "operand_mode": 0, "pair": 0,
                                      "split_k": 1, "seconds": 1.0}


def test_unwritable_cache_still_chooses(tmp_path):
    blocker = tmp_path / "file"
    blocker.write_text("x")
    tuner = PlanTuner(cache_path=str(blocker / "sub" / "tune.json"), device_name="x",
                      timer=lambda n, m, cfg: 1.0 if cfg["variant"] == "fp32" else 2.0)
    assert tuner.choose(64, 32)["variant"] == "fp32"
