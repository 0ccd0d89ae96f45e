"""The plan autotuner's choice and cache logic (CPU; timings injected)."""

import json

from dlux_gb300.autotune import PlanTuner, candidate_configs


def test_candidates():
    assert [c["variant"] for c in candidate_configs(256, 128)] == \
        ["split_bf16", "split_bf16", "fp32"]
    # the split form needs sides divisible by 8; no tensor cores: FP32 only
    assert candidate_configs(100, 64) == [{"variant": "fp32", "operand_mode": 0}]
    assert candidate_configs(256, 128, tensor_cores=False) == \
        [{"variant": "fp32", "operand_mode": 0}]


def test_chooses_fastest_and_caches(tmp_path):
    calls = []

    def timer(n, m, cfg):
        calls.append((n, m, cfg["variant"], cfg["operand_mode"]))
        t = {("split_bf16", 0): 3.0, ("split_bf16", 1): 2.0, ("fp32", 0): 5.0}
        if n == 128:   # a tiny transform: the CUDA-core form wins
            t[("fp32", 0)] = 1.0
        return t[(cfg["variant"], cfg["operand_mode"])]

    path = tmp_path / "tune.json"
    tuner = PlanTuner(cache_path=str(path), timer=timer, device_name="GB300-test")
    assert tuner.choose(512, 256)["variant"] == "split_bf16"
    assert tuner.choose(512, 256)["operand_mode"] == 1
    assert tuner.choose(128, 64)["variant"] == "fp32"
    assert len(calls) == 6                     # each shape timed once
    assert tuner.choose(512, 256)["operand_mode"] == 1
    assert len(calls) == 6                     # served from memory
    data = json.loads(path.read_text())
    assert data["GB300-test|512|256"]["operand_mode"] == 1
    # a new tuner reads the file instead of timing again
    other = PlanTuner(cache_path=str(path), timer=timer, device_name="GB300-test")
    assert other.choose(128, 64)["variant"] == "fp32"
    assert len(calls) == 6
    # another device name is a different key
    third = PlanTuner(cache_path=str(path), timer=timer, device_name="other-gpu")
    third.choose(128, 64)
    assert len(calls) == 9


def test_failing_candidates_are_skipped(tmp_path):
    def timer(n, m, cfg):
        if cfg["variant"] == "split_bf16":
            raise RuntimeError("not on this device")
        return 1.0
    tuner = PlanTuner(cache_path=str(tmp_path / "t.json"), timer=timer, device_name="x")
    assert tuner.choose(256, 128) == {"variant": "fp32", "operand_mode": 0, "seconds": 1.0}


def test_unwritable_cache_still_chooses(tmp_path):
    blocker = tmp_path / "file"
    blocker.write_text("x")
    tuner = PlanTuner(cache_path=str(blocker / "sub" / "tune.json"), device_name="x",
                      timer=lambda n, m, cfg: 1.0 if cfg["variant"] == "fp32" else 2.0)
    assert tuner.choose(64, 32)["variant"] == "fp32"
