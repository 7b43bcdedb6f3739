"""The autotuner's table on the CPU: keys, persistence, and the defaults it gives without timing."""

from __future__ import annotations

import json

import torch

from citrus_gb300.autotune import Autotuner


def test_choices_persist_and_defaults_hold(tmp_path):
    path = tmp_path / "tuning.json"
    key = Autotuner.key("small_k_gemm", torch.device("cpu"), M=120, K=36, J=64, batch=4, acc=1, aligned=1)
    assert key == "small_k_gemm|cpu|J=64,K=36,M=120,acc=1,aligned=1,batch=4"
    path.write_text(json.dumps({key: {"choice": [2, 8], "ms": {"[2, 8]": 1.0}}}))
    tuner = Autotuner(path, enabled=False)
    ran = []
    assert tuner.choose(key, ([1, 0], [2, 8]), ran.append, [0, 0]) == [2, 8]       # the stored choice
    assert tuner.choose("other", ([1, 0], [2, 8]), ran.append, [0, 0]) == [0, 0]   # off: the default, untimed
    assert ran == []
    # a stored choice that is no longer a candidate is not used
    assert tuner.choose(key, ([1, 0],), ran.append, [0, 0]) == [0, 0]
    broken = tmp_path / "broken.json"
    broken.write_text("{not json")
    assert Autotuner(broken, enabled=False).table == {}
