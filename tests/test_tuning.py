"""The launch-shape autotuner: candidates and cache on the CPU, tuning on the GPU."""

from __future__ import annotations

import json

import numpy as np
import pytest

from commkit_gb300 import LDPCCode, tuning, workloads as W


def test_candidates_respect_the_lifting():
    shapes = tuning.candidates({"quasi_cyclic": 1, "lifting": 384})
    ts = {t for t, _, _ in shapes}
    assert ts and all(t % 32 == 0 and (384 % t == 0 or t % 384 == 0) and t <= 768 for t in ts)
    assert 384 in ts and 768 in ts
    shapes = tuning.candidates({"quasi_cyclic": 1, "lifting": 54})  # padded to 64
    assert {t for t, _, _ in shapes} == {32, 64, 128}
    assert {t for t, _, _ in tuning.candidates({"quasi_cyclic": 0, "lifting": 0})} == {32, 64, 128, 256, 512}
    # One message per edge only with one thread per row slot (the specialised kernel), circulant codes only.
    from commkit_gb300 import _lib

    assert {t for t, _, p in shapes if p == _lib.CK_LDPC_PLACE_EDGES} == {64}
    assert not any(p == _lib.CK_LDPC_PLACE_EDGES for _, _, p in tuning.candidates({"quasi_cyclic": 0, "lifting": 0}))


def test_cache_roundtrip_and_key(tmp_path, monkeypatch):
    monkeypatch.setenv("COMMKIT_GB300_TUNING", str(tmp_path / "t.json"))
    code = LDPCCode.quasi_cyclic(W.CODE_A.base(), lifting=54)
    k1 = tuning.code_key(code, "GPU X")
    k2 = tuning.code_key(LDPCCode.quasi_cyclic(W.CODE_A.base(), lifting=54), "GPU X")
    k3 = tuning.code_key(LDPCCode.quasi_cyclic(W.CODE_B.base(), lifting=96), "GPU X")
    assert k1 == k2 != k3 and k1.startswith("GPU X|")
    tuning._store({k1: {"threads_per_frame": 64, "frames_per_block": 4, "placement": 1}})
    assert json.loads((tmp_path / "t.json").read_text())[k1]["frames_per_block"] == 4


@pytest.mark.gpu
def test_tune_picks_a_shape_and_keeps_results(tmp_path, monkeypatch):
    import torch

    import commkit_gb300 as ck

    monkeypatch.setenv("COMMKIT_GB300_TUNING", str(tmp_path / "t.json"))
    dev = torch.device("cuda", 0)
    code = ck.LDPCCode.quasi_cyclic(W.CODE_B.base(), lifting=96)
    b = W.coded_batch(W.CODE_B, 200, 16, 5.4, seed=3)
    llr = ck.compute_llr_frames(torch.from_numpy(b.symbols).to(dev), noise_var=b.noise_var,
                                constellation=ck.Constellation.qam(16))  # fmt: skip
    before = ck.decode(llr, code=code)
    best = tuning.tune(code, device=0, frames=304, iterations=3, reps=1)
    assert best["tried"] > 1 and best["ms"] > 0
    after = ck.decode(llr, code=code)
    np.testing.assert_array_equal(before.llrs.cpu().numpy(), after.llrs.cpu().numpy())
    np.testing.assert_array_equal(before.iterations.cpu().numpy(), after.iterations.cpu().numpy())
    # a fresh code object picks the cached shape up
    code2 = ck.LDPCCode.quasi_cyclic(W.CODE_B.base(), lifting=96)
    assert code2._plan(0).get_launch() == (best["threads_per_frame"], best["frames_per_block"], best["placement"])
    code._plan(0).set_launch(0, 0, 0)


@pytest.mark.gpu
def test_tuning_batch_sits_in_the_waterfall():
    """The default timing batch: frames near the code's waterfall, decoded
    with early stop, so iteration counts are uneven as in service."""
    import commkit_gb300 as ck

    code = ck.LDPCCode.quasi_cyclic(W.CODE_A.base(), lifting=54)
    llr, mu = tuning.waterfall_llrs(code, 512, device=0, iterations=50)
    assert llr.shape == (512, code.n) and mu > 0
    res = ck.decode(llr, code=code, method=ck.MinSum(max_iterations=50))
    fer = float((~res.valid).float().mean())
    its = res.iterations.cpu().numpy()
    assert 0.2 < fer < 0.8, fer
    assert its.min() < 25 and its.max() == 50
