"""Autotuner: times the candidate realizations / geometries on the GPU, rejects candidates
that miss the reference's accuracy gate on a prefix, and returns a plan that filters correctly."""
import json

import numpy as np
import pytest
import torch

import oracle
from cuda_recursive_filtering_gb300 import autotune

pytestmark = pytest.mark.gpu


def test_tune_picks_a_passing_candidate_and_caches(tmp_path, cuda_device):
    from scipy import signal
    sos = signal.butter(16, 0.1, output="sos")
    cache = str(tmp_path / "tune.json")
    best = autotune.tune(sos, 1 << 20, reps=2, cache_path=cache)
    assert best["gsps"] > 0 and best["kernel"] in ("TC", "PH", "STCR_UNROLL", "DTCR_UNROLL")
    assert any(t["gsps"] is not None for t in best["table"])
    assert json.load(open(cache))
    again = autotune.tune(sos, 1 << 20, cache_path=cache)
    assert again["kernel"] == best["kernel"]
    plan = autotune.tuned_plan(sos, 1 << 18)
    x = np.random.default_rng(0).uniform(-1, 1, 1 << 18).astype(np.float32)
    y = plan(torch.from_numpy(x).cuda())
    plan.check()
    _, ref = oracle.reference_golden(sos, x)
    assert oracle.errors(y.cpu().numpy(), ref)["rel_max"] <= 1e-4


def test_tune_rejects_direct_form_at_order_16(cuda_device):
    from scipy import signal
    sos = signal.butter(16, 0.2, output="sos")
    res = autotune.tune(sos, 1 << 18, candidates=[("PLR", 0, 0), ("PH", 32, 64)], reps=1)
    plr = [t for t in res["table"] if t["kernel"] == "PLR"]
    assert plr and plr[0]["gsps"] is None  # the float32 direct form misses the gate
    assert res["kernel"] == "PH"
