"""Autotuner logic on the CPU (fake plan, fake timer) and on the GPU."""
import numpy as np
import pytest


class FakePlan:
    def __init__(self, precision):
        self.n = 512
        self.precision = precision
        self.cfg = {}

    def set_tuning(self, **kw):
        self.cfg.update(kw)


def test_candidates_cover_the_space():
    from ntk import autotune

    c = autotune.candidates("fp64")
    assert {"f64_x_variant": 0, "f64_threads": 64} in c and len(c) == 4
    c = autotune.candidates("fp32_refine")
    assert len(c) == 17
    for w in (4, 8, 16):
        assert {"refine_kernel": 2, "refine_w": w, "refine_prefetch": 1, "refine_tps": 32} in c
        assert {"refine_kernel": 3, "refine_w": w, "refine_tps": 32} in c
    assert {"refine_kernel": 1, "refine_w": 8, "refine_spw": 2, "refine_tps": 32} in c
    assert {"refine_kernel": 1, "refine_w": 16, "refine_spw": 1, "refine_tps": 32} in c
    assert {"refine_kernel": 1, "refine_w": 16, "refine_spw": 2, "refine_tps": 32} not in c  # > 16 systems per CTA
    # threads per system: 64 (two 512-row windows) only for 512 < n <= 1024
    assert all(x.get("refine_tps", 32) == 32 for x in autotune.candidates("fp32_refine", 512))
    c1024 = autotune.candidates("fp32_refine", 1024)
    assert {"refine_kernel": 1, "refine_w": 8, "refine_spw": 1, "refine_tps": 64} in c1024
    assert len(c1024) == 17 + 5


def test_tune_picks_fastest_and_caches(tmp_path, monkeypatch):
    from ntk import autotune

    monkeypatch.setenv("NTK_AUTOTUNE_CACHE", str(tmp_path / "cache.json"))
    monkeypatch.setattr(autotune, "device_name", lambda: "FAKE-GPU")
    plan = FakePlan("fp32_refine")
    fake_ms = {(1, 4, 1): 2.0, (1, 8, 1): 1.0, (1, 16, 1): 0.75, (1, 4, 2): 1.5, (1, 8, 2): 0.5,
               (3, 4, 1): 0.9, (3, 8, 1): 0.6, (3, 16, 1): 0.7, (2, 4, 1): 0.95, (2, 8, 1): 0.65, (2, 16, 1): 0.8}
    best = {"refine_kernel": 1, "refine_w": 8, "refine_spw": 2, "refine_tps": 32}

    def timer(run, repeats):
        c = plan.cfg
        return fake_ms[(c["refine_kernel"], c["refine_w"], c.get("refine_spw", 1) if c["refine_kernel"] == 1 else 1)] \
            + 0.01 * c.get("refine_prefetch", 0)

    res = autotune.tune(plan, lambda: None, key="compact-x", timer=timer)
    assert res["config"] == best and all(plan.cfg[k] == v for k, v in best.items())
    plan2 = FakePlan("fp32_refine")
    assert autotune.apply_cached(plan2, "compact-x") == best
    assert all(plan2.cfg[k] == v for k, v in best.items())
    # a cache hit does not time again
    res2 = autotune.tune(FakePlan("fp32_refine"), lambda: None, key="compact-x",
                         timer=lambda *a: pytest.fail("timed despite cache"))
    assert res2["config"] == best


@pytest.mark.gpu
def test_tune_on_gpu_keeps_results_correct(cuda, oracle, tmp_path, monkeypatch):
    import torch

    import ntk
    from ntk import autotune

    monkeypatch.setenv("NTK_AUTOTUNE_CACHE", str(tmp_path / "cache.json"))
    n = 256
    f = np.random.default_rng(0).normal(size=(8, 64, n))
    ft = torch.from_numpy(f).to(cuda)
    out = torch.empty_like(ft)
    for prec, tol in (("fp64", 1e-13), ("fp32_refine", 1e-12)):
        with ntk.Plan(n, 0, ntk.COMPACT_COEFFS, precision=prec) as p:
            res = autotune.tune(p, lambda: p.compact_deriv(ft, out, axis=2, h=0.01), key="t")
            cur = p.get_tuning()
            assert all(cur[k] == v for k, v in res["config"].items())
            p.compact_deriv(ft, out, axis=2, h=0.01)
            torch.cuda.synchronize()
        assert oracle.rel_err(out.cpu().numpy(), oracle.banded_compact_deriv(f, 0.01, 2)) < tol
