"""Uneven batches (one persistent launch over systems of different lengths
and coefficients) against per-system long-double Thomas solves (the
reference's CPU path, a banded LAPACK solve, agrees with it to rounding on
these diagonally dominant systems).  Tolerance 1e-13 relative per system."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TOL = 1e-13


def _descriptors(lengths, systems):
    interior = np.array([s[0] for s in systems])
    head = np.array([s[1] for s in systems])
    tail = np.array([s[2] for s in systems])
    return interior, head, tail


def _bands(n, interior, head, tail):
    """Rows 0, 1 from head, rows n-2, n-1 from tail; for n = 3 the shared
    middle row is head's second row (ntk_batch_create's rule)."""
    a = np.full(n, interior[0])
    b = np.full(n, interior[1])
    c = np.full(n, interior[2])
    for r in range(2):
        if n - 2 + r >= 2:
            a[n - 2 + r], b[n - 2 + r], c[n - 2 + r] = tail[r]
    for r in range(2):
        a[r], b[r], c[r] = head[r]
    a[0] = 0.0
    c[-1] = 0.0
    return a, b, c


def _check(cuda, oracle, lengths, interior, head, tail, seed, offsets=None, precision="fp64"):
    import ntk

    with ntk.UnevenBatch(lengths, interior, head, tail, offsets=offsets, precision=precision) as bt:
        total = bt.elements
        d = np.random.default_rng(seed).normal(size=total)
        t = torch.from_numpy(d).to(cuda)
        bt.solve(t)
        torch.cuda.synchronize()
        x = t.cpu().numpy()
        info = bt.info()
        offs = bt.offsets
    worst = 0.0
    for s, n in enumerate(lengths):
        o = int(offs[s])
        a, b, c = _bands(int(n), interior[s], head[s], tail[s])
        ref = oracle.thomas_ld(a, b, c, d[o:o + n])
        worst = max(worst, oracle.rel_err(x[o:o + n], ref))
    return worst, info, x, d


def test_uneven_workload_4096(cuda, oracle):
    """4096 systems, lengths log-uniform in [32, 8192], b = 1, a, c ~ U(0.1, 0.3),
    random diagonally dominant end rows, RHS N(0, 1)."""
    from ntk.workloads import uneven_batch

    lengths, systems = uneven_batch(4096, seed=0)
    interior, head, tail = _descriptors(lengths, systems)
    worst, info, _, _ = _check(cuda, oracle, lengths, interior, head, tail, seed=1)
    assert worst < TOL
    assert info["max_n"] <= 8192 and info["segmented"] > 0


# FP64 windows: n <= 512 one padded window; 513 (the last window starts at
# the second head row, its own pivot sequence), 514, 600, 1000, 20000 first /
# middle / last windows.
@pytest.mark.parametrize("n", [3, 4, 5, 31, 130, 512, 513, 514, 600, 1000, 20000])
def test_single_lengths(cuda, oracle, n):
    rng = np.random.default_rng(n)
    k = 5
    lengths = np.full(k, n)
    interior = np.column_stack([rng.uniform(0.1, 0.3, k), np.ones(k), rng.uniform(0.1, 0.3, k)])
    head = rng.uniform(-0.3, 0.3, size=(k, 2, 3))
    head[:, :, 1] = 2.0
    tail = rng.uniform(-0.3, 0.3, size=(k, 2, 3))
    tail[:, :, 1] = 2.0
    worst, _, _, _ = _check(cuda, oracle, lengths, interior, head, tail, seed=n)
    assert worst < TOL


def test_weak_decay_falls_back_to_one_lane(cuda, oracle):
    """a = c = 0.49, b = 1: the factors decay too slowly for an exact halo,
    so the system runs unsegmented and is still exact."""
    n = 4096
    lengths = np.array([n, 300])
    interior = np.array([[0.49, 1.0, 0.49], [0.2, 1.0, 0.2]])
    head = np.array([[[0, 1.0, 0.49], [0.49, 1.0, 0.49]]] * 2)
    tail = np.array([[[0.49, 1.0, 0.49], [0.49, 1.0, 0]]] * 2)
    worst, info, _, _ = _check(cuda, oracle, lengths, interior, head, tail, seed=4)
    assert worst < 1e-12


def test_gapped_offsets_leave_gaps_untouched(cuda, oracle):
    lengths = np.array([50, 70, 90])
    offsets = np.array([5, 100, 300])
    interior = np.tile([0.2, 1.0, 0.25], (3, 1))
    head = np.tile([[0, 1.5, 0.3], [0.2, 1.2, 0.3]], (3, 1, 1))
    tail = np.tile([[0.2, 1.1, 0.3], [0.3, 1.4, 0]], (3, 1, 1))
    worst, _, x, d = _check(cuda, oracle, lengths, interior, head, tail, seed=5, offsets=offsets)
    assert worst < TOL
    untouched = np.ones(len(d), bool)
    for o, n in zip(offsets, lengths):
        untouched[o:o + n] = False
    assert np.array_equal(x[untouched], d[untouched])


def test_overlap_and_bad_length_rejected(cuda):
    import ntk

    inter = np.tile([0.2, 1.0, 0.2], (2, 1))
    hd = np.tile([[0, 1.0, 0.2], [0.2, 1.0, 0.2]], (2, 1, 1))
    with pytest.raises(ValueError, match="overlap"):
        ntk.UnevenBatch([10, 10], inter, hd, hd, offsets=[0, 5])
    with pytest.raises(ValueError):
        ntk.UnevenBatch([2, 10], inter, hd, hd)


def test_empty_batch(cuda):
    import ntk

    with ntk.UnevenBatch(np.zeros(0, int), np.zeros((0, 3)), np.zeros((0, 2, 3)), np.zeros((0, 2, 3))) as bt:
        bt.solve(torch.zeros(1, dtype=torch.float64, device=cuda))


# FP32 solve + double-word refinement over overlapping 512-row windows
# (systems up to 512 rows are one padded window): within 1e-12 relative of
# the long-double Thomas per system, the refinement tolerance.
REFINE_TOL = 1e-12


def test_refine_uneven_workload_4096(cuda, oracle):
    from ntk.workloads import uneven_batch

    lengths, systems = uneven_batch(4096, seed=0)
    interior, head, tail = _descriptors(lengths, systems)
    worst, _, _, _ = _check(cuda, oracle, lengths, interior, head, tail, seed=1, precision="fp32_refine")
    assert worst < REFINE_TOL, worst


@pytest.mark.parametrize("n", [3, 4, 5, 31, 130, 511, 512, 513, 1000, 20000])
def test_refine_single_lengths(cuda, oracle, n):
    rng = np.random.default_rng(n)
    k = 5
    lengths = np.full(k, n)
    interior = np.column_stack([rng.uniform(0.1, 0.3, k), np.ones(k), rng.uniform(0.1, 0.3, k)])
    head = rng.uniform(-0.3, 0.3, size=(k, 2, 3))
    head[:, :, 1] = 2.0
    tail = rng.uniform(-0.3, 0.3, size=(k, 2, 3))
    tail[:, :, 1] = 2.0
    worst, _, _, _ = _check(cuda, oracle, lengths, interior, head, tail, seed=n, precision="fp32_refine")
    assert worst < REFINE_TOL, worst


def test_refine_gapped_offsets_leave_gaps_untouched(cuda, oracle):
    lengths = np.array([50, 700, 90])
    offsets = np.array([5, 100, 1000])
    interior = np.tile([0.2, 1.0, 0.25], (3, 1))
    head = np.tile([[0, 1.5, 0.3], [0.2, 1.2, 0.3]], (3, 1, 1))
    tail = np.tile([[0.2, 1.1, 0.3], [0.3, 1.4, 0]], (3, 1, 1))
    worst, _, x, d = _check(cuda, oracle, lengths, interior, head, tail, seed=5, offsets=offsets,
                            precision="fp32_refine")
    assert worst < REFINE_TOL
    untouched = np.ones(len(d), bool)
    for o, n in zip(offsets, lengths):
        untouched[o:o + n] = False
    assert np.array_equal(x[untouched], d[untouched])


def test_refine_rejects_slow_decay(cuda):
    import ntk

    inter = np.array([[0.49, 1.0, 0.49]])
    hd = np.array([[[0, 1.0, 0.49], [0.49, 1.0, 0.49]]])
    with pytest.raises(Exception, match="NTK_FP64"):
        ntk.UnevenBatch([4096], inter, hd, hd, precision="fp32_refine")


@pytest.mark.parametrize("precision,tol", [("fp64", TOL), ("fp32_refine", 1e-12)])
def test_repeated_solves_in_one_stream(cuda, oracle, precision, tol):
    """Three solves of the same batch back to back: the windows' per-system
    counters (the last window of a system copies its border rows) reset
    themselves at the end of every launch, so each solve is complete."""
    import ntk
    from ntk.workloads import uneven_batch

    lengths, systems = uneven_batch(256, seed=7)
    interior, head, tail = _descriptors(lengths, systems)
    rng = np.random.default_rng(8)
    with ntk.UnevenBatch(lengths, interior, head, tail, precision=precision) as bt:
        offs = bt.offsets
        ds = [rng.normal(size=bt.elements) for _ in range(3)]
        ts = [torch.from_numpy(d).to(cuda) for d in ds]
        for t in ts:
            bt.solve(t)
        torch.cuda.synchronize()
        assert bt.status() == 0
    for d, t in zip(ds, ts):
        x = t.cpu().numpy()
        for s, n in enumerate(lengths):
            o = int(offs[s])
            a, b, c = _bands(int(n), interior[s], head[s], tail[s])
            ref = oracle.thomas_ld(a, b, c, d[o:o + n])
            assert oracle.rel_err(x[o:o + n], ref) < tol, (s, n)


def test_refine_benchmark_batch_takes_the_paired_chunk_windows(cuda):
    """The 4096-system batch (a, c <= 0.3): every 512-row window of the long
    systems qualifies for the paired-chunk solve (constant Toeplitz factors,
    end corrections per window kind)."""
    import ntk
    from ntk.workloads import uneven_batch

    lengths, systems = uneven_batch(4096, seed=0)
    interior, head, tail = _descriptors(lengths, systems)
    with ntk.UnevenBatch(lengths, interior, head, tail, precision="fp32_refine") as bt:
        w = bt.windows()
    short = int(np.sum(np.asarray(lengths) < 512))
    assert w["paired"] == w["windows"] - short, w


@pytest.mark.parametrize("precision,tol", [("fp32_refine", REFINE_TOL), ("fp32", 2e-5)])
def test_mixed_paired_and_chunked_windows(cuda, oracle, precision, tol):
    """Systems whose factors decay fast (a = c = 0.2: paired-chunk windows)
    beside systems that decay slowly (a = c = 0.45: the chunked windows with
    per-window tables) and short ones, at unaligned offsets, in one launch."""
    import ntk

    lengths = np.array([512, 1500, 3000, 700, 512, 2048, 300, 4099])
    k = len(lengths)
    slow = np.array([0, 1, 0, 1, 1, 0, 0, 1], bool)
    ac = np.where(slow, 0.45, 0.2)
    interior = np.column_stack([ac, np.ones(k), ac])
    rng = np.random.default_rng(21)
    head = rng.uniform(-0.3, 0.3, size=(k, 2, 3))
    head[:, :, 1] = 1.8
    tail = rng.uniform(-0.3, 0.3, size=(k, 2, 3))
    tail[:, :, 1] = 1.8
    offsets = np.cumsum(np.concatenate([[3], lengths[:-1] + 1]))
    with ntk.UnevenBatch(lengths, interior, head, tail, offsets=offsets, precision=precision) as bt:
        w = bt.windows()
    assert 0 < w["paired"] < w["windows"], w
    worst, _, _, _ = _check(cuda, oracle, lengths, interior, head, tail, seed=22, offsets=offsets,
                            precision=precision)
    assert worst < tol, worst
