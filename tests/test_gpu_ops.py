"""The reference's stand-alone operators on the GPU: bit-identical to the
oracle (no contracted multiply-adds) and to the reference's golden vectors."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_compact_rhs_bitwise(cuda, oracle, golden):
    from compact.rhs import compute_rhs

    f = golden["rhs_in"]
    t = torch.from_numpy(f).to(cuda)
    out = torch.empty_like(t)
    compute_rhs(t, out, float(golden["rhs_dx"]))
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), golden["rhs_out"])


@pytest.mark.parametrize("shape", [(8, 8, 8), (7, 33, 65), (1, 3, 300)])
def test_compact_rhs_any_shape(cuda, oracle, shape):
    from compact.rhs import compute_rhs

    f = np.random.default_rng(1).normal(size=shape)
    t = torch.from_numpy(f).to(cuda)
    out = torch.empty_like(t)
    compute_rhs(t, out, 0.37)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), oracle.compact_rhs(f, 0.37))


@pytest.mark.parametrize("perm", [(0, 2, 1), (1, 2, 0), (2, 0, 1), (0, 1, 2), (1, 0, 2), (2, 1, 0)])
@pytest.mark.parametrize("shape", [(8, 8, 8), (5, 40, 67), (64, 3, 33)])
def test_permute_bitwise(cuda, oracle, perm, shape):
    from compact.permute import permute

    a = np.random.default_rng(2).normal(size=shape)
    ta = torch.from_numpy(a).to(cuda)
    tb = torch.empty([shape[p] for p in perm], dtype=torch.float64, device=cuda)
    permute(ta, tb, perm)
    torch.cuda.synchronize()
    assert np.array_equal(tb.cpu().numpy(), np.transpose(a, perm))


def test_permute_golden(cuda, golden):
    from compact.permute import permute

    ta = torch.from_numpy(golden["perm_in"]).to(cuda)
    for perm in [(0, 2, 1), (1, 2, 0), (2, 0, 1)]:
        tb = torch.empty_like(ta)
        permute(ta, tb, perm)
        torch.cuda.synchronize()
        assert np.array_equal(tb.cpu().numpy(), golden["perm_%d%d%d" % perm])


@pytest.mark.parametrize("N", [32, 50, 256])
def test_adi_rhs_bitwise(cuda, oracle, N):
    from adi.rhs import compute_rhs

    u = np.random.default_rng(N).normal(size=(N, N))
    d = np.random.default_rng(N + 1).normal(size=(N, N))
    tu = torch.from_numpy(u).to(cuda)
    td = torch.from_numpy(d).to(cuda)
    compute_rhs(tu, td, 1.0 / (N - 1), 0.01, N)
    torch.cuda.synchronize()
    ref = d.copy()
    oracle.adi_rhs(u, ref, 1.0 / (N - 1), 0.01)
    assert np.array_equal(td.cpu().numpy(), ref)


def test_adi_rhs_golden(cuda, golden):
    from adi.rhs import compute_rhs

    tu = torch.from_numpy(golden["adi_rhs_u"]).to(cuda)
    td = torch.from_numpy(golden["adi_rhs_d"]).to(cuda)
    compute_rhs(tu, td, 1.0 / 31, 0.01, 32)
    torch.cuda.synchronize()
    assert np.array_equal(td.cpu().numpy(), golden["adi_rhs_out"])


@pytest.mark.parametrize("N", [32, 33, 100, 2048])
def test_transpose(cuda, N):
    from adi.transpose import transpose

    a = np.random.default_rng(N).normal(size=(N, N))
    ta = torch.from_numpy(a).to(cuda)
    tb = torch.empty_like(ta)
    transpose(ta, tb, N)
    torch.cuda.synchronize()
    assert np.array_equal(tb.cpu().numpy(), a.T)
