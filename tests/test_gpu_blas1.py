"""Transpose, axpy/scal, row extraction and the deterministic reductions
through the C ABI, against the reference's golden values and numpy."""
import numpy as np
import pytest

from tests.helpers import colmajor, from_dev, goldens, ptr, stream, to_dev

pytestmark = pytest.mark.gpu
G = goldens()
PFX = {np.float32: "s", np.float64: "d"}


def _flat(values, dt):
    import torch
    return torch.tensor(np.asarray(values, dtype=dt)).cuda()


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_transpose_golden_and_random(gbla_lib, cuda, dt):
    import torch
    A = colmajor(G["transpose_a"], 3, 2, 2)
    Ad = to_dev(A, dt)
    At = torch.empty_like(Ad)
    assert getattr(gbla_lib, f"gbla_{PFX[dt]}transpose_batched")(3, 2, ptr(Ad), 6, ptr(At), 6, 2, stream()) == 0
    assert np.array_equal(At.cpu().numpy().ravel(), np.array(G["transpose_expected"], dtype=dt))
    rng = np.random.default_rng(0)
    for (m, n, k) in [(1, 1, 1), (33, 65, 3), (8, 8, 70000), (128, 7, 5)]:
        X = rng.standard_normal((k, m, n)).astype(dt)
        Xd = to_dev(X, dt)
        Xt = torch.empty_like(Xd)
        assert getattr(gbla_lib, f"gbla_{PFX[dt]}transpose_batched")(m, n, ptr(Xd), m * n, ptr(Xt), m * n, k,
                                                                       stream()) == 0
        assert np.array_equal(from_dev(Xt, k, n, m), X.transpose(0, 2, 1))


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_axpy_scal_golden(gbla_lib, cuda, dt):
    a, b = _flat(G["tensor_234A"], dt), _flat(G["tensor_234B"], dt)
    p = PFX[dt]
    assert getattr(gbla_lib, f"gbla_{p}axpy")(24, 1.0, ptr(b), ptr(a), stream()) == 0
    assert np.array_equal(a.cpu().numpy(), np.array(G["tensor_234APB"], dtype=dt))
    a = _flat(G["tensor_234A"], dt)
    assert getattr(gbla_lib, f"gbla_{p}axpy")(24, -1.0, ptr(b), ptr(a), stream()) == 0
    assert np.array_equal(a.cpu().numpy(), np.array(G["tensor_234AMB"], dtype=dt))
    a = _flat(G["tensor_234A"], dt)
    assert getattr(gbla_lib, f"gbla_{p}scal")(24, 3.0, ptr(a), stream()) == 0
    assert np.array_equal(a.cpu().numpy(), 3 * np.array(G["tensor_234A"], dtype=dt))


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_reductions_golden(gbla_lib, cuda, dt):
    import torch
    p = PFX[dt]
    ws = torch.empty(gbla_lib.gbla_reduce_workspace_bytes(), dtype=torch.uint8, device="cuda")
    res = torch.zeros(1, dtype=torch.float32 if dt == np.float32 else torch.float64, device="cuda")
    a, b = _flat(G["tensor_234A"], dt), _flat(G["tensor_234B"], dt)
    amb = _flat(G["tensor_234AMB"], dt)
    tol = G["precision_low"] if dt == np.float32 else G["precision_high"]
    assert getattr(gbla_lib, f"gbla_{p}dot")(24, ptr(a), ptr(b), ptr(res), ptr(ws), stream()) == 0
    assert res.item() == G["dotF"]
    assert getattr(gbla_lib, f"gbla_{p}nrm2")(24, ptr(a), ptr(res), ptr(ws), stream()) == 0
    assert abs(res.item() - G["normF"]) < tol
    assert getattr(gbla_lib, f"gbla_{p}asum")(24, ptr(a), ptr(res), ptr(ws), stream()) == 0
    assert abs(res.item() - G["sumAbs"]) < tol
    assert getattr(gbla_lib, f"gbla_{p}amax")(24, ptr(amb), ptr(res), ptr(ws), stream()) == 0
    assert res.item() == G["maxAbs"]
    assert getattr(gbla_lib, f"gbla_{p}amin")(24, ptr(amb), ptr(res), ptr(ws), stream()) == 0
    assert res.item() == G["minAbs"]


@pytest.mark.parametrize("length", [1, 255, 256 * 4 * 1024 + 3, 50_000_000])
def test_reductions_random_and_deterministic(gbla_lib, cuda, length):
    import torch
    rng = np.random.default_rng(length)
    x = rng.standard_normal(length)
    y = rng.standard_normal(length)
    xd, yd = torch.tensor(x).cuda(), torch.tensor(y).cuda()
    ws = torch.empty(gbla_lib.gbla_reduce_workspace_bytes(), dtype=torch.uint8, device="cuda")
    r1 = torch.zeros(1, dtype=torch.float64, device="cuda")
    r2 = torch.zeros(1, dtype=torch.float64, device="cuda")
    assert gbla_lib.gbla_ddot(length, ptr(xd), ptr(yd), ptr(r1), ptr(ws), stream()) == 0
    assert gbla_lib.gbla_ddot(length, ptr(xd), ptr(yd), ptr(r2), ptr(ws), stream()) == 0
    assert r1.item() == r2.item()  # bitwise reproducible
    assert abs(r1.item() - float(x @ y)) < 1e-9 * max(1.0, np.abs(x).sum())
    assert gbla_lib.gbla_damax(length, ptr(xd), ptr(r1), ptr(ws), stream()) == 0
    assert r1.item() == np.abs(x).max()
    assert gbla_lib.gbla_damin(length, ptr(xd), ptr(r1), ptr(ws), stream()) == 0
    assert r1.item() == np.abs(x).min()
    xs = torch.tensor(x.astype(np.float32)).cuda()
    rs = torch.zeros(1, dtype=torch.float32, device="cuda")
    assert gbla_lib.gbla_snrm2(length, ptr(xs), ptr(rs), ptr(ws), stream()) == 0
    assert abs(rs.item() - np.linalg.norm(x.astype(np.float32).astype(np.float64))) < 1e-5 * np.sqrt(length)


def _norm_exact(x):
    """Euclidean norm in FP64 (float data) or through a power-of-two rescale
    (double data near the ends of the exponent range)."""
    x = np.asarray(x, dtype=np.float64)
    amax = np.abs(x).max()
    if amax == 0:
        return 0.0
    e = np.frexp(amax)[1]
    return float(np.ldexp(np.linalg.norm(np.ldexp(x, -e)), e))


@pytest.mark.parametrize("dt,scale", [(np.float32, 1e30), (np.float32, 1e-30), (np.float32, 1e19),
                                      (np.float32, 1e-20), (np.float64, 1e300), (np.float64, 1e-300),
                                      (np.float64, 1e160), (np.float64, 1e-160)])
@pytest.mark.parametrize("length", [7, 100_003])
def test_nrm2_extreme_magnitudes(gbla_lib, cuda, dt, scale, length):
    """nrm2 neither overflows nor underflows where the norm is representable
    (a plain sum of squares returns inf above ~1.8e19 and 0 below ~1e-23 in
    float, inf above ~1.3e154 and 0 below ~1.5e-162 in double)."""
    import torch
    rng = np.random.default_rng(length)
    x = (rng.standard_normal(length) * scale).astype(dt)
    x[length // 2] = dt(scale * 3.0)  # one entry well above the others
    xd = torch.tensor(x).cuda()
    ws = torch.empty(gbla_lib.gbla_reduce_workspace_bytes(), dtype=torch.uint8, device="cuda")
    res = torch.zeros(1, dtype=xd.dtype, device="cuda")
    assert getattr(gbla_lib, f"gbla_{PFX[dt]}nrm2")(length, ptr(xd), ptr(res), ptr(ws), stream()) == 0
    got, want = res.item(), _norm_exact(x)
    assert np.isfinite(got) and got > 0
    tol = (1e-5 if dt == np.float32 else 1e-12) * max(1.0, np.sqrt(length) / 10)
    assert abs(got - want) <= tol * want, (got, want)


def test_nrm2_mixed_magnitudes(gbla_lib, cuda):
    """Entries from all three magnitude classes in one vector, float and double."""
    import torch
    ws = torch.empty(gbla_lib.gbla_reduce_workspace_bytes(), dtype=torch.uint8, device="cuda")
    for dt, vals in ((np.float32, [3e20, 4e20, 1.0, 2.0, 1e-25, 5e-30]),
                     (np.float64, [3e200, 4e200, 1.0, 1e-200, 2e-300])):
        x = np.array(vals * 1000, dtype=dt)
        xd = torch.tensor(x).cuda()
        res = torch.zeros(1, dtype=xd.dtype, device="cuda")
        assert getattr(gbla_lib, f"gbla_{PFX[dt]}nrm2")(len(x), ptr(xd), ptr(res), ptr(ws), stream()) == 0
        want = _norm_exact(x)
        assert abs(res.item() - want) <= (1e-6 if dt == np.float32 else 1e-14) * want * 10
    zero = torch.zeros(5, dtype=torch.float32, device="cuda")
    res = torch.full((1,), 7.0, dtype=torch.float32, device="cuda")
    assert gbla_lib.gbla_snrm2(5, ptr(zero), ptr(res), ptr(ws), stream()) == 0
    assert res.item() == 0.0


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_copy_rows_golden(gbla_lib, cuda, dt):
    import torch
    A = colmajor(G["getRows_a"], 3, 3, 2)
    Ad = to_dev(A, dt)
    out = torch.empty(3, dtype=Ad.dtype, device="cuda")
    p = PFX[dt]
    assert getattr(gbla_lib, f"gbla_{p}copy_rows")(3, 3, 1, 1, ptr(Ad), ptr(out), stream()) == 0
    assert np.array_equal(out.cpu().numpy(), np.array(G["getRows_expected0"], dtype=dt))
    out = torch.empty(6, dtype=Ad.dtype, device="cuda")
    assert getattr(gbla_lib, f"gbla_{p}copy_rows")(3, 3, 1, 2, ptr(Ad) + 9 * Ad.element_size(), ptr(out),
                                                    stream()) == 0
    assert np.array_equal(out.cpu().numpy(), np.array(G["getRows_expected1"], dtype=dt))


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_givens_annihilate_batched(gbla_lib, cuda, dt):
    """Every matrix gets its own rotation of rows i, k zeroing (k, j): the
    batched form of GivensAnnihilator::annihilate, checked against a numpy
    restatement of k_givensAnnihilateRHypot + rot on each matrix."""
    import torch
    rng = np.random.default_rng(11)
    k, m, n = 37, 6, 9
    A = rng.standard_normal((k, m, n))
    Ad = to_dev(A, dt)
    co = torch.zeros(3 * k, dtype=Ad.dtype, device="cuda")
    p = PFX[dt]
    assert getattr(gbla_lib, f"gbla_{p}givens_annihilate_batched")(m, n, ptr(Ad), m * n, 4, 1, 3, ptr(co), k,
                                                                    stream()) == 0
    got = from_dev(Ad, k, m, n)
    want = A.copy()
    r = 1.0 / np.hypot(A[:, 4, 3], A[:, 1, 3])
    c, s = A[:, 4, 3] * r, A[:, 1, 3] * r
    want[:, 4, :] = c[:, None] * A[:, 4, :] + s[:, None] * A[:, 1, :]
    want[:, 1, :] = c[:, None] * A[:, 1, :] - s[:, None] * A[:, 4, :]
    tol = 1e-5 if dt == np.float32 else 1e-13
    assert np.abs(got - want).max() < tol
    assert np.abs(got[:, 1, 3]).max() < tol
    np.testing.assert_allclose(co.cpu().numpy().reshape(k, 3), np.stack([r, c, s], 1), rtol=tol)
    # invalid: i == k, out-of-range row
    assert getattr(gbla_lib, f"gbla_{p}givens_annihilate_batched")(m, n, ptr(Ad), m * n, 2, 2, 0, None, k,
                                                                    stream()) == 1
    assert getattr(gbla_lib, f"gbla_{p}givens_annihilate_batched")(m, n, ptr(Ad), m * n, 6, 1, 0, None, k,
                                                                    stream()) == 1


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_rot_batched_left_and_right(gbla_lib, cuda, dt):
    import torch
    rng = np.random.default_rng(12)
    k, m, n = 50, 8, 5
    A = rng.standard_normal((k, m, n))
    th = rng.uniform(0, 2 * np.pi, k)
    c, s = np.cos(th), np.sin(th)
    cd = torch.tensor(c, dtype=torch.float32 if dt == np.float32 else torch.float64, device="cuda")
    sd = torch.tensor(s, dtype=cd.dtype, device="cuda")
    p = PFX[dt]
    tol = 1e-5 if dt == np.float32 else 1e-13
    # left: rows 2 and 6 of every matrix
    Ad = to_dev(A, dt)
    base = ptr(Ad)
    es = Ad.element_size()
    assert getattr(gbla_lib, f"gbla_{p}rot_batched")(n, base + 2 * es, m, base + 6 * es, m, m * n, ptr(cd), ptr(sd),
                                                      1, k, stream()) == 0
    want = A.copy()
    want[:, 2, :] = c[:, None] * A[:, 2, :] + s[:, None] * A[:, 6, :]
    want[:, 6, :] = c[:, None] * A[:, 6, :] - s[:, None] * A[:, 2, :]
    assert np.abs(from_dev(Ad, k, m, n) - want).max() < tol
    # right: columns 0 and 3
    Ad = to_dev(A, dt)
    base = ptr(Ad)
    assert getattr(gbla_lib, f"gbla_{p}rot_batched")(m, base, 1, base + 3 * m * es, 1, m * n, ptr(cd), ptr(sd), 1,
                                                      k, stream()) == 0
    want = A.copy()
    want[:, :, 0] = c[:, None] * A[:, :, 0] + s[:, None] * A[:, :, 3]
    want[:, :, 3] = c[:, None] * A[:, :, 3] - s[:, None] * A[:, :, 0]
    assert np.abs(from_dev(Ad, k, m, n) - want).max() < tol
