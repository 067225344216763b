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
