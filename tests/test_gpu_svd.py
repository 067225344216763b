"""Batched one-sided Jacobi SVD, rank and null space through the C ABI,
against the FP64 oracle and the reference's golden values (Svd, Nullspace)."""
import numpy as np
import pytest

from gputils_gb300 import workloads
from oracle import oracle as O
from tests.helpers import colmajor, from_dev, goldens, ptr, rel_err, rowmajor, stream, to_dev

pytestmark = pytest.mark.gpu
G = goldens()
LOW = G["precision_low"]


def _svd(lib, A, compute_u=False, V0=None, tol=1e-6, max_sweeps=40, dt=np.float32):
    import torch
    k, m, n = A.shape
    tdt = torch.float32 if dt == np.float32 else torch.float64
    Ad = to_dev(A, dt)
    S = torch.zeros(k * n, dtype=tdt, device="cuda")
    Vt = torch.zeros(k * n * n, dtype=tdt, device="cuda")
    U = torch.zeros(k * m * m, dtype=tdt, device="cuda") if compute_u else None
    V0d = to_dev(V0, dt) if V0 is not None else None
    info = torch.full((k,), -1, dtype=torch.int32, device="cuda")
    sw = torch.zeros(k, dtype=torch.int32, device="cuda")
    fn = lib.gbla_sgesvj_batched if dt == np.float32 else lib.gbla_dgesvj_batched
    st = fn(m, n, ptr(Ad), m * n, ptr(S), n, ptr(Vt), n * n,
                                 ptr(U) if compute_u else None, m * m, ptr(V0d) if V0d is not None else None, n * n,
                                 tol, max_sweeps, ptr(info), ptr(sw), k, stream())
    assert st == 0
    out = {"S": S.cpu().numpy().reshape(k, n), "Vt": from_dev(Vt, k, n, n), "info": info.cpu().numpy(),
           "sweeps": sw.cpu().numpy()}
    if compute_u:
        out["U"] = from_dev(U, k, m, m)
    return out


def test_reference_golden_singular_values(gbla_lib, cuda):
    # singularValuesComputation (test/testTensor.cu:1059-1084)
    B = colmajor(G["svd_b"], 8, 3)
    r = _svd(gbla_lib, B, compute_u=True)
    assert r["info"][0] == 0
    assert abs(r["S"][0, 0] - G["svd_sigma1"]) < LOW
    assert abs(r["S"][0, 1] - G["svd_sigma2"]) < LOW


def test_reference_golden_signed_vectors(gbla_lib, cuda):
    # singularValuesMultipleMatrices (test/testTensor.cu:1126-1171), float tolerance 10 * 1e-4
    A = colmajor(G["svd_multi_a"], 3, 2, 3)
    r = _svd(gbla_lib, A, compute_u=True)
    vt_flat = np.concatenate([r["Vt"][i].T.ravel() for i in range(3)])
    np.testing.assert_allclose(vt_flat[:4], G["svd_multi_vt"][:4], atol=10 * LOW)
    np.testing.assert_allclose(r["S"].ravel(), G["svd_multi_s"], atol=10 * LOW)
    u_flat = np.concatenate([r["U"][i].T.ravel() for i in range(3)])
    np.testing.assert_allclose(u_flat, G["svd_multi_u"], atol=10 * LOW)


def test_reference_golden_rank(gbla_lib, cuda):
    # singularValuesRankMultipleMatrices (test/testTensor.cu:1178-1199)
    import torch
    A = colmajor(G["rank_a"], 4, 3, 3)
    r = _svd(gbla_lib, A)
    S = torch.tensor(r["S"].ravel(), device="cuda")
    rank = torch.zeros(3, dtype=torch.int32, device="cuda")
    assert gbla_lib.gbla_srank_batched(3, ptr(S), 3, LOW, ptr(rank), 3, stream()) == 0
    assert rank.cpu().tolist() == [G["rank0"], G["rank1"], G["rank2"]]


SHAPES = [(1, 1), (2, 2), (3, 2), (5, 5), (8, 3), (17, 17), (32, 32), (40, 7), (64, 32), (33, 33), (64, 64),
          (100, 50), (128, 64)]


@pytest.mark.parametrize("shape", SHAPES)
def test_random_vs_oracle(gbla_lib, cuda, shape):
    m, n = shape
    rng = np.random.default_rng(m * 1000 + n)
    k = 12
    A = rng.standard_normal((k, m, n)).astype(np.float32)
    r = _svd(gbla_lib, A, compute_u=True)
    o = O.gesvj(A, compute_u=True)
    assert (r["info"] == 0).all()
    assert rel_err(r["S"][:, None, :], o["S"][:, None, :]) < 1e-6
    V = r["Vt"].transpose(0, 2, 1)
    U = r["U"]
    A64 = A.astype(np.float64)
    rec = np.stack([U[i][:, :n] @ np.diag(r["S"][i]) @ r["Vt"][i] for i in range(k)])
    assert rel_err(rec, A64) < 5e-6
    assert np.abs(V.transpose(0, 2, 1) @ V - np.eye(n)).max() < 5e-6
    assert np.abs(U.transpose(0, 2, 1) @ U - np.eye(m)).max() < 5e-6
    # same sign rule as the oracle: every right singular vector points the
    # oracle's way, and agrees with it to the accuracy the stopping tolerance
    # allows for its gap (tol' sigma_max^2 / min_k |sigma_j^2 - sigma_k^2|)
    tol_eff = max(1e-6, 4 * np.sqrt(m) * 2.0 ** -24)
    for i in range(k):
        s2 = o["S"][i] ** 2
        d = np.abs(s2[:, None] - s2[None, :]) + np.diag(np.full(n, np.inf))
        bound = 1e-4 + 8 * tol_eff * s2[0] / d.min(axis=1)
        assert (np.abs(V[i] - o["V"][i]).max(axis=0) <= bound).all()
        well = bound < 0.1
        assert ((V[i] * o["V"][i]).sum(axis=0)[well] > 0.99).all()


def test_d4_config_full_size(gbla_lib, cuda):
    """Config D4 at full size: 8192 32x32 matrices of the parametric family,
    tol 1e-6.  Every matrix: info, reconstruction; a sample: sigma vs FP64."""
    A = workloads.d4_svd32()
    k = A.shape[0]
    r = _svd(gbla_lib, A, compute_u=True, tol=1e-6)
    assert (r["info"] == 0).all()
    assert r["sweeps"].max() <= 15
    rec = r["U"] @ (r["S"][:, :, None] * r["Vt"])
    assert rel_err(rec, A) < 5e-6
    idx = np.arange(0, k, 64)
    o = O.gesvj(A[idx])
    assert rel_err(r["S"][idx][:, None, :], o["S"][:, None, :]) < 1e-6


def test_warm_start_with_exact_vectors_converges_at_once(gbla_lib, cuda):
    A = workloads.svd_family(64, 32, seed=9)[0]
    o = O.gesvj(A)
    cold = _svd(gbla_lib, A)
    warm = _svd(gbla_lib, A, V0=o["V"].astype(np.float32))
    assert (warm["info"] == 0).all()
    assert warm["sweeps"].max() <= 3 < cold["sweeps"].min()
    assert rel_err(warm["S"][:, None, :], o["S"][:, None, :]) < 1e-6


def _nullspace(lib, A):
    import torch
    k, m, n = A.shape
    Ad = to_dev(A, np.float32)
    N = torch.zeros(k * n * n, dtype=torch.float32, device="cuda")
    P = torch.zeros(k * n * n, dtype=torch.float32, device="cuda")
    nul = torch.zeros(k, dtype=torch.int32, device="cuda")
    ws = torch.empty(lib.gbla_snullspace_workspace_bytes(m, n, k), dtype=torch.uint8, device="cuda")
    assert lib.gbla_snullspace_batched(m, n, ptr(Ad), m * n, ptr(N), ptr(P), ptr(nul), 1e-6, None, ptr(ws),
                                       ws.numel(), k, stream()) == 0
    return from_dev(N, k, n, n), from_dev(P, k, n, n), nul.cpu().numpy()


def test_reference_golden_nullspace(gbla_lib, cuda):
    # computeNullspaceTensor (test/testTensor.cu:1555-1592): 3x4x5, incl. a zero matrix
    A = colmajor(G["ns_a"], 3, 4, 5).astype(np.float32)
    N, P, nul = _nullspace(gbla_lib, A)
    for i in range(5):
        assert np.linalg.norm(A[i] @ N[i]) < LOW
        E = N[i].T @ N[i]
        assert abs(E[0, 0] - 1) < LOW
        assert np.abs(E - np.diag(np.diag(E))).max() < LOW
    assert nul[4] == 4  # the zero matrix
    # computeNullspaceTrivial (:1598-1618): full rank -> N == 0 exactly
    A = rowmajor(G["ns_trivial_rowmajor"], 3, 3, 2).astype(np.float32)
    N, P, nul = _nullspace(gbla_lib, A)
    assert np.linalg.norm(N) == 0 and (nul == 0).all()
    # projectOnNullspaceTensor (:1624-1663)
    A = rowmajor(G["ns_project_a_rowmajor"], 3, 7).astype(np.float32)
    N, P, nul = _nullspace(gbla_lib, A)
    x = np.array(G["ns_project_x"])
    proj = P[0] @ x
    assert np.linalg.norm(A[0] @ proj) < LOW
    other = np.array(G["ns_project_other"])
    y = N[0] @ other
    assert (y - proj) @ (proj - x) < LOW


def test_nullspace_random_rank_deficient(gbla_lib, cuda):
    rng = np.random.default_rng(3)
    k, m, n = 20, 12, 40
    A = rng.standard_normal((k, m, n)).astype(np.float32)
    A[::2, -3:, :] = 0.0   # rank 9 for even matrices
    N, P, nul = _nullspace(gbla_lib, A)
    for i in range(k):
        r = n - nul[i]
        assert r == (9 if i % 2 == 0 else 12)
        Ni = N[i][:, :nul[i]]
        assert np.abs(A[i] @ Ni).max() < 1e-4
        assert np.abs(Ni.T @ Ni - np.eye(nul[i])).max() < 1e-5
        assert np.abs(P[i] - Ni @ Ni.T).max() < 1e-5


def test_d5_family_64_converges(gbla_lib, cuda):
    """The 64x64 parametric family (config D5) on 1024 matrices: every matrix
    converges, sigma within 1e-6 of FP64 on a sample."""
    A = workloads.svd_family(1024, 64, seed=6)[0]
    r = _svd(gbla_lib, A, tol=1e-6, max_sweeps=60)
    assert (r["info"] == 0).all(), r["sweeps"].max()
    idx = np.arange(0, 1024, 37)
    o = O.gesvj(A[idx])
    assert rel_err(r["S"][idx][:, None, :], o["S"][:, None, :]) < 1e-6


@pytest.mark.parametrize("shape", [(3, 2), (8, 3), (32, 32), (20, 17), (64, 64), (100, 40)])
def test_double_precision_vs_oracle(gbla_lib, cuda, shape):
    m, n = shape
    rng = np.random.default_rng(7 * m + n)
    A = rng.standard_normal((6, m, n))
    r = _svd(gbla_lib, A, compute_u=True, tol=1e-14, max_sweeps=60, dt=np.float64)
    o = O.gesvj(A, compute_u=True)
    assert (r["info"] == 0).all()
    assert rel_err(r["S"][:, None, :], o["S"][:, None, :]) < 1e-13
    rec = r["U"][:, :, :n] @ (r["S"][:, :, None] * r["Vt"])
    assert rel_err(rec, A) < 1e-12


def test_double_reference_goldens(gbla_lib, cuda):
    HIGH = G["precision_high"]
    B = colmajor(G["svd_b"], 8, 3)
    r = _svd(gbla_lib, B, compute_u=True, tol=1e-15, dt=np.float64)
    assert abs(r["S"][0, 0] - G["svd_sigma1"]) < HIGH and abs(r["S"][0, 1] - G["svd_sigma2"]) < HIGH
    A = colmajor(G["svd_multi_a"], 3, 2, 3)
    r = _svd(gbla_lib, A, compute_u=True, tol=1e-15, dt=np.float64)
    vt_flat = np.concatenate([r["Vt"][i].T.ravel() for i in range(3)])
    np.testing.assert_allclose(vt_flat[:4], G["svd_multi_vt"][:4], atol=HIGH)
    u_flat = np.concatenate([r["U"][i].T.ravel() for i in range(3)])
    np.testing.assert_allclose(u_flat, G["svd_multi_u"], atol=HIGH)
