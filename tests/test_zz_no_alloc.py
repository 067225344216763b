"""gbla_sdot_noalloc: the dot product for callers that cannot allocate
device memory (a control loop that must not call cudaMalloc once it runs, code
that executes while a stream is captured, a host that owns every device
allocation).  Its partial sums live in a fixed array inside the library
instead of a caller workspace.

Checked through the C ABI against the workspace entry point gbla_sdot, on two
calls in a row (the second call is shorter, so partial sums the first call
left in the shared array must not leak into it).  The file name sorts last so
that a run stopping at the first failure has run everything else already; it
also passes alone in a fresh process, where its first call is the one that
looks up the array's device address.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dot_with_workspace(lib, x, y, stream):
    import torch

    ws = torch.empty(lib.gbla_reduce_workspace_bytes(), dtype=torch.uint8, device="cuda")
    out = torch.zeros(1, dtype=torch.float32, device="cuda")
    assert lib.gbla_sdot(x.numel(), x.data_ptr(), y.data_ptr(), out.data_ptr(), ws.data_ptr(), stream) == 0
    return out.item()


def test_noalloc_dot_matches_workspace_dot_on_two_calls(gbla_lib, cuda):
    import torch

    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(2026)
    # first call: long enough to use all 1024 partial sums; second: short (4 partials)
    for length in (5_000_000, 3_333):
        x = torch.tensor(rng.standard_normal(length).astype(np.float32), device="cuda")
        y = torch.tensor(rng.standard_normal(length).astype(np.float32), device="cuda")
        out = torch.full((1,), float("nan"), dtype=torch.float32, device="cuda")
        assert gbla_lib.gbla_sdot_noalloc(length, x.data_ptr(), y.data_ptr(), out.data_ptr(), stream) == 0
        got = out.item()
        want = _dot_with_workspace(gbla_lib, x, y, stream)
        # same kernels, block count and summation order as gbla_sdot: identical bits
        assert np.float32(got).tobytes() == np.float32(want).tobytes(), (length, got, want)
        assert abs(got - want) <= 1e-6 * max(1.0, abs(want)), (length, got, want)
        exact = float(x.double().cpu().numpy() @ y.double().cpu().numpy())
        assert abs(got - exact) <= 1e-4 * np.sqrt(length), (length, got, exact)


def test_noalloc_dot_rejects_bad_arguments(gbla_lib, cuda):
    assert gbla_lib.gbla_sdot_noalloc(-1, None, None, None, None) == 1      # GBLA_INVALID_VALUE
    assert gbla_lib.gbla_sdot_noalloc(8, None, None, None, None) == 1
