"""The C ABI without a GPU: the library builds and loads, exports exactly
what include/gbla.h declares, and rejects invalid arguments before touching
the device (no compute call runs here)."""
import ctypes as C
import subprocess

import pytest

from gputils_gb300 import _lib


def test_header_parses_and_every_symbol_is_exported(gbla_lib):
    decls = _lib.parse_header()
    assert len(decls) >= 30
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True, check=True)
    exported = {line.split()[-1] for line in out.stdout.splitlines() if " T " in line}
    missing = [name for name in decls if name not in exported]
    assert not missing, f"declared in gbla.h but not exported: {missing}"
    extra = sorted(s for s in exported if s.startswith("gbla_") and s not in decls)
    assert not extra, f"exported but not declared in gbla.h: {extra}"


def test_status_strings(gbla_lib):
    assert gbla_lib.gbla_status_string(0) == b"GBLA_SUCCESS"
    assert gbla_lib.gbla_status_string(1) == b"GBLA_INVALID_VALUE"
    assert gbla_lib.gbla_status_string(99) == b"GBLA_UNKNOWN_STATUS"
    assert gbla_lib.gbla_version() >= 100


INVALID = 1


def test_invalid_arguments_are_rejected_host_side(gbla_lib):
    L = gbla_lib
    fake = C.c_void_p(0x1000)  # never dereferenced: validation fails first
    assert L.gbla_spotrf_batched(-1, fake, 1, None, 1, None) == INVALID
    assert L.gbla_spotrf_batched(4, None, 16, None, 1, None) == INVALID
    assert L.gbla_spotrf_batched(4, fake, 15, None, 1, None) == INVALID      # stride < n*n
    assert L.gbla_spotrs_batched(4, 1, fake, 16, None, 4, 1, None) == INVALID
    assert L.gbla_sposv_batched(4, 1, fake, 16, fake, 4, None, -1, 1, None) == INVALID
    assert L.gbla_sgemm_batched(-1, 1, 1, 1.0, fake, 1, fake, 1, 0.0, fake, 1, 1, 0, None) == INVALID
    assert L.gbla_sgemm_batched(2, 2, 2, 1.0, fake, 3, fake, 4, 0.0, fake, 4, 1, 0, None) == INVALID
    # C overlapping A is rejected (the reference's Nullspace::project aliasing is handled by the header)
    assert L.gbla_sgemm_batched(2, 2, 2, 1.0, fake, 4, fake, 4, 0.0, fake, 4, 1, 0, None) == INVALID
    assert L.gbla_sgemm_batched(2, 2, 2, 1.0, C.c_void_p(0x1000), 4, C.c_void_p(0x2000), 4, 0.0,
                                C.c_void_p(0x3000), 4, 1, 7, None) == INVALID  # unknown mode
    assert L.gbla_stranspose_batched(3, 2, fake, 5, fake, 6, 1, None) == INVALID
    assert L.gbla_scopy_rows(3, 2, 2, 2, fake, fake, None) == INVALID        # rows out of range
    assert L.gbla_saxpy(-1, 1.0, fake, fake, None) == INVALID
    assert L.gbla_sdot(4, fake, None, fake, fake, None) == INVALID
    # two-kernel least squares: workspace size, m < n, and a workspace that is too small
    ws = L.gbla_sgels_batched_workspace_bytes(128, 32, 8192)
    assert ws >= 4 * (8192 * 128 * 32 + 8192 * 32)
    assert L.gbla_sgels_batched_workspace_bytes(-1, 32, 8) == 0
    assert L.gbla_sgels_batched_ws(4, 5, 1, fake, 20, fake, 4, None, 1, fake, 1 << 20, 1, None) == INVALID
    assert L.gbla_sgels_batched_ws(8, 4, 1, fake, 32, fake, 8, None, 1, fake, 64, 2, None) == 4
    assert L.gbla_sgels_batched_ws(8, 4, 1, fake, 32, fake, 8, None, 1, None, 1 << 20, 2, None) == 4
    assert L.gbla_sgels_batched_ws(130, 4, 1, fake, 520, fake, 130, None, 1, fake, 1 << 20, 2, None) == 2
    # host-buffer pipeline calls: no pipeline, bad stream counts
    assert L.gbla_pipeline_create(0, C.byref(C.c_void_p())) == INVALID
    assert L.gbla_pipeline_create(3, None) == INVALID
    assert L.gbla_sgemm_batched_host(None, 4, 4, 4, 1.0, fake, 16, fake, 16, 0.0, fake, 16, 1, 0, 0, None) == INVALID
    assert L.gbla_sgels_batched_host(None, 8, 4, 1, fake, 32, None, fake, 8, fake, None, 1, 1, 0, None) == INVALID
    assert L.gbla_pipeline_destroy(None) == 0


def test_empty_problems_are_noops(gbla_lib):
    L = gbla_lib
    assert L.gbla_spotrf_batched(0, None, 0, None, 5, None) == 0
    assert L.gbla_spotrf_batched(4, None, 16, None, 0, None) == 0
    assert L.gbla_sgemm_batched(0, 3, 3, 1.0, None, 0, None, 0, 0.0, None, 0, 3, 0, None) == 0
    assert L.gbla_saxpy(0, 1.0, None, None, None) == 0
    assert L.gbla_stranspose_batched(0, 5, None, 0, None, 0, 3, None) == 0
    assert L.gbla_sgels_batched_ws(8, 4, 1, None, 32, None, 8, None, 1, None, 0, 0, None) == 0


@pytest.mark.parametrize("name", ["gbla_spotrf_batched", "gbla_sgemm_batched", "gbla_sdot"])
def test_argtypes_come_from_header(gbla_lib, name):
    f = getattr(gbla_lib, name)
    assert f.restype is C.c_int and len(f.argtypes) >= 5


def test_large_cholesky_entry_points_validate_host_side(gbla_lib):
    """gbla_spotrf_large / gbla_spotrs_large reject bad sizes, strides and
    workspaces before touching the device; empty problems are no-ops."""
    L = gbla_lib
    fake = C.c_void_p(0x1000)
    assert L.gbla_spotrf_large(-1, fake, 1, None, None, 0, None) == INVALID
    assert L.gbla_spotrf_large(300, fake, 299, None, None, 0, None) == INVALID     # lda < n
    assert L.gbla_spotrf_large(300, None, 300, None, None, 0, None) == INVALID     # no matrix
    assert L.gbla_spotrf_large(300, fake, 300, None, fake, 1024, None) == 4        # workspace too small
    assert L.gbla_spotrf_large(300, fake, 300, None, None, 1 << 30, None) == 4     # no workspace
    assert L.gbla_spotrf_large(0, None, 1, None, None, 0, None) == 0
    assert L.gbla_spotrf_large_workspace_bytes(128) == 0
    assert L.gbla_spotrf_large_workspace_bytes(129) >= 2 * 2 * 129 * 768 * 2       # two sets of two operands
    assert L.gbla_spotrs_large(-1, 1, fake, 1, fake, 1, None) == INVALID
    assert L.gbla_spotrs_large(300, 1, fake, 299, fake, 300, None) == INVALID       # lda < n
    assert L.gbla_spotrs_large(300, 1, fake, 300, fake, 299, None) == INVALID       # ldb < n
    assert L.gbla_spotrs_large(300, 1, None, 300, fake, 300, None) == INVALID
    assert L.gbla_spotrs_large(0, 3, None, 1, None, 1, None) == 0
    assert L.gbla_spotrs_large(300, 0, None, 300, None, 300, None) == 0
