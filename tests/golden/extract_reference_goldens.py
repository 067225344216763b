"""Regenerates ``reference_goldens.json`` and ``b_d.bt`` from the reference.

Run in a checkout that has the reference mounted (it is not needed at test
time):  ``python tests/golden/extract_reference_goldens.py /root/reference``

Every golden value below is read from the reference's own test file
(test/testTensor.cu) at the cited line range; nothing is typed in by hand.
``b_d.bt`` is written by the reference's own Python API
(python/gputils_api/gputils_api.py:25-51) with the array its unit test uses
(python/test/test.py:9-13), which its C++ test reads back
(test/testTensor.cu:193-202).
"""
from __future__ import annotations

import json
import os
import re
import sys

import numpy as np

NUM = re.compile(r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?")

# name -> (first line, last line, what) ; lines are 1-based, inclusive.
BRACED = {
    "tensor_234A": (21, 21, "TENSOR_DATA_234A"),
    "tensor_234B": (22, 22, "TENSOR_DATA_234B"),
    "tensor_234APB": (23, 23, "TENSOR_DATA_234APB"),
    "tensor_234AMB": (24, 24, "TENSOR_DATA_234AMB"),
    "addAB_a": (830, 834, "tensorAddAB aData (2x3x3)"),
    "addAB_b": (835, 839, "tensorAddAB bData (3x2x3)"),
    "addAB_expected": (844, 844, "tensorAddAB expected C (2x2x3)"),
    "getRows_a": (901, 908, "tensorGetRows aData (3x3x2)"),
    "getRows_expected0": (911, 911, "getRows(1,1,0)"),
    "getRows_expected1": (917, 917, "getRows(1,2,1)"),
    "transpose_a": (935, 935, "tensorTranspose aData (3x2x2)"),
    "transpose_expected": (941, 941, "tensorTranspose expected (2x3x2)"),
    "ls1_a": (1015, 1022, "tensorLeastSquares1 aData (2x2x3)"),
    "ls1_b": (1023, 1023, "tensorLeastSquares1 bData (2x1x3)"),
    "svd_b": (1062, 1066, "singularValuesComputation bData (8x3)"),
    "svd_multi_a": (1129, 1129, "singularValuesMultipleMatrices aData (3x2x3)"),
    "svd_multi_vt": (1137, 1141, "expected_v (Vt, only first 4 checked)"),
    "svd_multi_s": (1146, 1146, "expected_s"),
    "svd_multi_u": (1151, 1161, "expected_u (3x3x3)"),
    "rank_a": (1181, 1185, "singularValuesRankMultipleMatrices aData (4x3x3)"),
    "chol_a": (1221, 1225, "choleskyFactorisation aData (3x3)"),
    "chol_b": (1257, 1257, "choleskyFactorisationSolution bData"),
    "chol_x": (1262, 1262, "choleskyFactorisationSolution expected x"),
    "chol_low_rowmajor": (1377, 1381, "choleskyBatchSolve lowData (row-major L)"),
    "qr_ls_a_rowmajor": (1502, 1507, "qrLeastSquares vecA (4x3 row-major)"),
    "qr_ls_b": (1508, 1513, "qrLeastSquares vecB"),
    "ns_a": (1558, 1564, "computeNullspaceTensor aData (3x4x5)"),
    "ns_trivial_rowmajor": (1601, 1608, "computeNullspaceTrivial data (3x3x2 row-major)"),
    "ns_project_a_rowmajor": (1630, 1634, "projectOnNullspaceTensor mat (3x7 row-major)"),
    "ns_project_x": (1641, 1641, "projectOnNullspaceTensor vec"),
    "ns_project_other": (1652, 1652, "projectOnNullspaceTensor h_other"),
}

# scalar constants: name -> (line, index of the numeric literal on that line)
SCALARS = {
    "dotF": (496, 0),
    "normF": (517, 0),
    "sumAbs": (534, 0),
    "maxAbs": (551, 0),
    "minAbs": (568, 0),
    "svd_sigma1": (1074, 0),
    "svd_sigma2": (1075, 0),
    "rank0": (1191, 0),
    "rank1": (1192, 0),
    "rank2": (1193, 0),
    "chol_L00": (1229, 0),
    "chol_L21": (1230, 0),
    "chol_L22": (1231, 0),
    "qr_ls_residual": (1529, 0),
    "givens_a00": (1726, 0),
    "givens_a03": (1727, 0),
    "givens_a13": (1728, 0),
    "precision_low": (5, 0),
    "precision_high": (6, 0),
}


def _braced_numbers(text: str):
    lo, hi = text.index("{"), text.rindex("}")
    return [float(x) for x in NUM.findall(text[lo + 1:hi])]


def main(ref_root: str) -> None:
    here = os.path.dirname(os.path.abspath(__file__))
    src = os.path.join(ref_root, "test", "testTensor.cu")
    lines = open(src).read().split("\n")
    out = {"source": "test/testTensor.cu", "values": {}, "cite": {}}
    for name, (a, b, what) in BRACED.items():
        text = "\n".join(lines[a - 1:b])
        out["values"][name] = _braced_numbers(text)
        out["cite"][name] = f"test/testTensor.cu:{a}-{b} ({what})"
    for name, (ln, idx) in SCALARS.items():
        text = lines[ln - 1]
        # drop identifiers containing digits (e.g. "PRECISION_LOW 1e-4" keeps 1e-4)
        nums = NUM.findall(re.sub(r"[A-Za-z_]\w*\d\w*", " ", text.split("//")[0]))
        out["values"][name] = float(nums[idx])
        out["cite"][name] = f"test/testTensor.cu:{ln}"
    with open(os.path.join(here, "reference_goldens.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)

    sys.path.insert(0, os.path.join(ref_root, "python"))
    import gputils_api.gputils_api as gapi  # the reference's own writer

    b = np.array([[[1, 2], [3, 4], [5, 6]], [[7, 8], [9, 10], [11, 12]], [[13, 14], [15, 16], [17, 18]]],
                 dtype=np.dtype("d"))  # python/test/test.py:9-13
    gapi.write_array_to_gputils_binary_file(b, os.path.join(here, "b_d.bt"))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
