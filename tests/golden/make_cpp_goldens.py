"""Writes tests/cpp/goldens.h from reference_goldens.json, so the C++ port of
the reference's tests uses exactly the values read from test/testTensor.cu.
Run: python tests/golden/make_cpp_goldens.py"""
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    d = json.load(open(os.path.join(HERE, "reference_goldens.json")))
    lines = ["// Generated by tests/golden/make_cpp_goldens.py from reference_goldens.json;",
             "// every value is cited there (test/testTensor.cu line ranges).",
             "#pragma once", "#include <vector>", "namespace golden {"]
    for name in sorted(d["values"]):
        v = d["values"][name]
        cite = d["cite"][name]
        if isinstance(v, list):
            body = ", ".join(repr(float(x)) for x in v)
            lines.append(f"static const std::vector<double> {name} = {{{body}}};  // {cite}")
        else:
            lines.append(f"static const double {name} = {float(v)!r};  // {cite}")
    lines.append("}  // namespace golden")
    with open(os.path.join(os.path.dirname(HERE), "cpp", "goldens.h"), "w") as f:
        f.write("\n".join(lines) + "\n")


if __name__ == "__main__":
    main()
