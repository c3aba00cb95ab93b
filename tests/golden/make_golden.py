"""Regenerate tests/golden/reference_kats.json from CppIrlba's own unit tests.

Reads the reference test sources (as text; nothing is compiled or run) and
extracts the known-answer tests of the hot path:
  * the hard-coded 5x4 orthonormal basis and 5-vector of the Gram-Schmidt test
    (tests/src/lanczos.cpp:13-27);
  * the expectations of requested_greater_than_or_equal_to_half_smaller and
    choose_requested_plus_extra_work_or_smaller (tests/src/compute.cpp:33-50);
  * the grid of update_k arguments (tests/src/compute.cpp:52-76), with the
    expected values from the test's own restatement of R irlba's convtests()
    logic (compute.cpp:53-64), transcribed below.
Usage: python tests/golden/make_golden.py [/path/to/CppIrlba]
"""
import json
import os
import re
import sys

ROOT = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_kats.json")


def numbers(text):
    return [float(x) for x in re.findall(r"-?\d+\.\d+(?:[eE][-+]?\d+)?", text)]


def main():
    lz = open(os.path.join(ROOT, "tests/src/lanczos.cpp")).read()
    m_block = lz[lz.index("m <<"):lz.index(";", lz.index("m <<"))]
    v_block = lz[lz.index("v <<"):lz.index(";", lz.index("v <<"))]
    m_vals = numbers(m_block)
    v_vals = numbers(v_block)
    assert len(m_vals) == 20 and len(v_vals) == 5

    cp = open(os.path.join(ROOT, "tests/src/compute.cpp")).read()
    half = [(int(a), int(b), kind == "TRUE") for kind, a, b in
            re.findall(r"EXPECT_(TRUE|FALSE)\(irlba::requested_greater_than_or_equal_to_half_smaller\((\d+), (\d+)\)\)", cp)]
    choose = [(int(a), int(b), int(c), int(d)) for a, b, c, d in
              re.findall(r"EXPECT_EQ\(irlba::choose_requested_plus_extra_work_or_smaller\((\d+), (\d+), (\d+)\), (\d+)\)", cp)]
    grid_txt = re.search(r"std::vector<int> values\{([^}]*)\}", cp).group(1)
    grid = [int(x) for x in grid_txt.split(",")]

    def ref_update_k(k, requested, n_converged, work):  # compute.cpp:53-64
        if k < requested + n_converged:
            k = requested + n_converged
        if k > work - 3:
            k = work - 3
        if k < 1:
            k = 1
        return k

    upd = [(k, r, c, w, ref_update_k(k, r, c, w)) for k in grid for r in grid for c in grid for w in grid]
    out = {
        "source": "CppIrlba tests/src/lanczos.cpp:13-27, tests/src/compute.cpp:33-76",
        "cgs_basis_rowmajor_5x4": m_vals,
        "cgs_vector": v_vals,
        "requested_ge_half_smaller": half,
        "choose_requested_plus_extra_work_or_smaller": choose,
        "update_k": upd,
    }
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", OUT, len(half), len(choose), len(upd))


if __name__ == "__main__":
    main()
