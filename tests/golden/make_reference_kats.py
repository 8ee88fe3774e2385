"""Extract the reference test suite's known-answer values into reference_kats.json.

Reads the reference's gtest sources AS TEXT (nothing of the reference is built
or run) and records the numbers its hot-path tests assert:

* direction matrix for phase centre / direction of the MWA test MS
    (src/icrar/leap-accelerate/tests/model/MetaDataTests.cc:146-165 and
     src/icrar/leap-accelerate/tests/algorithm/PhaseRotateTests.cc:196-212)
* channel-0 wavelength, dlm_ra/dlm_dec constants (PhaseRotateTests.cc:202-207,
  MetaDataTests.cc:186)
* pseudoinverse known answers (src/icrar/leap-accelerate/tests/math/MatrixTests.cc:154-250)
* the calibration directions of the end-to-end multi-direction run
    (src/icrar/leap-accelerate-cli/tests/E2EPerformanceTests.cc:65-76) and of the
    phase-rotate test (PhaseRotateTests.cc:97-103), as (ra, dec) in radians

Usage:  python tests/golden/make_reference_kats.py <reference_root>
"""
from __future__ import annotations

import json
import os
import re
import sys

NUM = r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?"


def _lines(path, a, b):
    with open(path) as f:
        return "".join(f.readlines()[a - 1:b])


def _nums(text):
    return [float(x) for x in re.findall(NUM, text)]


def _matrix_after(text, name, rows, cols):
    """Numbers of an Eigen comma-initialiser `name << ...;`."""
    m = re.search(re.escape(name) + r"\s*<<(.*?);", text, re.S)
    vals = _nums(m.group(1))
    assert len(vals) == rows * cols, (name, vals)
    return [vals[r * cols:(r + 1) * cols] for r in range(rows)]


def main(root):
    t = os.path.join(root, "src", "icrar", "leap-accelerate", "tests")
    md = os.path.join(t, "model", "MetaDataTests.cc")
    pr = os.path.join(t, "algorithm", "PhaseRotateTests.cc")
    mx = os.path.join(t, "math", "MatrixTests.cc")

    dd_txt = _lines(md, 146, 166)
    direction = _nums(re.search(r"SphericalDirection\(([^)]*)\)", dd_txt).group(1))
    dd_vals = [float(v) for v in re.findall(r"EXPECT_DOUBLE_EQ\((" + NUM + r"),\s*meta\.GetDD\(\)\((\d),(\d)\)\)", dd_txt)
               for v in [v[0]]]
    idx = re.findall(r"meta\.GetDD\(\)\((\d),(\d)\)", dd_txt)
    dd = [[0.0] * 3 for _ in range(3)]
    for v, (i, j) in zip(dd_vals, idx):
        dd[int(i)][int(j)] = v

    c_txt = _lines(pr, 196, 212)
    consts = {}
    for key in ("nbaselines", "channels", "num_pols", "stations", "rows", "freq_start_hz", "freq_inc_hz",
                "phase_centre_ra_rad", "phase_centre_dec_rad", "dlm_ra", "dlm_dec"):
        consts[key] = float(re.search(r"expectedConstants\." + key + r"\s*=\s*(" + NUM + ")", c_txt).group(1))
    dd2 = _matrix_after(c_txt, "expectedDD", 3, 3)
    lam = float(re.search(r"EXPECT_DOUBLE_EQ\((" + NUM + r"),\s*meta\.GetConstants\(\)\.GetChannelWavelength\(0\)\)",
                          _lines(md, 181, 187)).group(1))

    m_txt = _lines(mx, 154, 250)
    blocks = re.split(r"void\s+Test", m_txt)
    pinv = []
    for blk in blocks:
        name = blk.split("(")[0].strip()
        if not name.startswith(("PseudoInverse", "SVDPseudoInverse")):
            continue
        dims = re.search(r"m1\s*=\s*Eigen::MatrixXd\((\d+),\s*(\d+)\)", blk)
        r, c = int(dims.group(1)), int(dims.group(2))
        a = _matrix_after(blk, "m1", r, c)
        e = _matrix_after(blk, "expected_m1d", c, r)
        pinv.append({"name": name, "A": a, "expected": e})

    e2e = os.path.join(root, "src", "icrar", "leap-accelerate-cli", "tests", "E2EPerformanceTests.cc")
    e2e_dirs = [_nums(x) for x in re.findall(r"MVDirection\(([^)]*)\)", _lines(e2e, 65, 76))]
    assert len(e2e_dirs) == 9 and all(len(d) == 2 for d in e2e_dirs), e2e_dirs
    pr_dirs = [_nums(x) for x in re.findall(r"\{\s*(" + NUM + r"\s*,\s*" + NUM + r")\s*\}", _lines(pr, 97, 103))]
    assert len(pr_dirs) == 4, pr_dirs

    out = {
        "source": "reference gtest sources (values asserted by the hot-path tests)",
        "dd": {"phase_centre": [consts["phase_centre_ra_rad"], consts["phase_centre_dec_rad"]],
               "direction": direction, "expected": dd, "expected_phase_rotate_test": dd2},
        "constants": consts,
        "wavelength0": lam,
        "pinv_tolerance": 1e-4,
        "pinv": pinv,
        "phase_matrix_empty_input_throws": {"refAnt": 0},
        "e2e_directions": {"source": "E2EPerformanceTests.cc:65-76 (MultiDirectionTest: Slice(0,1,1), refAnt 0)",
                           "radec": e2e_dirs},
        "phase_rotate_directions": {"source": "PhaseRotateTests.cc:97-103", "radec": pr_dirs},
    }
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "reference_kats.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out)[:400])


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_reference_kats.py <reference_root>")
    main(sys.argv[1])
