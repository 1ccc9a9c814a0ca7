"""Regenerates tests/golden/reference_goldens.json from the numrs2 source tree.

Run with the path of a numrs2 0.4.1 source tree:

    python tests/golden/make_golden.py REF

It copies, verbatim, the reference's own test data for this path:
  * the NumPy-generated goldens read by tests/test_array_operations_reference.rs
    (tests/py/array_operations_reference_data.json): sum/mean/min/max/var/std
    overall/axis0/axis1, exp_*, add/subtract/multiply/divide and scalar_* ops;
  * the pinned bit patterns of tests/test_reduction_determinism.rs:126-197
    (x_i = 0.5*i - 12345, N = 50,000), extracted from the Rust source text.
The fixture is committed; tests never read the reference tree at run time.
"""
from __future__ import annotations

import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref: str) -> None:
    data = json.load(open(os.path.join(ref, "tests/py/array_operations_reference_data.json")))
    stats = {k: v for k, v in data["statistical_operations"].items()
             if v["operation"] in ("sum", "mean", "min", "max", "var", "std")}
    maths = {k: v for k, v in data["mathematical_functions"].items() if v["operation"] == "exp"}
    arith = dict(data["arithmetic_operations"])

    src = open(os.path.join(ref, "tests/test_reduction_determinism.rs")).read()
    n = int(re.search(r"const N: usize = ([\d_]+);", src).group(1).replace("_", ""))
    kats = {}
    for fn, name in (("sum_f64_is_deterministic", "sum_f64"), ("mean_f64_is_deterministic", "mean_f64"),
                     ("var_f64_ddof0_is_deterministic", "var_f64_ddof0"),
                     ("std_f64_ddof0_is_deterministic", "std_f64_ddof0"),
                     ("sum_f32_is_deterministic", "sum_f32")):
        body = src[src.index(fn):]
        m = re.search(r"got\.to_bits\(\),\s*(\d+)u(64|32)", body)
        kats[name] = {"bits": int(m.group(1)), "width": int(m.group(2))}
    out = {
        "source": "numrs2 0.4.1 tests/py/array_operations_reference_data.json and "
                  "tests/test_reduction_determinism.rs",
        "determinism": {"n": n, "x": "0.5*i - 12345", "pins": kats},
        "statistical_operations": stats,
        "mathematical_functions": maths,
        "arithmetic_operations": arith,
    }
    with open(os.path.join(HERE, "reference_goldens.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <numrs2 source tree>")
    main(sys.argv[1])
