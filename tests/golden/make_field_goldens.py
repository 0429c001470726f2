#!/usr/bin/env python3
"""Extract the reference's known-answer vectors for the field summators.

Reads the test module of the reference crate's ``src/field.rs`` (fixtures
``Setup`` :258-292 and ``SetupFourier`` :294-332, expected results of
``test_summate_fourier_2d`` :334-357, ``test_summate_2d`` :359-382 and
``test_summate_incompr_2d`` :384-430) as text and writes them, with the
line number of every literal, to ``field_rs_goldens.json`` beside this
script.  The JSON is committed; the tests never read the reference tree.

Usage:  python tests/golden/make_field_goldens.py path/to/reference
"""
from __future__ import annotations

import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))

def _literals(text: str, start: int):
    """Yield (kind, line, value) for every arr1/arr2 literal after ``start``."""
    pat = re.compile(r"\barr([12])\(&\[")
    pos = start
    while True:
        m = pat.search(text, pos)
        if not m:
            return
        depth, i = 1, m.end()
        while depth:
            c = text[i]
            depth += c == "["
            depth -= c == "]"
            i += 1
        body = text[m.end() - 1:i]
        body = re.sub(r",\s*\]", "]", body)           # trailing commas
        value = json.loads(body)
        line = text.count("\n", 0, m.start()) + 1
        yield ("arr" + m.group(1), line, value)
        pos = i


def main(ref_root: str) -> None:
    path = os.path.join(ref_root, "src", "field.rs")
    with open(path) as fh:
        text = fh.read()
    start = text.index("mod tests")
    lits = list(_literals(text, start))
    names = [
        "setup.cov_samples", "setup.z_1", "setup.z_2", "setup.pos",
        "fourier.spectrum_factor", "fourier.modes", "fourier.z_1", "fourier.z_2",
        "fourier.pos",
        "expected.summate_fourier", "expected.summate", "expected.summate_incompr",
    ]
    if len(lits) != len(names):
        raise SystemExit(f"expected {len(names)} literals, found {len(lits)}")
    out = {"source": "src/field.rs (gstools-core 1.1.0)", "arrays": {}}
    for name, (kind, line, value) in zip(names, lits):
        out["arrays"][name] = {"line": line, "kind": kind, "value": value}
    out["tolerance"] = {
        "summate": "exact (assert_eq!, src/field.rs:364)",
        "summate_fourier": "exact (assert_eq!, src/field.rs:337)",
        "summate_incompr": "assert_ulps_eq!(max_ulps = 6), approx 0.5 default "
                           "epsilon = f64::EPSILON (src/field.rs:388,428)",
    }
    dst = os.path.join(HERE, "field_rs_goldens.json")
    lines = ["{", f' "source": {json.dumps(out["source"])},', ' "arrays": {']
    items = list(out["arrays"].items())
    for i, (k, v) in enumerate(items):
        sep = "," if i < len(items) - 1 else ""
        lines.append(f"  {json.dumps(k)}: {json.dumps(v)}{sep}")
    lines += [" },", f' "tolerance": {json.dumps(out["tolerance"])}', "}"]
    with open(dst, "w") as fh:
        fh.write("\n".join(lines) + "\n")
    print("wrote", dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_field_goldens.py path/to/reference  (the GSTools-Core source tree)")
    main(sys.argv[1])
