"""Golden vectors of Sim-kClist++ at k = 2 (kCDensestCmpSync.c:189-192, the
edge branch): the reference's own CDF_Main loop through the cmpsync harness
on the golden graphs, FP64 reports and rho stored bit for bit in
tests/golden/sim2.json / sim2.npz.

Runs in the build container only (it needs the reference sources).

usage: python tests/golden/make_golden_sim2.py
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(ROOT, "oracle", "_ref")
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from tests.golden.cases import CASES, make_pairs  # noqa: E402
from tests.golden.make_golden import parse_cmpsync  # noqa: E402


def main() -> None:
    O.build(ref=True)
    index, arrays = {}, {}
    T = 16
    for case in CASES:
        name = case["name"]
        pairs = make_pairs(case)
        with tempfile.NamedTemporaryFile("w", suffix=".txt", delete=False) as f:
            for s, t in pairs:
                f.write(f"{s} {t}\n")
            path = f.name
        out = subprocess.run([os.path.join(REF, "cmpsync_harness"), "4", str(T), "2", path], check=True,
                             capture_output=True, text=True).stdout
        os.unlink(path)
        infos, rho = parse_cmpsync(out)
        index[name] = {"T": T, "infos": [[i[0], i[1], i[2], i[3].hex(), i[4].hex()] for i in infos]}
        arrays[f"{name}_rho_bits"] = rho.view(np.uint64)
        print(name, infos[-1])
    np.savez_compressed(os.path.join(HERE, "sim2.npz"), **arrays)
    with open(os.path.join(HERE, "sim2.json"), "w") as f:
        json.dump(index, f, indent=1)


if __name__ == "__main__":
    main()
