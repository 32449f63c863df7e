"""Golden vectors of the k = 2 trim: the reference's NormalGraphCoreTrim run on
the golden graphs (and two extra seeded ones).

Runs in the build container only (it needs the reference sources): builds
the program with `make -C oracle ref` (sources compiled where they lie,
output in oracle/_ref/), runs `NormalGraphCoreTrim edges.txt t` per graph and
stores the statistics line of stat_trim_t_2.txt (vertices, edges, 2-cliques
left) and the trimmed edge list in tests/golden/trim2.npz / trim2.json.

usage: python tests/golden/make_golden_trim2.py
"""
from __future__ import annotations

import hashlib
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


def extra_cases():
    import kclistpp_gb300 as K

    return [("planted_k2", K.planted(4000, 6.0, 2.2, 2, 40, 90, 0.5, seed=21).pairs()),
            ("chung_lu_k2", K.chung_lu(5000, 12.0, 2.2, seed=22).pairs())]


def main() -> None:
    O.build(ref=True)
    graphs = [(c["name"], make_pairs(c)) for c in CASES] + extra_cases()
    index, arrays = {}, {}
    for name, pairs in graphs:
        d = tempfile.mkdtemp()
        path = os.path.join(d, "edges.txt")
        with open(path, "w") as f:
            for s, t in pairs:
                f.write(f"{s} {t}\n")
        subprocess.run([os.path.join(REF, "NormalGraphCoreTrim"), path, "t"], cwd=d, check=True,
                       capture_output=True, text=True)
        stat = open(os.path.join(d, "stat_trim_t_2.txt")).read().split("\n")
        nodes, edges, cliques = (int(x) for x in stat[1].split("\t")[:3])
        tr = np.loadtxt(os.path.join(d, "trimmed_t_2.txt"), dtype=np.uint32, ndmin=2).reshape(-1, 2)
        index[name] = {"sha256": hashlib.sha256(np.ascontiguousarray(pairs, dtype=np.uint32).tobytes()).hexdigest(),
                       "ntrim": nodes, "mtrim": edges, "ncktrim": cliques, "trimmed_edges": int(len(tr))}
        arrays[f"{name}_trimmed"] = tr
        print(name, index[name])
    np.savez_compressed(os.path.join(HERE, "trim2.npz"), **arrays)
    with open(os.path.join(HERE, "trim2.json"), "w") as f:
        json.dump(index, f, indent=1)


if __name__ == "__main__":
    main()
