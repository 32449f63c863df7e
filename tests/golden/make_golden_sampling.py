"""Golden vectors of Seq-Sampling++ (kCDensestSamplingKclistpp.c), from the
reference program's own functions run through oracle/ref_harness/
sampling_harness.c on the golden graphs:

* the clique count (KCLIST_CliqueEnum COUNT) and every clique the SAMPLING
  task stores at p = 1 (stored as a count and a SHA-256 of the sorted rows);
* for a sample drawn by the oracle's counter-based rule (the library's), the
  order in which one InMemoryFrankWolfe call visits it after srand(seed) and
  the loads it leaves, ExtractDensest(T = 1) on those loads (FP64 by bit
  pattern), and Solve's printed report line for the same pass.

The oracle's restatement is checked against all of it here, before anything
is written, and again by tests/test_oracle_golden.py from the stored files.

Runs in the build container only (it needs the reference sources).

usage: python tests/golden/make_golden_sampling.py
"""
from __future__ import annotations

import hashlib
import json
import os
import re
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

KS = {"config1_chung_lu_1e4": [3, 4], "cl_2000": [3, 4, 5], "er_1500": [3, 4], "rmat12": [3],
      "planted_3000": [3, 4, 5], "kat_complete10": [3, 4], "kat_disjoint_cliques": [3, 4],
      "kat_clique_tree": [3, 4], "kat_star": [3], "kat_triangle_k4": [3, 4]}
TARGET = 600          # cliques the oracle's sample aims at
SAMPLE_SEED = 20201   # seed of the counter-based sample
RAND_SEED = 12345     # srand() seed of the reference's shuffle
WAVES = 4

LINE = re.compile(r"Approximate densest subgraph: (\d+) nodes, (\d+) edges, edge density = (\S+), "
                  r"k-clique density = (\S+), upper bound = (\S+)\. ")


def rows_digest(rows: np.ndarray) -> str:
    """SHA-256 of the rows sorted by (largest member, next largest, ...)."""
    r = np.ascontiguousarray(rows, dtype=np.uint32)
    if len(r):
        r = r[np.lexsort(r.T)]
    return hashlib.sha256(r.tobytes()).hexdigest()


def parse(out: str, k: int) -> dict:
    res = {"rows": []}
    for line in out.splitlines():
        w = line.split()
        if not w:
            continue
        if w[0] == "graph":
            res["graph"] = [int(x) for x in w[1:4]]
        elif w[0] == "count":
            res["count"] = int(w[1])
        elif w[0] == "all":
            res["all"] = int(w[1])
        elif w[0] == "row":
            res["rows"].append([int(x) for x in w[1:]])
        elif w[0] == "order":
            res["order"] = np.array([int(x) for x in w[1:]], dtype=np.uint32)
        elif w[0] == "rho":
            res["rho"] = np.array([int(x) for x in w[1:]], dtype=np.uint32)
        elif w[0] == "info":
            res["info"] = [int(w[1]), int(w[2]), float.fromhex(w[3]), float.fromhex(w[4])]
        else:
            m = LINE.match(line)
            if m:
                res["line"] = [int(m.group(1)), int(m.group(2)), m.group(3), m.group(4), m.group(5)]
    res["rows"] = np.array(res["rows"], dtype=np.uint32).reshape(-1, k)
    return res


def fmt(x: float) -> str:
    return "%f" % x


def check_line(rep: dict, line: list) -> None:
    """The oracle's report against Solve's printed line (%f; NaN by kind)."""
    assert rep["sub_n"] == line[0] and rep["sub_e"] == line[1], (rep, line)
    for val, txt in zip((rep["edge_density"], rep["clique_density"], rep["upper_bound"]), line[2:]):
        if "nan" in txt:
            assert np.isnan(val), (val, txt)
        else:
            assert fmt(val) == txt, (fmt(val), txt)


def main() -> None:
    O.build(ref=True)
    index, arrays = {}, {}
    for case in CASES:
        name = case["name"]
        pairs = make_pairs(case)
        g = O.Graph(pairs)
        with tempfile.NamedTemporaryFile("w", suffix=".txt", delete=False) as f:
            for s, t in pairs:
                f.write(f"{s} {t}\n")
            path = f.name
        for k in KS[name]:
            total = g.count_cliques(k)[0]
            all_, prob, thr = O.sampling_threshold(TARGET, total)
            rows, wave = g.sampling_collect(k, SAMPLE_SEED, thr, all_, WAVES)
            with tempfile.NamedTemporaryFile("w", suffix=".smp", delete=False) as f:
                f.write(f"{len(rows)} {prob!r}\n")
                for r in rows:
                    f.write(" ".join(str(int(x)) for x in r) + "\n")
                spath = f.name
            out = subprocess.run([os.path.join(REF, "sampling_harness"), str(k), path, spath, str(RAND_SEED)],
                                 check=True, capture_output=True, text=True).stdout
            os.unlink(spath)
            ref = parse(out, k)
            # The oracle against the reference, before anything is stored.
            assert ref["graph"] == [g.n, g.m, g.core], (name, ref["graph"])
            assert ref["count"] == total and ref["all"] == total, (name, k)
            assert np.all(np.diff(ref["rows"].astype(np.int64), axis=1) > 0) if total else True
            full, _ = g.sampling_collect(k, SAMPLE_SEED, 0, True, WAVES)
            assert rows_digest(full) == rows_digest(ref["rows"]), (name, k, "clique lists differ")
            assert sorted(ref["order"].tolist()) == list(range(len(rows))), (name, k)
            rho = O.sampling_pass_order(k, rows, ref["order"], np.zeros(g.n, np.uint32))
            assert np.array_equal(rho, ref["rho"]), (name, k, "loads differ")
            info, _ = O.sampling_extract(g.n, k, rows, ref["rho"], 1)
            got = [info.n, info.m, info.density, info.ub]
            assert got[:2] == ref["info"][:2] and all(
                np.float64(a).tobytes() == np.float64(b).tobytes() for a, b in zip(got[2:], ref["info"][2:])), (
                name, k, got, ref["info"])
            check_line(O.sampling_report(g, k, rows, ref["rho"], 1, prob), ref["line"])
            key = f"{name}_k{k}"
            index[key] = {"case": name, "k": k, "target": TARGET, "sample_seed": SAMPLE_SEED,
                          "rand_seed": RAND_SEED, "waves": WAVES, "total": total, "prob": prob.hex(),
                          "sampled": int(len(rows)), "all_digest": rows_digest(ref["rows"]),
                          "info": [ref["info"][0], ref["info"][1], ref["info"][2].hex(), ref["info"][3].hex()],
                          "line": ref["line"]}
            arrays[f"{key}_order"] = ref["order"]
            arrays[f"{key}_rho"] = ref["rho"]
            print(key, total, len(rows), ref["info"][:2], ref["line"])
        os.unlink(path)
    np.savez_compressed(os.path.join(HERE, "sampling.npz"), **arrays)
    with open(os.path.join(HERE, "sampling.json"), "w") as f:
        json.dump(index, f, indent=1)


if __name__ == "__main__":
    main()
