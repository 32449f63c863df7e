"""Golden vectors of the headline workload's trim: the reference's own
kClistCoreTrim run on the benchmark graph (RMAT scale 20, (0.57, 0.19, 0.19,
0.05), edge factor 16, seed 1, symmetrised and deduplicated).

Runs in the build container only (it needs the reference sources): compiles
the reference with `oracle.build(ref=True)` (sources compiled where they lie,
outputs in oracle/_ref/), writes the graph as an edge list, runs
`kClistCoreTrim k edges ckdeg ckcore ckdens r20` for each k and stores, in
tests/golden/rmat20_trim.json:

  * the graph's size and a SHA-256 of its canonical pairs (u32 little endian);
  * the reference's statistics: n2, e2 (survivors of the (k-1)-core), the
    k-clique count, the k-clique core number, ckrho / rho / size as printed
    in the ckdens file, ntrim, mtrim and ncktrim of the trimmed graph;
  * SHA-256 digests of the ckdeg and ckcore files and of the trimmed edge
    list (the files are 5-12 MB, too large to commit);
  * the kept vertices (original ids) in the order of the reference's new
    labels, which with the input order defines the trimmed edge list exactly:
    the input edges with both ends kept, each written with its end of larger
    new label first (relabelnodes, kClistCoreTrim.c:274-294).

    python tests/golden/make_golden_rmat20.py [--k 4 5] [--reuse DIR]

--reuse DIR takes the reference's output files from DIR where they already
exist (a previous run of this script), instead of running it again.  One k = 4
run of the reference takes about seven minutes on one core.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")
OUT = os.path.join(HERE, "rmat20_trim.json")


def sha(path: str) -> str:
    h = hashlib.sha256()
    with open(path, "rb") as f:
        for chunk in iter(lambda: f.read(1 << 20), b""):
            h.update(chunk)
    return h.hexdigest()


def write_edges(pairs: np.ndarray, path: str) -> None:
    with open(path, "w") as f:
        for i in range(0, len(pairs), 1 << 20):
            blk = pairs[i:i + (1 << 20)]
            f.write("".join(f"{u} {v}\n" for u, v in blk.tolist()))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--k", type=int, nargs="+", default=[4])
    ap.add_argument("--reuse", default=None)
    a = ap.parse_args()
    O.build(ref=True)
    pairs = O.rmat(20, 16, 0.57, 0.19, 0.19, seed=1)
    d = a.reuse or os.path.join("/tmp", "kclpp_rmat20_golden")
    os.makedirs(d, exist_ok=True)
    edges = os.path.join(d, "rmat20.txt")
    if not os.path.exists(edges):
        write_edges(pairs, edges)
    out = json.load(open(OUT)) if os.path.exists(OUT) else {}
    out["graph"] = {"generator": "rmat scale 20, edge factor 16, (0.57, 0.19, 0.19), seed 1",
                    "n": int(pairs.max()) + 1, "e": int(len(pairs)),
                    "sha256": hashlib.sha256(np.ascontiguousarray(pairs, dtype="<u4").tobytes()).hexdigest()}
    for k in a.k:
        names = [f"ckdeg{k}.txt", f"ckcore{k}.txt", f"ckdens{k}.txt"]
        trimmed = os.path.join(d, f"trimmed_r20_{k}.txt")
        stat = os.path.join(d, f"stat_trim_r20_{k}.txt")
        log = os.path.join(d, f"trim{k}.out")
        secs = None
        if not all(os.path.exists(os.path.join(d, x)) for x in names + [os.path.basename(trimmed)]):
            t0 = time.time()
            with open(log, "w") as f:
                subprocess.run([os.path.join(REF, "kClistCoreTrim"), str(k), edges] + names + ["r20"], cwd=d,
                               stdout=f, stderr=subprocess.STDOUT, check=True)
            secs = time.time() - t0
        text = open(log).read()
        phases = []
        for ln in text.splitlines():
            if "Time = " in ln:
                h, rest = ln.split("Time = ")[1].split("h")
                m, sec = rest.split("m")
                phases.append(int(h) * 3600 + int(m) * 60 + int(sec.rstrip("s")))
        total = int(text.split(f"Number of {k}-cliques: ")[1].split()[0])
        ckcore = int(text.split(f"{k}-clique core number of the graph = ")[1].split()[0])
        n2 = int(text.split(f"Number of nodes (with core value > {k - 2}): ")[1].split()[0])
        e2 = int(text.split(f"Number of edges (between nodes with core value > {k - 2}): ")[1].split()[0])
        ckd = open(os.path.join(d, f"ckdens{k}.txt")).read().split()
        st = open(stat).read().splitlines()[1].split("\t")
        deg = np.loadtxt(os.path.join(d, f"ckdeg{k}.txt"), dtype=np.uint64).reshape(-1, 2)
        tr = np.loadtxt(trimmed, dtype=np.uint32).reshape(-1, 2)
        kept = set(np.unique(tr).tolist())
        kept_order = [int(v) for v in deg[:, 0].tolist() if v in kept]
        # The trimmed file is the input edges with both ends kept, larger new label first.
        label = {v: i for i, v in enumerate(kept_order)}
        keep = np.zeros(int(pairs.max()) + 1, dtype=bool)
        keep[np.array(kept_order, dtype=np.int64)] = True
        sel = pairs[keep[pairs[:, 0]] & keep[pairs[:, 1]]]
        lab = np.full(int(pairs.max()) + 1, -1, dtype=np.int64)
        lab[np.array(kept_order, dtype=np.int64)] = np.arange(len(kept_order))
        swap = lab[sel[:, 0]] < lab[sel[:, 1]]
        rebuilt = sel.copy()
        rebuilt[swap] = sel[swap][:, ::-1]
        assert np.array_equal(rebuilt, tr), "the trimmed file is not the relabelled input order"
        assert len(label) == int(st[0])
        out[str(k)] = {
            "n2": n2, "e2": e2, "total": total, "ckcore": ckcore,
            "ckrho": ckd[0], "rho": ckd[1], "size": int(ckd[2]),
            "ntrim": int(st[0]), "mtrim": int(st[1]), "ncktrim": int(st[2]),
            "ckdeg_sha256": sha(os.path.join(d, f"ckdeg{k}.txt")),
            "ckcore_sha256": sha(os.path.join(d, f"ckcore{k}.txt")),
            "ckdens_sha256": sha(os.path.join(d, f"ckdens{k}.txt")),
            "trimmed_sha256": sha(trimmed),
            "kept_in_label_order": kept_order,
            # the program's own phase times (one core): read, kcore + relabel,
            # k-clique degrees, k-clique core peel + output; and the total
            "reference_phase_seconds": phases[:4],
            "reference_seconds": sum(phases) if phases else (round(secs, 1) if secs is not None else None),
        }
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
