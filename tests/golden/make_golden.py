"""Generate the golden vectors in tests/golden/ by running the reference itself.

Runs in the build container only (it needs the reference sources): compiles
the reference programs and harnesses with `make -C oracle ref` (sources
compiled where they lie, outputs in oracle/_ref/), runs them on seeded graphs
and known-answer graphs, and stores their exact outputs:

  seq_p1   kCDensestNoAtom's own CDF_Main loop at p = 1 (noatom_harness seq)
  seq_edge the same functions, one stream per root edge (noatom_harness edge)
  sim      kCDensestCmpSync's CDF_Main loop (cmpsync_harness), FP64 as hex
  trim     kClistCoreTrim's output files (ckdeg, ckcore, ckdens, trimmed graph)

Graphs come from the library's seeded generators; each fixture stores a
SHA-256 of the edge list so that a change in a generator is caught, and the
small graphs store the edge list itself.

usage: python tests/golden/make_golden.py
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


def sha(pairs: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(pairs, dtype=np.uint32).tobytes()).hexdigest()


def run(cmd, cwd=None) -> str:
    r = subprocess.run(cmd, capture_output=True, text=True, cwd=cwd, timeout=3600)
    if r.returncode != 0:
        raise RuntimeError(f"{cmd} failed: {r.stderr[-2000:]}")
    return r.stdout


def parse_noatom(out: str):
    infos, rhos = [], []
    for line in out.splitlines():
        f = line.split()
        if not f:
            continue
        if f[0] == "info":
            infos.append([int(f[1]), int(f[2]), int(f[3]), float.fromhex(f[4]), float.fromhex(f[5])])
        elif f[0] == "rho":
            rhos.append(np.array(f[1:], dtype=np.uint64))
        elif f[0] == "graph":
            graph = [int(f[1]), int(f[2]), int(f[3])]
    return graph, infos, (rhos[-1] if rhos else np.zeros(0, np.uint64))


def parse_cmpsync(out: str):
    infos, rhos = [], []
    for line in out.splitlines():
        f = line.split()
        if not f:
            continue
        if f[0] == "info":
            infos.append([int(f[1]), int(f[2]), int(f[3]), float.fromhex(f[4]), float.fromhex(f[5])])
        elif f[0] == "rho":
            rhos.append(np.array([float.fromhex(x) for x in f[1:]], dtype=np.float64))
    return infos, (rhos[-1] if rhos else np.zeros(0, np.float64))


def trim_ref(path: str, k: int) -> dict:
    d = tempfile.mkdtemp()
    out = run([os.path.join(REF, "kClistCoreTrim"), str(k), path, "ckdeg", "ckcore", "ckdens", "t"], cwd=d)
    deg = np.loadtxt(os.path.join(d, "ckdeg"), dtype=np.uint64, ndmin=2).reshape(-1, 2)
    core = np.loadtxt(os.path.join(d, "ckcore"), dtype=np.uint64, ndmin=2).reshape(-1, 2)
    dens = open(os.path.join(d, "ckdens")).read().split()
    tr = np.loadtxt(os.path.join(d, f"trimmed_t_{k}.txt"), dtype=np.uint32, ndmin=2).reshape(-1, 2)
    line = [l for l in out.splitlines() if "trimmed graph has" in l][0].split()
    total = [l for l in out.splitlines() if l.startswith(f"Number of {k}-cliques")][0].split()[-1]
    return {
        "ckdeg": deg, "ckcore": core, "ckdens": dens, "trimmed": tr,
        "ntrim": int(line[4]), "mtrim": int(line[6]), "ncktrim": int(line[9]), "total": int(total),
    }


def main() -> None:
    O.build(ref=True)
    index = {}
    for case in CASES:
        name = case["name"]
        pairs = make_pairs(case)
        with tempfile.NamedTemporaryFile("w", suffix=".txt", delete=False) as f:
            for s, t in pairs:
                f.write(f"{s} {t}\n")
            path = f.name
        arrays = {}
        meta = {"name": name, "sha256": sha(pairs), "e": int(len(pairs)), "runs": {}}
        if case.get("store_edges", True):
            arrays["pairs"] = pairs
        T = case["T"]
        for k in case["ks"]:
            run_meta = {}
            graph, infos, rho = parse_noatom(run([os.path.join(REF, "noatom_harness"), "1", str(T), str(k), path, "seq"]))
            meta["graph"] = graph
            run_meta["seq_p1"] = infos
            arrays[f"k{k}_seq_p1_rho"] = rho
            _, infos, rho = parse_noatom(run([os.path.join(REF, "noatom_harness"), "1", str(T), str(k), path, "edge"]))
            run_meta["seq_edge"] = infos
            arrays[f"k{k}_seq_edge_rho"] = rho
            infos, rho = parse_cmpsync(run([os.path.join(REF, "cmpsync_harness"), "4", str(T), str(k), path]))
            run_meta["sim"] = infos
            arrays[f"k{k}_sim_rho_bits"] = rho.view(np.uint64)
            if case.get("trim", True):
                tr = trim_ref(path, k)
                run_meta["trim"] = {x: tr[x] for x in ("ckdens", "ntrim", "mtrim", "ncktrim", "total")}
                arrays[f"k{k}_trim_ckdeg"] = tr["ckdeg"]
                arrays[f"k{k}_trim_ckcore"] = tr["ckcore"]
                arrays[f"k{k}_trim_trimmed"] = tr["trimmed"]
            meta["runs"][str(k)] = run_meta
        os.unlink(path)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **arrays)
        index[name] = meta
        print(name, meta["graph"], "e =", meta["e"])
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(index, f, indent=1)


if __name__ == "__main__":
    main()
