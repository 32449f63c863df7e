"""Graphs behind the golden vectors: seeded synthetic graphs (stand-ins for the
paper's datasets, which are not distributed) and known-answer graphs."""
from __future__ import annotations

import itertools

import numpy as np


def complete(n: int, base: int = 0) -> list[tuple[int, int]]:
    return [(base + i, base + j) for i, j in itertools.combinations(range(n), 2)]


def disjoint_cliques(sizes) -> list[tuple[int, int]]:
    out, base = [], 0
    for s in sizes:
        out += complete(s, base)
        base += s
    return out


def clique_with_tree(c: int, tree: int) -> list[tuple[int, int]]:
    """K_c on 0..c-1 plus a path-and-branch tree of `tree` vertices hanging off vertex 0."""
    out = complete(c)
    for i in range(tree):
        v = c + i
        parent = 0 if i == 0 else c + (i - 1) // 2
        out.append((parent, v))
    return out


def star(leaves: int) -> list[tuple[int, int]]:
    return [(0, i) for i in range(1, leaves + 1)]


CASES = [
    # Config 1: the parity config (Chung-Lu n=10,000, average degree 20, exponent 2.5, seed 1).
    {"name": "config1_chung_lu_1e4", "gen": ("chung_lu", dict(n=10000, avg_degree=20.0, gamma=2.5, seed=1)),
     "ks": [4], "T": 10, "store_edges": False},
    {"name": "cl_2000", "gen": ("chung_lu", dict(n=2000, avg_degree=16.0, gamma=2.3, seed=5)),
     "ks": [3, 4, 5], "T": 8},
    {"name": "er_1500", "gen": ("erdos_renyi", dict(n=1500, avg_degree=30.0, seed=2)), "ks": [4, 5, 6], "T": 8},
    {"name": "rmat12", "gen": ("rmat", dict(scale=12, edge_factor=16, seed=3)), "ks": [4, 5], "T": 8,
     "store_edges": False},
    {"name": "planted_3000", "gen": ("planted", dict(n=3000, avg_degree=8.0, gamma=2.2, communities=3,
                                                     comm_min=30, comm_max=80, p_in=0.6, seed=4)),
     "ks": [5, 6, 7], "T": 8},
    # Known answers: K_10 has C(10, k) k-cliques and density C(10, k) / 10.
    {"name": "kat_complete10", "pairs": complete(10), "ks": [3, 4, 5, 6, 7, 8], "T": 4},
    {"name": "kat_disjoint_cliques", "pairs": disjoint_cliques([6, 7, 5]), "ks": [3, 4, 5], "T": 4},
    {"name": "kat_clique_tree", "pairs": clique_with_tree(7, 12), "ks": [3, 4], "T": 4},
    # No triangles at all (the trim would drop every vertex; the reference's trim
    # program does not terminate on an empty core, so it is not run here).
    {"name": "kat_star", "pairs": star(20), "ks": [3], "T": 2, "trim": False},
    {"name": "kat_triangle_k4", "pairs": complete(3), "ks": [4], "T": 2, "trim": False},
]


def make_pairs(case: dict) -> np.ndarray:
    if "pairs" in case:
        return np.asarray(case["pairs"], dtype=np.uint32).reshape(-1, 2)
    import kclistpp_gb300 as K

    fn, kw = case["gen"]
    return getattr(K, fn)(**kw).pairs()
