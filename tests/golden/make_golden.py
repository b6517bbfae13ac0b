"""Writes tests/golden/tiny_graphs.json: hand-derived known answers.

The reference project ships no tests or golden vectors, so these fixtures pin
the semantics of its plugins on graphs small enough to work out by hand
(derivations inline), and every value is cross-checked here against
networkx / numpy, which share no code with the oracle or the GPU path.

Semantics pinned (Grudon src/graph_algorithms/*.cpp):
  CC    label[v] = min gid over every u that reaches v along out-edges
        (cc.cpp:66-79 propagates along out-edges only)
  SSSP  hop count from gid 0 (sssp.cpp:69) and the weighted variant
  PR    delta-push fixed point pr[v] = 0.15*[outdeg>0] + 0.85*sum pr[u]/outdeg(u)
        (pr.cpp:30-49 gives dangling vertices no base rank) and the round
        count of the delta-push protocol.

Run: python tests/golden/make_golden.py
"""
import json
from pathlib import Path

import networkx as nx
import numpy as np

INF = 0xFFFFFFFF
D = 0.85

FIXTURES = [
    {
        "name": "path4_directed", "n": 4,
        "edges": [[0, 1, 2], [1, 2, 3], [2, 3, 4]],
        # hop: 0,1,2,3; weighted: 0, 2, 2+3, 2+3+4; CC: 0 reaches everyone
        "cc": [0, 0, 0, 0], "hop": [0, 1, 2, 3], "sssp_w": [0, 2, 5, 9],
        "hop_rounds": 4, "cc_rounds": 4,
    },
    {
        "name": "star_sym", "n": 6,
        "edges": [[0, k, k] for k in range(1, 6)] + [[k, 0, k] for k in range(1, 6)],
        "cc": [0] * 6, "hop": [0, 1, 1, 1, 1, 1], "sssp_w": [0, 1, 2, 3, 4, 5],
    },
    {
        "name": "two_components_sym", "n": 6,
        "edges": [[0, 1, 1], [1, 0, 1], [1, 2, 1], [2, 1, 1], [0, 2, 5], [2, 0, 5], [3, 4, 1], [4, 3, 1]],
        # triangle {0,1,2}, edge {3,4}, isolated 5; 0->2 costs 5 direct, 2 via 1
        "cc": [0, 0, 0, 3, 3, 5], "hop": [0, 1, 1, INF, INF, INF], "sssp_w": [0, 1, 2, INF, INF, INF],
    },
    {
        "name": "cycle4_directed", "n": 4,
        "edges": [[0, 1, 5], [1, 2, 1], [2, 3, 2], [3, 0, 7]],
        # 0->1 (5), ->2 (6), ->3 (8); everyone reachable from 0 so CC = 0
        "cc": [0, 0, 0, 0], "hop": [0, 1, 2, 3], "sssp_w": [0, 5, 6, 8],
    },
    {
        "name": "dangling", "n": 3,
        "edges": [[0, 1, 1], [0, 2, 1], [1, 2, 1]],
        # delta push by hand (TOL 1e-6):
        #  init  prop = [.85*.15/2, .85*.15/1, 0] = [.06375, .1275, 0], pr = [.15, .15, 0]
        #  r1    upd1 = .06375, upd2 = .06375 + .1275 = .19125 -> pr = [.15, .21375, .19125]
        #        prop1 = .85*.06375 = .0541875; vertex 2 has no out-edges
        #  r2    upd2 = .0541875 -> pr2 = .2454375
        #  r3    frontier {2} pushes nothing -> empty frontier, stop after 3 rounds
        "cc": [0, 0, 0], "hop": [0, 1, 1], "sssp_w": [0, 1, 1],
        "pr": [0.15, 0.21375, 0.2454375], "pr_rounds": 3,
    },
]


def csr(n, edges):
    e = sorted((s, d, w) for s, d, w in edges)
    ro = [0] * (n + 1)
    for s, _, _ in e:
        ro[s + 1] += 1
    for i in range(n):
        ro[i + 1] += ro[i]
    return ro, [d for _, d, _ in e], [w for _, _, w in e]


def check(fx):
    n = fx["n"]
    G = nx.DiGraph()
    G.add_nodes_from(range(n))
    for s, d, w in fx["edges"]:
        G.add_edge(s, d, weight=w)
    hop = nx.single_source_shortest_path_length(G, 0)
    assert [hop.get(v, INF) for v in range(n)] == fx["hop"], fx["name"]
    dist = nx.single_source_dijkstra_path_length(G, 0)
    assert [dist.get(v, INF) for v in range(n)] == fx["sssp_w"], fx["name"]
    cc = [min(u for u in range(n) if u == v or nx.has_path(G, u, v)) for v in range(n)]
    assert cc == fx["cc"], fx["name"]
    if "pr" in fx:
        outdeg = np.array([G.out_degree(v) for v in range(n)], dtype=float)
        A = np.zeros((n, n))
        for s, d, _ in fx["edges"]:
            A[d, s] += D / outdeg[s]
        b = 0.15 * (outdeg > 0)
        pr = np.linalg.solve(np.eye(n) - A, b)
        assert np.allclose(pr, fx["pr"], atol=1e-12), fx["name"]


def main():
    out = []
    for fx in FIXTURES:
        check(fx)
        ro, col, w = csr(fx["n"], fx["edges"])
        out.append(dict(fx, row_offsets=ro, col_indices=col, weights=w))
    path = Path(__file__).with_name("tiny_graphs.json")
    path.write_text(json.dumps(out, indent=1) + "\n")
    print(f"wrote {path} ({len(out)} graphs)")


if __name__ == "__main__":
    main()
