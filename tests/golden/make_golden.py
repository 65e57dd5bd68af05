"""Writes the golden fixtures under tests/golden/ (run: python tests/golden/make_golden.py).

The reference's Go toolchain is not available, so the fixtures are produced by
the CPU oracle (oracle/sph_oracle.c, a -ffp-contract=off restatement of
sim/core.go, sim/nearest-neighbour.go and sim/sph.go) running the reference's
own tree search. Each fixture stores its inputs as well, so that tests on any
host (x86 or Arm) can check that the oracle and the GPU path reproduce it bit
for bit.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

CASES = {
    # name: (n, k, seed, steps, alpha, beta, dth)
    "blast600_k32": (600, 32, 11, 3, 1.0, 2.0, 5e-5),
    "blast400_k16_refconsts": (400, 16, 12, 2, 0.75, 1.5, 1e-4),
}


def splitmix_uniform(n, seed):
    """SplitMix64 (Steele, Lea and Flood) -> 53-bit doubles, as sph_ic_uniform_blast."""
    out = np.empty(2 * n)
    s = seed & 0xFFFFFFFFFFFFFFFF
    M = 0xFFFFFFFFFFFFFFFF
    for i in range(2 * n):
        s = (s + 0x9E3779B97F4A7C15) & M
        z = s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
        z ^= z >> 31
        out[i] = (z >> 11) * 2.0 ** -53
    return out[0::2].copy(), out[1::2].copy()


def make(name):
    n, k, seed, steps, alpha, beta, dth = CASES[name]
    x, y = splitmix_uniform(n, seed)
    u = np.where((x - 0.5) ** 2 + (y - 0.5) ** 2 < 0.1 * 0.1, 10.0, 1.0)
    p = O.make_params(n, k, knn_mode=O.KNN_TREE, alpha=alpha, beta=beta, dth=dth)
    s = O.OracleSim(p, x, y, None, None, u)
    s.set_check_tree(True)
    s.step(steps)
    if s.tree_mismatches():
        raise SystemExit(f"{name}: tree and exact neighbour sets differ; pick another seed")
    st = s.state()
    ids, dist, img = s.neighbours()
    np.savez_compressed(
        os.path.join(HERE, name + ".npz"), n=n, k=k, seed=seed, steps=steps, alpha=alpha, beta=beta, dth=dth,
        x0=x, y0=y, u0=u, ids=ids.astype(np.int32), dist=dist, img=img.astype(np.int8),
        **{f"out_{key}": val for key, val in st.items()})


if __name__ == "__main__":
    for name in CASES:
        make(name)
        print("wrote", name)
