"""Extract the Witherden-Vincent cubature rules the reference integrates simplices with into wv_rules.npz.

Run once where the reference tree is mounted (the rules are not needed from it afterwards):

    python dpgsolver_gb300/host/make_wv_rules.py <path of the reference checkout>

The reference reads them from input/nodes/{tri,tet}/WV<degree>.txt (element/nodes.c:640-760): a header with the
number of point groups and of symmetry classes, per class the number of groups and the orbit size, then one line of
barycentric coordinates (on the regular reference simplex) per group and one weight per group. The weights are
already scaled to the regular reference element's measure (sqrt 3 for the TRI, 2 sqrt 2 / 3 for the TET). Degrees
2, 4, 6 and 8 are the volume and face cubature of orders p = 1..4 (degree 2p, nodes_operators.c:313-350, 474-516).
The file keeps the compact form (group representatives, orbit sizes, weights); simplex.wv_rule expands the orbits.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
DEGREES = (2, 4, 6, 8)


def read_rule(path: str, n_bary: int):
    with open(path) as fh:
        lines = [ln.strip() for ln in fh if ln.strip()]
    n_groups, n_symms = (int(t) for t in lines[0].split()[:2])
    counts, perms = [], []
    for ln in lines[1:1 + n_symms]:
        c, p = (int(t) for t in ln.split()[:2])
        counts.append(c)
        perms.append(p)
    i = 1 + n_symms
    assert lines[i].startswith("Barycentric"), lines[i]
    bary = np.array([[float(t) for t in ln.split()[:n_bary]] for ln in lines[i + 1:i + 1 + n_groups]])
    i += 1 + n_groups
    assert lines[i].startswith("Weights"), lines[i]
    w = np.array([float(ln.split()[0]) for ln in lines[i + 1:i + 1 + n_groups]])
    orbit = np.concatenate([np.full(c, p) for c, p in zip(counts, perms)]).astype(np.int64)
    assert len(orbit) == n_groups
    return bary, w, orbit


def main(ref_dir: str) -> None:
    out = {}
    for name, n_bary in (("tri", 3), ("tet", 4)):
        for deg in DEGREES:
            bary, w, orbit = read_rule(os.path.join(ref_dir, "input", "nodes", name, f"WV{deg}.txt"), n_bary)
            out[f"{name}{deg}_bary"] = bary
            out[f"{name}{deg}_w"] = w
            out[f"{name}{deg}_orbit"] = orbit
    path = os.path.join(HERE, "wv_rules.npz")
    np.savez_compressed(path, **out)
    print(f"{path}: {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: {sys.argv[0]} <path of the reference checkout>")
    main(sys.argv[1])
