"""Extract the reference's mesh integration-test fixtures into a JSON fixture for the mesh reader's tests.

Run once where the reference tree is mounted (it is not needed afterwards):

    python tests/golden/make_mesh_golden.py <path of the reference checkout>

Sources (read as text, values copied verbatim): input/testing/integration/mesh/<name>.msh, the gmsh files the
reference's test_integration_mesh.c reads, and <name>.msh.data, the Mesh_Data, Mesh_Connectivity and
Mesh_Vertices it compares them against (test_integration_mesh.c:71-150), for the three meshes that have data.
"""
from __future__ import annotations

import json
import os
import sys

MESHES = ["straight_2d_quad_periodic", "blended_2d_mixed", "parametric_2d_quad_periodic_reflected"]


def _container(lines, i):
    """lines[i] == 'container <type>'; returns (value, next index)."""
    kind = lines[i].split()[1]
    i += 1
    if kind == "Vector_i":
        vals = [int(v) for v in lines[i].split()]
        assert vals[0] == len(vals) - 1
        return vals[1:], i + 1
    if kind in ("Matrix_d", "Matrix_i"):
        layout, m, n = lines[i].split()
        assert layout == "R"
        conv = float if kind == "Matrix_d" else int
        rows = [[conv(v) for v in lines[i + 1 + r].split()] for r in range(int(m))]
        assert all(len(r) == int(n) for r in rows)
        return rows, i + 1 + int(m)
    if kind == "Multiarray_Vector_i":
        assert lines[i].split() == ["order", "1"]
        n = int(lines[i + 1].split()[1])
        assert lines[i + 2].strip() == "ext_0/data"
        out = []
        for r in range(n):
            vals = [int(v) for v in lines[i + 3 + r].split()]
            assert vals[0] == len(vals) - 1
            out.append(vals[1:])
        return out, i + 3 + n
    raise ValueError(kind)


def parse_data(path):
    lines = [ln.rstrip("\n") for ln in open(path)]
    out = {}
    i = 0
    while i < len(lines):
        ln = lines[i].strip()
        if ln.endswith(":") and i + 1 < len(lines) and lines[i + 1].startswith("container"):
            out[ln[:-1]], i = _container(lines, i + 1)
            continue
        i += 1
    return out


def main(ref_root):
    base = os.path.join(ref_root, "input", "testing", "integration", "mesh")
    fixture = {}
    for name in MESHES:
        fixture[name] = {"d": 2, "msh": open(os.path.join(base, name + ".msh")).read(),
                         "expected": parse_data(os.path.join(base, name + ".msh.data"))}
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_mesh_data.json")
    with open(dst, "w") as fh:
        json.dump(fixture, fh, indent=0)
    print("wrote", dst, {k: sorted(v["expected"]) for k, v in fixture.items()})


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: {sys.argv[0]} <path of the reference checkout>")
    main(sys.argv[1])
