"""Extract the reference's unit-test golden data that pins the TP element layer into JSON fixtures.

Run once where the reference tree is mounted (it is not needed afterwards):

    python tests/golden/make_golden.py <path of the reference checkout>

Sources (read as text, values copied verbatim):
  input/testing/unit/operators/operators_tp.data  -- test_unit_operators_tp.c:56-170 (TP op_std assembly and
                                                     sum-factorised apply, tolerance EPS)
  input/testing/unit/nodes/nodes_tp.data          -- test_unit_nodes.c (EQ / GLL / GL TP nodes and weights)
  input/testing/unit/nodes/nodes_correspondence.data -- test_unit_nodes.c:62-89 (face-node correspondence
                                                     permutations per ind_ord)
"""
from __future__ import annotations

import json
import os
import re
import sys


def _tokens(path):
    with open(path) as fh:
        return [ln.rstrip("\n") for ln in fh]


def _read_matrix(lines, i):
    """At lines[i] == 'container Matrix_d' or 'container Multiarray_d'; returns (matrix rows, next index)."""
    kind = lines[i].split()[1]
    i += 1
    hdr = lines[i].split()
    if hdr[0] == "NULL":
        return None, i + 1
    if kind == "Matrix_d":
        layout, m, n = hdr[0], int(hdr[1]), int(hdr[2])
    else:
        layout, order, m, n = hdr[0], int(hdr[1]), int(hdr[2]), int(hdr[3])
        assert order == 2
    rows = []
    for r in range(m):
        rows.append([float(v) for v in lines[i + 1 + r].split()])
        assert len(rows[-1]) == n, (lines[i + 1 + r], n)
    return {"layout": layout, "rows": rows}, i + 1 + m


def parse_operators_tp(path):
    lines = _tokens(path)
    out = {}
    i = 0
    current = None
    while i < len(lines):
        ln = lines[i].strip()
        m = re.match(r"^(\w+)_ops_tp:$", ln)
        if m:
            current = m.group(1)
            ext = int(lines[i + 3].split()[1])
            i += 4
            ops = []
            for _ in range(ext):
                assert lines[i].startswith("container Matrix_d")
                mat, i = _read_matrix(lines, i)
                ops.append(mat["rows"] if mat else None)
            out.setdefault(current, {})["ops_tp"] = ops
            continue
        m = re.match(r"^(\w+)_(op_std|b|c):$", ln)
        if m:
            mat, i = _read_matrix(lines, i + 1)
            out.setdefault(m.group(1), {})[m.group(2)] = mat["rows"]
            continue
        i += 1
    return out


def parse_nodes_tp(path):
    lines = _tokens(path)
    out = {}
    i = 0
    while i < len(lines):
        ln = lines[i].strip()
        m = re.match(r"^Nodes_d(\d)_p(\d)_(\w+)$", ln)
        if m:
            key = ln
            entry = {"d": int(m.group(1)), "p": int(m.group(2)), "type": m.group(3)}
            i += 1
            while i < len(lines) and not lines[i].startswith("Nodes_") and not lines[i].startswith("----"):
                if lines[i].strip() == "rst:":
                    mat, i = _read_matrix(lines, i + 1)
                    entry["rst"] = mat["rows"]
                    continue
                if lines[i].strip() == "w:":
                    mat, i = _read_matrix(lines, i + 1)
                    entry["w"] = [r[0] for r in mat["rows"]]
                    continue
                i += 1
            out[key] = entry
            continue
        i += 1
    return out


def parse_correspondence(path):
    lines = _tokens(path)
    out = {}
    i = 0
    while i < len(lines):
        ln = lines[i].strip()
        m = re.match(r"^((line|quad)_\d+):$", ln)
        if m:
            ext = int(lines[i + 3].split()[1])
            perms = []
            for r in range(ext):
                vals = lines[i + 5 + r].split()
                n = int(vals[0])
                perms.append([int(v) for v in vals[1:1 + n]])
            out[m.group(1)] = perms
            i += 5 + ext
            continue
        i += 1
    return out


def main(ref_root):
    base = os.path.join(ref_root, "input", "testing", "unit")
    data = {
        "source": "DPGSolver input/testing/unit (operators_tp.data, nodes_tp.data, nodes_correspondence.data)",
        "operators_tp": parse_operators_tp(os.path.join(base, "operators", "operators_tp.data")),
        "nodes_tp": parse_nodes_tp(os.path.join(base, "nodes", "nodes_tp.data")),
        "nodes_correspondence": parse_correspondence(os.path.join(base, "nodes", "nodes_correspondence.data")),
    }
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_unit_data.json")
    with open(dst, "w") as fh:
        json.dump(data, fh, indent=1)
    print("wrote", dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: {sys.argv[0]} <path of the reference checkout>")
    main(sys.argv[1])
