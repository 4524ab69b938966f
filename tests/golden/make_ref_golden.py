"""Golden vectors computed by the reference itself: its compute_rhs and time_step_ssp_rk_33 on the 2D parity cases.

Run where the reference tree is mounted (it is not needed afterwards):

    python tests/golden/make_ref_golden.py <path of the reference checkout> [case ...]

It compiles the reference's own src/ into oracle/_ref (oracle/ref/Makefile), runs every case of
oracle.reference.CASES but the full-size "c2" through it (oracle.reference.run_named), and writes
tests/golden/reference_<case>.npz: the reference's geometry as its Solver_Volume / Solver_Face lists hold it
(metrics_vc, jacobian_det_vc, normals_fc, jacobian_det_fc), its volume and face lists (solution-node coordinates,
volumes / local faces / node orders per face side), the initial state, the residual and max|rhs| of compute_rhs,
and the state and max|rhs| after the case's SSP-RK3 steps. The mixed-order cases (oracle.reference.MIXED_CASES) go
through the reference's own p-adaptation first; their fixtures add every volume's order (p_vol). Case names after
the path limit it to those cases.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def main(ref_dir: str, names=()) -> None:
    import oracle.reference as R
    R.build(ref_dir)
    for name, (pde, n, p, flux, steps) in R.CASES.items():
        if name == "c2" or (names and name not in names):
            continue
        arrays = R.to_arrays(R.run_named(name))
        arrays.update(n=np.int64(n), p=np.int64(p), num_flux=np.int64(flux), steps=np.int64(steps),
                      dt=np.float64(R.host_problem(name).dt))
        _save(name, arrays)
    for name in R.MIXED_CASES:
        if not names or name in names:
            _save(name, R.run_mixed(name))


def _save(name, arrays) -> None:
    path = os.path.join(HERE, f"reference_{name}.npz")
    np.savez_compressed(path, **arrays)
    print(f"{path}: {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit(f"usage: {sys.argv[0]} <path of the reference checkout> [case ...]")
    main(sys.argv[1], tuple(sys.argv[2:]))
