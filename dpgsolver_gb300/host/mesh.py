"""Structured QUAD/HEX meshes (periodic, or bounded in chosen directions) and the reference's face list.

The reference reads gmsh files and builds its connectivity in src/simulation/mesh; the
face list itself is built by computational_elements/face.c:86-160: volumes are visited in
list order, local faces in index order, and a face is created the first time it is met, so
the volume that comes first in the list is side 0 (``neigh_info[0]``, the "left" volume
whose normal the numerical flux uses) and its neighbour is side 1.  This module reproduces
that rule for generated periodic meshes, which is what makes the Roe-Pike flux (whose
entropy fix is not symmetric in L/R, numerical_flux_euler_T.c:560-562) agree with the
reference's choice of sides.

Volume order: first index fastest (x, then y, then z).
"""
from __future__ import annotations

import numpy as np

from .element import QUAD, HEX


class StructuredMesh:
    """n_x x n_y (x n_z) mesh of [lo, hi]^d, periodic in the directions `periodic` selects (all by default); the
    ends of the other directions are boundary faces with face_vol[f, 1] = face_lf[f, 1] = -1.

    Attributes
    ----------
    d, e_type, n_volumes, n_faces
    vertices_lo : (n_volumes, d) lower corner of each volume (undeformed)
    h : (d,) element size per direction
    face_vol : (n_faces, 2) volume index of side 0 / side 1
    face_lf : (n_faces, 2) local face index of each side
    face_ord : (n_faces, 2) reference ``ind_ord`` of each side (0 for these aligned meshes)
    vol_faces : (n_volumes, 2d) face index of each local face
    vol_side : (n_volumes, 2d) which side (0/1) the volume is on for that face
    """

    def __init__(self, d: int, n, lo, hi, periodic=True):
        if d not in (2, 3):
            raise ValueError("d must be 2 or 3")
        n = [int(v) for v in (n if np.ndim(n) else [n] * d)]
        lo = np.broadcast_to(np.asarray(lo, dtype=np.float64), (d,)).copy()
        hi = np.broadcast_to(np.asarray(hi, dtype=np.float64), (d,)).copy()
        if any(v < 2 for v in n):
            raise ValueError("periodic structured mesh needs at least 2 elements per direction")
        self.d = d
        self.e_type = QUAD if d == 2 else HEX
        self.n = n
        self.lo, self.hi = lo, hi
        self.h = (hi - lo) / np.array(n)
        nv = int(np.prod(n))
        self.n_volumes = nv
        idx = np.arange(nv)
        ijk = []
        rem = idx.copy()
        for k in range(d):
            ijk.append(rem % n[k])
            rem //= n[k]
        self.ijk = np.stack(ijk, axis=1)
        self.vertices_lo = lo[None, :] + self.ijk * self.h[None, :]

        per = [bool(x) for x in (periodic if np.ndim(periodic) else [periodic] * d)]
        self.periodic = per
        n_lf = 2 * d
        vol_faces = -np.ones((nv, n_lf), dtype=np.int64)
        vol_side = -np.ones((nv, n_lf), dtype=np.int64)
        face_vol, face_lf = [], []
        for v in range(nv):
            for lf in range(n_lf):
                if vol_faces[v, lf] >= 0:
                    continue
                dim, side = lf // 2, lf % 2
                nb = self.ijk[v].copy()
                step = nb[dim] + (1 if side == 1 else -1)
                if not per[dim] and (step < 0 or step >= n[dim]):
                    # boundary face: the volume is side 0, no side 1 (face.c:86-160 for a face with one neighbour)
                    f = len(face_vol)
                    face_vol.append((v, -1))
                    face_lf.append((lf, -1))
                    vol_faces[v, lf] = f
                    vol_side[v, lf] = 0
                    continue
                nb[dim] = step % n[dim]
                vn = self._index(nb)
                lf_n = lf ^ 1
                f = len(face_vol)
                face_vol.append((v, vn))
                face_lf.append((lf, lf_n))
                vol_faces[v, lf] = f
                vol_side[v, lf] = 0
                vol_faces[vn, lf_n] = f
                vol_side[vn, lf_n] = 1
        self.face_vol = np.array(face_vol, dtype=np.int64)
        self.face_lf = np.array(face_lf, dtype=np.int64)
        self.face_ord = np.zeros_like(self.face_lf)
        self.vol_faces = vol_faces
        self.vol_side = vol_side
        self.n_faces = len(face_vol)

    def _index(self, ijk):
        idx = 0
        stride = 1
        for k in range(self.d):
            idx += int(ijk[k]) * stride
            stride *= self.n[k]
        return idx

    def element_map(self, v: int, xi: np.ndarray) -> np.ndarray:
        """Undeformed affine map of volume v: reference coords (m, d) in [-1,1]^d -> physical (m, d)."""
        return self.vertices_lo[v][None, :] + 0.5 * (xi + 1.0) * self.h[None, :]
