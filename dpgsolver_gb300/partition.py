"""Element partitions of a mesh across GPUs, with the face-trace exchange of every residual / RK stage.

The reference runs on one process (its MPI set-up records rank and size, src/simulation/simulation.c:360-369, and
its older code partitioned meshes with ParMETIS, deprecated/src/gmsh_reader.c:647). Here a mesh is split by volumes:

* ``partition_volumes`` gives every volume an owner rank by recursive coordinate bisection of the volume centroids
  (equal counts, the longest extent split first);
* ``Partition`` is one rank's share: its volumes in global list order, every face with at least one of them in
  global face order, and the halo plan. A face whose other side belongs to another rank keeps the global side
  numbering and the global face-node order, and marks that side with ``REMOTE_VOLUME`` (``DGPU_REMOTE_VOLUME`` of
  include/dgpu.h). Both ranks of such a face evaluate its numerical flux from the same two traces with the same side
  convention, so they get the same flux bit for bit, and each lifts it into its own volume only;
* per stage each rank sends the traces of its side of every cut face (n_fc x n_var doubles per face) and receives
  the other side's, in global face order per neighbour. ``exchange`` does that with torch.distributed point-to-point
  calls (NCCL for device buffers, gloo for host buffers); the max |rhs| of the ranks is one all-reduce, which the
  caller may defer (it only drives progress output and the exit test, solve_explicit.c:103-112).

Volume residuals depend only on a volume's own faces, accumulated in its local-face order on the GPU (and in
global face order in the CPU oracle, which a partition keeps), so the partitioned residual equals the single-domain
one bit for bit.
"""
from __future__ import annotations

import copy
from dataclasses import dataclass, field

import numpy as np

REMOTE_VOLUME = -2


def _centroids(prob) -> np.ndarray:
    X = prob.geom.X_geom
    return X.mean(axis=1)


def partition_volumes(prob, n_parts: int) -> np.ndarray:
    """Owner rank of every volume: recursive coordinate bisection of the volume centroids into n_parts parts of
    equal size (to one volume)."""
    if n_parts < 1:
        raise ValueError("n_parts must be positive")
    c = _centroids(prob)
    owner = np.zeros(len(c), dtype=np.int32)

    def split(idx, first, parts):
        if parts == 1:
            owner[idx] = first
            return
        left = parts // 2
        ext = c[idx].max(axis=0) - c[idx].min(axis=0)
        axis = int(np.argmax(ext))
        order = idx[np.argsort(c[idx, axis], kind="stable")]
        cut = (len(idx) * left) // parts
        split(order[:cut], first, left)
        split(order[cut:], first + left, parts - left)

    split(np.arange(len(c)), 0, int(n_parts))
    return owner


@dataclass
class _SubMesh:
    d: int
    e_type: int
    n_volumes: int
    n_faces: int
    face_vol: np.ndarray
    face_lf: np.ndarray
    h: np.ndarray
    nc: np.ndarray | None = None

    def nc_fc(self, q):
        return self.nc


@dataclass
class _SubGeom:
    d: int
    curved: bool
    p_g: int
    X_geom: np.ndarray
    metrics_vc: np.ndarray
    jacobian_det_vc: np.ndarray
    normals_fc: np.ndarray
    jacobian_det_fc: np.ndarray
    extra: dict = field(default_factory=dict)


class Partition:
    """One rank's share of a uniform QUAD/HEX problem (see the module docstring).

    Attributes
    ----------
    volumes : global indices of the local volumes (global list order)
    faces : global indices of the local faces (global face order)
    face_vol, face_lf : (n_local_faces, 2) local volume index / local face of each side; REMOTE_VOLUME (and -1
        for ind_lf) for a side of another rank, -1 / -1 for the absent side of a boundary face
    neighbours : list of (rank, first, count): the halo slots exchanged with that rank are
        send_slots[first:first+count] / recv_slots[first:first+count]
    send_slots, recv_slots : trace slots 2 * local_face + side, in global face order per neighbour: the local side
        of a cut face, and its remote side
    """

    def __init__(self, prob, owner: np.ndarray, rank: int):
        self.rank = int(rank)
        self.n_parts = int(owner.max()) + 1
        mesh = prob.mesh
        owner = np.asarray(owner, dtype=np.int32)
        self.volumes = np.nonzero(owner == rank)[0]
        g2l = np.full(mesh.n_volumes, -1, dtype=np.int64)
        g2l[self.volumes] = np.arange(len(self.volumes))
        fv = np.asarray(mesh.face_vol)
        flf = np.asarray(mesh.face_lf)
        side_owner = np.where(fv >= 0, owner[np.maximum(fv, 0)], -1)
        local = np.any(side_owner == rank, axis=1)
        self.faces = np.nonzero(local)[0]
        fv_l = fv[self.faces].astype(np.int64)
        flf_l = flf[self.faces].astype(np.int64)
        own_l = side_owner[self.faces]
        out_v = np.where(fv_l < 0, -1, np.where(own_l == rank, g2l[np.maximum(fv_l, 0)], REMOTE_VOLUME))
        out_lf = np.where(out_v >= 0, flf_l, -1)
        self.face_vol = out_v.astype(np.int32)
        self.face_lf = out_lf.astype(np.int32)
        # halo: cut faces, grouped by the neighbour rank, in global face order
        send, recv, nbrs = [], [], []
        remote_side = (self.face_vol == REMOTE_VOLUME)
        cut = np.nonzero(remote_side.any(axis=1))[0]
        nbr_of = np.where(remote_side[cut, 0], own_l[cut, 0], own_l[cut, 1])
        for r in np.unique(nbr_of):
            sel = cut[nbr_of == r]
            rs = np.where(remote_side[sel, 0], 0, 1)
            nbrs.append((int(r), len(send), len(sel)))
            send.extend((2 * sel + (1 - rs)).tolist())
            recv.extend((2 * sel + rs).tolist())
        self.neighbours = nbrs
        self.send_slots = np.asarray(send, dtype=np.int32)
        self.recv_slots = np.asarray(recv, dtype=np.int32)

    @property
    def n_halo(self) -> int:
        return len(self.send_slots)

    def local_problem(self, prob):
        """The rank's share as a problem the oracle and the GPU context take (state, geometry and face data
        sliced; face-node orders, sides and numerical flux unchanged)."""
        mesh, g = prob.mesh, prob.geom
        sub = copy.copy(prob)
        nc = prob.nc_fc()[self.faces]
        sub.mesh = _SubMesh(d=mesh.d, e_type=getattr(mesh, "e_type", prob.ops.e_type), n_volumes=len(self.volumes),
                            n_faces=len(self.faces), face_vol=self.face_vol, face_lf=self.face_lf,
                            h=np.asarray(getattr(mesh, "h", np.ones(mesh.d))), nc=np.ascontiguousarray(nc))
        sub.geom = _SubGeom(d=g.d, curved=g.curved, p_g=g.p_g, X_geom=g.X_geom[self.volumes],
                            metrics_vc=g.metrics_vc[self.volumes], jacobian_det_vc=g.jacobian_det_vc[self.volumes],
                            normals_fc=g.normals_fc[self.faces], jacobian_det_fc=g.jacobian_det_fc[self.faces])
        sub.sol = np.ascontiguousarray(prob.sol[self.volumes])
        if prob.bc is not None:
            sub.bc = np.ascontiguousarray(prob.bc[self.faces])
        if prob.bc_state is not None:
            sub.bc_state = np.ascontiguousarray(prob.bc_state[self.faces])
        if getattr(prob, "source_vc", None) is not None:
            sub.source_vc = np.ascontiguousarray(prob.source_vc[self.volumes])
        return sub

    def local_state(self, sol: np.ndarray) -> np.ndarray:
        return np.ascontiguousarray(sol[self.volumes])


def exchange(part: Partition, send, recv, group=None) -> None:
    """Send this rank's halo traces (send: n_halo x slot doubles, ordered as part.send_slots) and receive the
    neighbours' into recv (ordered as part.recv_slots), with torch.distributed point-to-point calls. send / recv are
    torch tensors of shape (n_halo, slot): on the GPU for NCCL, on the host for gloo."""
    import torch.distributed as dist
    ops = []
    for r, first, count in part.neighbours:
        ops.append(dist.P2POp(dist.isend, send[first:first + count], r, group=group))
        ops.append(dist.P2POp(dist.irecv, recv[first:first + count], r, group=group))
    if ops:
        for req in dist.batch_isend_irecv(ops):
            req.wait()


def all_max(value: float, device=None, group=None) -> float:
    """max over the ranks (the deferred all-reduce of max |rhs|)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
