"""Element partitions with the per-stage face-trace exchange (dpgsolver_gb300/partition.py) on CPU ranks.

The oracle is each rank's compute engine here (its oracle_face_traces / oracle_compute_rhs_remote split the residual
at the same point the GPU path does: traces of the local sides, exchange, face term and lift). The stitched residual
and SSP-RK3 states of the partitions must equal the single-domain ones bit for bit, in one process (all ranks in
turn) and on two and three gloo ranks over 127.0.0.1 exchanging through torch.distributed.
"""
import os
import socket
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp

import oracle
from dpgsolver_gb300 import partition as PT
from dpgsolver_gb300.host import problem as P

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROBLEMS = {
    "vortex2d_roe_p3_8": lambda: P.euler_vortex_2d(8, 3),
    "adv2d_p2_6": lambda: P.advection_2d(6, 2),
    "hex_roe_p2_4": lambda: P.euler_hex_3d(4, 2, num_flux=P.NUM_FLUX_ROE_PIKE),
    "hex_lf_p1_5": lambda: P.euler_hex_3d(5, 1),
    "channel2d_bc": lambda: P.euler_channel_2d(6, 2),
    "adv2d_source_p3_6": lambda: P.advection_default_2d(6, 3, periodic=False),
}


def test_plan_covers_every_volume_and_pairs_the_halos():
    prob = P.euler_hex_3d(6, 1)
    for n in (1, 2, 3, 5, 8):
        owner = PT.partition_volumes(prob, n)
        counts = np.bincount(owner, minlength=n)
        assert counts.sum() == prob.n_volumes and counts.max() - counts.min() <= 1
        parts = [PT.Partition(prob, owner, r) for r in range(n)]
        assert sorted(np.concatenate([p.volumes for p in parts]).tolist()) == list(range(prob.n_volumes))
        for p in parts:
            assert np.all(np.diff(p.faces) > 0)
            for r, first, count in p.neighbours:
                q = parts[r]
                back = [b for b in q.neighbours if b[0] == p.rank]
                assert len(back) == 1 and back[0][2] == count
                # the same global faces, in the same order, seen from both sides
                mine = p.faces[p.send_slots[first:first + count] // 2]
                theirs = q.faces[q.recv_slots[back[0][1]:back[0][1] + count] // 2]
                assert np.array_equal(mine, theirs)
                # send the local side, receive the remote one
                assert np.all(p.face_vol[p.send_slots[first:first + count] // 2,
                                         p.send_slots[first:first + count] % 2] >= 0)
                assert np.all(p.face_vol[p.recv_slots[first:first + count] // 2,
                                         p.recv_slots[first:first + count] % 2] == PT.REMOTE_VOLUME)


class _Rank:
    """One rank's oracle-backed share: traces of its cut faces, residual from the received ones, RK3 stages."""

    def __init__(self, prob, part):
        self.part = part
        self.sub = part.local_problem(prob)
        self.o = oracle.Oracle(self.sub)
        self.prob = prob

    def send_traces(self, sol):
        return self.o.face_traces(sol, self.part.send_slots)

    def rhs(self, sol, recv):
        remote = np.zeros((self.sub.mesh.n_faces, self.prob.n_var, self.prob.ops.n_fc))
        remote[self.part.recv_slots // 2] = recv
        return self.o.compute_rhs_remote(sol, remote)

    def stage_update(self, rk, s, sp, r, dt):
        """The reference's stage expressions (solve_explicit.c:273-290), then positivity per volume."""
        if rk == 0:
            sp[...] = s
            s = s + dt * r
        elif rk == 1:
            s = (1.0 / 4.0) * (3.0 * sp + s + dt * r)
        else:
            s = (1.0 / 3.0) * (sp + 2.0 * s + 2.0 * dt * r)
        if self.prob.positivity:
            s, _ = self.o.enforce_positivity(s)
        return s


def _serial_exchange(ranks, sends):
    """What every rank receives: the neighbours' send blocks addressed to it, in its recv_slots order."""
    recvs = []
    for rk in ranks:
        p = rk.part
        recv = np.zeros((p.n_halo, rk.prob.n_var, rk.prob.ops.n_fc))
        for nb, first, count in p.neighbours:
            q = ranks[nb].part
            blk = [b for b in q.neighbours if b[0] == p.rank][0]
            recv[first:first + count] = sends[nb][blk[1]:blk[1] + blk[2]]
        recvs.append(recv)
    return recvs


@pytest.mark.parametrize("name", sorted(PROBLEMS))
@pytest.mark.parametrize("n_parts", [2, 3, 4])
def test_partitioned_residual_and_rk3_are_bitwise_single_domain(name, n_parts):
    prob = PROBLEMS[name]()
    ref = oracle.Oracle(prob)
    r_ref, mx_ref = ref.compute_rhs(prob.sol)
    owner = PT.partition_volumes(prob, n_parts)
    ranks = [_Rank(prob, PT.Partition(prob, owner, r)) for r in range(n_parts)]
    sols = [rk.sub.sol.copy() for rk in ranks]
    recvs = _serial_exchange(ranks, [rk.send_traces(s) for rk, s in zip(ranks, sols)])
    out = np.empty_like(prob.sol)
    mx = 0.0
    for rk, s, rv in zip(ranks, sols, recvs):
        r, m = rk.rhs(s, rv)
        out[rk.part.volumes] = r
        mx = max(mx, m)
    assert np.array_equal(out, r_ref) and mx == mx_ref

    dt = prob.dt if prob.dt > 0 else 1e-3
    s_ref, _, _ = ref.ssp_rk3_step(prob.sol, dt)
    sps = [np.empty_like(s) for s in sols]
    for stage in range(3):
        recvs = _serial_exchange(ranks, [rk.send_traces(s) for rk, s in zip(ranks, sols)])
        rs = [rk.rhs(s, rv)[0] for rk, s, rv in zip(ranks, sols, recvs)]
        sols = [rk.stage_update(stage, s, sp, r, dt) for rk, s, sp, r in zip(ranks, sols, sps, rs)]
    stitched = np.empty_like(prob.sol)
    for rk, s in zip(ranks, sols):
        stitched[rk.part.volumes] = s
    assert np.array_equal(stitched, s_ref)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _gloo_rank(rank, world, port, name, out):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, REPO)
    from dpgsolver_gb300 import partition as PT_
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        prob = PROBLEMS[name]()
        owner = PT_.partition_volumes(prob, world)
        rk = _Rank(prob, PT_.Partition(prob, owner, rank))
        s = rk.sub.sol.copy()
        sp = np.empty_like(s)
        dt = prob.dt if prob.dt > 0 else 1e-3
        res = {}
        for step in range(2):
            for stage in range(3):
                send = torch.from_numpy(rk.send_traces(s))
                recv = torch.empty_like(send)
                PT_.exchange(rk.part, send, recv)
                r, m = rk.rhs(s, recv.numpy())
                if step == 0 and stage == 0:
                    res["rhs"] = r
                    res["max_rhs"] = PT_.all_max(m)
                s = rk.stage_update(stage, s, sp, r, dt)
        res["sol"] = s
        res["volumes"] = rk.part.volumes
        out[rank] = res
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("name,world", [("vortex2d_roe_p3_8", 2), ("hex_roe_p2_4", 3)])
def test_gloo_ranks_exchange_traces_and_match_single_domain(name, world):
    prob = PROBLEMS[name]()
    ref = oracle.Oracle(prob)
    r_ref, mx_ref = ref.compute_rhs(prob.sol)
    dt = prob.dt if prob.dt > 0 else 1e-3
    s_ref = prob.sol
    for _ in range(2):
        s_ref, _, _ = ref.ssp_rk3_step(s_ref, dt)
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        mp.start_processes(_gloo_rank, args=(world, port, name, out), nprocs=world, join=True, start_method="spawn")
        res = dict(out)
    rhs = np.empty_like(prob.sol)
    sol = np.empty_like(prob.sol)
    for r in range(world):
        rhs[res[r]["volumes"]] = res[r]["rhs"]
        sol[res[r]["volumes"]] = res[r]["sol"]
        assert res[r]["max_rhs"] == mx_ref
    assert np.array_equal(rhs, r_ref)
    assert np.array_equal(sol, s_ref)
