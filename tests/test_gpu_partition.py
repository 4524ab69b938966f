"""Element partitions on the GPU: the halo calls of the C ABI (dgpu_halo_*), with every rank of a 2-, 3- or 4-way
partition on this one GPU in turn (each rank's kernels run to completion before the exchange, which is a device copy
here and NCCL send/recv between GPUs). The stitched residual and SSP-RK3 states must equal the single-domain context's
bit for bit, and a partitioned context must refuse the whole-mesh calls."""
import numpy as np
import pytest

from dpgsolver_gb300 import partition as PT
from dpgsolver_gb300.host import problem as P

pytestmark = pytest.mark.gpu

PROBLEMS = {
    "vortex2d_roe_p3_8": lambda: P.euler_vortex_2d(8, 3),
    "adv2d_p2_12": lambda: P.advection_2d(12, 2),
    "hex_roe_p2_6": lambda: P.euler_hex_3d(6, 2, num_flux=P.NUM_FLUX_ROE_PIKE),
    "hex_lf_p3_8": lambda: P.euler_hex_3d(8, 3),
    "channel2d_bc": lambda: P.euler_channel_2d(6, 2),
    "adv2d_source_p3_8": lambda: P.advection_default_2d(8, 3, periodic=False),
}


def _exchange(sims):
    """Every rank's received traces: the neighbours' send blocks addressed to it (device copies)."""
    import torch
    for s in sims:
        s.synchronize()
    bufs = [s.halo_tensors() for s in sims]
    for s, (_, recv) in zip(sims, bufs):
        for nb, first, count in s.part.neighbours:
            q = sims[nb].part
            blk = [b for b in q.neighbours if b[0] == s.part.rank][0]
            recv[first:first + count].copy_(bufs[nb][0][blk[1]:blk[1] + blk[2]])
    torch.cuda.synchronize()


@pytest.mark.parametrize("name", sorted(PROBLEMS))
@pytest.mark.parametrize("n_parts", [2, 3, 4])
def test_partitioned_gpu_residual_and_rk3_are_bitwise_single_domain(gpu_lib, name, n_parts):
    from dpgsolver_gb300.solver import PartitionSimulation, Simulation
    prob = PROBLEMS[name]()
    dt = prob.dt if prob.dt > 0 else 1e-3
    with Simulation(prob) as sim:
        mx_ref = sim.compute_rhs()
        r_ref = sim.rhs
        mx_step_ref = sim.ssp_rk3_steps(dt, 2)
        s_ref = sim.sol_coef
    owner = PT.partition_volumes(prob, n_parts)
    sims = [PartitionSimulation(prob, PT.Partition(prob, owner, r)) for r in range(n_parts)]
    try:
        for s in sims:
            s.rhs_begin()
        _exchange(sims)
        rhs = np.empty_like(prob.sol)
        mx = max(s.rhs_end() for s in sims)
        for s in sims:
            rhs[s.part.volumes] = s.rhs
        assert np.array_equal(rhs, r_ref) and mx == mx_ref

        for step in range(2):
            for stage in range(3):
                for s in sims:
                    s.stage_begin(stage)
                _exchange(sims)
                mxs = [s.stage_end(dt, stage, want_max=(step == 1 and stage == 2)) for s in sims]
        assert max(mxs) == mx_step_ref
        sol = np.empty_like(prob.sol)
        for s in sims:
            sol[s.part.volumes] = s.sol_coef
        assert np.array_equal(sol, s_ref)
    finally:
        for s in sims:
            s.close()


def test_partitioned_context_refuses_whole_mesh_calls(gpu_lib):
    from dpgsolver_gb300.solver import DGPUError, PartitionSimulation
    prob = P.euler_hex_3d(4, 2)
    owner = PT.partition_volumes(prob, 2)
    with PartitionSimulation(prob, PT.Partition(prob, owner, 0)) as s:
        with pytest.raises(DGPUError):
            s.compute_rhs()
        with pytest.raises(DGPUError):
            s.ssp_rk3_steps(1e-3, 1)
