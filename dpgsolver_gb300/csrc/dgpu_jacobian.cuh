// Block-sparse Jacobian of the residual, assembled from coloured directional derivatives.
//
// The reference assembles its implicit-solver Jacobian block by block on the host: constructor_lhs_v_1_T
// (compute_volume_rlhs_T.c:179-220) for each volume's diagonal block, constructor_lhs_f_1_T
// (compute_face_rlhs_T.c:163-220) for the face couplings, each added to a PETSc matrix (add_to_petsc_Mat,
// solve.c:321-338). Here the blocks come from the dual-number JVP kernels (dgpu_jvp.cuh) by compression
// (Curtis-Powell-Reid): the volumes are coloured so that no block row holds two volumes of one colour (a distance-2
// colouring of the face-neighbour graph); a directional derivative whose direction is the unit vector of local
// degree of freedom k in every volume of colour c then yields, in each volume v's rows, column k of the block
// (v, w) of the one volume w of colour c coupled to v. n_colours x block_size derivatives give every block.
//
// The kernels here only seed the directions, apply the mass matrix (for the raw residual the reference's blocks
// belong to) and scatter the derivative into the blocks; the derivative itself is the JVP's.
#pragma once

#include "dgpu_tp.cuh"

namespace dgpu {

// du[w nb + k] = value for the volumes w of one colour.
__global__ void __launch_bounds__(256) jac_seed_kernel(double* du, const int* __restrict__ members, int n_members,
                                                      int nb, int k, double value)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n_members)
		du[(size_t)members[i] * nb + k] = value;
}

// Column k of every block (v, w(v, c)): values[(s nb + i) nb + k] = jv[v nb + i], s = slot[v n_colours + c] the block's
// index in the block-sparse rows (row-major blocks: row i = eq n_vs + node, column k = var n_vs + node).
__global__ void __launch_bounds__(256) jac_scatter_kernel(const double* __restrict__ jv, const int* __restrict__ slot,
                                                         int n_colours, int c, int n_vol, int nb, int k,
                                                         double* values)
{
	const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
	if (gid >= (long long)n_vol * nb)
		return;
	const int v = (int)(gid / nb), i = (int)(gid % nb);
	const int s = slot[(size_t)v * n_colours + c];
	if (s >= 0)
		values[((size_t)s * nb + i) * nb + k] = jv[gid];
}

// out = M in per volume, M = V^T diag(w J) V the mass matrix of each variable (the reference's residual before
// scale_rhs_by_m_inv_std, solve_dg.c:265-272, is M times the explicit right-hand side).
template <int D, int Q, int NV>
__global__ void __launch_bounds__(TPShape<D, Q>::THREADS)
tp_mass_kernel(const TPOps ops, const TPParams P, const double* __restrict__ in, double* __restrict__ out)
{
	using S = TPShape<D, Q>;
	constexpr int N = S::N, E = S::E;
	extern __shared__ double smem[];
	TPOps* sops = reinterpret_cast<TPOps*>(smem);
	double* base = smem + sizeof(TPOps) / 8;
	load_ops(sops, ops);
	const int tid = threadIdx.x;
	const int v0 = blockIdx.x * E;
	const int n_here = min(E, P.n_vol - v0);
	for (int i = tid; i < n_here * NV * N; i += blockDim.x)
		base[(i / (NV * N)) * 3 * NV * N + i % (NV * N)] = in[(size_t)v0 * NV * N + i];
	__syncthreads();
	const int e = tid / N, node = tid % N;
	const bool active = e < n_here;
	double* sa = base + e * 3 * NV * N;
	double* sb = sa + NV * N;
	double* sc = sb + NV * N;
	tp_apply<D, Q, NV>(sa, sb, sc, sops->B, node, active);   // GL values V x
	if (active) {
		const double wJ = 1.0 / P.inv_wJ[(size_t)(v0 + e) * N + node];
#pragma unroll
		for (int k = 0; k < NV; ++k)
			sa[k * N + node] = wJ * sb[k * N + node];
	}
	__syncthreads();
	tp_apply<D, Q, NV>(sa, sb, sc, sops->BT, node, active);  // V^T (w J V x)
	if (active)
#pragma unroll
		for (int k = 0; k < NV; ++k)
			out[((size_t)(v0 + e) * NV + k) * N + node] = sb[k * N + node];
}

}  // namespace dgpu
