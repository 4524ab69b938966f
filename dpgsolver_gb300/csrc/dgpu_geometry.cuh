// Geometry precompute of TP volumes and their faces on the device: the reference's set_up_solver_geometry_T
// (src/simulation/geometry/geometry_T.c:165-185) for QUAD/HEX volumes.
//
// Input per volume: the geometry coefficients geom_coef (Solver_Volume_T::geom_coef), the physical coordinates at
// the GLL nodes of order p_g (p for curved volumes, 1 for straight ones, geometry_T.c:740-742), which are also the
// metric nodes vm. Per volume (geo_volume_kernel, compute_geometry_volume_T :208-272 through
// constructor_volume_metric_terms_T :734-801):
//   * the Jacobian dx_i/dr_j at vm by the GLL derivative of the coefficients (cv1_vg_vm);
//   * the metric terms at vm, m(i, j) = J dr_j/dx_i: the cofactors in 2D (compute_cofactors_T :546-590); in 3D the
//     conservative curl form m(i, .) = -1/2 curl_r(X_l grad_r X_m - X_m grad_r X_l), (i, m, l) cyclic, whose
//     discrete divergence vanishes (the reference aborts there with EXIT_ADD_SUPPORT and points to the curl form);
//   * metrics_vc = the interpolant of the vm metric terms at the GL cubature nodes (vv0_vm_vc);
//   * jacobian_det_vc from the Jacobian evaluated at the cubature nodes directly (cv1_vg_vc, compute_detJV_T).
// Per face node (geo_face_kernel, compute_geometry_face_T :274-325): the side-0 volume's vm metric terms interpolated
// to the face cubature node (vv0_vm_fc), n = m . n_ref of the local face (compute_normals_T :412-445), normals_fc
// = n / |n|, jacobian_det_fc = |n|, and xyz_fc (cv0_vg_fc).
//
// Setup work, run once per mesh: one CTA per volume with every intermediate in shared memory, sum-factorised
// passes with run-time extents; the face kernel sums over the volume's geometry nodes directly.
#pragma once

#include <cuda_runtime.h>

#include "dgpu_tp.cuh"

namespace dgpu {

constexpr int kGeoNodes = kQMax * kQMax * kQMax;   // geometry or cubature nodes of one volume, at most

struct GeoOps {
	int d;
	int qg;                         // geometry (= metric) nodes per direction: p_g + 1
	int q;                          // GL cubature nodes per direction: p + 1
	double Dgg[kQMax][kQMax];       // Dgg[m][a] = l_a'(x_g[m])   (GLL basis derivative at its own nodes)
	double Lgc[kQMax][kQMax];       // Lgc[c][a] = l_a(x_c[c])    (GLL basis at the GL nodes)
	double Dgc[kQMax][kQMax];       // Dgc[c][a] = l_a'(x_c[c])
	double Lgb[2][kQMax];           // l_a(-1), l_a(+1)
	double nref[6][3];              // reference unit normals of the local faces (element.c:708-780)
	double w[kQMax];                // GL weights (the context form multiplies them in)
};

// Where the results go: the reference's layouts (any pointer may be null), or the context's pre-multiplied form.
struct GeoOut {
	double* metrics_vc;       // [v][c + n_vc (i + d j)] = m(c, i, j)
	double* jacobian_det_vc;  // [v][c]
	double* normals_fc;       // [f][(t d + k)]
	double* jacobian_det_fc;  // [f][t]
	double* xyz_fc;           // [f][(t d + k)]
	double* gmet;             // context: [v][(j d + i)][c] = w_c m(c, i, j)
	double* inv_wJ;           // context: [v][c] = 1 / (w_c J_c)
	double* fgeo;             // context: [f][d + 1][t] = unit normal, w_t J_f
	double* metrics_vm;       // scratch [v][(i d + j)][g], written by the volume kernel, read by the face kernel
	int* err;                 // set to 1 where a Jacobian determinant is not positive
};

// out = M applied along direction `dir` to `nc` components of `in` (extents e, first direction fastest); M has
// `rows` rows. Component c of in starts at c * (e0 e1 e2), of out at c * (e'0 e'1 e'2). All threads of the CTA.
__device__ __forceinline__ void geo_pass(const double* in, double* out, const int* e, int dir,
                                         const double (*M)[kQMax], int rows, int nc)
{
	int eo[3] = {e[0], e[1], e[2]};
	eo[dir] = rows;
	const int n_in = e[0] * e[1] * e[2], n_out = eo[0] * eo[1] * eo[2];
	for (int t = threadIdx.x; t < n_out * nc; t += blockDim.x) {
		const int c = t / n_out, o = t % n_out;
		int idx[3] = {o % eo[0], (o / eo[0]) % eo[1], o / (eo[0] * eo[1])};
		const int a = idx[dir];
		double s = 0.0;
		for (int m = 0; m < e[dir]; ++m) {
			idx[dir] = m;
			s += M[a][m] * in[c * n_in + idx[0] + e[0] * (idx[1] + e[1] * idx[2])];
		}
		out[c * n_out + o] = s;
	}
	__syncthreads();
}

// Shared memory of geo_volume_kernel, in doubles: X, Jm, mvm, V, dV, mvc, Jc and two pass temporaries.
constexpr int kGeoSmem = (3 + 9 + 9 + 3 + 9 + 9 + 9) * kGeoNodes + 2 * 9 * kGeoNodes;

__global__ void __launch_bounds__(128) geo_volume_kernel(const GeoOps G, int n_vol, const double* __restrict__ geom_coef,
                                                        GeoOut out)
{
	extern __shared__ double sm[];
	const int d = G.d, qg = G.qg, q = G.q;
	const int ng = (d == 2 ? qg * qg : qg * qg * qg), nc = (d == 2 ? q * q : q * q * q);
	double* X = sm;                       // [k][g]
	double* Jm = X + 3 * kGeoNodes;       // [(j d + i)][g] = dx_i/dr_j at vm
	double* mvm = Jm + 9 * kGeoNodes;     // [(i d + j)][g]
	double* V = mvm + 9 * kGeoNodes;      // [j][g] (3D curl form)
	double* dV = V + 3 * kGeoNodes;       // [(jj 3 + c)][g] = d V_c / dr_jj
	double* mvc = dV + 9 * kGeoNodes;     // [(i d + j)][c] at vc
	double* Jc = mvc + 9 * kGeoNodes;     // [(j d + i)][c] at vc
	double* t0 = Jc + 9 * kGeoNodes;      // pass temporaries
	double* t1 = t0 + 9 * kGeoNodes;
	const int v = blockIdx.x;
	if (v >= n_vol)
		return;
	const double* xg = geom_coef + (size_t)v * ng * d;
	for (int i = threadIdx.x; i < ng * d; i += blockDim.x)
		X[i] = xg[i];
	__syncthreads();
	const int eg[3] = {qg, qg, d == 3 ? qg : 1};

	// Jacobian at vm: d/dr_j of every coordinate
	for (int j = 0; j < d; ++j)
		geo_pass(X, Jm + j * d * ng, eg, j, G.Dgg, qg, d);

	// metric terms at vm
	if (d == 2) {
		for (int g = threadIdx.x; g < ng; g += blockDim.x) {
			const double xr = Jm[(0 * 2 + 0) * ng + g], yr = Jm[(0 * 2 + 1) * ng + g];
			const double xs = Jm[(1 * 2 + 0) * ng + g], ys = Jm[(1 * 2 + 1) * ng + g];
			mvm[0 * ng + g] = ys;
			mvm[1 * ng + g] = -yr;
			mvm[2 * ng + g] = -xs;
			mvm[3 * ng + g] = xr;
		}
		__syncthreads();
	} else {
		for (int i = 0; i < 3; ++i) {
			const int mm = (i + 1) % 3, ll = (i + 2) % 3;
			for (int t = threadIdx.x; t < 3 * ng; t += blockDim.x) {
				const int j = t / ng, g = t % ng;
				V[j * ng + g] = X[ll * ng + g] * Jm[(j * 3 + mm) * ng + g] - X[mm * ng + g] * Jm[(j * 3 + ll) * ng + g];
			}
			__syncthreads();
			for (int jj = 0; jj < 3; ++jj)
				geo_pass(V, dV + jj * 3 * ng, eg, jj, G.Dgg, qg, 3);
			for (int g = threadIdx.x; g < ng; g += blockDim.x) {
				// curl of V: (d2 V3 - d3 V2, d3 V1 - d1 V3, d1 V2 - d2 V1), dV[(jj 3 + c)] = d_jj V_c
				const double c0 = dV[(1 * 3 + 2) * ng + g] - dV[(2 * 3 + 1) * ng + g];
				const double c1 = dV[(2 * 3 + 0) * ng + g] - dV[(0 * 3 + 2) * ng + g];
				const double c2 = dV[(0 * 3 + 1) * ng + g] - dV[(1 * 3 + 0) * ng + g];
				mvm[(i * 3 + 0) * ng + g] = -0.5 * c0;
				mvm[(i * 3 + 1) * ng + g] = -0.5 * c1;
				mvm[(i * 3 + 2) * ng + g] = -0.5 * c2;
			}
			__syncthreads();
		}
	}
	if (out.metrics_vm)
		for (int t = threadIdx.x; t < d * d * ng; t += blockDim.x)
			out.metrics_vm[(size_t)v * d * d * ng + t] = mvm[t];

	// metrics at vc: interpolate every component along each direction
	{
		int e[3] = {eg[0], eg[1], eg[2]};
		const double* src = mvm;
		double* bufs[2] = {t0, t1};
		for (int k = 0; k < d; ++k) {
			double* dst = (k == d - 1) ? mvc : bufs[k & 1];
			geo_pass(src, dst, e, k, G.Lgc, q, d * d);
			e[k] = q;
			src = dst;
		}
	}
	// Jacobian at vc: derivative along j, interpolation along the others
	for (int j = 0; j < d; ++j) {
		int e[3] = {eg[0], eg[1], eg[2]};
		const double* src = X;
		double* bufs[2] = {t0, t1};
		for (int k = 0; k < d; ++k) {
			double* dst = (k == d - 1) ? Jc + j * d * nc : bufs[k & 1];
			geo_pass(src, dst, e, k, k == j ? G.Dgc : G.Lgc, q, d);
			e[k] = q;
			src = dst;
		}
	}
	for (int c = threadIdx.x; c < nc; c += blockDim.x) {
		double J;
		auto jac = [&](int i, int j) { return Jc[(j * d + i) * nc + c]; };   // dx_i/dr_j
		if (d == 2) {
			J = jac(0, 0) * jac(1, 1) - jac(0, 1) * jac(1, 0);
		} else {
			J = jac(0, 0) * (jac(1, 1) * jac(2, 2) - jac(1, 2) * jac(2, 1))
			  - jac(0, 1) * (jac(1, 0) * jac(2, 2) - jac(1, 2) * jac(2, 0))
			  + jac(0, 2) * (jac(1, 0) * jac(2, 1) - jac(1, 1) * jac(2, 0));
		}
		if (!(J > 0.0))
			atomicOr(out.err, 1);
		int r = c;
		double w = 1.0;
		for (int k = 0; k < d; ++k) {
			w *= G.w[r % q];
			r /= q;
		}
		if (out.jacobian_det_vc)
			out.jacobian_det_vc[(size_t)v * nc + c] = J;
		if (out.inv_wJ)
			out.inv_wJ[(size_t)v * nc + c] = 1.0 / (w * J);
		for (int i = 0; i < d; ++i)
			for (int j = 0; j < d; ++j) {
				const double m = mvc[(i * d + j) * nc + c];
				if (out.metrics_vc)
					out.metrics_vc[(size_t)v * d * d * nc + c + (size_t)nc * (i + d * j)] = m;
				if (out.gmet)
					out.gmet[((size_t)v * d * d + j * d + i) * nc + c] = w * m;
			}
	}
}

// One thread per face cubature node: side 0's vm metric terms and coordinates at the node, the normal and the face
// Jacobian.
__global__ void __launch_bounds__(128) geo_face_kernel(const GeoOps G, int n_face, const int* __restrict__ face_vol,
                                                      const int* __restrict__ face_lf,
                                                      const double* __restrict__ geom_coef, GeoOut out)
{
	const int d = G.d, qg = G.qg, q = G.q;
	const int ng = (d == 2 ? qg * qg : qg * qg * qg), nf = (d == 2 ? q : q * q);
	const int gid = blockIdx.x * blockDim.x + threadIdx.x;
	if (gid >= n_face * nf)
		return;
	const int f = gid / nf, t = gid % nf;
	const int v = face_vol[2 * f], lf = face_lf[2 * f];
	const int nd = lf >> 1, side = lf & 1;
	// face node t -> cubature index along each tangential direction (increasing direction, first fastest)
	int tc[3] = {0, 0, 0};
	{
		int r = t;
		for (int k = 0; k < d; ++k)
			if (k != nd) {
				tc[k] = r % q;
				r /= q;
			}
	}
	const double* mv = out.metrics_vm + (size_t)v * d * d * ng;
	const double* xg = geom_coef + (size_t)v * ng * d;
	double m[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, x[3] = {0, 0, 0};
	for (int g = 0; g < ng; ++g) {
		int r = g;
		double wgt = 1.0;
		for (int k = 0; k < d; ++k) {
			const int a = r % qg;
			r /= qg;
			wgt *= (k == nd ? G.Lgb[side][a] : G.Lgc[tc[k]][a]);
		}
		if (wgt == 0.0)
			continue;
		for (int c = 0; c < d * d; ++c)
			m[c] += wgt * mv[c * ng + g];
		for (int k = 0; k < d; ++k)
			x[k] += wgt * xg[k * ng + g];
	}
	double n[3] = {0, 0, 0}, len2 = 0.0;
	for (int i = 0; i < d; ++i) {
		for (int j = 0; j < d; ++j)
			n[i] += m[i * d + j] * G.nref[lf][j];
		len2 += n[i] * n[i];
	}
	const double len = sqrt(len2);
	for (int k = 0; k < d; ++k) {
		const double nk = n[k] / len;
		if (out.normals_fc)
			out.normals_fc[((size_t)f * nf + t) * d + k] = nk;
		if (out.fgeo)
			out.fgeo[((size_t)f * (d + 1) + k) * nf + t] = nk;
		if (out.xyz_fc)
			out.xyz_fc[((size_t)f * nf + t) * d + k] = x[k];
	}
	if (out.jacobian_det_fc)
		out.jacobian_det_fc[(size_t)f * nf + t] = len;
	if (out.fgeo) {
		int r = t;
		double w = 1.0;
		for (int k = 0; k < d - 1; ++k) {
			w *= G.w[r % q];
			r /= q;
		}
		out.fgeo[((size_t)f * (d + 1) + d) * nf + t] = w * len;
	}
}


// ---- blended geometry of curved QUAD volumes -------------------------------------------------------------------
// compute_geom_coef_blended_T (geometry_T.c:845-855) with constructor_xyz_blended_ce (geometry_blended_T.c:286-315)
// for tensor-product volumes (Gordon-Hall blending, compute_p_base_min :320-335) on the reference's blended domains,
// the n-cylinder meshes with the radial projection (constructor_xyz_surface_cylinder_radial_proj_T,
// geometry_surface_T.c:103-147). Per volume, starting from the straight (bilinear) map at the GLL geometry nodes of
// order p_g, each curved local face b in turn:
//   surface   the face's straight nodes (its two vertices interpolated at the face's GLL nodes) projected radially
//             onto the circle through its first vertex: r (cos theta, sin theta), theta = atan2(y, x);
//   diff      surface - the current coordinates at the face's nodes, extended along the volume's lines normal to
//             the face (vv0_fgc_vgc: the face node with the same tangential coordinate);
//   blend     the sum of the face's two vertex basis functions at the node (constructor_blend_values :337-351),
//             i.e. the linear hat that is 1 on face b and 0 on the opposite face;
//   xyz += blend * diff.
// The reference has no 3D TP blending (its edge step stops with EXIT_ADD_SUPPORT), so this is 2D only.
struct BlendArgs {
	int n_vol;
	int qg;                  // geometry nodes per direction, p_g + 1
	double x[kQMax];         // GLL nodes of order p_g on [-1, 1]
	const double* xyz_ve;    // [v][c][vertex]: the straight volume's vertices (the p_g = 1 geom_coef layout)
	const int* face_curved;  // [v][lf]: 1 for a curved boundary face (Face::bc > BC_CURVED_START)
	double* geom_coef;       // [v][c][node]
};

__global__ void __launch_bounds__(128) blend_quad_kernel(const BlendArgs A)
{
	const int v = blockIdx.x * blockDim.x + threadIdx.x;
	if (v >= A.n_vol)
		return;
	const int q = A.qg, n_g = q * q;
	// local faces of a QUAD and their vertices (element.c f_ve, TP vertex order v = a + 2 b)
	const int f_ve[4][2] = {{0, 2}, {1, 3}, {0, 1}, {2, 3}};
	double ve[2][4];
	for (int c = 0; c < 2; ++c)
		for (int k = 0; k < 4; ++k)
			ve[c][k] = A.xyz_ve[((size_t)v * 2 + c) * 4 + k];
	double X[2][kQMax * kQMax];
	for (int j = 0; j < q; ++j)
		for (int i = 0; i < q; ++i) {
			double phi[4];
			for (int k = 0; k < 4; ++k)
				phi[k] = 0.5 * ((k & 1) ? 1.0 + A.x[i] : 1.0 - A.x[i]) * 0.5 * ((k & 2) ? 1.0 + A.x[j] : 1.0 - A.x[j]);
			for (int c = 0; c < 2; ++c) {
				double s = 0.0;
				for (int k = 0; k < 4; ++k)
					s += phi[k] * ve[c][k];
				X[c][i + q * j] = s;
			}
		}
	for (int b = 0; b < 4; ++b) {
		if (!A.face_curved[(size_t)v * 4 + b])
			continue;
		const int va = f_ve[b][0], vb = f_ve[b][1];
		const double r = sqrt(ve[0][va] * ve[0][va] + ve[1][va] * ve[1][va]);
		double diff[2][kQMax];
		for (int k = 0; k < q; ++k) {
			const double la = 0.5 * (1.0 - A.x[k]), lb = 0.5 * (1.0 + A.x[k]);
			const double sx = la * ve[0][va] + lb * ve[0][vb], sy = la * ve[1][va] + lb * ve[1][vb];
			const double th = atan2(sy, sx);
			const int n = (b < 2) ? (b == 0 ? 0 : q - 1) + q * k : k + q * (b == 2 ? 0 : q - 1);
			diff[0][k] = r * cos(th) - X[0][n];
			diff[1][k] = r * sin(th) - X[1][n];
		}
		for (int j = 0; j < q; ++j)
			for (int i = 0; i < q; ++i) {
				double blend = 0.0;
				for (int e = 0; e < 2; ++e) {
					const int k = f_ve[b][e];
					blend += 0.5 * ((k & 1) ? 1.0 + A.x[i] : 1.0 - A.x[i]) * 0.5 * ((k & 2) ? 1.0 + A.x[j] : 1.0 - A.x[j]);
				}
				const int t = (b < 2) ? j : i;
				X[0][i + q * j] += blend * diff[0][t];
				X[1][i + q * j] += blend * diff[1][t];
			}
	}
	for (int c = 0; c < 2; ++c)
		for (int n = 0; n < n_g; ++n)
			A.geom_coef[((size_t)v * 2 + c) * n_g + n] = X[c][n];
}

}  // namespace dgpu
