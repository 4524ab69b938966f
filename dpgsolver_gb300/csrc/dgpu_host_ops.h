// Host-side derivation of the GL-space 1D operators from a caller's TP operator set (shared by the contexts).
#pragma once

#include <math.h>
#include <string.h>

#include "../../include/dgpu.h"
#include "dgpu_tp.cuh"

namespace dgpu {

// Gauss-Jordan inverse with partial pivoting of a small row-major matrix.
inline bool host_invert_small(int n, const double* A, double* Ainv)
{
	double a[kQMax * kQMax];
	for (int i = 0; i < n * n; ++i)
		a[i] = A[i];
	for (int i = 0; i < n; ++i)
		for (int j = 0; j < n; ++j)
			Ainv[i * n + j] = (i == j) ? 1.0 : 0.0;
	for (int col = 0; col < n; ++col) {
		int piv = col;
		for (int r = col + 1; r < n; ++r)
			if (fabs(a[r * n + col]) > fabs(a[piv * n + col]))
				piv = r;
		if (!(fabs(a[piv * n + col]) > 1e-300))
			return false;
		if (piv != col)
			for (int j = 0; j < n; ++j) {
				double t = a[col * n + j]; a[col * n + j] = a[piv * n + j]; a[piv * n + j] = t;
				t = Ainv[col * n + j]; Ainv[col * n + j] = Ainv[piv * n + j]; Ainv[piv * n + j] = t;
			}
		const double inv = 1.0 / a[col * n + col];
		for (int j = 0; j < n; ++j) {
			a[col * n + j] *= inv;
			Ainv[col * n + j] *= inv;
		}
		for (int r = 0; r < n; ++r) {
			if (r == col)
				continue;
			const double f = a[r * n + col];
			for (int j = 0; j < n; ++j) {
				a[r * n + j] -= f * a[col * n + j];
				Ainv[r * n + j] -= f * Ainv[col * n + j];
			}
		}
	}
	return true;
}

// Gauss-Jordan inverse with partial pivoting of a row-major n x n matrix of any size.
inline bool host_invert(int n, const double* A, double* Ainv)
{
	double* a = new double[(size_t)n * n];
	for (size_t i = 0; i < (size_t)n * n; ++i)
		a[i] = A[i];
	for (int i = 0; i < n; ++i)
		for (int j = 0; j < n; ++j)
			Ainv[(size_t)i * n + j] = (i == j) ? 1.0 : 0.0;
	bool ok = true;
	for (int col = 0; col < n && ok; ++col) {
		int piv = col;
		for (int r = col + 1; r < n; ++r)
			if (fabs(a[(size_t)r * n + col]) > fabs(a[(size_t)piv * n + col]))
				piv = r;
		if (!(fabs(a[(size_t)piv * n + col]) > 1e-300)) {
			ok = false;
			break;
		}
		if (piv != col)
			for (int j = 0; j < n; ++j) {
				double t = a[(size_t)col * n + j]; a[(size_t)col * n + j] = a[(size_t)piv * n + j]; a[(size_t)piv * n + j] = t;
				t = Ainv[(size_t)col * n + j]; Ainv[(size_t)col * n + j] = Ainv[(size_t)piv * n + j]; Ainv[(size_t)piv * n + j] = t;
			}
		const double inv = 1.0 / a[(size_t)col * n + col];
		for (int j = 0; j < n; ++j) {
			a[(size_t)col * n + j] *= inv;
			Ainv[(size_t)col * n + j] *= inv;
		}
		for (int r = 0; r < n; ++r) {
			if (r == col)
				continue;
			const double f = a[(size_t)r * n + col];
			for (int j = 0; j < n; ++j) {
				a[(size_t)r * n + j] -= f * a[(size_t)col * n + j];
				Ainv[(size_t)r * n + j] -= f * Ainv[(size_t)col * n + j];
			}
		}
	}
	delete[] a;
	return ok;
}

// Legendre polynomial P_n and its derivative at x (three-term recurrence).
inline void legendre(int n, double x, double* p, double* dp)
{
	double p0 = 1.0, p1 = x;
	if (n == 0) {
		*p = 1.0;
		*dp = 0.0;
		return;
	}
	for (int k = 2; k <= n; ++k) {
		const double pk = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
		p0 = p1;
		p1 = pk;
	}
	*p = p1;
	*dp = n * (x * p1 - p0) / (x * x - 1.0);
}

// Gauss-Legendre nodes (ascending) by Newton iteration from Chebyshev guesses.
inline void gauss_legendre_nodes(int q, double* x)
{
	for (int i = 0; i < q; ++i) {
		double z = -cos(M_PI * (i + 0.75) / (q + 0.5));
		for (int it = 0; it < 100; ++it) {
			double p, dp;
			legendre(q, z, &p, &dp);
			const double dz = p / dp;
			z -= dz;
			if (fabs(dz) < 1e-16)
				break;
		}
		x[i] = z;
	}
	for (int i = 0; i < q / 2; ++i) {   // exact symmetry
		const double s = 0.5 * (x[q - 1 - i] - x[i]);
		x[i] = -s;
		x[q - 1 - i] = s;
	}
	if (q % 2)
		x[q / 2] = 0.0;
}

// Value of the i-th Lagrange polynomial on nodes xn (q of them) at x.
inline double lagrange_value(const double* xn, int q, int i, double x)
{
	double num = 1.0, den = 1.0;
	for (int k = 0; k < q; ++k)
		if (k != i) {
			num *= x - xn[k];
			den *= xn[i] - xn[k];
		}
	return num / den;
}

// Derivative of the i-th Lagrange polynomial on nodes xn (q of them) at x.
inline double lagrange_derivative(const double* xn, int q, int i, double x)
{
	double den = 1.0, s = 0.0;
	for (int k = 0; k < q; ++k)
		if (k != i)
			den *= xn[i] - xn[k];
	for (int j = 0; j < q; ++j) {
		if (j == i)
			continue;
		double t = 1.0;
		for (int k = 0; k < q; ++k)
			if (k != i && k != j)
				t *= x - xn[k];
		s += t;
	}
	return s / den;
}

// Gauss-Lobatto-Legendre nodes (ascending, q >= 2): the end points and the roots of P_{q-1}', by Newton iteration on
// (1 - x^2) P_n'(x), whose derivative is -n (n + 1) P_n(x), from the Chebyshev-Gauss-Lobatto points.
inline void gauss_lobatto_nodes(int q, double* x)
{
	const int n = q - 1;
	for (int i = 0; i < q; ++i)
		x[i] = -cos(M_PI * i / n);
	for (int i = 1; i < n; ++i) {
		double z = x[i];
		for (int it = 0; it < 100; ++it) {
			double p, dp;
			legendre(n, z, &p, &dp);
			const double dz = ((1.0 - z * z) * dp) / (-n * (n + 1) * p);
			z -= dz;
			if (fabs(dz) < 1e-17)
				break;
		}
		x[i] = z;
	}
	x[0] = -1.0;
	x[n] = 1.0;
	for (int i = 0; i < q / 2; ++i) {   // exact symmetry
		const double s = 0.5 * (x[q - 1 - i] - x[i]);
		x[i] = -s;
		x[q - 1 - i] = s;
	}
	if (q % 2)
		x[q / 2] = 0.0;
}

// B, B^-1, Dgl, l_gl(+-1), Bezier maps, positivity constants, transposes: see TPOps.
inline bool derive_tp_ops(const dgpu_tp_operators* ops, int d, TPOps* out)
{
	const int q = ops->p + 1;
	memset(out, 0, sizeof *out);
	double Bm[kQMax * kQMax], Bi[kQMax * kQMax];
	for (int i = 0; i < q * q; ++i)
		Bm[i] = ops->cv0_vs_vc[i];
	if (!host_invert_small(q, Bm, Bi))
		return false;
	for (int a = 0; a < q; ++a)
		for (int m = 0; m < q; ++m) {
			out->B[a][m] = Bm[a * q + m];
			out->Binv[a][m] = Bi[a * q + m];
			double s = 0.0;
			for (int k = 0; k < q; ++k)
				s += ops->cv1_vs_vc[a * q + k] * Bi[k * q + m];
			out->Dgl[a][m] = s;
			if (ops->ccSB0_vs_vs) out->SB[a][m] = ops->ccSB0_vs_vs[a * q + m];
			if (ops->ccBS0_vs_vs) out->BS[a][m] = ops->ccBS0_vs_vs[a * q + m];
		}
	for (int s = 0; s < 2; ++s)
		for (int m = 0; m < q; ++m) {
			double acc = 0.0;
			for (int k = 0; k < q; ++k)
				acc += ops->cv0_vs_fc[s * q + k] * Bi[k * q + m];
			out->lb[s][m] = acc;
		}
	double L = 0.0;
	for (int a = 0; a < q; ++a) {
		double row = 0.0;
		for (int m = 0; m < q; ++m) {
			double sbg = 0.0, bsg = 0.0;
			for (int k = 0; k < q; ++k) {
				sbg += out->SB[a][k] * Bi[k * q + m];
				bsg += Bm[a * q + k] * out->BS[k][m];
			}
			out->SBg[a][m] = sbg;
			out->BSg[a][m] = bsg;
			out->SBf[a][m] = (float)sbg;
			row += fabs(sbg);
		}
		L = fmax(L, row);
	}
	out->pos_err = (float)(2.0 * (d * (q + 1) + 1) * ldexp(1.0, -24) * pow(L, d));
	for (int a = 0; a < q; ++a)
		for (int m = 0; m < q; ++m) {
			out->BT[a][m] = out->B[m][a];
			out->BinvT[a][m] = out->Binv[m][a];
		}
	return true;
}

}  // namespace dgpu
