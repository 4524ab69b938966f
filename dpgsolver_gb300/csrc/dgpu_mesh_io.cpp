// Mesh reader and connectivity (declared in include/dgpu_mesh.h): the reference's mesh preprocessing
// (src/simulation/mesh/ and constructor_Faces) on the host, in C++.
//
// The results are the reference's (the same v_to_v, v_to_lf, v_to_lf_wp, vertex flags and face list); the way to
// them is sort-based: every local face of every volume gets a key (its sorted vertex numbers), periodic slave faces
// take the key of their master face, and equal keys after one sort are the interior faces.
#include <algorithm>
#include <array>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <string>
#include <vector>

#include "../../include/dgpu_mesh.h"

struct dgpu_gmsh {
	int d = 0;
	std::vector<double> nodes;                 // n_nodes x d
	std::vector<int> elem_types, elem_tags;    // n_elements, n_elements x 2
	std::vector<int> node_ptr, node_nums;      // vertices per element (reference order, 0-based)
	std::vector<int> periodic_corr;            // n_periodic x 2
	int elem_per_dim[4] = {0, 0, 0, 0};
	int ind_v = 0, n_v = 0;                    // first volume element, number of volumes
	bool has_periodic = false;
	std::vector<int> lf_ptr, v_to_v, v_to_lf, v_to_lf_wp;
	std::vector<int> ve_curved, ve_boundary, ve_bc_ptr, ve_bc;
	int n_faces = 0;
	std::vector<int> face_vol, face_lf, face_bc, face_wp, face_match, face_ord;
};

namespace {

thread_local std::string g_mesh_error;

constexpr int kBcStepSC = 10000;   // definitions_bc.h:33
constexpr double kEps = 1.0e-15;   // definitions_tol.h:23

// gmsh element codes (the reference's element type indices)
enum { kLine = 1, kTri = 2, kQuad = 3, kTet = 4, kHex = 5, kWedge = 6, kPyr = 7, kPoint = 15 };

int type_dim(int t)
{
	switch (t) {
	case kPoint: return 0;
	case kLine: return 1;
	case kTri: case kQuad: return 2;
	case kTet: case kHex: case kWedge: case kPyr: return 3;
	default: return -1;
	}
}

int type_n_nodes(int t)   // get_n_nodes, mesh_readers.c:165-188
{
	switch (t) {
	case kPoint: return 1;
	case kLine: return 2;
	case kTri: return 3;
	case kQuad: return 4;
	case kTet: return 4;
	case kHex: return 8;
	case kWedge: return 6;
	case kPyr: return 5;
	default: return -1;
	}
}

// Local faces of each element type and the vertices of each (element.c:440-530; the reference's local face order
// and vertex order within a face, which the face list, v_to_lf and the vertex correspondences all refer to).
struct LocalFaces {
	int n_f;
	int n_ve[6];
	int ve[6][4];
};

const LocalFaces* local_faces(int t)
{
	static const LocalFaces line = {2, {1, 1}, {{0}, {1}}};
	static const LocalFaces tri = {3, {2, 2, 2}, {{1, 2}, {0, 2}, {0, 1}}};
	static const LocalFaces quad = {4, {2, 2, 2, 2}, {{0, 2}, {1, 3}, {0, 1}, {2, 3}}};
	static const LocalFaces tet = {4, {3, 3, 3, 3}, {{2, 3, 1}, {2, 3, 0}, {0, 1, 3}, {0, 1, 2}}};
	static const LocalFaces hex = {6, {4, 4, 4, 4, 4, 4},
	                               {{0, 2, 4, 6}, {1, 3, 5, 7}, {0, 1, 4, 5}, {2, 3, 6, 7}, {0, 1, 2, 3}, {4, 5, 6, 7}}};
	static const LocalFaces wedge = {5, {4, 4, 4, 3, 3},
	                                 {{1, 2, 4, 5}, {0, 2, 3, 5}, {0, 1, 3, 4}, {0, 1, 2}, {3, 4, 5}}};
	static const LocalFaces pyr = {5, {3, 3, 3, 3, 4}, {{0, 2, 4}, {1, 3, 4}, {0, 1, 4}, {2, 3, 4}, {0, 1, 2, 3}}};
	switch (t) {
	case kLine: return &line;
	case kTri: return &tri;
	case kQuad: return &quad;
	case kTet: return &tet;
	case kHex: return &hex;
	case kWedge: return &wedge;
	case kPyr: return &pyr;
	default: return nullptr;
	}
}

// gmsh's counter-clockwise quadrilateral vertex order -> the reference's tensor-product order
// (reorder_nodes_gmsh, mesh_readers.c:132-163).
void reorder_gmsh(int t, int* v)
{
	static const int quad[4] = {0, 1, 3, 2}, hex[8] = {0, 1, 3, 2, 4, 5, 7, 6}, pyr[5] = {0, 1, 3, 2, 4};
	const int* ord = (t == kQuad ? quad : t == kHex ? hex : t == kPyr ? pyr : nullptr);
	if (!ord)
		return;
	int tmp[8];
	const int n = type_n_nodes(t);
	for (int i = 0; i < n; ++i)
		tmp[i] = v[ord[i]];
	std::memcpy(v, tmp, n * sizeof(int));
}

// Periodic codes (definitions_mesh.h:37-45): 51/52 x, 53/54 y, 55/56 z (left = master, right = slave), 61/62 x with
// y reflected.
int periodic_base(int bc)
{
	const int b = bc % kBcStepSC;
	return ((b >= 51 && b <= 56) || b == 61 || b == 62) ? b : 0;
}
bool periodic_master(int b) { return b == 51 || b == 53 || b == 55 || b == 61; }
int periodic_dir(int b) { return (b == 51 || b == 52 || b == 61 || b == 62) ? 0 : (b <= 54 ? 1 : 2); }

// The non-periodic boundary codes the reference accepts (check_pfe_boundary, mesh_connectivity.c:130-170).
bool known_boundary(int bc)
{
	const int b = bc % kBcStepSC;
	return (b >= 1 && b <= 3) || (b >= 11 && b <= 13) || (b >= 41 && b <= 46) || b == 21 || b == 22 || b == 31 ||
	       b == 32 || (b >= 101 && b <= 106) || (b >= 111 && b <= 113);
}

dgpu_status fail(dgpu_status st, const std::string& msg)
{
	g_mesh_error = msg;
	return st;
}

// Whitespace-separated numbers of one line.
bool parse_doubles(const std::string& line, std::vector<double>* out)
{
	out->clear();
	const char* p = line.c_str();
	char* end = nullptr;
	for (;;) {
		while (*p == ' ' || *p == '\t' || *p == '\r')
			++p;
		if (!*p)
			return true;
		const double x = std::strtod(p, &end);
		if (end == p)
			return false;
		out->push_back(x);
		p = end;
	}
}

bool parse_ints(const std::string& line, std::vector<long long>* out)
{
	out->clear();
	const char* p = line.c_str();
	char* end = nullptr;
	for (;;) {
		while (*p == ' ' || *p == '\t' || *p == '\r')
			++p;
		if (!*p)
			return true;
		const long long x = std::strtoll(p, &end, 10);
		if (end == p)
			return false;
		out->push_back(x);
		p = end;
	}
}

// ---- reading: mesh_reader_gmsh (mesh_readers.c:215-235, 298-445) ----------------------------------------------------
dgpu_status read_gmsh(const char* path, int d, dgpu_gmsh* m)
{
	std::ifstream in(path);
	if (!in)
		return fail(DGPU_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path);
	std::string line;
	std::vector<double> dv;
	std::vector<long long> iv;
	bool have_nodes = false, have_elements = false;
	auto next = [&](std::string* l) { return (bool)std::getline(in, *l); };
	while (next(&line)) {
		if (line.find("$Nodes") != std::string::npos) {
			if (!next(&line) || !parse_ints(line, &iv) || iv.size() != 1 || iv[0] < 0)
				return fail(DGPU_ERR_INVALID_ARGUMENT, "bad $Nodes count");
			const long long n = iv[0];
			m->nodes.assign((size_t)n * d, 0.0);
			for (long long i = 0; i < n; ++i) {
				if (!next(&line) || !parse_doubles(line, &dv) || (int)dv.size() < 1 + d)
					return fail(DGPU_ERR_INVALID_ARGUMENT, "bad node line " + std::to_string(i + 1));
				for (int k = 0; k < d; ++k)
					m->nodes[(size_t)i * d + k] = dv[1 + k];   // the first value is the node number
			}
			have_nodes = true;
		} else if (line.find("$Elements") != std::string::npos) {
			if (!next(&line) || !parse_ints(line, &iv) || iv.size() != 1 || iv[0] < 0)
				return fail(DGPU_ERR_INVALID_ARGUMENT, "bad $Elements count");
			const long long n = iv[0];
			m->node_ptr.assign(1, 0);
			for (long long i = 0; i < n; ++i) {
				if (!next(&line) || !parse_ints(line, &iv) || iv.size() < 3)
					return fail(DGPU_ERR_INVALID_ARGUMENT, "bad element line " + std::to_string(i + 1));
				const int t = (int)iv[1], n_tags = (int)iv[2], nn = type_n_nodes(t);
				if (nn < 0)
					return fail(DGPU_ERR_UNSUPPORTED, "element type " + std::to_string(t) + " is not read");
				if (n_tags != 2)
					return fail(DGPU_ERR_UNSUPPORTED, "elements must carry 2 tags (physical, entity)");
				if ((int)iv.size() != 3 + n_tags + nn)
					return fail(DGPU_ERR_INVALID_ARGUMENT, "bad element line " + std::to_string(i + 1));
				m->elem_types.push_back(t);
				m->elem_tags.push_back((int)iv[3]);
				m->elem_tags.push_back((int)iv[4]);
				int v[8];
				for (int k = 0; k < nn; ++k)
					v[k] = (int)iv[5 + k] - 1;
				reorder_gmsh(t, v);
				m->node_nums.insert(m->node_nums.end(), v, v + nn);
				m->node_ptr.push_back((int)m->node_nums.size());
			}
			have_elements = true;
		} else if (line.rfind("$Periodic", 0) == 0) {
			if (!next(&line) || !parse_ints(line, &iv) || iv.size() != 1)
				return fail(DGPU_ERR_INVALID_ARGUMENT, "bad $Periodic count");
			const long long n_all = iv[0];
			for (long long e = 0; e < n_all; ++e) {
				if (!next(&line) || !parse_ints(line, &iv) || iv.size() < 3)
					return fail(DGPU_ERR_INVALID_ARGUMENT, "bad periodic entity line");
				const bool keep = iv[0] >= d - 1;   // lower-dimensional entities are skipped
				if (keep) {
					m->periodic_corr.push_back((int)iv[1]);
					m->periodic_corr.push_back((int)iv[2]);
				}
				std::vector<long long> cnt;
				if (!next(&line) || !parse_ints(line, &cnt) || cnt.size() != 1 || cnt[0] < 0)
					return fail(DGPU_ERR_INVALID_ARGUMENT, "bad periodic node count");
				for (long long k = 0; k < cnt[0]; ++k)
					if (!next(&line))
						return fail(DGPU_ERR_INVALID_ARGUMENT, "truncated $Periodic");
			}
			if (m->periodic_corr.empty())
				return fail(DGPU_ERR_UNSUPPORTED, "$Periodic without entities of dimension d-1");
		}
	}
	if (!have_nodes || !have_elements)
		return fail(DGPU_ERR_INVALID_ARGUMENT, "no $Nodes or $Elements section");
	const int n_nodes = (int)(m->nodes.size() / d);
	for (int v : m->node_nums)
		if (v < 0 || v >= n_nodes)
			return fail(DGPU_ERR_INVALID_ARGUMENT, "element vertex out of the node list");
	return DGPU_OK;
}

}  // namespace

namespace {

using Key = std::array<int, 4>;   // sorted vertex numbers of a face, INT_MAX padded

Key face_key(const int* v, int n)
{
	Key k = {INT_MAX, INT_MAX, INT_MAX, INT_MAX};
	for (int i = 0; i < n; ++i) {   // insertion sort of at most 4 values
		int j = i;
		while (j > 0 && k[j - 1] > v[i]) {
			k[j] = k[j - 1];
			--j;
		}
		k[j] = v[i];
	}
	return k;
}

// ---- connectivity: constructor_Mesh_Connectivity (mesh_connectivity.c:85-113) ---------------------------------------
dgpu_status build_connectivity(dgpu_gmsh* m)
{
	const int d = m->d, n_el = (int)m->elem_types.size();
	for (int e = 0; e < n_el; ++e) {
		const int dim = type_dim(m->elem_types[e]);
		if (dim > d)
			return fail(DGPU_ERR_INVALID_ARGUMENT, "element of dimension above d");
		m->elem_per_dim[dim]++;
	}
	m->ind_v = 0;
	for (int k = 0; k < d; ++k)
		m->ind_v += m->elem_per_dim[k];
	m->n_v = m->elem_per_dim[d];
	if (m->n_v < 1)
		return fail(DGPU_ERR_INVALID_ARGUMENT, "no volumes of dimension d");
	for (int e = 0; e < n_el; ++e)   // the reference expects the elements sorted by dimension (gmsh writes them so)
		if ((e < m->ind_v) != (type_dim(m->elem_types[e]) < d))
			return fail(DGPU_ERR_INVALID_ARGUMENT, "elements are not sorted by dimension");
	const int ind_pfe = m->ind_v - m->elem_per_dim[d - 1];   // physical face elements: dimension d-1

	// volume faces and their keys (f_ve), before and after the periodic substitution
	m->lf_ptr.assign(1, 0);
	std::vector<Key> key, key0;
	std::vector<int> fv_v, fv_lf;
	for (int v = 0; v < m->n_v; ++v) {
		const int e = m->ind_v + v;
		const LocalFaces* L = local_faces(m->elem_types[e]);
		const int* vn = &m->node_nums[m->node_ptr[e]];
		for (int lf = 0; lf < L->n_f; ++lf) {
			int fv[4];
			for (int i = 0; i < L->n_ve[lf]; ++i)
				fv[i] = vn[L->ve[lf][i]];
			key.push_back(face_key(fv, L->n_ve[lf]));
			fv_v.push_back(v);
			fv_lf.push_back(lf);
		}
		m->lf_ptr.push_back((int)key.size());
	}
	key0 = key;
	const int n_f = (int)key.size();
	auto pfe_key = [&](int e) { return face_key(&m->node_nums[m->node_ptr[e]], m->node_ptr[e + 1] - m->node_ptr[e]); };

	// periodic: slave faces take the key of their master face (correct_f_ve_for_periodic, mesh_periodic.c:102-130);
	// masters and slaves are paired in the order of (direction, centroid in the other directions), slave
	// centroids reflected where the code says so
	m->has_periodic = !m->periodic_corr.empty();
	if (m->has_periodic) {
		struct PF {
			int dir;
			double c[2];
			Key k;
		};
		std::vector<PF> ms[2];
		for (int e = ind_pfe; e < m->ind_v; ++e) {
			const int bc = m->elem_tags[2 * e], b = periodic_base(bc);
			if (!b) {
				if (!known_boundary(bc))
					return fail(DGPU_ERR_UNSUPPORTED, "boundary code " + std::to_string(bc) + " is not known");
				continue;
			}
			const int s = periodic_master(b) ? 0 : 1, dir = periodic_dir(b);
			PF pf;
			pf.dir = dir;
			pf.c[0] = pf.c[1] = 0.0;
			const int n = m->node_ptr[e + 1] - m->node_ptr[e];
			for (int i = 0; i < n; ++i) {
				const double* x = &m->nodes[(size_t)m->node_nums[m->node_ptr[e] + i] * d];
				for (int k = 0, j = 0; k < d; ++k) {
					if (k == dir)
						continue;
					const double scale = (s == 1 && (b == 61 || b == 62) && k == 1) ? -1.0 : 1.0;
					pf.c[j++] += scale * x[k];
				}
			}
			pf.c[0] /= n;
			pf.c[1] /= n;
			pf.k = pfe_key(e);
			ms[s].push_back(pf);
		}
		if (ms[0].size() != ms[1].size())
			return fail(DGPU_ERR_INVALID_ARGUMENT, "periodic master and slave face counts differ");
		for (auto& list : ms)
			std::sort(list.begin(), list.end(), [](const PF& a, const PF& b) {
				if (a.dir != b.dir)
					return a.dir < b.dir;
				if (a.c[0] != b.c[0])
					return a.c[0] < b.c[0];
				return a.c[1] < b.c[1];
			});
		std::map<Key, std::vector<int>> where;
		for (int f = 0; f < n_f; ++f)
			where[key0[f]].push_back(f);
		for (size_t i = 0; i < ms[1].size(); ++i) {
			auto it = where.find(ms[1][i].k);
			if (it == where.end() || it->second.size() != 1)
				return fail(DGPU_ERR_INVALID_ARGUMENT, "a periodic slave face is not the face of one volume");
			key[it->second[0]] = ms[0][i].k;
		}
	}

	// interior faces: equal keys after one sort (compute_v_to__v_lf, mesh_connectivity.c:303-361)
	m->v_to_v.assign(n_f, -1);
	m->v_to_lf.assign(n_f, -1);
	m->v_to_lf_wp.assign(n_f, -1);
	std::vector<int> ord(n_f);
	for (int f = 0; f < n_f; ++f)
		ord[f] = f;
	std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return key[a] < key[b]; });
	for (int i = 0; i < n_f; ++i) {
		if (i + 1 < n_f && key[ord[i]] == key[ord[i + 1]]) {
			if (i + 2 < n_f && key[ord[i]] == key[ord[i + 2]])
				return fail(DGPU_ERR_INVALID_ARGUMENT, "a face is shared by more than two volumes");
			const int a = ord[i], b = ord[i + 1];
			m->v_to_v[a] = fv_v[b];
			m->v_to_lf[a] = fv_lf[b];
			m->v_to_v[b] = fv_v[a];
			m->v_to_lf[b] = fv_lf[a];
			if (m->has_periodic && key0[a] == key0[b]) {
				m->v_to_lf_wp[a] = m->v_to_lf[a];
				m->v_to_lf_wp[b] = m->v_to_lf[b];
			}
			++i;
		}
	}

	// boundary faces: the BC code of the physical face element with the same vertices (add_bc_info,
	// mesh_connectivity.c:372-420), first without, then (v_to_lf_wp) with the periodic elements
	for (int pass = 0; pass < (m->has_periodic ? 2 : 1); ++pass) {
		const bool with_periodic = pass == 1;
		std::map<Key, int> bcs;
		for (int e = ind_pfe; e < m->ind_v; ++e) {
			const int bc = m->elem_tags[2 * e], b = periodic_base(bc);
			if (!b && !known_boundary(bc))
				return fail(DGPU_ERR_UNSUPPORTED, "boundary code " + std::to_string(bc) + " is not known");
			if (!b || with_periodic)
				bcs[pfe_key(e)] = bc;
		}
		std::vector<int>& dst = with_periodic ? m->v_to_lf_wp : m->v_to_lf;
		const std::vector<Key>& k = with_periodic ? key0 : key;
		for (int f = 0; f < n_f; ++f) {
			if (dst[f] != -1)
				continue;
			auto it = bcs.find(k[f]);
			if (it == bcs.end())
				return fail(DGPU_ERR_INVALID_ARGUMENT, "volume " + std::to_string(fv_v[f]) + " local face " +
				                                           std::to_string(fv_lf[f]) +
				                                           " has no neighbour and no boundary element");
			dst[f] = it->second;
		}
	}
	return DGPU_OK;
}

// ---- vertices on boundaries: set_up_mesh_vertices (mesh_vertices.c:95-132) -----------------------------------------
void build_vertices(dgpu_gmsh* m)
{
	const int n_nodes = (int)(m->nodes.size() / m->d);
	m->ve_curved.assign(n_nodes, 0);
	m->ve_boundary.assign(n_nodes, 0);
	std::vector<std::vector<int>> bc(n_nodes);
	for (int v = 0; v < m->n_v; ++v) {
		const int e = m->ind_v + v;
		const LocalFaces* L = local_faces(m->elem_types[e]);
		for (int lf = 0; lf < L->n_f; ++lf) {
			const int code = m->v_to_lf[m->lf_ptr[v] + lf];
			if (code < kBcStepSC)
				continue;
			for (int i = 0; i < L->n_ve[lf]; ++i) {
				const int ve = m->node_nums[m->node_ptr[e] + L->ve[lf][i]];
				m->ve_boundary[ve] = 1;
				bc[ve].push_back(code);
				if (code > 2 * kBcStepSC)
					m->ve_curved[ve] = 1;
			}
		}
	}
	m->ve_bc_ptr.assign(1, 0);
	m->ve_bc.clear();
	for (auto& b : bc) {
		std::sort(b.begin(), b.end());
		b.erase(std::unique(b.begin(), b.end()), b.end());
		m->ve_bc.insert(m->ve_bc.end(), b.begin(), b.end());
		m->ve_bc_ptr.push_back((int)m->ve_bc.size());
	}
}

// ---- the face list: constructor_Faces (face.c:86-154), vertex correspondence and ordering index (face.c:498-660) -----
dgpu_status build_faces(dgpu_gmsh* m)
{
	const int d = m->d;
	std::vector<int> assigned(m->v_to_v.size(), -1);
	m->n_faces = 0;
	for (int v = 0; v < m->n_v; ++v) {
		const int e = m->ind_v + v;
		const LocalFaces* L = local_faces(m->elem_types[e]);
		for (int lf = 0; lf < L->n_f; ++lf) {
			const int i0 = m->lf_ptr[v] + lf;
			if (assigned[i0] >= 0)
				continue;
			const int f = m->n_faces++;
			const int vn = m->v_to_v[i0], il = m->v_to_lf[i0];
			const int wp = m->has_periodic ? m->v_to_lf_wp[i0] : 0;
			assigned[i0] = f;
			m->face_vol.push_back(v);
			m->face_vol.push_back(vn);
			m->face_lf.push_back(lf);
			m->face_lf.push_back(vn >= 0 ? il : -1);
			m->face_bc.push_back(il > kBcStepSC ? il : -1);
			m->face_wp.push_back(wp);
			int match[4] = {-1, -1, -1, -1}, ord[2] = {-1, -1};
			if (vn >= 0) {
				assigned[m->lf_ptr[vn] + il] = f;
				// the face's vertex coordinates as each side lists them; a periodic face skips its periodic
				// direction, a reflected one compares y with the sign turned (constructor_Vertex_Correspondence)
				const int en = m->ind_v + vn;
				const LocalFaces* Ln = local_faces(m->elem_types[en]);
				const int n = L->n_ve[lf];
				if (Ln->n_ve[il] != n)
					return fail(DGPU_ERR_INVALID_ARGUMENT, "neighbouring faces with different vertex counts");
				const int b = (wp > kBcStepSC) ? periodic_base(wp) : 0;
				const int skip = (b && b != 61 && b != 62) ? periodic_dir(b) : -1, reflect = (b == 61 || b == 62) ? 1 : -1;
				auto xyz = [&](int el, const LocalFaces* T, int face, int i) {
					return &m->nodes[(size_t)m->node_nums[m->node_ptr[el] + T->ve[face][i]] * d];
				};
				auto matches = [&](int ea, const LocalFaces* Ta, int fa, int eb, const LocalFaces* Tb, int fb, int* out) {
					for (int i = 0; i < n; ++i) {
						out[i] = -1;
						const double* xa = xyz(ea, Ta, fa, i);
						double scale = 1.0;
						for (int k = 0; k < d; ++k)
							scale = std::max(scale, std::fabs(xa[k]));
						for (int j = 0; j < n && out[i] < 0; ++j) {
							const double* xb = xyz(eb, Tb, fb, j);
							double diff = 0.0;
							for (int k = 0; k < d; ++k)
								if (k != skip)
									diff += std::fabs(xa[k] + (k == reflect ? 1.0 : -1.0) * xb[k]);
							if (diff < std::max(kEps, 1e-12 * scale))
								out[i] = j;
						}
						if (out[i] < 0)
							return false;
					}
					return true;
				};
				int back[4];
				if (!matches(e, L, lf, en, Ln, il, match) || !matches(en, Ln, il, e, L, lf, back))
					return fail(DGPU_ERR_INVALID_ARGUMENT, "face " + std::to_string(f) + ": no vertex correspondence");
				// the reference's permutation lists (face.c:515-527)
				static const int line_p[2][2] = {{0, 1}, {1, 0}};
				static const int tri_p[6][3] = {{0, 1, 2}, {1, 2, 0}, {2, 0, 1}, {0, 2, 1}, {2, 1, 0}, {1, 0, 2}};
				static const int quad_p[8][4] = {{0, 1, 2, 3}, {1, 0, 3, 2}, {2, 3, 0, 1}, {3, 2, 1, 0},
				                                 {0, 2, 1, 3}, {2, 0, 3, 1}, {1, 3, 0, 2}, {3, 1, 2, 0}};
				const int n_perm = (n == 2 ? 2 : n == 3 ? 6 : n == 4 ? 8 : 1);
				for (int p = 0; p < n_perm; ++p) {
					const int* row = (n == 2 ? line_p[p] : n == 3 ? tri_p[p] : n == 4 ? quad_p[p] : nullptr);
					if (!row) {   // points (d = 1)
						ord[0] = ord[1] = 0;
						break;
					}
					if (std::equal(match, match + n, row))
						ord[1] = p;
					if (std::equal(back, back + n, row))
						ord[0] = p;
				}
			}
			m->face_match.insert(m->face_match.end(), match, match + 4);
			m->face_ord.push_back(ord[0]);
			m->face_ord.push_back(ord[1]);
		}
	}
	return DGPU_OK;
}

template <typename T>
void put(T* dst, const std::vector<T>& src)
{
	if (dst && !src.empty())
		std::memcpy(dst, src.data(), src.size() * sizeof(T));
}

}  // namespace

extern "C" dgpu_status dgpu_gmsh_read(const char* path, int d, dgpu_gmsh** out)
{
	g_mesh_error.clear();
	if (!path || !out)
		return fail(DGPU_ERR_INVALID_ARGUMENT, "NULL argument");
	*out = nullptr;
	if (d < 1 || d > 3)
		return fail(DGPU_ERR_UNSUPPORTED, "d must be 1, 2 or 3");
	dgpu_gmsh* m = new dgpu_gmsh();
	m->d = d;
	dgpu_status st = read_gmsh(path, d, m);
	if (st == DGPU_OK)
		st = build_connectivity(m);
	if (st == DGPU_OK)
		build_vertices(m);
	if (st == DGPU_OK)
		st = build_faces(m);
	if (st != DGPU_OK) {
		delete m;
		return st;
	}
	*out = m;
	return DGPU_OK;
}

extern "C" dgpu_status dgpu_gmsh_destroy(dgpu_gmsh* m)
{
	delete m;
	return DGPU_OK;
}

extern "C" const char* dgpu_gmsh_last_error(void) { return g_mesh_error.c_str(); }

extern "C" dgpu_status dgpu_gmsh_get_sizes(const dgpu_gmsh* m, dgpu_gmsh_sizes* s)
{
	if (!m || !s)
		return fail(DGPU_ERR_INVALID_ARGUMENT, "NULL argument");
	s->d = m->d;
	s->n_nodes = (int)(m->nodes.size() / m->d);
	s->n_elements = (int)m->elem_types.size();
	s->n_node_nums = (int)m->node_nums.size();
	s->n_periodic = (int)(m->periodic_corr.size() / 2);
	s->n_volumes = m->n_v;
	s->n_volume_faces = (int)m->v_to_v.size();
	s->n_ve_bc = (int)m->ve_bc.size();
	s->n_faces = m->n_faces;
	s->has_periodic = m->has_periodic ? 1 : 0;
	return DGPU_OK;
}

extern "C" dgpu_status dgpu_gmsh_data(const dgpu_gmsh* m, double* nodes, int* elem_types, int* elem_tags,
                                      int* node_ptr, int* node_nums, int* periodic_corr, int* elem_per_dim)
{
	if (!m)
		return fail(DGPU_ERR_INVALID_ARGUMENT, "NULL argument");
	put(nodes, m->nodes);
	put(elem_types, m->elem_types);
	put(elem_tags, m->elem_tags);
	put(node_ptr, m->node_ptr);
	put(node_nums, m->node_nums);
	put(periodic_corr, m->periodic_corr);
	if (elem_per_dim)
		std::memcpy(elem_per_dim, m->elem_per_dim, sizeof m->elem_per_dim);
	return DGPU_OK;
}

extern "C" dgpu_status dgpu_gmsh_connectivity(const dgpu_gmsh* m, int* lf_ptr, int* v_to_v, int* v_to_lf,
                                              int* v_to_lf_wp)
{
	if (!m)
		return fail(DGPU_ERR_INVALID_ARGUMENT, "NULL argument");
	put(lf_ptr, m->lf_ptr);
	put(v_to_v, m->v_to_v);
	put(v_to_lf, m->v_to_lf);
	put(v_to_lf_wp, m->v_to_lf_wp);
	return DGPU_OK;
}

extern "C" dgpu_status dgpu_gmsh_vertices(const dgpu_gmsh* m, int* ve_curved, int* ve_boundary, int* ve_bc_ptr,
                                          int* ve_bc)
{
	if (!m)
		return fail(DGPU_ERR_INVALID_ARGUMENT, "NULL argument");
	put(ve_curved, m->ve_curved);
	put(ve_boundary, m->ve_boundary);
	put(ve_bc_ptr, m->ve_bc_ptr);
	put(ve_bc, m->ve_bc);
	return DGPU_OK;
}

extern "C" dgpu_status dgpu_gmsh_faces(const dgpu_gmsh* m, int* face_vol, int* face_lf, int* face_bc, int* face_wp,
                                       int* face_match, int* face_ord)
{
	if (!m)
		return fail(DGPU_ERR_INVALID_ARGUMENT, "NULL argument");
	put(face_vol, m->face_vol);
	put(face_lf, m->face_lf);
	put(face_bc, m->face_bc);
	put(face_wp, m->face_wp);
	put(face_match, m->face_match);
	put(face_ord, m->face_ord);
	return DGPU_OK;
}
