/* dgpu_mesh.h -- C ABI of the mesh reader and connectivity that feed the GB300 residual.
 *
 * Host code only (no device is needed). A gmsh 2.2 ASCII file is read and preprocessed the way the reference does
 * it before its solvers run, and the results come out in the reference's containers and in dgpu_mesh's face list:
 *   dgpu_gmsh_read          constructor_Mesh (src/simulation/mesh/mesh.c): the reader mesh_reader_gmsh
 *                           (mesh_readers.c:215-235, nodes, elements with 2 tags, d-1 dimensional periodic entity
 *                           pairs; vertices reordered by reorder_nodes_gmsh :132-163), the connectivity
 *                           constructor_Mesh_Connectivity (mesh_connectivity.c:85-113: v_to_v, v_to_lf with the
 *                           boundary faces' BC codes, v_to_lf_wp keeping the periodic codes; periodic faces matched
 *                           by correct_f_ve_for_periodic, mesh_periodic.c:102-130), the vertex flags
 *                           constructor_Mesh_Vertices (mesh_vertices.c:56-75), and the face list of
 *                           constructor_Faces (computational_elements/face.c:86-154) with each face's vertex
 *                           correspondence and ordering index (set_ind_ord, face.c:498-546).
 *   dgpu_gmsh_data          Mesh_Data members          dgpu_gmsh_connectivity  Mesh_Connectivity members
 *   dgpu_gmsh_vertices      Mesh_Vertices members      dgpu_gmsh_faces         the face list
 * Element types are gmsh's codes, which the reference uses as its own: POINT 15, LINE 1, TRI 2, QUAD 3, TET 4,
 * HEX 5, WEDGE 6, PYR 7. Vertex orders are the reference's (TP order for QUAD/HEX/PYR bases). Volume v is the v-th
 * element of dimension d in file order.
 */
#ifndef DGPU_MESH_H
#define DGPU_MESH_H

#include "dgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct dgpu_gmsh dgpu_gmsh;

typedef struct {
	int d;
	int n_nodes;
	int n_elements;       /* all elements of the file (points, lines, faces, volumes) */
	int n_node_nums;      /* sum over elements of their vertex counts */
	int n_periodic;       /* rows of periodic_corr */
	int n_volumes;
	int n_volume_faces;   /* sum over volumes of their local faces: the length of v_to_v, v_to_lf, v_to_lf_wp */
	int n_ve_bc;          /* total length of ve_bc */
	int n_faces;
	int has_periodic;     /* 1 when v_to_lf_wp exists (the file has periodic entities) */
} dgpu_gmsh_sizes;

/* Read and preprocess. DGPU_ERR_INVALID_ARGUMENT for a file that cannot be read or is not a conforming mesh of
 * dimension d (the reason: dgpu_gmsh_last_error), DGPU_ERR_UNSUPPORTED for element types, tag counts or BC codes
 * the reference does not read. */
dgpu_status dgpu_gmsh_read(const char* path, int d, dgpu_gmsh** out);
dgpu_status dgpu_gmsh_destroy(dgpu_gmsh* mesh);
/* Message of the last failed dgpu_gmsh_* call of this thread ("" if none). */
const char* dgpu_gmsh_last_error(void);
dgpu_status dgpu_gmsh_get_sizes(const dgpu_gmsh* mesh, dgpu_gmsh_sizes* sizes);

/* Mesh_Data (mesh_readers.h): nodes n_nodes x d row-major; elem_types; elem_tags n_elements x 2 (physical tag =
 * BC code or volume tag, entity tag); node_ptr (n_elements + 1) and node_nums (0-based, reference vertex order);
 * periodic_corr n_periodic x 2 (slave entity, master entity); elem_per_dim[4]. Any output may be NULL. */
dgpu_status dgpu_gmsh_data(const dgpu_gmsh* mesh, double* nodes, int* elem_types, int* elem_tags, int* node_ptr,
                           int* node_nums, int* periodic_corr, int* elem_per_dim);

/* Mesh_Connectivity (mesh_connectivity.h), per volume and local face, flattened with lf_ptr (n_volumes + 1):
 * v_to_v the neighbouring volume or -1; v_to_lf its local face, or on a boundary face the face's BC code (> 10000);
 * v_to_lf_wp as v_to_lf but with the periodic faces' periodic codes (all -1 when has_periodic is 0). */
dgpu_status dgpu_gmsh_connectivity(const dgpu_gmsh* mesh, int* lf_ptr, int* v_to_v, int* v_to_lf, int* v_to_lf_wp);

/* Mesh_Vertices (mesh_vertices.h): ve_curved, ve_boundary (n_nodes, 0/1); ve_bc_ptr (n_nodes + 1) and ve_bc (the
 * sorted BC codes of the boundary faces each vertex lies on). */
dgpu_status dgpu_gmsh_vertices(const dgpu_gmsh* mesh, int* ve_curved, int* ve_boundary, int* ve_bc_ptr, int* ve_bc);

/* The face list in constructor_Faces order, in dgpu_mesh's layout: face_vol and face_lf n_faces x 2 (side 1 = -1
 * on boundary faces), face_bc (Face::bc: the BC code of a boundary face, -1 otherwise), face_wp (the side-0 entry
 * of v_to_lf_wp: a periodic code on a periodic face, 0 without periodic entities), face_match n_faces x 4
 * (matches_R_to_L of the vertex correspondence: side 0's face vertex i is side 1's face vertex face_match[i], in the
 * element's local face vertex order; -1 padded and on boundary faces), face_ord n_faces x 2 (Neigh_Info::ind_ord,
 * the index of the correspondence in the reference's permutation list; -1 on boundary faces). */
dgpu_status dgpu_gmsh_faces(const dgpu_gmsh* mesh, int* face_vol, int* face_lf, int* face_bc, int* face_wp,
                            int* face_match, int* face_ord);

#ifdef __cplusplus
}
#endif

#endif
