/*
 * lymph3d_mesh.h -- host-side mesh set-up utilities of the GB300 library.
 *
 * These produce the flat arrays of lymph_mesh_desc (lymph3d_gpu.h).  They
 * replace the set-up part of the reference that feeds the hot path:
 * face matching and neighbour tables (CREATE_NEIGH_EL_TRIA /
 * FIND_NEIGHBOUR_EL, src/MAKE_PARTITION_AND_MPI_FILES.f90:1914-2461 and
 * :2536-2580, an O(n^2) scan in the reference, hashed here), the hard-coded
 * boundary-tag convention (:2105-2109) and the grouping of tetrahedra into
 * polyhedra (MESH_AGGLOMERATION :327-478, which calls METIS; here a seeded
 * breadth-first grouping, see lymph_mesh_agglomerate).  Plain host code: no
 * device is needed to call any of them.
 */
#ifndef LYMPH3D_MESH_H
#define LYMPH3D_MESH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Boundary-condition assignment modes for lymph_mesh_apply_bc. */
#define LYMPH_BCMODE_REFERENCE      0  /* tags 2,3,4 Dirichlet; 5,6,7 Neumann
                                          (MAKE_PARTITION_AND_MPI_FILES.f90:2105-2109) */
#define LYMPH_BCMODE_ALL_DIRICHLET  1  /* every tagged boundary face Dirichlet */

/* Value left in neigh[] for a face with no neighbour and no boundary tag. */
#define LYMPH_MESH_UNMATCHED (-9)

/* Sizes of the structured unit-cube mesh of nx*ny*nz hexahedra, each cut
 * into 6 tetrahedra. */
int lymph_mesh_cube_sizes(int32_t nx, int32_t ny, int32_t nz, int32_t* n_node, int32_t* n_tet);

/* Structured mesh of [0,1]^3: node (i,j,k) at (i/nx, j/ny, k/nz), hexahedron
 * (a,b,c) cut along its main diagonal into the 6 Kuhn tetrahedra, each
 * ordered so that det J > 0 (outward normals with the reference's face
 * vertex order).  face_tag[t*4+f] receives the cube-face tag of a boundary
 * face with the reference decks' numbering (2: z=0, 3: z=1, 4: x=1, 5: y=1,
 * 6: x=0, 7: y=0; src/tests/analytical/tet_5/cube_size05.mesh) and 0 for an
 * interior face. */
int lymph_mesh_cube(int32_t nx, int32_t ny, int32_t nz, double* coords, int32_t* tet_vert, int32_t* face_tag);

/* Face matching by hashing the sorted vertex triple of every tetrahedron
 * face (faces {1,2,3},{1,2,4},{2,3,4},{3,1,4} in 1-based local numbering).
 * neigh[t*4+f] = the tetrahedron across face f or LYMPH_MESH_UNMATCHED;
 * neigh_face (nullable) = that tetrahedron's local face.  Returns
 * LYMPH_EXIT_NEIGHBOUR_EL_ERROR if a face is shared by more than two
 * tetrahedra. */
int lymph_mesh_match_faces(int32_t n_tet, const int32_t* tet_vert, int32_t* neigh, int32_t* neigh_face);

/* Boundary tags from a list of tagged boundary triangles (the "tria" records
 * of a reference .mesh file): face_tag[t*4+f] = tag of the triangle with the
 * same vertex set, 0 if none.  Returns the number of triangles not found on
 * any tetrahedron face through *n_unfound (nullable). */
int lymph_mesh_tag_boundary(int32_t n_tet, const int32_t* tet_vert, int32_t n_tri, const int32_t* tri_vert,
                            const int32_t* tri_tag, int32_t* face_tag, int32_t* n_unfound);

/* Writes LYMPH_BC_DIRI / LYMPH_BC_NEUM into neigh[] for unmatched faces that
 * carry a boundary tag, and the space-function tag into fun_tag[] (tags 2..4
 * -> 1..3 and 5..7 -> 1..3, the .mate DIRI/NEUM records of the reference
 * decks; 0 for interior faces).  Returns LYMPH_EXIT_SETUP if an unmatched
 * face has no tag. */
int lymph_mesh_apply_bc(int32_t n_tet, const int32_t* face_tag, int32_t mode, int32_t* neigh, int32_t* fun_tag);

/* Seeded breadth-first agglomeration of tetrahedra into connected
 * polyhedra.  Tetrahedra are visited in index order; an unassigned one starts
 * a group whose target size is drawn uniformly from [min_size, max_size]
 * (splitmix64 stream of `seed`); the group grows breadth-first through face
 * neighbours (face order 1..4) until it reaches the target or runs out of
 * unassigned neighbours.  Groups left below min_size are merged into the
 * smallest face-adjacent group, so sizes end in [min_size, max_size +
 * min_size - 1] (a group with no face neighbour may stay smaller).  Polyhedra are
 * numbered by their first tetrahedron.  min_size = max_size = 1 gives one
 * polyhedron per tetrahedron. */
int lymph_mesh_agglomerate(int32_t n_tet, const int32_t* neigh, uint64_t seed, int32_t min_size, int32_t max_size,
                           int32_t* tet_poly, int32_t* n_poly);

/* Groups the 6 tetrahedra of every hexahedron of a lymph_mesh_cube mesh
 * into one polyhedron (tet t -> polyhedron t/6). */
int lymph_mesh_agglomerate_hex(int32_t n_tet, int32_t* tet_poly, int32_t* n_poly);

/* Polyhedron containing a point: the tetrahedron whose barycentric
 * coordinates are all >= -tol, else the one with the nearest barycentre
 * (FIND_ELEM_FROM_POINT, src/find_tet.f90:82-124). Returns the tet index. */
int lymph_mesh_find_tet(int32_t n_tet, const int32_t* tet_vert, const double* coords, const double* point, int32_t* tet);

#ifdef __cplusplus
}
#endif

#endif /* LYMPH3D_MESH_H */
