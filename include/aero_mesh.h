/* aero_mesh.h -- host mesh generators of libaero_gb300.so (C ABI).
 *
 * Two generators produce meshes in the reference UnstructuredMesh layout
 * (src/cfd_core/include/cfd_core/mesh.hpp:14-35, paths relative to the AeroCFD root):
 *
 *  - aero_mesh_ogrid_reference: the reference's own O-grid
 *    (make_airfoil_ogrid_mesh, src/cfd_core/mesh/airfoil_mesh.cpp:459-544, including
 *    generate_naca4_profile :395-457 and build_triangular_mesh :184-392), computed with the
 *    same float arithmetic so that run_case on the device path sees the reference's mesh
 *    bit for bit. It replaces make_airfoil_ogrid_mesh behind the cfd_core boundary.
 *  - aero_mesh_ogrid_synthetic: the benchmark O-grids (no reference counterpart): analytic
 *    closed-trailing-edge NACA 00xx contour, cosine clustering at LE/TE, prescribed first
 *    wall spacing with per-line geometric growth to a circular far field, quads or
 *    triangles with a seeded diagonal, seeded jitter of interior nodes and seeded
 *    permutations of cells and of faces within the interior/wall/far-field blocks.
 *    Geometry is computed in double.
 */
#ifndef AERO_MESH_H
#define AERO_MESH_H

#include "aero_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct aero_mesh aero_mesh;

typedef struct aero_ogrid_spec {
  int n_circ;            /* points (and cells) around the airfoil */
  int n_radial;          /* cell layers from the wall to the far field */
  int cell_type;         /* 3 = triangles (two per quad), 4 = quads */
  int permute;           /* 1: seeded permutation of cells and faces */
  double chord;
  double thickness;      /* t of NACA 00xx, 0.12 for NACA 0012 */
  double wall_spacing;   /* first radial spacing at the wall, in chords */
  double farfield_radius;/* in chords, circle centred at mid-chord */
  double jitter;         /* interior node jitter as a fraction of local spacing */
  unsigned long long seed;
} aero_ogrid_spec;

/* Sizes of a generated mesh. */
typedef struct aero_mesh_sizes {
  int num_cells, num_faces, num_points, num_wall_faces, num_farfield_faces, conn_length;
} aero_mesh_sizes;

AERO_API int aero_mesh_ogrid_reference(const char* naca_code, int n_circ, int n_radial,
                              double farfield_radius, double radial_stretch, double chord,
                              aero_mesh** out);
AERO_API int aero_mesh_ogrid_synthetic(const aero_ogrid_spec* spec, aero_mesh** out);
AERO_API void aero_mesh_free(aero_mesh* m);
AERO_API const char* aero_mesh_last_error(void);

AERO_API int aero_mesh_get_sizes(const aero_mesh* m, aero_mesh_sizes* s);
/* Fill a descriptor that points into the mesh's own arrays (valid while m lives). */
AERO_API int aero_mesh_describe(const aero_mesh* m, aero_mesh_desc* d);
/* Copy the auxiliary arrays: points [3P], face_vertices [2F], cell connectivity [conn],
 * cell offsets [N] (running end offsets, VTU style), cell types [N] (5 tri, 9 quad),
 * far-field faces [num_farfield_faces]. Any pointer may be null. */
AERO_API int aero_mesh_get_aux(const aero_mesh* m, double* points, int* face_vertices, int* conn,
                      int* offsets, unsigned char* types, int* farfield_faces);

/* Deep copy of a mesh (free it with aero_mesh_free). */
AERO_API int aero_mesh_clone(const aero_mesh* m, aero_mesh** out);

/* Move the nodes to points [3P] and recompute the geometry (cell areas and centres, face
 * normals, lengths and centres) with the synthetic generator's double formulas. Fails
 * (mesh unchanged) if a cell inverts or a face degenerates. */
AERO_API int aero_mesh_set_points(aero_mesh* m, const double* points);

/* Derivatives of that geometry along a node displacement dpoints [3P]: d_normal [3F],
 * d_center [3F], d_area [F], d_volume [N], d_cell_center [3N]. Fill an aero_mesh_desc with
 * them (connectivity from aero_mesh_describe) to pass to aero_adjoint_geometry. */
AERO_API int aero_mesh_geometry_tangent(const aero_mesh* m, const double* dpoints, double* d_normal,
                                        double* d_center, double* d_area, double* d_volume,
                                        double* d_cell_center);

/* Transpose of aero_mesh_geometry_tangent (no reference counterpart): from the derivatives of a
 * scalar with respect to face_normal [3F], face_center [3F], face_area [F], cell_volume [N] and
 * cell_center [3N], its derivatives with respect to the node coordinates, b_points [3P] (z
 * entries 0), in one reverse pass; for every node displacement dX, the sum of b_points * dX
 * equals the sum of the given derivatives times aero_mesh_geometry_tangent(dX). */
AERO_API int aero_mesh_geometry_vjp(const aero_mesh* m, const double* b_normal, const double* b_center,
                                    const double* b_area, const double* b_volume, const double* b_cell_center,
                                    double* b_points);

/* Shape modes of n Hicks-Henne bumps, modes [n][3P]: mode k moves the wall-patch nodes of
 * the upper (upper[k] != 0, y > 0) or lower (y < 0) surface in y by
 * sin(pi xi^(ln 0.5 / ln peak_x[k]))^width_exponent, xi the chordwise position in [0, 1]
 * along the patch, keeps the far-field nodes fixed and carries the displacement into the
 * volume by inverse-distance weighting (weights |x - x_s|^-3 over the wall and far-field
 * nodes). The deformed nodes for amplitudes a are points + sum_k a_k modes[k]. */
AERO_API int aero_mesh_hicks_henne_modes(const aero_mesh* m, int n_bumps, const double* peak_x,
                                         const int* upper, double width_exponent, double* modes);

#ifdef __cplusplus
}
#endif

#endif /* AERO_MESH_H */
