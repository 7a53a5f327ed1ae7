/* include/vibe_nest.h
 *
 * One-level nest transfers on the GPU, replacing grid::Nest
 * (include/vibe/grid/nest.hpp:41-98, src/grid/nest.cpp:34-124):
 *   vibe_davies_profile              davies_profile (nest.cpp:34-44)
 *   vibe_nest_interpolate_from_parent Nest::interpolate_from_parent (:58-84)
 *   vibe_nest_restrict_to_parent     Nest::restrict_to_parent (:86-105)
 *   vibe_nest_apply_lateral_boundary Nest::apply_lateral_boundary (:107-124)
 * with the reference's arithmetic and index maps bit for bit: child point
 * (i, j) sits at parent coordinate ((i0 + i) + 0.5)/r - 0.5 (bilinear,
 * parent clamped to its cells); the parent point (i0 + i, j0 + j) receives
 * the mean of the child's r x r points (i < iext, j < jext); the Davies
 * weight of a child point is alpha(d), d = its distance in points to the
 * nearest lateral edge (d < boundary_zone). As in the reference, every
 * stagger uses the cell formulas over the grid's nx x ny (the extra face of
 * a staggered field is not touched) and the placement offsets i0/j0 enter
 * the interpolation in child points but the restriction in parent points.
 *
 * Fields are passed as arrays of nvars pointers (FieldT storage, halo 4) and
 * nvars staggers (0 cell, 1 x-face, 2 y-face, 3 z-face); one call transfers
 * all of them. The _dev forms take device pointers and a stream; the plain
 * forms take host arrays. The restriction writes the parent box
 * (i0 .. i0+iext-1, j0 .. j0+jext-1), which must lie inside the parent's
 * storage (the reference does not check; here it is VIBE_C_ERR_BAD_ARG).
 */
#ifndef VIBE_GB300_NEST_H
#define VIBE_GB300_NEST_H

#include "vibe_c_kernels.h"

#ifdef __cplusplus
extern "C" {
#endif

/* NestPlacement (nest.hpp:41-48) */
typedef struct vibe_nest_placement {
  int i0, j0, k0;
  int iext, jext;
  int ratio;          /* >= 2 */
  int boundary_zone;  /* >= 1, Davies zone width in child points */
  int two_way;
} vibe_nest_placement;

/* n_zone weights alpha_max * (1 - cos(pi (n_zone - n) / n_zone)) / 2. */
int vibe_davies_profile(int n_zone, double alpha_max, double *out);

int vibe_nest_interpolate_from_parent(const vibe_nest_placement *p, int nvars, const int *stagger, int pnx,
                                      int pny, int pnz, const double *const *parent, int cnx, int cny, int cnz,
                                      double *const *child);
int vibe_nest_restrict_to_parent(const vibe_nest_placement *p, int nvars, const int *stagger, int cnx, int cny,
                                 int cnz, const double *const *child, int pnx, int pny, int pnz,
                                 double *const *parent);
int vibe_nest_apply_lateral_boundary(const vibe_nest_placement *p, int nvars, const int *stagger, int cnx, int cny,
                                     int cnz, double *const *child, const double *const *parent_interp);

int vibe_nest_interpolate_from_parent_dev(const vibe_nest_placement *p, int nvars, const int *stagger, int pnx,
                                          int pny, int pnz, const double *const *parent, int cnx, int cny,
                                          int cnz, double *const *child, vibe_stream_t stream);
int vibe_nest_restrict_to_parent_dev(const vibe_nest_placement *p, int nvars, const int *stagger, int cnx,
                                     int cny, int cnz, const double *const *child, int pnx, int pny, int pnz,
                                     double *const *parent, vibe_stream_t stream);
int vibe_nest_apply_lateral_boundary_dev(const vibe_nest_placement *p, int nvars, const int *stagger, int cnx,
                                         int cny, int cnz, double *const *child,
                                         const double *const *parent_interp, vibe_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif
