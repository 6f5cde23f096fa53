/*
 * exfem_host.h — host side that plays the role of damian.par's Fortran host:
 * problem.in parsing (io.cpp:113-228), materials (model.f90:893-945), the
 * single-process quadtree mesher (mesh_utils.f90:64-112, 454-681, 720-750 with
 * the divide selection of communicator.f90:627-768 and mesh_utils.f90:114-201),
 * problem_setup (model.f90:958-1106), recalculate_deltat
 * (communicator.f90:1629-1662) and the receiver search of find_highest
 * (visualization.f90:286-305, quadtree.f90:253-291).
 *
 * The result is exposed as the exfem_mesh / exfem_problem pair that
 * exfem_gpu_create() consumes, plus writers for the reference's binary and
 * text formats (mesh.bin, mass.bin, step.bin, sheet.txt; io.cpp:333-482,
 * 844-911) so files round-trip with the reference's own reader.
 *
 * Deck format: the reference's problem.in sections (DOMAIN:, TIME:,
 * CH PERIOD:, CONTROL:, MATERIALS:, PROBLEM:, GEOMETRY:), plus optional
 * sections the reference parser skips as unknown lines:
 *   RECEIVERS:      xmin xmax dist            (the SHEET parameters)
 *   RHS:            n, then n lines "WAVEP|WAVESV angle amp freq t0"
 *   REFINE:         levels band               (extra rim/boundary refinement)
 *   HETEROGENEITY:  sigma seed                (per-element log-normal factors)
 * and the extra GEOMETRY kind EVALLY (xc, yc, a, b): semi-elliptical valley.
 */
#ifndef EXFEM_HOST_H
#define EXFEM_HOST_H

#include "exfem_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct exfem_model exfem_model;

typedef struct exfem_model_info {
    double width, height, duration, inttime, chper, nperlen, sperlen;
    double blength;      /* base element length m_blength                      */
    double mlength;      /* finest element length reached m_mlength             */
    int    totcols, totrows;
    int    wrows, wcols; /* DRM box in base-grid columns/rows (init_wave)       */
    int    nmat_base;    /* materials listed in the deck                        */
    int    nmat;         /* materials in the problem (> base with heterogeneity) */
    int    nelems, nnodes, nhanging, nseismic, nrecv, nrhs;
    int    nsteps, io_interval;
    double deltat;
    int    nlevels;      /* quadtree levels present                             */
    double min_h, max_h; /* smallest/largest element length                     */
} exfem_model_info;

/* Parse a deck (text of problem.in) and build the full model.  Returns 0 or a
 * negative EXFEM_E_* code; exfem_model_error() then holds the message. */
int  exfem_model_build(const char *deck_text, exfem_model **out);
const char *exfem_model_error(void);

/* Pointers into the model's own storage (valid until exfem_model_free). */
void exfem_model_views(const exfem_model *m, exfem_mesh *mesh, exfem_problem *prob);
void exfem_model_get_info(const exfem_model *m, exfem_model_info *info);

/* Limit the run to nsteps (<= the deck's); used to bound test and bench runs. */
int  exfem_model_set_nsteps(exfem_model *m, int nsteps);

/* Reference file formats. */
int  exfem_model_save_mesh(const exfem_model *m, const char *path);            /* io.cpp:333-367 */
int  exfem_write_mass(const char *path, int ndofs, const double *mass);        /* io.cpp:409-429 */
int  exfem_write_step(const char *path, int append, int step, int ndofs,
                      const double *u);                                        /* io.cpp:454-482 */
int  exfem_write_sheet(const char *path, int npoints, const double *points /* [2*npoints] */,
                       int nsave, const double *field, double samp);           /* io.cpp:844-889 */

/* ANIMAT sampling grid (create_visualization, visualization.f90:24-54).
 * visu_points (visualization.f90:129-154): nx = int((xmax-xmin)/dist),
 * ny = int((ymax-ymin)/dist), points (xmin + i dist, ymin + j dist) with i
 * outer and j inner.  Each point's element comes from a restatement of the
 * reference's quadtree (order_quadtree/search_quadtree, quadtree.f90:21-251):
 * ties on shared edges go to the larger coordinate, and points in no element
 * (cut voids, outside the domain) get 0.  material holds visu_material's
 * (material id, vp) at found points and 0 elsewhere (visualization.f90:
 * 183-190, share_field's zero fill, communicator.f90:1580-1584).  The cells
 * are create_struct_mesh's quads (mesh_utils.f90:846-878), 1-based. */
typedef struct exfem_grid {
    int    nx, ny;
    double origin[2], space;
    int    npoints;              /* (nx+1)*(ny+1)                                */
    const double *points;        /* [2*npoints]                                   */
    const int    *elem;          /* [npoints] 1-based element, 0 = not found      */
    const double *material;      /* [2*npoints]                                   */
    int    ncells;               /* nx*ny                                         */
    const int    *eptr;          /* [ncells+1] 1-based                            */
    const int    *eind;          /* [4*ncells] 1-based point ids                  */
    int    nfound;
} exfem_grid;

int  exfem_model_grid(const exfem_model *m, double xmin, double xmax, double ymin, double ymax, double dist,
                      exfem_grid **out);
void exfem_grid_free(exfem_grid *g);

/* VTK XML unstructured grid with base64 appended data, byte for byte the
 * layout of write_vtk_unst_field (io.cpp:699-842): a 3-component Float32
 * point array named fieldname (field is 2 values per point, the third 0),
 * the points, connectivity/offsets/types of the cells.  io.cpp encodes the
 * fourth byte of each block-length word from one byte past the int
 * (io.cpp:657); this writer encodes the int's own fourth byte. */
int  exfem_write_vtu(const char *path, int ncells, const int *eptr, const int *eind, int npoints,
                     const double *points, const char *fieldname, const double *field);

void exfem_model_free(exfem_model *m);

#ifdef __cplusplus
}
#endif
#endif /* EXFEM_HOST_H */
