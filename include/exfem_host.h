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

void exfem_model_free(exfem_model *m);

#ifdef __cplusplus
}
#endif
#endif /* EXFEM_HOST_H */
