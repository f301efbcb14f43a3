/*
 * sbte.h -- C entry points of the host layer (libstaticbtesolver_gb300.so):
 * read the reference's input files, run its preprocessing, and hand the
 * result to a bte_ctx.  Used by the Python front end and by anyone who wants
 * the reference's file formats without the C++ classes.
 *
 * geo is an .mphtxt path or a decimal cell count for the uniform 1D mesh, as
 * BTEcmd's -g flag (src/BTEMain.cpp:118-141).
 */
#ifndef SBTE_H
#define SBTE_H
#include "bte_cuda.h"
#ifdef __cplusplus
extern "C" {
#endif

typedef struct sbte_problem sbte_problem;

/* Returns NULL on failure; sbte_error() then says why. */
sbte_problem* sbte_open(const char* geo, const char* bc_file, const char* band_file, int DM,
                        int num_theta, int num_phi, double T_ref, double L_x, double L_y, double L_z);
const char* sbte_error(void);
void sbte_close(sbte_problem* p);
/* counts: n_cell, n_dir, n_band, n_face, n_bc, dim */
void sbte_counts(const sbte_problem* p, int* counts);
/* scalars: solid_angle, T_ref (after the 1D override), WFACTOR, ms_quadrature, ms_geometry */
void sbte_quadrature(const sbte_problem* p, double* s, double* S, double* omega, double* scalars);
void sbte_geometry(const sbte_problem* p, double* volume, double* centroid, double* area, double* normal,
                   int* nbr);
void sbte_bands(const sbte_problem* p, double* vg, double* tau, double* C, double* Lr);
void sbte_bcs(const sbte_problem* p, int* index, int* type, double* T);
/* bte_set_geometry/quadrature/bands/bcs on ctx; returns a bte_status. */
int sbte_upload(const sbte_problem* p, bte_ctx* ctx);
/* Write T [n] at the cell centroids [n][3] in the reference's Tempcell.dat
 * format (src/StaticBTESolver.cpp:818-831, commented out there); 0 on success. */
int sbte_write_tempcell(const char* path, int n, int dim, const double* centroid, const double* T, double L_x,
                        double L_y, double L_z);
/* BTEcmd's main (argv[0] is the program name). */
int sbte_main(int argc, char** argv);

#ifdef __cplusplus
}
#endif
#endif
