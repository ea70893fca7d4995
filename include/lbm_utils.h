/* lbm_utils.h -- drop-in for lbc include/lbm_utils.h (host utilities). */
#ifndef LBM_UTILS_H
#define LBM_UTILS_H

#include "lbm_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* lbc include/lbm_utils.h:4, src/utils/filesystem.c:38-57: 0 if the directory
 * exists or was created, -1 otherwise. */
int ensure_directory_exists(const char *path);

/* lbc include/lbm_utils.h:6-15, src/utils/write_vtk_binary_2D.c:25-84: legacy
 * binary (big-endian FP32) VTK STRUCTURED_POINTS with velocity and density. */
void write_vtk_binary_2D(const char *filename, int Nx, int Ny, double dx, LBM_FLD(u), LBM_FLD(v),
                         LBM_FLD(rho), double cu, double crho);

#ifdef __cplusplus
}
#endif
#endif
