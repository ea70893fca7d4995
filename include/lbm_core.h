/* lbm_core.h -- drop-in for lbc include/lbm_core.h (same names, argument lists
 * and meaning). Every function runs on the GPU (sm_103a); arrays are the
 * caller's host arrays in lbc's layout and are read and written in place
 * exactly as lbc does. Errors are recorded in lbm_gpu_last_error() (lbm_gpu.h);
 * on error the output arrays are left untouched.
 */
#ifndef LBM_CORE_H
#define LBM_CORE_H

#include "lbm_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* One time step (lbc include/lbm_core.h:6-31, src/core/main_lbm.c:5-62):
 * collide f in place, bounce-back (IBB when use_IBB), momentum-exchange force
 * into *D (x) and *L (y), stream into f_new, Boundary list in order, moments
 * into rho/u/v. The caller swaps f and f_new afterwards. */
void main_lbm(int Nx, int Ny, int Q, LBM_POP(f), LBM_POP(f_new), LBM_FLD(rho), LBM_FLD(u),
              LBM_FLD(v), int cx[], int cy[], double w[], int opp[], LBM_FLD(omega_eff),
              LBM_MASK(solid_mask), Boundary boundaries[], int num_boundaries, int isperiodic_x,
              int isperiodic_y, double Fx, double Fy, double *L, double *D, LBM_FLD(phi),
              int use_IBB);

/* lbc include/lbm_core.h:33-48, src/core/collision.c */
void collision(int Nx, int Ny, int Q, LBM_POP(f), LBM_FLD(rho), LBM_FLD(u), LBM_FLD(v),
               LBM_FLD(omega_eff), LBM_MASK(solid_mask), int cx[], int cy[], double w[],
               double Fx, double Fy);

/* lbc include/lbm_core.h:50-61, src/core/streaming.c */
void streaming(int Nx, int Ny, int Q, LBM_POP(f), LBM_POP(f_new), LBM_MASK(solid_mask), int cx[],
               int cy[], int isperiodic_x, int isperiodic_y);

/* lbc include/lbm_core.h:63-76, src/core/compute_macroscopic_fields.c */
void compute_macroscopic_fields(int Nx, int Ny, int Q, LBM_POP(f_new), LBM_MASK(solid_mask),
                                int cx[], int cy[], LBM_FLD(rho), LBM_FLD(u), LBM_FLD(v),
                                double Fx, double Fy);

/* lbc include/lbm_core.h:78-92, src/core/compute_force_mem.c */
void compute_force_mem(int Nx, int Ny, int Q, LBM_POP(f), LBM_POP(f_new), LBM_MASK(solid_mask),
                       int isperiodic_x, int isperiodic_y, const int cx[], const int cy[],
                       const int opp[], double *Fx, double *Fy);

/* lbc include/lbm_core.h:94-115, src/core/mei_initialization.c */
void mei_initialization(int Nx, int Ny, int Q, LBM_POP(f), LBM_POP(f_new), LBM_FLD(rho_in),
                        LBM_FLD(U_in), LBM_FLD(V_in), LBM_FLD(rho), LBM_FLD(u), LBM_FLD(v),
                        int cx[], int cy[], double w[], LBM_FLD(omega_eff), int isperiodic_x,
                        int isperiodic_y, int init_iter_max, double tol_rho,
                        LBM_MASK(solid_mask));

/* lbc include/lbm_core.h:117-128, src/core/sponge_layer.c (filled on the device) */
void sponge_layer(int Nx, int Ny, double dx, double xc, double yc, double r_inner,
                  double r_outer, double tau_base, double incr_tau, double exp_coeff,
                  LBM_FLD(omega_eff));

#ifdef __cplusplus
}
#endif
#endif
