/* lbm_bc.h -- drop-in for lbc include/lbm_bc.h (same 20 functions).
 *
 * Called directly, each function runs on the GPU on the caller's arrays. Passed
 * as Boundary.apply to main_lbm, the function pointer selects the matching BC
 * kernel of the fused step (compared by identity).
 */
#ifndef LBM_BC_H
#define LBM_BC_H

#include "lbm_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* lbc include/lbm_bc.h:4-16, src/bc/bounce_back.c */
void bounce_back(int Nx, int Ny, int Q, LBM_POP(f), LBM_POP(f_new), LBM_MASK(solid_mask), int cx[],
                 int cy[], int opp[], int isperiodic_x, int isperiodic_y);

/* lbc include/lbm_bc.h:18-31, src/bc/interpolated_bounce_back.c */
void interpolated_bounce_back(int Nx, int Ny, int Q, LBM_POP(f), LBM_POP(f_new),
                              LBM_MASK(solid_mask), LBM_FLD(phi), int opp[], int cx[], int cy[],
                              int isperiodic_x, int isperiodic_y);

#define LBM_BC_PARAMS                                                                     \
    int Nx, int Ny, int Q, int index, const double *val1, const double *val2, LBM_POP(f), \
        LBM_POP(f_new), LBM_FLD(rho), LBM_FLD(u), LBM_FLD(v), LBM_MASK(solid_mask),       \
        int cx[], int cy[], double w[]

/* lbc include/lbm_bc.h:33-49, src/bc/convective_inlet.c */
void convective_inlet(LBM_BC_PARAMS);

/* lbc include/lbm_bc.h:51-67, src/bc/convective_outlet.c */
void convective_outlet(LBM_BC_PARAMS);

/* lbc include/lbm_bc.h:69-85, src/bc/pressure_inlet.c */
void pressure_inlet(LBM_BC_PARAMS);

/* lbc include/lbm_bc.h:87-103, src/bc/pressure_outlet.c */
void pressure_outlet(LBM_BC_PARAMS);

/* lbc include/lbm_bc.h:105-121, src/bc/periodic_x.c */
void periodic_x(LBM_BC_PARAMS);

/* lbc include/lbm_bc.h:123-139, src/bc/periodic_y.c */
void periodic_y(LBM_BC_PARAMS);

/* lbc include/lbm_bc.h:141-157, src/bc/velocity_inlet.c */
void velocity_inlet(LBM_BC_PARAMS);

/* lbc include/lbm_bc.h:159-175, src/bc/velocity_outlet.c */
void velocity_outlet(LBM_BC_PARAMS);

/* lbc include/lbm_bc.h:177-193, src/bc/velocity_top.c */
void velocity_top(LBM_BC_PARAMS);

/* lbc include/lbm_bc.h:195-211, src/bc/velocity_bottom.c */
void velocity_bottom(LBM_BC_PARAMS);

/* lbc include/lbm_bc.h:213-229, src/bc/velocity_outlet_regularized.c */
void velocity_outlet_regularized(LBM_BC_PARAMS);

/* lbc include/lbm_bc.h:231-247, src/bc/velocity_inlet_regularized.c */
void velocity_inlet_regularized(LBM_BC_PARAMS);

/* lbc include/lbm_bc.h:249-265, src/bc/velocity_top_regularized.c */
void velocity_top_regularized(LBM_BC_PARAMS);

/* lbc include/lbm_bc.h:267-283, src/bc/velocity_bottom_regularized.c */
void velocity_bottom_regularized(LBM_BC_PARAMS);

/* lbc include/lbm_bc.h:285-301, src/bc/pressure_outlet_regularized.c */
void pressure_outlet_regularized(LBM_BC_PARAMS);

/* lbc include/lbm_bc.h:303-319, src/bc/pressure_inlet_regularized.c */
void pressure_inlet_regularized(LBM_BC_PARAMS);

/* lbc include/lbm_bc.h:321-337, src/bc/pressure_top_regularized.c */
void pressure_top_regularized(LBM_BC_PARAMS);

/* lbc include/lbm_bc.h:339-355, src/bc/pressure_bottom_regularized.c */
void pressure_bottom_regularized(LBM_BC_PARAMS);

/* Extension (no counterpart in lbc): velocity_bottom with the Zou-He closure
 * for population 6, f6 = f8 + (f1 - f3)/2 - rho U/2 + rho V/6. lbc's
 * velocity_bottom (src/bc/velocity_bottom.c:39) writes that value to
 * population 7 a second time and leaves 6 as streamed; velocity_bottom keeps
 * lbc's behaviour for drop-in parity, and a case opts into the corrected
 * closure by putting this function in its Boundary list. */
void velocity_bottom_corrected(LBM_BC_PARAMS);


#ifdef __cplusplus
}
#endif
#endif
