/* lbm_types.h -- lbc's BC callback type and Boundary list entry.
 *
 * Drop-in for lbc include/lbm_types.h:4-26: same typedef, same struct layout.
 * A Boundary's `apply` is compared by function identity against this
 * library's own BC symbols (lbm_bc.h), the way lbc's cases derive their
 * periodic flags (cases/nit/nit.c:187-192).
 */
#ifndef LBM_TYPES_H
#define LBM_TYPES_H

#ifdef __cplusplus
/* C++ cannot spell variably modified parameters; at the ABI level they are
 * plain pointers (AoS f[Ny][Nx][Q] with k fastest, fields [Ny][Nx]). */
#define LBM_POP(name) double *name
#define LBM_FLD(name) double *name
#define LBM_MASK(name) int *name
extern "C" {
#else
#define LBM_POP(name) double name[Ny][Nx][Q]
#define LBM_FLD(name) double name[Ny][Nx]
#define LBM_MASK(name) int name[Ny][Nx]
#endif

/* lbc include/lbm_types.h:4-19 */
typedef void (*BCFunction)(
    int Nx, int Ny, int Q, int index,
    const double *val1, const double *val2,
    LBM_POP(f), LBM_POP(f_new),
    LBM_FLD(rho), LBM_FLD(u), LBM_FLD(v),
    LBM_MASK(solid_mask),
    int cx[], int cy[], double w[]);

/* lbc include/lbm_types.h:21-26 */
typedef struct {
    int index;
    const double *val1;
    const double *val2;
    BCFunction apply;
} Boundary;

#ifdef __cplusplus
}
#endif
#endif
