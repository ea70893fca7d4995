/* Test infrastructure, not product code: lbc's step (src/core/main_lbm.c:32-61
 * with collision.c:18-40, streaming.c:14-45, bounce_back.c:15-49 and
 * compute_macroscopic_fields.c:19-48) on the 256 x 64 Poiseuille channel
 * (cases/poiseuille/poiseuille.c:47-107: solid rows 0 and 63, periodic in x,
 * Fx = 1e-6, tau = 0.8, f = w, stored rho = 1, u = 0) in long double.
 *
 * On x86-64 long double carries a 64-bit significand, 2^11 times finer than
 * FP64, so this run is the FP64 step's exact-arithmetic solution to within
 * about 1e-16: it measures how far an FP64 implementation's rounding moves the
 * result. Its inputs are the FP64 values an FP64 run uses (weights, omega and
 * force rounded to double first), so only the arithmetic differs.
 *
 * Prints rho and u of column 0 after N steps, one row per line (the channel is
 * uniform in x), with 21 significant digits. Usage: poiseuille_extended N
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef long double R;
static const int CX[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
static const int CY[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
static const int OPP[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};

int main(int argc, char **argv) {
    const int NX = 256, NY = 64;
    const int steps = argc > 1 ? atoi(argv[1]) : 20000;
    const double wd[9] = {4.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0,
                          1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0};
    R W[9];
    for (int k = 0; k < 9; k++) W[k] = wd[k];
    const R OM = (double)(1.0 / 0.8), FX = (double)1e-6;
    const size_t N = (size_t)NX * NY * 9;
    R *f = malloc(N * sizeof(R)), *fn = malloc(N * sizeof(R));
    R *rho = calloc(NY, sizeof(R)), *u = calloc(NY, sizeof(R));
    if (!f || !fn || !rho || !u) return 1;
#define IDX(j, i, k) ((((size_t)(j)) * NX + (i)) * 9 + (k))
    for (size_t q = 0; q < N; q++) f[q] = W[q % 9];
    const R g = 1 - 0.5L * OM;
    /* the first collision with the stored fields rho = 1, u = 0 */
    for (int j = 1; j < NY - 1; j++)
        for (int i = 0; i < NX; i++)
            for (int k = 0; k < 9; k++) {
                R *p = f + IDX(j, i, k);
                *p = *p + (-OM * (*p - W[k]) + g * W[k] * (3 * (CX[k] * FX)));
            }
    for (int t = 0; t < steps; t++) {
        for (int j = 1; j < NY - 1; j++)
            for (int i = 0; i < NX; i++) {
                R a[9];
                for (int k = 0; k < 9; k++) {
                    const int is = (i - CX[k] + NX) % NX, js = j - CY[k];
                    a[k] = (js == 0 || js == NY - 1) ? f[IDX(j, i, OPP[k])] : f[IDX(js, is, k)];
                }
                R s = 0, sx = 0, sy = 0;
                for (int k = 0; k < 9; k++) {
                    s += a[k];
                    sx += CX[k] * a[k];
                    sy += CY[k] * a[k];
                }
                const R ux = (sx + 0.5L * FX) / s, uy = sy / s;
                if (i == 0) {
                    rho[j] = s;
                    u[j] = ux;
                }
                if (t < steps - 1) {
                    const R usq = ux * ux + uy * uy, uF = ux * FX;
                    for (int k = 0; k < 9; k++) {
                        const R cu = CX[k] * ux + CY[k] * uy, cF = CX[k] * FX;
                        const R feq = W[k] * s * (1 + 3 * cu + 4.5L * cu * cu - 1.5L * usq);
                        const R Fk = W[k] * (3 * cF + 9 * cu * cF - 3 * uF);
                        a[k] = a[k] + (-OM * (a[k] - feq) + g * Fk);
                    }
                }
                memcpy(fn + IDX(j, i, 0), a, sizeof a);
            }
        R *tmp = f;
        f = fn;
        fn = tmp;
    }
    for (int j = 0; j < NY; j++) printf("%.21Le %.21Le\n", rho[j], u[j]);
    free(f);
    free(fn);
    free(rho);
    free(u);
    return 0;
}
