/*
 * ORACLE (test infrastructure only; never part of the product path).
 *
 * CPU restatement of the FDFK2D hybrid FD time step (`updatedispl_`, shipped
 * closed in lib_gnu/libHybrid.so + libPML.so) and of the time loop of
 * `simulate_wavefield` (src/FDFK2D.f90:465-532).  The closed parts were
 * recovered by running the shipped libraries as a black box (see
 * oracle/refharness.py); the restatement is pinned against them by
 * tests/test_oracle.py and the fixtures in tests/golden/.
 *
 * All arrays use the reference's Fortran layout (src/FDFK2D.f90:253-355).
 */
#ifndef FDFK_ORACLE_H
#define FDFK_ORACLE_H

#include "fdfk_ops.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int norder, nx, nz, npml, izt, npower, nbd, nt;
    real_t dx, dz;
    double dt;
    real_t vpml;
    double R0;
} fdfk_oracle_params;

/* Strip order = the argument order of updatedispl_ (src/FDFK2D.f90:517-518):
 * uxl_reg uzl_reg uxr_reg uzr_reg uxb_reg uzb_reg uxl_pml uzl_pml uxr_pml uzr_pml uxb_pml uzb_pml.
 * bp order: bpxlx bpzlx bpxrx bpzrx bpxtx bpxtz bpztx bpztz bpxbx bpxbz bpzbx bpzbz.
 * bu order: bux1l bux2l bux3l buz1l buz2l buz3l, same for r, then b, then t. */
int fdfk_oracle_updatedispl(const fdfk_oracle_params *p, int it, const real_t *const strips[12], const real_t *c,
                            const double *coef0, const double *coef1, real_t *ux, real_t *uz, real_t *const bp[12],
                            real_t *const bu[24]);

/* The time loop it = 0..nt of src/FDFK2D.f90:465-532 with receiver sampling
 * every nstp steps (loadseis, src/Submain.f90:33-116) into seis[(nsis+1) x nrcv]
 * (sample fastest, as seisx(0:nsis, 1:nrcv)).  State arrays start at zero.
 * steps_limit < 0 runs all nt+1 steps; otherwise only the first steps_limit
 * steps (used to time a bounded sample).  Returns 0 or a negative error. */
int fdfk_oracle_simulate(const fdfk_oracle_params *p, const real_t *const strips[12], const real_t *c, int nrcv,
                         const real_t *rx, const real_t *rz, real_t x0, real_t z0, int nstp, int nsis,
                         real_t *seisx, real_t *seisz, int steps_limit);

#ifdef __cplusplus
}
#endif
#endif
