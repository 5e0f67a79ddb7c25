/*
 * ORACLE (test infrastructure only).  Restatement of the open FD operators of
 * FDFK2D src/Submain.f90; see fdfk_ops.c.
 */
#ifndef FDFK_ORACLE_OPS_H
#define FDFK_ORACLE_OPS_H

/* Field precision of the restatement: float (the reference's own arithmetic, with
 * its mixed-precision accumulation) by default; FDFK_ORACLE_FP64 builds the same
 * restatement with every field and intermediate in double (the FP64 oracle). */
#ifdef FDFK_ORACLE_FP64
typedef double real_t;
#define REAL_SQRT(x) sqrt(x)
#else
typedef float real_t;
#define REAL_SQRT(x) sqrtf(x)
#endif

#ifdef __cplusplus
extern "C" {
#endif

void fdfk_op_fd_coef0(int norder, double *coef);
void fdfk_op_fd_coef1(int norder, double *coef);
void fdfk_op_fd_coef2(int norder, double *coef);
real_t fdfk_op_dt_stable(int nx, int nz, int npml, int izt, int norder, real_t dx, real_t dz,
                        const double *coef2, const real_t *c);

real_t fdfk_op_diff1(int norder, int dire, int nx, int nz, int npml, int izt, int ix, int iz,
                    real_t d, const double *coef, const real_t *u);
real_t fdfk_op_diffx1(int norder, int nx, int npml, int ix, real_t dx, const double *coef, const real_t *u);

void fdfk_op_diffzx_reg(int norder, int nx, int nz, int npml, int izt, real_t dx, real_t dz,
                        const double *coef, const real_t *mat, const real_t *u, real_t *out);
void fdfk_op_diffzx_pml(int norder, int nx, int nz, int npml, int izt, real_t dx, real_t dz,
                        const double *coef, const real_t *mat, const real_t *u, real_t *out);
void fdfk_op_diffxz_reg(int norder, int nx, int nz, int npml, int izt, real_t dx, real_t dz,
                        const double *coef, const real_t *mat, const real_t *u, real_t *out);
void fdfk_op_diffxz_pml(int norder, int nx, int nz, int npml, int izt, real_t dx, real_t dz,
                        const double *coef, const real_t *mat, const real_t *u, real_t *out);
void fdfk_op_diffx2_reg(int norder, int nx, int nz, int npml, int izt, real_t dx,
                        const double *coef, const real_t *mat, const real_t *u, real_t *out);
void fdfk_op_diffx2_pml(int norder, int nx, int nz, int npml, int izt, real_t dx,
                        const double *coef, const real_t *mat, const real_t *u, real_t *out);
void fdfk_op_diffz2_reg(int norder, int nx, int nz, int npml, int izt, real_t dz,
                        const double *coef, const real_t *mat, const real_t *u, real_t *out);
void fdfk_op_diffz2_pml(int norder, int nx, int nz, int npml, int izt, real_t dz,
                        const double *coef, const real_t *mat, const real_t *u, real_t *out);

double fdfk_op_delta_weight(double x);
void fdfk_op_loadseis(int nx, int nz, int npml, int izt, real_t x0, real_t z0, real_t dx, real_t dz,
                      real_t rx, real_t rz, const real_t *ux, const real_t *uz, real_t *dispx, real_t *dispz);

void fdfk_trace_hook(const char *name, int norder, int nx, int nz, int npml, int izt,
                     const real_t *mat, const real_t *u, real_t *out);
void fdfk_trace_point(int which, const void *caller, int ix, int iz, int dire, real_t d, const real_t *u,
                      real_t val);
void fdfk_trace_post(const char *name, int nx, int nz, int npml, int izt, real_t *out);

#ifdef __cplusplus
}
#endif
#endif
