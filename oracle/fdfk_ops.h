/*
 * ORACLE (test infrastructure only).  Restatement of the open FD operators of
 * FDFK2D src/Submain.f90; see fdfk_ops.c.
 */
#ifndef FDFK_ORACLE_OPS_H
#define FDFK_ORACLE_OPS_H

#ifdef __cplusplus
extern "C" {
#endif

void fdfk_op_fd_coef0(int norder, double *coef);
void fdfk_op_fd_coef1(int norder, double *coef);
void fdfk_op_fd_coef2(int norder, double *coef);
float fdfk_op_dt_stable(int nx, int nz, int npml, int izt, int norder, float dx, float dz,
                        const double *coef2, const float *c);

float fdfk_op_diff1(int norder, int dire, int nx, int nz, int npml, int izt, int ix, int iz,
                    float d, const double *coef, const float *u);
float fdfk_op_diffx1(int norder, int nx, int npml, int ix, float dx, const double *coef, const float *u);

void fdfk_op_diffzx_reg(int norder, int nx, int nz, int npml, int izt, float dx, float dz,
                        const double *coef, const float *mat, const float *u, float *out);
void fdfk_op_diffzx_pml(int norder, int nx, int nz, int npml, int izt, float dx, float dz,
                        const double *coef, const float *mat, const float *u, float *out);
void fdfk_op_diffxz_reg(int norder, int nx, int nz, int npml, int izt, float dx, float dz,
                        const double *coef, const float *mat, const float *u, float *out);
void fdfk_op_diffxz_pml(int norder, int nx, int nz, int npml, int izt, float dx, float dz,
                        const double *coef, const float *mat, const float *u, float *out);
void fdfk_op_diffx2_reg(int norder, int nx, int nz, int npml, int izt, float dx,
                        const double *coef, const float *mat, const float *u, float *out);
void fdfk_op_diffx2_pml(int norder, int nx, int nz, int npml, int izt, float dx,
                        const double *coef, const float *mat, const float *u, float *out);
void fdfk_op_diffz2_reg(int norder, int nx, int nz, int npml, int izt, float dz,
                        const double *coef, const float *mat, const float *u, float *out);
void fdfk_op_diffz2_pml(int norder, int nx, int nz, int npml, int izt, float dz,
                        const double *coef, const float *mat, const float *u, float *out);

double fdfk_op_delta_weight(double x);
void fdfk_op_loadseis(int nx, int nz, int npml, int izt, float x0, float z0, float dx, float dz,
                      float rx, float rz, const float *ux, const float *uz, float *dispx, float *dispz);

void fdfk_trace_hook(const char *name, int norder, int nx, int nz, int npml, int izt,
                     const float *mat, const float *u, float *out);
void fdfk_trace_point(int which, const void *caller, int ix, int iz, int dire, float d, const float *u,
                      float val);
void fdfk_trace_post(const char *name, int nx, int nz, int npml, int izt, float *out);

#ifdef __cplusplus
}
#endif
#endif
