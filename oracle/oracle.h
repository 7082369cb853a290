/*
 * oracle.h -- CPU restatement of the GMlib mesh-kernel path (test
 * infrastructure: the checker, never part of the library).
 */
#ifndef ORACLE_H
#define ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

int    orc_ver_tet_ball(int nv, int nt, const int *tet, int BalSiz, int MaxSiz,
                        int *deg, int *MaxPos, int *HghSiz, int *base, int *high);
int    orc_tet_edges(int nt, const int *tet, int *edges);
double orc_quality_ref1(const float *crd, const int *t);
void   orc_quality_ref(int nt, const float *crd, const int *tet, double *q);
double orc_mean_ratio1(const float *crd, const int *t);
void   orc_mean_ratio(int nt, const float *crd, const int *tet, double *q);
double orc_det1(const float *crd, const int *t);
double orc_reduce(int op, int n, const float *x);
void   orc_minmax_arg(int n, const double *x, double *vmin, int *imin, double *vmax, int *imax);
void   orc_scatter(int nt, const float *crd, const int *tet, double *opt);
void   orc_gather(int nv, const float *crd, const int *deg, const int *ball, int width,
                  const double *opt, double *newcrd, double *res);

/* oracle_mesh.c */
long long orc_point_ball(int nv, int nt, const int *tet, const int *fixed,
                         long long *ptr, int *col, long long cap);
void   orc_boundary_vertices(int nv, int nt, const int *tet, int *fixed);
void   orc_laplace(int nv, double *crd, const long long *ptr, const int *col, double w, int nsweeps);
void   orc_quality_stats(int nt, const float *crd, const int *tet, double *q, unsigned *hist,
                         unsigned *flags, unsigned *ninv);

/* oracle_linalg.c */
void   orc_bsr_spmv(int nrow, int b, const int *lin, const int *col, const double *val,
                    const double *x, double *y);
double orc_rel_residual(int nrow, int b, const int *lin, const int *col, const double *val,
                        const double *rhs, const double *x);
int    orc_cg(int nrow, int b, const int *lin, const int *col, const double *val,
              const double *rhs, double *x, double tol, int maxit);

double orc_p2_quality1(const double ver[4][3], const double mid[6][3]);
void   orc_p2_quality(int nt, const int *tet, const int *tedg, const float *crd,
                      const float *mid, double *q);

#ifdef __cplusplus
}
#endif

#endif
