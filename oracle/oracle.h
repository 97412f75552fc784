/* TEST INFRASTRUCTURE -- the oracle (checker) for the band-projection path.
 *
 * A CPU restatement, in plain C with OpenMP, of the reference pawpyseed
 * algorithm (the C sources of pawpyseed/core). Only the tests, the smoke
 * check and the CPU baseline leg of bench.py use it; the product library
 * never links it.
 * Every function cites the reference lines it follows. All arithmetic is
 * double precision; pseudo overlaps can also be accumulated in single
 * precision to mimic the reference's cblas_cdotc_sub. */
#ifndef PAWPY_ORACLE_H
#define PAWPY_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- radial helpers (utils.c:699-764, 461-489, 377-448) ---- */
void oracle_spline_coeff(const double *x, const double *y, int n, double *b,
                         double *c, double *d);
double oracle_spline_integral(const double *x, const double *a, const double *b,
                              const double *c, const double *d, int n);
double oracle_legendre(int l, int m, double x);
void oracle_ylm(int l, int m, double theta, double phi, double *re, double *im);

/* ---- spherical Bessel transform (sbt.c:24-215, Talman's NumSBT) ---- */
/* Fills ks[n] (reciprocal grid) and returns nothing; transform of r*f (n pts). */
void oracle_sbt_forward(double encut, int lmax, int n, const double *r,
                        const double *f, int l, double *ks, double *out);
void oracle_sbt_inverse(double encut, int lmax, int n, const double *r,
                        const double *fk, int l, double *out);

/* ---- species setup (projector.c:20-171, 507-558) ----
 * Inputs: ls[nproj], proj[nproj*ndata] on rmax*j/ndata, ae/ps[nproj*ngrid]
 * (r*phi) on wave_grid[ngrid]. Outputs (caller allocated):
 *   proj_grid[ndata], proj_spl[nproj*3*ndata]      (b,c,d per function)
 *   smooth_grid[ndata], sdw[nproj*ndata], sdw_spl[nproj*3*ndata]
 *   kgrid[ngrid], kwave[nproj*ngrid], kwave_spl[nproj*3*ngrid]
 *   aeov/psov/diov[nproj*nproj] */
void oracle_species_setup(int nproj, const int *ls, int ndata, int ngrid,
                          double rmax, const double *wave_grid,
                          const double *proj, const double *ae, const double *ps,
                          double grid_encut, double *proj_grid, double *proj_spl,
                          double *smooth_grid, double *sdw, double *sdw_spl,
                          double *kgrid, double *kwave, double *kwave_spl,
                          double *aeov, double *psov, double *diov);

/* ---- sphere tables (utils.c:590-696) ----
 * One site (of element with functions f[nproj*size] + spl on grid x[size],
 * real radius rmax used for both R0 and interpolation) centred at frac
 * coord[3]; r0_size is the proj_gridsize the reference reads through
 * pps[labels[s]] for the cutoff denominator. Writes up to cap points:
 * indices[cap], paths[3*cap], values[cap*total] (complex pairs, point-major:
 * values[2*(pt*total+p)]). Returns the point count, or -1 if it exceeds cap. */
int oracle_site_table(const double *lattice, const int *fftg, const double *coord,
                      double rmax, int size, int r0_size, const double *x,
                      int nproj, const int *ls, const double *f, const double *spl,
                      int cap, int *indices, double *paths, double *values);

/* ---- fft3d (linalg.c:14-45) ---- */
void oracle_fft3d(double *x, const int *Gs, const float *Cs, int nw,
                  const int *fftg, double vol);

/* ---- projections for many bands (projector.c:223-274, 333-357, 394-418) ----
 * For each band b in [0,nb): FFT of Cs[b*stride .. ) with Gs and gather onto
 * the given site tables: out[(b*ntot) + off_s + p] = sum_i conj(v)*x*dv*e^{ik.path}.
 * Sites are described by flat arrays (npts[s], toff[s] into indices/paths,
 * voff[s] into values (complex), total[s], ooff[s] into out). OpenMP over b. */
void oracle_project_bands(int nb, const float *Cs, long stride, const int *Gs,
                          int nw, const int *fftg, const double *lattice,
                          const double *kcart, int nsites, const int *npts,
                          const long *toff, const long *voff, const int *total,
                          const int *ooff, int ntot, const int *indices,
                          const double *paths, const double *values, double *out);

/* ---- off-site partial-wave overlap (radial.c:116-196) ---- */
void oracle_aug_coefficients(int nb, const double *P, long pstride, const int *pcol, const int *Gs, int nw,
                             const int *fftg, const double *L, const double *kcart, int nsites,
                             const int *npts, const long *toff, const long *voff, const int *total,
                             const int *indices, const double *paths, const double *values, double *out);
void oracle_offsite(const double *dcoord, const double *k1, const double *f1,
                    const double *s1, int size1, const double *k2, const double *f2,
                    const double *s2, int size2, int l1, int m1, int l2, int m2,
                    const double *sbtfacs, double *re, double *im);
void oracle_offsite_matrix(const double *dc, const double *k1, const double *f1, const double *s1,
                           int size1, int T1, const int *n1, const int *l1, const int *m1,
                           const double *k2, const double *f2, const double *s2, int size2, int T2,
                           const int *n2, const int *l2, const int *m2, const double *sbtfacs,
                           double *out);

/* ---- pseudoprojection, all S bands (pseudoprojector.c:63-90) ----
 * out[(bS*nbR + bR)] = sum_w conj(CR[bR][w]) CS[bS][w] for one k; fp32 != 0
 * accumulates in float like the reference's cblas_cdotc_sub. OpenMP over bR. */
void oracle_pseudo_k(int nbR, int nbS, int nw, const float *CR, long strideR,
                     const float *CS, long strideS, int fp32, double *out);

#ifdef __cplusplus
}
#endif
#endif
