// Host-side declarations shared by the translation units of libpawpy_gpu.
#pragma once

#include <cmath>
#include <cstddef>
#include <vector>

#include "common.h"

namespace pawpy {

// --- wavefunction files and ownership (host_wavecar.cpp) ---
double det3(const double *m);
void reciprocal(const double *lat, double *rec);
// hbar^2/2m in eV A^2, the reader's c (reader.c:11)
constexpr double kGsphereC = 0.262465831;
// nb{1,2,3}max of reader.c:55-127 (kept in double precision)
void gsphere_bounds(const double *rec, double encut, double nb[3]);
// The reader's cutoff test of one plane wave k + g (reader.c:243-251), in its
// order of operations: |s| = pow(s.s, 0.5), pow(|s|, 2.0) / c <= ENCUT.
inline bool gsphere_keep(const double *rec, const double *k, int g1, int g2, int g3, double encut) {
  double s[3];
  for (int j = 0; j < 3; j++) s[j] = (k[0] + g1) * rec[j] + (k[1] + g2) * rec[3 + j] + (k[2] + g3) * rec[6 + j];
  const double g = std::pow(s[0] * s[0] + s[1] * s[1] + s[2] * s[2], 0.5);
  return std::pow(g, 2.0) / kGsphereC <= encut;
}
// The plane-wave list of one k-point in VASP order (int triples), on the host.
std::vector<int> enumerate_gvectors(const double *rec, const double *k, double encut);
// The lists of nk k-points (kpts [nk][3]); on the device where a CUDA device is
// present (gsphere.cu), on the host threads otherwise.
std::vector<std::vector<int>> gsphere_lists(const double *rec, double encut, const double *kpts, int nk);
// Whether the process sees a CUDA device.
bool device_present();
pswf_t *read_wavecar(const char *path, const double *kws);
// The same from the bytes of a WAVECAR in memory; len = SIZE_MAX when the
// caller does not know it (read_wavefunctions_from_str, reader.c:324-329).
pswf_t *read_wavecar_bytes(const char *data, size_t len, const double *kws);
pswf_t *pswf_from_arrays(int nspin, int nwk, int nband, double encut, const double *lattice,
                         const double *kpts, const double *weights, const int *nplane,
                         const int *const *Gs, const pawpy_c64 *const *Cs, const double *energies,
                         const double *occs, int is_ncl);
void free_pswf_all(pswf_t *wf);
void free_ppot_array(ppot_t *pps, int n);
void free_wave_projections(pswf_t *wf);

// --- radial setup (host_radial.cpp) ---
// Cubic spline coefficients in the reference's convention (utils.c:699-749):
// b, c, d such that f(x) = y_i + t(b_i + t(c_i + t d_i)), t = x - x_i.
void spline_coeffs(const double *x, const double *y, int n, double *b, double *c, double *d);
double spline_integral(const double *x, const double *y, const double *b, const double *c,
                       const double *d, int n);
double interp_log(double r, int n, const double *x, const double *f, double *const *s);
// w with spline_integral(x, y, spline(y)) = sum_i w_i y_i (the integral is linear in y)
void spline_integral_weights(const double *x, int n, double *w);
// get_projector_list served from a cache of earlier results with identical
// inputs (a deep copy the caller owns), computed by device_projector_list otherwise
// Whether get_projector_list keeps its results per exact input (on by default);
// off, every call runs the whole element setup.
void set_projector_list_cache(bool on);
ppot_t *cached_projector_list(int num_els, const int *labels, const int *ls, const double *wave_grids,
                              const double *projectors, const double *aewaves, const double *pswaves,
                              const double *rmaxs, double grid_encut);
// get_projector_list on the device (radial.cu)
ppot_t *device_projector_list(int num_els, const int *labels, const int *ls, const double *wave_grids,
                              const double *projectors, const double *aewaves, const double *pswaves,
                              const double *rmaxs, double grid_encut);
// conj(<(phi-phit)_1 lm | (phi-phit)_2 l'm'>) matrix of one site pair
// (reciprocal_offsite_wave_overlap, radial.c:116-196), row-major [P1 x P2],
// from its radial integrals I[f1][f2][L] (L <= Lmax).
void offsite_pair_matrix(const ppot_t *pp1, const ppot_t *pp2, const double *dcoord, const double *I,
                         int Lmax, pawpy_c128 *out);
double pair_distance(const double *dcoord);
// ppot_t.num_cart_gridpts of add_num_cart_gridpts (projector.c:455-505)
int cart_gridpts_bound(const ppot_t &pp, const double *lattice, const int *fftg);
// I[p][f1][f2][L] = int f1(k) f2(k) k^2 j_L(k R_p) dk of every pair on the device (radial.cu)
void offsite_radial_integrals(const ppot_t *ppR, const ppot_t *ppS, const std::vector<int> &eR,
                              const std::vector<int> &eS, const std::vector<double> &R,
                              std::vector<std::vector<double>> &I, std::vector<int> &Lmax);
// Minimum-image Cartesian path coord - center (utils.c:51-73).
void min_image_path(const double *coord, const double *center, const double *lattice, double *path,
                    double *r);

// --- device mirror lifetime (engine.cu) ---
void release_device(pswf_t *wf);

}  // namespace pawpy
