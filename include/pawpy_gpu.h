/* pawpy_gpu.h -- C ABI of the GB300 band-projection library (libpawpy_gpu.so).
 *
 * Drop-in for the hot path of pawpyseed's C core: the structs below have the
 * binary layout of pawpyseed/core/utils.h:30-166 (the Cython layer reads
 * pswf_t members directly, e.g. pawpyc.pyx:537), and the entry points in
 * section 2 keep the exact names and signatures that pawpyc_extern.pxd
 * declares, so the Cython extension links against this library unchanged:
 * the aug_real path, the aug_recip pair overlap_setup_recip /
 * compensation_terms_recip, and the real-space functions of density.c.
 * Section 3 adds batched entry points, status reporting and host helpers;
 * they use a pawpy_gpu_ prefix so that they never collide with reference
 * symbols.
 *
 * Every computation runs on one CUDA device (the current device when the
 * library first touches a wavefunction); there is no CPU fallback. No entry
 * point aborts the process: on failure a call leaves its outputs unspecified
 * and records a status that pawpy_gpu_last_error() returns (0 = success).
 */
#ifndef PAWPY_GPU_H
#define PAWPY_GPU_H

#include <stddef.h>

#ifdef __cplusplus
#include <complex>
typedef std::complex<double> pawpy_c128;
typedef std::complex<float> pawpy_c64;
extern "C" {
#else
#include <complex.h>
typedef double complex pawpy_c128;
typedef float complex pawpy_c64;
#endif

/* ---------------------------------------------------------------------- */
/* 1. Structs (layout of pawpyseed/core/utils.h:30-166)                    */
/* ---------------------------------------------------------------------- */

typedef struct funcset {
  int l;
  double *proj;
  double **proj_spline;
  double *aewave;
  double **aewave_spline;
  double *pswave;
  double **pswave_spline;
  double *diffwave;
  double **diffwave_spline;
  double *kwave;
  double **kwave_spline;
  double *smooth_diffwave;
  double **smooth_diffwave_spline;
  double *dense_kwave;
  double **dense_kwave_spline;
} funcset_t;

typedef struct ppot {
  int num_projs;
  int total_projs;
  int lmax;
  funcset_t *funcs;
  double rmax;
  double wave_rmax;
  double *pspw_overlap_matrix;
  double *aepw_overlap_matrix;
  double *diff_overlap_matrix;
  int proj_gridsize;
  int wave_gridsize;
  int num_cart_gridpts;
  double *wave_grid;
  double *kwave_grid;
  double *proj_grid;
  double *smooth_grid;
  double *dense_kgrid;
} ppot_t;

typedef struct projection {
  int num_projs;
  int total_projs;
  int *ns;
  int *ls;
  int *ms;
  pawpy_c128 *overlaps;
} projection_t;

typedef struct band {
  int n;
  int num_waves;
  double occ;
  double N;
  double energy;
  pawpy_c64 *Cs;
  pawpy_c128 *CRs;
  pawpy_c64 *CAs;
  projection_t *projections;
  projection_t *up_projections;
  projection_t *down_projections;
  projection_t *wave_projections;
} band_t;

typedef struct rayleigh_set {
  int l;
  pawpy_c128 *terms;
} rayleigh_set_t;

typedef struct kpoint {
  short int up;
  int num_waves;
  int *Gs;
  double *k;
  double weight;
  int num_bands;
  band_t **bands;
  rayleigh_set_t **expansion;
} kpoint_t;

typedef struct pswf {
  double encut;
  int num_elems;
  int *num_projs;
  int num_sites;
  ppot_t *pps;
  int *G_bounds;
  kpoint_t **kpts;
  int nspin;
  int nband;
  int nwk;
  double *lattice;
  double *reclattice;
  int *fftg;
  int is_ncl;
  int wp_num;
  int num_aug_overlap_sites;
  double *dcoords;
  pawpy_c128 **overlaps;
} pswf_t;

typedef struct real_proj {
  int l;
  int m;
  int func_num;
  pawpy_c128 *values;
} real_proj_t;

typedef struct real_proj_site {
  int index;
  int elem;
  int num_projs;
  int total_projs;
  int num_indices;
  int gridsize;
  double rmax;
  double *coord;
  int *indices;
  double *paths;
  real_proj_t *projs;
} real_proj_site_t;

/* ---------------------------------------------------------------------- */
/* 2. Drop-in entry points (names and signatures of pawpyc_extern.pxd)     */
/* ---------------------------------------------------------------------- */

/* Replaces pseudoprojection (pseudoprojector.c:63-90; declared
 * pawpyc_extern.pxd, called pawpyc.pyx:324). projections[b*NK + k] =
 * <C_ref,b,k'|C_proj,BAND_NUM,k> for every basis band b and k = 0..NK-1
 * (NK = nwk*nspin; k' = k with the spins swapped when flip_spin and nspin==2).
 * Overwrites projections. Computed on the device as part of the full
 * basis x defect overlap matrix, which is cached per (wf_ref, wf_proj, flip)
 * so that a loop over BAND_NUM costs one matrix product. */
void pseudoprojection(pawpy_c128 *projections, pswf_t *wf_ref, pswf_t *wf_proj,
                      int BAND_NUM, int flip_spin);

/* Replaces get_projector_list (projector.c:20-171 with
 * make_pwave_overlap_matrices projector.c:507-558 and the spherical Bessel
 * transforms of sbt.c; called pawpyc.pyx:392-395). labels holds 4 ints per
 * element: [label, nproj, ndata, ngrid]. Returns a malloc'd ppot_t[num_els]
 * whose members are laid out and owned as the reference's (freed by
 * free_pswf once setup_projections has attached it). The radial work runs on
 * the device in double precision. */
ppot_t *get_projector_list(int num_els, int *labels, int *ls, double *wave_grids,
                           double *projectors, double *aewaves, double *pswaves,
                           double *rmaxs, double grid_encut);

/* Replaces setup_projections (projector.c:560-602; called pawpyc.pyx:406-410).
 * Attaches pps to wf (takes ownership), builds the augmentation-sphere tables
 * of every site on the device, and computes <p_i|psi> for every band and
 * k-point (batched scatter + 3D FFT + sphere gather). Unless disabled with
 * pawpy_gpu_set_host_projections(0), also fills band->projections as malloc'd
 * projection_t arrays, as the reference does. */
void setup_projections(pswf_t *wf, ppot_t *pps, int num_elems, int num_sites,
                       int *fftg, int *labels, double *coords);

/* Replaces onto_projector (projector.c:333-357): <p_i|psi> of one band from
 * host sphere tables; fills kpt->bands[band_num]->projections. */
void onto_projector(kpoint_t *kpt, int band_num, real_proj_site_t *sites,
                    int num_sites, int *G_bounds, double *lattice,
                    double *reclattice, int num_cart_gridpts, int *fftg);

/* Replaces overlap_setup_real (projector.c:604-725; called pawpyc.pyx:680-683).
 * <(phi-phit)|psi> on the other structure's sites (smoothed partial waves,
 * N_R for wf_S bands and N_S for wf_R bands) and the N_RS pair matrices
 * conj(<(phi-phit)_R|(phi-phit)_S>) with the minimum-image displacements.
 * Empty site lists may be NULL. Sets wf_S->overlaps/dcoords/
 * num_aug_overlap_sites and wp_num as the reference does; wave_projections
 * are filled on the host unless host projections are disabled. */
void overlap_setup_real(pswf_t *wf_R, pswf_t *wf_S, int *labels_R, int *labels_S,
                        double *coords_R, double *coords_S, int *N_R, int *N_S,
                        int *N_RS_R, int *N_RS_S, int num_N_R, int num_N_S,
                        int num_N_RS);

/* Replaces compensation_terms (projector.c:850-963; called pawpyc.pyx:698-702;
 * argument order wf_S = defect, wf_R = basis). Adds O_M + O_R + O_S + O_N of
 * defect band BAND_NUM into overlap[b*NK + k], computed on the device in
 * double precision from the device copies of the projector coefficients. */
void compensation_terms(pawpy_c128 *overlap, int BAND_NUM, pswf_t *wf_S,
                        pswf_t *wf_R, int num_M, int num_N_R, int num_N_S,
                        int num_N_RS, int *M_R, int *M_S, int *N_R, int *N_S,
                        int *N_RS_R, int *N_RS_S, int *proj_labels,
                        double *proj_coords, int *ref_labels, double *ref_coords,
                        int *fft_grid, int flip_spin);

/* Replaces overlap_setup_recip (projector.c:727-848; called pawpyc.pyx:674-678),
 * the setup of the aug_recip method. Same arguments as overlap_setup_real.
 * Instead of real-space smoothed-wave projections it forms the augmentation
 * coefficients CAs of get_aug_freqs (projector.c:276-331, 420-453): for every
 * band of wf_R (sites N_R) and of wf_S (sites N_S), the band's projector
 * coefficients times the smoothed (phi - phit) Y_lm of those sites, spread on
 * the grid and transformed forward (fwd_fft3d, linalg.c:47-79) onto the
 * plane waves -- on the device, in single precision. Also the N_RS pair
 * matrices as overlap_setup_real. band->CAs are filled (malloc'd complex64 in
 * the file's plane-wave order) unless host projections are disabled; they are
 * recomputed for every setup of a pair (the reference keeps the first ones).
 * The overlaps of the pair (compensation_terms_recip, pawpy_gpu_project_all,
 * pawpy_gpu_band_character) then follow the aug_recip method until the next
 * overlap setup of the pair. */
void overlap_setup_recip(pswf_t *wf_R, pswf_t *wf_S, int *labels_R, int *labels_S,
                         double *coords_R, double *coords_S, int *N_R, int *N_S,
                         int *N_RS_R, int *N_RS_S, int num_N_R, int num_N_S,
                         int num_N_RS);

/* Replaces compensation_terms_recip (projector.c:965-1077; called
 * pawpyc.pyx:717-721): adds <CA_R|C_S> + <C_R|CA_S> + O_M + O_N of defect
 * band BAND_NUM into overlap[b*NK + k]. The cross terms come from the
 * device contraction of the pair (precision as pawpy_gpu_set_precision), the
 * O_M and O_N terms in double precision. Needs overlap_setup_recip. */
void compensation_terms_recip(pawpy_c128 *overlap, int BAND_NUM, pswf_t *wf_S,
                              pswf_t *wf_R, int num_M, int num_N_R, int num_N_S,
                              int num_N_RS, int *M_R, int *M_S, int *N_R, int *N_S,
                              int *N_RS_R, int *N_RS_S, int *proj_labels,
                              double *proj_coords, int *ref_labels, double *ref_coords,
                              int *fft_grid, int flip_spin);

/* The 'realspace' method and all-electron densities (density.c; declared
 * pawpyc_extern.pxd:252-262). All-electron wavefunction of band BAND_NUM,
 * k-point KPOINT_NUM (spin-major) on the grid fftg:
 *   x[(i N2 + j) N3 + k] = V^-1/2 sum_G C_G e^{iG.r} e^{2 pi i k.r}
 *     + sum_sites sum_nlm <p_nlm|psi> (phi_nl - phit_nl)(|r-R|)/|r-R| Y_lm e^{2 pi i k.(R+T)}
 * within the last radius of each element's partial-wave grid (realspace_state,
 * density.c:245-310). Computed on the device (single precision grids; double
 * precision sphere tables); the sphere terms of overlapping sites are added in
 * site order. Needs setup_projections on wf; labels/coords are its sites. */
void realspace_state(pawpy_c128 *x, int BAND_NUM, int KPOINT_NUM, pswf_t *wf, int *fftg,
                     int *labels, double *coords);
/* x *= exp(-2 pi i k.r) on the grid fftg (remove_phase, density.c:312-326). */
void remove_phase(pawpy_c128 *x, int KPOINT_NUM, pswf_t *wf, int *fftg);
/* P[i] += |realspace_state|^2 of one band (ae_state_density, density.c:27-37). */
void ae_state_density(double *P, int BAND_NUM, int KPOINT_NUM, pswf_t *wf, int *fftg,
                      int *labels, double *coords);
/* P[i] += sum over k and occupied bands of |psi|^2 * k-weight * occupation *
 * 2 / nspin (ae_chg_density, density.c:158-178); accumulated in double
 * precision on the device. */
void ae_chg_density(double *P, pswf_t *wf, int *fftg, int *labels, double *coords);
/* projs[b*NK + k] = <psi_R,b,k|psi_S,BAND_NUM,k> of the all-electron
 * real-space wavefunctions on fftg: the grid sum times V/N^3
 * (project_realspace_state, density.c:206-243), the contraction in the
 * overlap precision (pawpy_gpu_set_precision). wf = S (its sites labels/
 * coords), wf_R = R (labels_R/coords_R). */
void project_realspace_state(pawpy_c128 *projs, int BAND_NUM, pswf_t *wf, pswf_t *wf_R,
                             int *fftg, int *labels, double *coords, int *labels_R,
                             double *coords_R);

/* Replaces fft3d (linalg.c:14-45; called from C only). x[i*N2*N3 + j*N3 + k] =
 * V^-1/2 sum_w Cs[w] exp(2 pi i (g1 i/N1 + g2 j/N2 + g3 k/N3)). The transform
 * runs on the device in single precision (|error| well below the 1e-5 that
 * the reference's fft_check allows, tests.c:61). */
void fft3d(pawpy_c128 *x, int *G_bounds, double *lattice, double *kpt, int *Gs,
           pawpy_c64 *Cs, int num_waves, int *fftg);

/* ---------------------------------------------------------------------- */
/* 3. Library extensions (no counterpart in the reference)                 */
/* ---------------------------------------------------------------------- */

enum pawpy_gpu_precision {
  PAWPY_GPU_FP32 = 0,   /* complex FP32 overlap GEMM on the CUDA cores */
  PAWPY_GPU_BF16X3 = 1, /* split-BF16 (3 terms) on the tensor cores, FP32 accumulate */
  PAWPY_GPU_TF32 = 2    /* TF32 tensor cores, FP32 accumulate (reported variant) */
};

/* Status of the last entry point called on this thread: 0 on success. */
int pawpy_gpu_last_error(void);
/* Human-readable message for the last failure on this thread ("" if none). */
const char *pawpy_gpu_error_string(void);
/* Clears the recorded status. */
void pawpy_gpu_clear_error(void);

/* Overlap precision for the device overlap matrices (default FP32). */
void pawpy_gpu_set_precision(int precision);
int pawpy_gpu_get_precision(void);
/* K split of the tensor-core overlap contraction (0 = chosen with the tile
 * width, the default). No counterpart in the reference. */
void pawpy_gpu_set_tc_splits(int splits);
/* Tile width of the tensor-core overlap contraction: 128 or 64 defect bands
 * per tile (64: two CTAs per SM, for few defect bands), or 0 (the default) to
 * time the candidate widths and split counts once per problem shape and keep
 * the fastest (PAWPY_GPU_TUNE_VERBOSE=1 prints each decision). No counterpart
 * in the reference. */
void pawpy_gpu_set_tc_tile(int bn);
/* Form of the sphere contraction (the projections <p|psi> of
 * onto_projector_helper, projector.c:223-274): 1 (the default) on the tensor
 * cores (split-BF16) whenever the precision is a tensor-core one, FP32 CUDA
 * cores otherwise; 0 always the FP32 CUDA-core form; 2 always the tensor-core
 * form. No counterpart in the reference. */
void pawpy_gpu_set_sphere_contraction(int mode);

/* Batched overlap matrices of host arrays, no counterpart in the reference
 * (pseudoprojection's contraction, pseudoprojector.c:63-90, on raw matrices):
 * for z < nz, out[z][n][m] = sum_k conj(A_z[m][k]) B_z[n][k] with A_z of
 * M x K[z] and B_z of N x K[z], each row-major and packed one batch after
 * the other; out is nz x N x M. precision is a pawpy_gpu_precision. Returns
 * 0, or -1 with the status set. */
int pawpy_gpu_overlap_matrix(const pawpy_c64 *A, const pawpy_c64 *B, int M, int N, int nz, const int *K,
                             pawpy_c64 *out, int precision);

/* Whether get_projector_list keeps its results per exact input (default 1:
 * requests with the same species and grid share the element setup, as a
 * resident basis does; a deep copy is returned every call). With 0 every call
 * runs the whole element setup, as the reference does. */
void pawpy_gpu_set_element_cache(int on);

/* Whether setup_projections / overlap_setup_real also fill the host
 * projection_t arrays (default 1, as the reference). */
void pawpy_gpu_set_host_projections(int on);

/* Full PAW overlap matrix of every defect band against every basis band:
 * out[bS*(NB_R*NK) + bR*NK + k] = single_band_projection(bS)[bR*NK + k],
 * i.e. pseudo overlap plus O_M + O_R + O_S + O_N, computed as one augmented
 * overlap contraction per k-point. Needs setup_projections on both and
 * overlap_setup_real with the same site lists. Returns 0 on success. */
int pawpy_gpu_project_all(pawpy_c128 *out, pswf_t *wf_R, pswf_t *wf_S, int num_M,
                          int num_N_R, int num_N_S, int num_N_RS, int *M_R,
                          int *M_S, int *N_R, int *N_S, int *N_RS_R, int *N_RS_S,
                          int flip_spin);

/* Band character of every defect band, from the full overlap matrix that
 * pawpy_gpu_project_all forms, without moving the matrix to the host: the
 * reductions of Projector.proportion_conduction (projector.py:384-435) for all
 * bands at once. With S[bS][bR*NK + k] that matrix (k = s*nwk + kk),
 *   v[bS*nch + ch] = sum over bR and the k of channel ch of |S|^2 w_v[bR*NK + k]
 * and c likewise with w_c. nch = 1 sums every k; nch = 2 gives the two spins
 * separately (k < nwk is spin 0). The weights (occupations or their complement,
 * k-point weights) come from the caller. Same prerequisites as
 * pawpy_gpu_project_all. Returns 0 on success. */
int pawpy_gpu_band_character(double *v, double *c, pswf_t *wf_R, pswf_t *wf_S, int num_M,
                             int num_N_R, int num_N_S, int num_N_RS, int *M_R, int *M_S,
                             int *N_R, int *N_S, int *N_RS_R, int *N_RS_S, const double *w_v,
                             const double *w_c, int nch, int flip_spin);

/* Noncollinear all-electron real-space wavefunction (ncl_realspace_state, density.c:328-408):
 * x receives the up then the down spinor component, 2 N1 N2 N3 complex values, each the
 * collinear realspace_state of its half with its own projections (up_projections,
 * down_projections). Replaces ncl_realspace_state (pawpyc_extern.pxd:257). */
void ncl_realspace_state(pawpy_c128 *x, int BAND_NUM, int KPOINT_NUM, pswf_t *wf, int *fftg, int *labels,
                         double *coords);
/* Noncollinear all-electron charge density (ncl_ae_chg_density, density.c:181-204): P +=
 * sum over occupied bands of (|psi_up|^2 + |psi_down|^2) weight occupation. Replaces
 * ncl_ae_chg_density (pawpyc_extern.pxd:260). The collinear real-space functions report
 * status 5 for a noncollinear wavefunction, as these do for a collinear one. */
void ncl_ae_chg_density(double *P, pswf_t *wf, int *fftg, int *labels, double *coords);
/* project_realspace_state for every band of wf at once: out[bS*(NB_R*NK) +
 * bR*NK + k], one contraction per k-point. No counterpart in the reference.
 * Returns 0, or the status. */
int pawpy_gpu_project_realspace_all(pawpy_c128 *out, pswf_t *wf, pswf_t *wf_R, int *fftg, int *labels,
                                    double *coords, int *labels_R, double *coords_R);

/* WAVECAR reader producing a pswf_t with the reference's layout and VASP plane-
 * wave order (reader.c:129-315 semantics); free with pawpy_gpu_free_pswf.
 * Replaces read_wavefunctions (reader.c:317-322). The plane-wave spheres of all
 * k-points are enumerated in one device launch where a CUDA device is present
 * (on the host threads otherwise), while the coefficient records are read in
 * parallel straight into the bands' arrays. */
pswf_t *pawpy_gpu_read_wavefunctions(const char *filename, const double *kpt_weights);
/* The same from the bytes of a WAVECAR in memory (an inflated .gz or .bz2 file,
 * pawpyc.pyx:217-222). Replaces read_wavefunctions_from_str (reader.c:324-329),
 * which has no length argument: the header's record length and counts bound the
 * reads. */
pswf_t *pawpy_gpu_read_wavefunctions_from_str(const char *start, const double *kpt_weights);
/* As pawpy_gpu_read_wavefunctions_from_str with the buffer's length: a record
 * past len is an error (status 4) instead of a read past the buffer. */
pswf_t *pawpy_gpu_read_wavefunctions_from_bytes(const char *data, size_t len, const double *kpt_weights);
/* The plane-wave sphere of one k-point (kpt in reciprocal-lattice units) of a
 * cell (lattice rows, A) at ENCUT (eV), enumerated on the device in VASP order
 * (reader.c:230-271): writes the int triples to out (3*cap ints; out may be NULL
 * to count) and returns their number, or -1 (status 5 without a CUDA device). */
int pawpy_gpu_gvectors(const double *lattice, const double *kpt, double encut, int *out, int cap);
/* Builds a pswf_t from in-memory arrays: Gs[iwk] int32[3*nplane[iwk]] and
 * Cs[iwk] complex64[nband*nplane[iwk]] for iwk = spin*nwk + k. Copies them.
 * is_ncl: noncollinear (spinor) coefficients; nplane counts both halves (up
 * then down) and Gs holds the nplane/2 vectors of one half. */
pswf_t *pawpy_gpu_wavefunction_from_arrays(int nspin, int nwk, int nband, double encut,
                                           const double *lattice, const double *kpts,
                                           const double *weights, const int *nplane,
                                           const int *const *Gs, const pawpy_c64 *const *Cs,
                                           const double *energies, const double *occs, int is_ncl);
/* Frees a pswf_t and everything attached to it (also releases its device copy). */
void pawpy_gpu_free_pswf(pswf_t *wf);
/* Frees an element array returned by get_projector_list that was not handed
 * to setup_projections (free_ppot_list, utils.h:248, under a library name). */
void pawpy_gpu_free_ppot_list(ppot_t *pps, int length);
/* Releases the device copy of a wavefunction (call before a foreign free). */
void pawpy_gpu_release(pswf_t *wf);
/* Makes the device copy of a wavefunction's coefficients resident now. */
int pawpy_gpu_upload(pswf_t *wf);

/* No counterpart in the reference. Overlap contraction for callers that cannot
 * allocate device memory (a process whose device memory belongs to another
 * allocator or a fixed up-front budget, or a loop that must not pay the device
 * synchronisation of cudaMalloc/cudaFree):
 *   out[n*M + m] = sum_{k<K} conj(A[m*lda + k]) * B[n*ldb + k]
 * on caller-owned device buffers (complex64, A/B 16-byte aligned, lda/ldb even
 * and >= K, K a multiple of 16 with zero padding) -- the contraction of
 * pseudoprojection in its plain FP32 form: FP32 accumulation on the CUDA
 * cores, split-K partial sums reduced in a fixed order. Its error against FP64
 * grows with K for coherent sums: a unit-norm band against itself over K =
 * 78,517 plane waves is off by up to 4.8e-5 (random-phase overlaps by ~3e-7);
 * the split-BF16 form of pawpy_gpu_project_all stays under 1e-5.
 * It allocates nothing: the partial sums live in a static device array of
 * 32 MiB that every GPU loading the library holds until exit; outputs larger
 * than M*N = 4,194,304 values are rejected. The first call on each device
 * sets up that device (looks up the array's device address and the SM count;
 * with lazy module loading it also loads the module, which reserves the
 * 32 MiB then), so a caller with a fixed memory budget makes it early, and
 * before any stream capture. The address is kept for the process: a
 * cudaDeviceReset invalidates it. Calls share the array, so calls whose work
 * overlaps on the GPU (e.g. on different streams) race and may leave wrong
 * values in each other's outputs (each call writes only its own out).
 * stream: a cudaStream_t, or NULL for the library's stream; the call is
 * asynchronous. Returns the split count used (>= 1) or a negative status. */
int pawpy_gpu_overlap_noalloc(const pawpy_c64 *A, long long lda, const pawpy_c64 *B, long long ldb,
                              int M, int N, int K, pawpy_c64 *out, void *stream);

/* Uploads a wavefunction that setup_projections has seen and computes its
 * projector coefficients, so that it can serve as a shared, read-only basis
 * for work on several threads. With keep_real_space, its real-space
 * wavefunctions stay on the device too (nk nband N1 N2 N3 complex64) and
 * later projections of it onto new sites gather from them instead of
 * transforming again. No counterpart in the reference. Returns 1 when the
 * real-space wavefunctions are resident, 0 when not, -1 with the status set on
 * failure. */
int pawpy_gpu_prepare_basis(pswf_t *wf, int keep_real_space);

/* Projection server: requests (a defect wavefunction against a resident
 * basis) run on `slots` worker threads, each on its own CUDA stream, and are
 * admitted first-in first-out when a worker is free and their estimated device
 * memory fits the budget. A request's work is the sequence setup_projections,
 * overlap_setup_real, pawpy_gpu_project_all; the server owns the request's
 * wavefunction and element array from submission (it frees both) and writes
 * the nband_S x (nband_R nk) result to `out` before the request completes.
 * No counterpart in the reference. */
typedef struct pawpy_gpu_request {
  int basis;                 /* index from pawpy_gpu_server_add_basis */
  pswf_t *wf;                /* defect wavefunction (owned by the server) */
  ppot_t *pps;               /* its element array from get_projector_list (owned by the server) */
  int num_elems, num_sites;
  const int *fftg;           /* [3] */
  const int *labels;         /* [num_sites] */
  const double *coords;      /* [3 num_sites] fractional */
  int num_M, num_N_R, num_N_S, num_N_RS;
  const int *M_R, *M_S, *N_R, *N_S, *N_RS_R, *N_RS_S;
  pawpy_c128 *out;           /* [nband_S][nband_R nk], kept alive by the caller until completion */
} pawpy_gpu_request_t;

void *pawpy_gpu_server_create(long long hbm_budget_bytes, int slots);
/* Registers a basis (setup_projections done; labels and coords of its sites);
 * prepares it (pawpy_gpu_prepare_basis with keep_real_space). Returns its
 * index or -1. */
int pawpy_gpu_server_add_basis(void *server, pswf_t *basis, const int *labels, const double *coords,
                               int num_sites, int keep_real_space);
/* Queues a request (arrays copied); returns its id or -1. */
long long pawpy_gpu_server_submit(void *server, const pawpy_gpu_request_t *request);
/* Waits for request id; returns 0 on success or its error code (message in
 * msg, up to msg_len bytes). times_ms (may be NULL, else 7 values) receives
 * queue, run and total (submission to completion) milliseconds, then the run's
 * setup_projections, overlap_setup_real, pawpy_gpu_project_all and release
 * parts; est_bytes the admission estimate. */
int pawpy_gpu_server_wait(void *server, long long id, double *times_ms, long long *est_bytes, char *msg,
                          int msg_len);
/* Requests completed, running, queued; peak estimated bytes in flight. */
void pawpy_gpu_server_counts(void *server, long long *done, int *running, int *queued, long long *peak_bytes);
/* Waits for every request, stops the workers and frees the server. */
void pawpy_gpu_server_destroy(void *server);

/* Orders the calling thread's library work on a CUDA stream of its own (on = 1)
 * or on the library's shared stream again (on = 0, after waiting for it), so
 * that several host threads keep independent work in flight on the device
 * (different wavefunctions per thread; a basis shared by threads must have
 * been prepared before, pawpy_gpu_prepare_basis). No counterpart in the
 * reference. Returns 0, or -1 with the status set. */
int pawpy_gpu_thread_stream(int on);

/* Device-side timing on the library's stream (CUDA events). */
void pawpy_gpu_timer_start(void);
float pawpy_gpu_timer_stop_ms(void); /* synchronizes */
void pawpy_gpu_synchronize(void);
/* Host-side check of the library's worker pool (no device work): `callers`
 * threads each run a loop of n items through it at once, then a loop whose item
 * 1 throws. Returns the number of items not run exactly once plus the loops
 * whose exception was not passed back (0 = correct), or -1 on a bad argument. */
int pawpy_gpu_host_pool_check(int callers, int n);
/* Kernels launched by this library since the counter was last reset. */
long long pawpy_gpu_launch_count(int reset);
/* Per-kernel-family device time: enables CUDA-event bracketing of launches;
 * pawpy_gpu_kernel_stats writes "name ms launches first last work\n" lines into
 * buf (first start and last end of the family's launches, or of the host phase
 * "host.<name>", in ms after profiling was switched on; work: the algorithmic
 * bytes the launches declared -- 8 N1 N2 N3 per band and FFT pass, 8 per picked
 * value read by the sphere contraction -- or, for the overlap contractions,
 * their useful flops, 8 M N K per batch). */
void pawpy_gpu_profile(int on);
int pawpy_gpu_kernel_stats(char *buf, int len, int reset);
/* Bytes of device memory the library holds. */
long long pawpy_gpu_device_bytes(void);
/* Whether the current device reads pageable host memory coherently (bit 0:
 * cudaDevAttrPageableMemoryAccess, bit 1: ...UsesHostPageTables); -1 on error. */
int pawpy_gpu_pageable_memory_access(void);
/* Byte offset / size of each struct member, for layout checks:
 * writes "struct member offset\n" lines; returns the length needed. */
int pawpy_gpu_struct_layout(char *buf, int len);

#ifdef __cplusplus
}
#endif
#endif
