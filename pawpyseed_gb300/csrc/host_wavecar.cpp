// Host side of libpawpy_gpu: WAVECAR reading into pswf_t, construction from
// arrays, and freeing with the reference's ownership rules.
//
// The WAVECAR record layout and the plane-wave order are properties of the
// file format; they follow the reference reader (pawpyseed/core/reader.c):
// reciprocal lattice with 2*pi and the double-valued bounds nb{1,2,3}max
// (reader.c:55-127), header records (reader.c:129-221), the G loop ig3 outer,
// ig2, ig1 inner with the wrap ig -> ig - 2*nbmax - 1 evaluated in double and
// truncated (reader.c:230-271), the noncollinear doubling (reader.c:274-284).
// Every member is allocated with malloc/calloc so that the reference's
// free_pswf (utils.c:275-301) and pawpy_gpu_free_pswf release the same objects.
#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <cerrno>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "common.h"
#include "host.h"

namespace pawpy {

static const double kC = kGsphereC;

static void cross(const double *a, const double *b, double *o) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}
static double dot3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static double norm3(const double *a) { return std::pow(dot3(a, a), 0.5); }

double det3(const double *m) {
  return m[0] * m[4] * m[8] + m[1] * m[5] * m[6] + m[2] * m[3] * m[7] - m[2] * m[4] * m[6] -
         m[1] * m[3] * m[8] - m[0] * m[5] * m[7];
}

void reciprocal(const double *lat, double *rec) {
  cross(lat + 3, lat + 6, rec + 0);
  cross(lat + 6, lat + 0, rec + 3);
  cross(lat + 0, lat + 3, rec + 6);
  double v = det3(lat);
  for (int i = 0; i < 9; i++) rec[i] *= 2.0 * M_PI / v;
}

void gsphere_bounds(const double *rec, double encut, double nb[3]) {
  const double *b1 = rec, *b2 = rec + 3, *b3 = rec + 6;
  double m1 = norm3(b1), m2 = norm3(b2), m3 = norm3(b3);
  double kc = std::pow(encut * kC, 0.5), v[3];
  double p12 = std::acos(dot3(b1, b2) / (m1 * m2));
  cross(b1, b2, v);
  double s123 = dot3(b3, v) / (norm3(v) * m3);
  double A[3] = {kc / (m1 * std::fabs(std::sin(p12))) + 1, kc / (m2 * std::fabs(std::sin(p12))) + 1,
                 kc / (m3 * std::fabs(s123)) + 1};
  double p13 = std::acos(dot3(b1, b3) / (m1 * m3));
  cross(b1, b3, v);
  s123 = dot3(b2, v) / (norm3(v) * m2);
  double B[3] = {kc / (m1 * std::fabs(std::sin(p13))) + 1, kc / (m2 * std::fabs(s123)) + 1,
                 kc / (m3 * std::fabs(std::sin(p13))) + 1};
  double p23 = std::acos(dot3(b3, b2) / (m3 * m2));
  cross(b2, b3, v);
  s123 = dot3(b1, v) / (norm3(v) * m1);
  double Cc[3] = {kc / (m1 * std::fabs(s123)) + 1, kc / (m2 * std::fabs(std::sin(p23))) + 1,
                  kc / (m3 * std::fabs(std::sin(p23))) + 1};
  for (int i = 0; i < 3; i++) nb[i] = std::fmax(A[i], std::fmax(B[i], Cc[i]));
}

// The plane-wave list of one k-point in VASP order; returns int triples.
std::vector<int> enumerate_gvectors(const double *rec, const double *k, double encut) {
  double nb[3];
  gsphere_bounds(rec, encut, nb);
  std::vector<int> out;
  for (int i3 = 0; i3 <= 2 * nb[2]; i3++) {
    int g3 = i3 > nb[2] ? (int)(i3 - 2 * nb[2] - 1) : i3;
    for (int i2 = 0; i2 <= 2 * nb[1]; i2++) {
      int g2 = i2 > nb[1] ? (int)(i2 - 2 * nb[1] - 1) : i2;
      for (int i1 = 0; i1 <= 2 * nb[0]; i1++) {
        int g1 = i1 > nb[0] ? (int)(i1 - 2 * nb[0] - 1) : i1;
        if (gsphere_keep(rec, k, g1, g2, g3, encut)) {
          out.push_back(g1);
          out.push_back(g2);
          out.push_back(g3);
        }
      }
    }
  }
  return out;
}

template <typename T>
static T *xmalloc(size_t n) {
  T *p = static_cast<T *>(std::malloc(n * sizeof(T) + 1));
  if (!p) throw std::bad_alloc();
  return p;
}
template <typename T>
static T *xcalloc(size_t n) {
  T *p = static_cast<T *>(std::calloc(n + 1, sizeof(T)));
  if (!p) throw std::bad_alloc();
  return p;
}

static pswf_t *new_pswf(int nspin, int nwk, int nband, double encut, const double *lattice) {
  pswf_t *wf = xcalloc<pswf_t>(1);
  wf->encut = encut;
  wf->nspin = nspin;
  wf->nwk = nwk;
  wf->nband = nband;
  wf->lattice = xmalloc<double>(9);
  wf->reclattice = xmalloc<double>(9);
  for (int i = 0; i < 9; i++) wf->lattice[i] = lattice[i];
  reciprocal(wf->lattice, wf->reclattice);
  wf->G_bounds = xcalloc<int>(6);
  wf->kpts = xcalloc<kpoint_t *>((size_t)nwk * nspin);
  return wf;
}

static kpoint_t *new_kpoint(int nband, int nplane, const double *k, double weight) {
  kpoint_t *kp = xcalloc<kpoint_t>(1);
  kp->num_bands = nband;
  kp->num_waves = nplane;
  kp->k = xmalloc<double>(3);
  for (int i = 0; i < 3; i++) kp->k[i] = k[i];
  kp->weight = weight;
  kp->bands = xcalloc<band_t *>(nband);
  for (int b = 0; b < nband; b++) {
    band_t *bd = xcalloc<band_t>(1);
    bd->n = b;
    bd->num_waves = nplane;
    kp->bands[b] = bd;
  }
  return kp;
}

static void update_bounds(pswf_t *wf, const int *g, int n) {
  for (int w = 0; w < n; w++)
    for (int a = 0; a < 3; a++) {
      int v = g[3 * w + a];
      if (v < wf->G_bounds[2 * a]) wf->G_bounds[2 * a] = v;
      if (v > wf->G_bounds[2 * a + 1]) wf->G_bounds[2 * a + 1] = v;
    }
}

// Where the bytes of a WAVECAR come from: a file read with pread (one file
// descriptor shared by the reading threads) or memory.
struct WcSource {
  int fd = -1;
  const char *mem = nullptr;
  size_t len = 0;  // bytes available (SIZE_MAX: unknown, memory only)
  void read(long long off, size_t n, void *dst) const {
    if (off < 0 || (len != SIZE_MAX && ((size_t)off > len || n > len - (size_t)off)))
      throw Error(ERR_IO, "short WAVECAR record");
    if (mem) {
      std::memcpy(dst, mem + off, n);
      return;
    }
    char *d = static_cast<char *>(dst);
    while (n) {
      const ssize_t r = ::pread(fd, d, n, (off_t)off);
      if (r < 0 && errno == EINTR) continue;
      if (r <= 0) throw Error(ERR_IO, "short WAVECAR record");
      d += r;
      off += r;
      n -= (size_t)r;
    }
  }
};

// read_wavecar (reader.c:129-315) in three stages: the header records of every
// k-point; the plane-wave spheres of all k-points in one device launch
// (gsphere_lists), while the host threads read the coefficient records straight
// into the bands' arrays (records in parallel, no staging copy); the spheres
// checked against the records' plane-wave counts.
static pswf_t *read_wavecar_from(const WcSource &src, const double *kws) {
  double head[3];
  src.read(0, sizeof head, head);
  long nrecl = std::lround(head[0]);
  int nspin = (int)std::lround(head[1]);
  long rtag = std::lround(head[2]);
  if (rtag != 45200)
    throw Error(ERR_UNSUPPORTED, "only complex64 WAVECARs (rtag 45200) are supported");
  if (nrecl < 96 || nrecl % 8) throw Error(ERR_IO, "bad WAVECAR record length");
  std::vector<double> rec(nrecl / 8);
  src.read(nrecl, nrecl, rec.data());
  int nwk = (int)std::lround(rec[0]), nband = (int)std::lround(rec[1]);
  double encut = rec[2];
  double lat[9];
  for (int i = 0; i < 9; i++) lat[i] = rec[3 + i];
  if (nspin < 1 || nspin > 2 || nwk < 1 || nband < 1) throw Error(ERR_IO, "bad WAVECAR dimensions");
  if ((long)(4 + 3 * nband) * 8 > nrecl) throw Error(ERR_IO, "WAVECAR record too short for its band header");
  pswf_t *wf = new_pswf(nspin, nwk, nband, encut, lat);
  const int nk = nwk * nspin;
  try {
    std::vector<double> kvec(3 * (size_t)nk);
    for (int iwk = 0; iwk < nk; iwk++) {
      const long long irec = (long long)iwk * (1 + nband);
      src.read((irec + 2) * nrecl, nrecl, rec.data());
      int nplane = (int)std::lround(rec[0]);
      if (nplane < 1 || (long)nplane * 8 > nrecl) throw Error(ERR_IO, "WAVECAR record too short for its bands");
      kpoint_t *kp = new_kpoint(nband, nplane, &rec[1], kws ? kws[iwk % nwk] : 0.0);
      wf->kpts[iwk] = kp;
      kp->up = (short)(iwk / nwk);
      for (int b = 0; b < nband; b++) {
        kp->bands[b]->energy = rec[4 + 3 * b];
        kp->bands[b]->occ = rec[6 + 3 * b];
        kp->bands[b]->Cs = xmalloc<pawpy_c64>(nplane);
      }
      for (int a = 0; a < 3; a++) kvec[3 * iwk + a] = kp->k[a];
    }
    // coefficient records: band b of k-point iwk is record 3 + iwk (1 + nband) + b
    // (reader.c:288-299); only the plane-wave count's bytes are read
    std::exception_ptr read_err;
    std::thread reader([&] {
      try {
        host_parallel_for(nk * nband, [&](int i) {
          const int iwk = i / nband, b = i - iwk * nband;
          kpoint_t *kp = wf->kpts[iwk];
          const long long irec = (long long)iwk * (1 + nband) + 3 + b;
          src.read(irec * nrecl, sizeof(pawpy_c64) * kp->num_waves, kp->bands[b]->Cs);
        });
      } catch (...) {
        read_err = std::current_exception();
      }
    });
    std::vector<std::vector<int>> gl;
    std::exception_ptr g_err;
    try {
      gl = gsphere_lists(wf->reclattice, encut, kvec.data(), nk);
    } catch (...) {
      g_err = std::current_exception();
    }
    reader.join();
    if (g_err) std::rethrow_exception(g_err);
    if (read_err) std::rethrow_exception(read_err);
    for (int iwk = 0; iwk < nk; iwk++) {
      kpoint_t *kp = wf->kpts[iwk];
      std::vector<int> &g = gl[iwk];
      const int nplane = kp->num_waves, ncnt = (int)g.size() / 3;
      if (2 * ncnt == nplane) {
        wf->is_ncl = 1;
        g.insert(g.end(), g.begin(), g.end());
      } else if (ncnt != nplane) {
        throw Error(ERR_IO, "plane-wave count of the WAVECAR does not match its ENCUT sphere");
      }
      kp->Gs = xmalloc<int>((size_t)3 * nplane);
      std::copy(g.begin(), g.end(), kp->Gs);
      update_bounds(wf, kp->Gs, ncnt);
    }
  } catch (...) {
    free_pswf_all(wf);
    throw;
  }
  return wf;
}

pswf_t *read_wavecar(const char *path, const double *kws) {
  WcSource src;
  src.fd = ::open(path, O_RDONLY | O_CLOEXEC);
  if (src.fd < 0) throw Error(ERR_IO, std::string("cannot open ") + path);
  struct Closer {
    int fd;
    ~Closer() { ::close(fd); }
  } closer{src.fd};
  struct stat st;
  if (::fstat(src.fd, &st) != 0) throw Error(ERR_IO, std::string("cannot stat ") + path);
  src.len = (size_t)st.st_size;
  return read_wavecar_from(src, kws);
}

pswf_t *read_wavecar_bytes(const char *data, size_t len, const double *kws) {
  PAWPY_REQUIRE(data != nullptr, "WAVECAR bytes are NULL");
  WcSource src;
  src.mem = data;
  src.len = len;
  return read_wavecar_from(src, kws);
}

pswf_t *pswf_from_arrays(int nspin, int nwk, int nband, double encut, const double *lattice,
                         const double *kpts, const double *weights, const int *nplane,
                         const int *const *Gs, const pawpy_c64 *const *Cs, const double *energies,
                         const double *occs, int is_ncl) {
  PAWPY_REQUIRE(nspin >= 1 && nspin <= 2 && nwk >= 1 && nband >= 1, "bad wavefunction dimensions");
  pswf_t *wf = new_pswf(nspin, nwk, nband, encut, lattice);
  wf->is_ncl = is_ncl ? 1 : 0;
  try {
    for (int iwk = 0; iwk < nwk * nspin; iwk++) {
      int np = nplane[iwk];
      kpoint_t *kp = new_kpoint(nband, np, kpts + 3 * (iwk % nwk), weights ? weights[iwk % nwk] : 0.0);
      kp->up = (short)(iwk / nwk);
      wf->kpts[iwk] = kp;
      kp->Gs = xmalloc<int>((size_t)3 * np);
      // noncollinear (reader.c:275-284): np counts both spinor halves; the G list of
      // one half is given, and stored twice as the WAVECAR reader stores it
      const int ng = is_ncl ? np / 2 : np;
      PAWPY_REQUIRE(!is_ncl || np % 2 == 0, "noncollinear plane-wave count must be even");
      std::memcpy(kp->Gs, Gs[iwk], sizeof(int) * 3 * ng);
      if (is_ncl) std::memcpy(kp->Gs + 3 * ng, Gs[iwk], sizeof(int) * 3 * ng);
      update_bounds(wf, kp->Gs, ng);
      for (int b = 0; b < nband; b++) {
        band_t *bd = kp->bands[b];
        bd->Cs = xmalloc<pawpy_c64>(np);
        std::memcpy(static_cast<void *>(bd->Cs), Cs[iwk] + (size_t)b * np, sizeof(pawpy_c64) * np);
        bd->energy = energies ? energies[(size_t)iwk * nband + b] : 0.0;
        bd->occ = occs ? occs[(size_t)iwk * nband + b] : 0.0;
      }
    }
  } catch (...) {
    free_pswf_all(wf);
    throw;
  }
  return wf;
}

static void free_projection_list(projection_t *p, int n) {
  if (!p) return;
  for (int i = 0; i < n; i++) {
    std::free(p[i].ms);
    std::free(p[i].ls);
    std::free(p[i].ns);
    std::free(p[i].overlaps);
  }
  std::free(p);
}

void free_wave_projections(pswf_t *wf) {
  for (int i = 0; i < wf->nwk * wf->nspin; i++) {
    kpoint_t *kp = wf->kpts[i];
    if (!kp) continue;
    for (int b = 0; b < kp->num_bands; b++) {
      free_projection_list(kp->bands[b]->wave_projections, wf->wp_num);
      kp->bands[b]->wave_projections = nullptr;
    }
  }
}

static void free_spline(double **s) {
  if (!s) return;
  for (int j = 0; j < 3; j++) std::free(s[j]);
  std::free(s);
}

void free_ppot_array(ppot_t *pps, int n) {
  if (!pps) return;
  for (int i = 0; i < n; i++) {
    ppot_t *p = pps + i;
    for (int k = 0; p->funcs && k < p->num_projs; k++) {
      funcset_t *f = p->funcs + k;
      std::free(f->proj);
      std::free(f->pswave);
      std::free(f->aewave);
      std::free(f->diffwave);
      std::free(f->kwave);
      std::free(f->smooth_diffwave);
      free_spline(f->proj_spline);
      free_spline(f->aewave_spline);
      free_spline(f->pswave_spline);
      free_spline(f->diffwave_spline);
      free_spline(f->kwave_spline);
      free_spline(f->smooth_diffwave_spline);
    }
    std::free(p->funcs);
    std::free(p->wave_grid);
    std::free(p->kwave_grid);
    std::free(p->proj_grid);
    std::free(p->smooth_grid);
    std::free(p->pspw_overlap_matrix);
    std::free(p->aepw_overlap_matrix);
    std::free(p->diff_overlap_matrix);
  }
  std::free(pps);
}

}  // namespace pawpy

extern "C" void pawpy_gpu_free_ppot_list(ppot_t *pps, int length) { pawpy::free_ppot_array(pps, length); }

namespace pawpy {

void free_pswf_all(pswf_t *wf) {
  if (!wf) return;
  for (int i = 0; wf->kpts && i < wf->nwk * wf->nspin; i++) {
    kpoint_t *kp = wf->kpts[i];
    if (!kp) continue;
    for (int b = 0; kp->bands && b < kp->num_bands; b++) {
      band_t *bd = kp->bands[b];
      if (!bd) continue;
      std::free(bd->Cs);
      free_projection_list(bd->projections, wf->num_sites);
      free_projection_list(bd->wave_projections, wf->wp_num);
      free_projection_list(bd->up_projections, wf->num_sites);
      free_projection_list(bd->down_projections, wf->num_sites);
      std::free(bd->CRs);
      std::free(bd->CAs);
      std::free(bd);
    }
    std::free(kp->Gs);
    std::free(kp->bands);
    std::free(kp->k);
    std::free(kp);
  }
  if (wf->overlaps) {
    for (int i = 0; i < wf->num_aug_overlap_sites; i++) std::free(wf->overlaps[i]);
    std::free(wf->overlaps);
  }
  std::free(wf->num_projs);
  std::free(wf->kpts);
  std::free(wf->G_bounds);
  std::free(wf->lattice);
  std::free(wf->reclattice);
  free_ppot_array(wf->pps, wf->num_elems);
  std::free(wf->dcoords);
  std::free(wf->fftg);
  std::free(wf);
}

}  // namespace pawpy

using namespace pawpy;

extern "C" {

pswf_t *pawpy_gpu_read_wavefunctions(const char *filename, const double *kpt_weights) {
  PAWPY_API_BEGIN
  PAWPY_REQUIRE(filename != nullptr, "filename is NULL");
  return read_wavecar(filename, kpt_weights);
  PAWPY_API_END(nullptr)
}

pswf_t *pawpy_gpu_read_wavefunctions_from_str(const char *start, const double *kpt_weights) {
  PAWPY_API_BEGIN
  return read_wavecar_bytes(start, SIZE_MAX, kpt_weights);
  PAWPY_API_END(nullptr)
}

pswf_t *pawpy_gpu_read_wavefunctions_from_bytes(const char *data, size_t len, const double *kpt_weights) {
  PAWPY_API_BEGIN
  return read_wavecar_bytes(data, len, kpt_weights);
  PAWPY_API_END(nullptr)
}

pswf_t *pawpy_gpu_wavefunction_from_arrays(int nspin, int nwk, int nband, double encut,
                                           const double *lattice, const double *kpts,
                                           const double *weights, const int *nplane,
                                           const int *const *Gs, const pawpy_c64 *const *Cs,
                                           const double *energies, const double *occs, int is_ncl) {
  PAWPY_API_BEGIN
  return pswf_from_arrays(nspin, nwk, nband, encut, lattice, kpts, weights, nplane, Gs, Cs,
                          energies, occs, is_ncl);
  PAWPY_API_END(nullptr)
}

void pawpy_gpu_free_pswf(pswf_t *wf) {
  PAWPY_API_BEGIN
  if (!wf) return;
  release_device(wf);
  free_pswf_all(wf);
  PAWPY_API_END()
}

#define PAWPY_MEMBER(S, m) out += std::string(#S) + " " + #m + " " + std::to_string(offsetof(S, m)) + "\n"
#define PAWPY_SIZE(S) out += std::string(#S) + " __sizeof__ " + std::to_string(sizeof(S)) + "\n"

int pawpy_gpu_struct_layout(char *buf, int len) {
  std::string out;
  PAWPY_MEMBER(funcset_t, l); PAWPY_MEMBER(funcset_t, proj); PAWPY_MEMBER(funcset_t, proj_spline);
  PAWPY_MEMBER(funcset_t, aewave); PAWPY_MEMBER(funcset_t, aewave_spline); PAWPY_MEMBER(funcset_t, pswave);
  PAWPY_MEMBER(funcset_t, pswave_spline); PAWPY_MEMBER(funcset_t, diffwave); PAWPY_MEMBER(funcset_t, diffwave_spline);
  PAWPY_MEMBER(funcset_t, kwave); PAWPY_MEMBER(funcset_t, kwave_spline); PAWPY_MEMBER(funcset_t, smooth_diffwave);
  PAWPY_MEMBER(funcset_t, smooth_diffwave_spline); PAWPY_MEMBER(funcset_t, dense_kwave);
  PAWPY_MEMBER(funcset_t, dense_kwave_spline); PAWPY_SIZE(funcset_t);
  PAWPY_MEMBER(ppot_t, num_projs); PAWPY_MEMBER(ppot_t, total_projs); PAWPY_MEMBER(ppot_t, lmax);
  PAWPY_MEMBER(ppot_t, funcs); PAWPY_MEMBER(ppot_t, rmax); PAWPY_MEMBER(ppot_t, wave_rmax);
  PAWPY_MEMBER(ppot_t, pspw_overlap_matrix); PAWPY_MEMBER(ppot_t, aepw_overlap_matrix);
  PAWPY_MEMBER(ppot_t, diff_overlap_matrix); PAWPY_MEMBER(ppot_t, proj_gridsize); PAWPY_MEMBER(ppot_t, wave_gridsize);
  PAWPY_MEMBER(ppot_t, num_cart_gridpts); PAWPY_MEMBER(ppot_t, wave_grid); PAWPY_MEMBER(ppot_t, kwave_grid);
  PAWPY_MEMBER(ppot_t, proj_grid); PAWPY_MEMBER(ppot_t, smooth_grid); PAWPY_MEMBER(ppot_t, dense_kgrid);
  PAWPY_SIZE(ppot_t);
  PAWPY_MEMBER(projection_t, num_projs); PAWPY_MEMBER(projection_t, total_projs); PAWPY_MEMBER(projection_t, ns);
  PAWPY_MEMBER(projection_t, ls); PAWPY_MEMBER(projection_t, ms); PAWPY_MEMBER(projection_t, overlaps);
  PAWPY_SIZE(projection_t);
  PAWPY_MEMBER(band_t, n); PAWPY_MEMBER(band_t, num_waves); PAWPY_MEMBER(band_t, occ); PAWPY_MEMBER(band_t, N);
  PAWPY_MEMBER(band_t, energy); PAWPY_MEMBER(band_t, Cs); PAWPY_MEMBER(band_t, CRs); PAWPY_MEMBER(band_t, CAs);
  PAWPY_MEMBER(band_t, projections); PAWPY_MEMBER(band_t, up_projections); PAWPY_MEMBER(band_t, down_projections);
  PAWPY_MEMBER(band_t, wave_projections); PAWPY_SIZE(band_t);
  PAWPY_MEMBER(rayleigh_set_t, l); PAWPY_MEMBER(rayleigh_set_t, terms); PAWPY_SIZE(rayleigh_set_t);
  PAWPY_MEMBER(kpoint_t, up); PAWPY_MEMBER(kpoint_t, num_waves); PAWPY_MEMBER(kpoint_t, Gs); PAWPY_MEMBER(kpoint_t, k);
  PAWPY_MEMBER(kpoint_t, weight); PAWPY_MEMBER(kpoint_t, num_bands); PAWPY_MEMBER(kpoint_t, bands);
  PAWPY_MEMBER(kpoint_t, expansion); PAWPY_SIZE(kpoint_t);
  PAWPY_MEMBER(pswf_t, encut); PAWPY_MEMBER(pswf_t, num_elems); PAWPY_MEMBER(pswf_t, num_projs);
  PAWPY_MEMBER(pswf_t, num_sites); PAWPY_MEMBER(pswf_t, pps); PAWPY_MEMBER(pswf_t, G_bounds); PAWPY_MEMBER(pswf_t, kpts);
  PAWPY_MEMBER(pswf_t, nspin); PAWPY_MEMBER(pswf_t, nband); PAWPY_MEMBER(pswf_t, nwk); PAWPY_MEMBER(pswf_t, lattice);
  PAWPY_MEMBER(pswf_t, reclattice); PAWPY_MEMBER(pswf_t, fftg); PAWPY_MEMBER(pswf_t, is_ncl); PAWPY_MEMBER(pswf_t, wp_num);
  PAWPY_MEMBER(pswf_t, num_aug_overlap_sites); PAWPY_MEMBER(pswf_t, dcoords); PAWPY_MEMBER(pswf_t, overlaps);
  PAWPY_SIZE(pswf_t);
  PAWPY_MEMBER(real_proj_t, l); PAWPY_MEMBER(real_proj_t, m); PAWPY_MEMBER(real_proj_t, func_num);
  PAWPY_MEMBER(real_proj_t, values); PAWPY_SIZE(real_proj_t);
  PAWPY_MEMBER(real_proj_site_t, index); PAWPY_MEMBER(real_proj_site_t, elem); PAWPY_MEMBER(real_proj_site_t, num_projs);
  PAWPY_MEMBER(real_proj_site_t, total_projs); PAWPY_MEMBER(real_proj_site_t, num_indices);
  PAWPY_MEMBER(real_proj_site_t, gridsize); PAWPY_MEMBER(real_proj_site_t, rmax); PAWPY_MEMBER(real_proj_site_t, coord);
  PAWPY_MEMBER(real_proj_site_t, indices); PAWPY_MEMBER(real_proj_site_t, paths); PAWPY_MEMBER(real_proj_site_t, projs);
  PAWPY_SIZE(real_proj_site_t);
  PAWPY_MEMBER(pawpy_gpu_request_t, basis); PAWPY_MEMBER(pawpy_gpu_request_t, wf); PAWPY_MEMBER(pawpy_gpu_request_t, pps);
  PAWPY_MEMBER(pawpy_gpu_request_t, num_elems); PAWPY_MEMBER(pawpy_gpu_request_t, num_sites);
  PAWPY_MEMBER(pawpy_gpu_request_t, fftg); PAWPY_MEMBER(pawpy_gpu_request_t, labels);
  PAWPY_MEMBER(pawpy_gpu_request_t, coords); PAWPY_MEMBER(pawpy_gpu_request_t, num_M);
  PAWPY_MEMBER(pawpy_gpu_request_t, num_N_R); PAWPY_MEMBER(pawpy_gpu_request_t, num_N_S);
  PAWPY_MEMBER(pawpy_gpu_request_t, num_N_RS); PAWPY_MEMBER(pawpy_gpu_request_t, M_R);
  PAWPY_MEMBER(pawpy_gpu_request_t, M_S); PAWPY_MEMBER(pawpy_gpu_request_t, N_R); PAWPY_MEMBER(pawpy_gpu_request_t, N_S);
  PAWPY_MEMBER(pawpy_gpu_request_t, N_RS_R); PAWPY_MEMBER(pawpy_gpu_request_t, N_RS_S);
  PAWPY_MEMBER(pawpy_gpu_request_t, out);
  PAWPY_SIZE(pawpy_gpu_request_t);
  if (buf && len > 0) {
    std::strncpy(buf, out.c_str(), (size_t)len - 1);
    buf[len - 1] = 0;
  }
  return (int)out.size() + 1;
}

}  // extern "C"
