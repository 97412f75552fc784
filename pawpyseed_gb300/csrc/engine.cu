// Device engine and drop-in entry points of libpawpy_gpu.
//
// Each pswf_t that reaches the library gets a device mirror (DevWF), keyed by
// its address and checked against a fingerprint of its host layout:
//   * coefficients per k-point as [nband][Wpad] complex64, plane waves sorted
//     by (g1, g2, g3) so that every g1 plane is a contiguous run (the FFT reads
//     whole planes, the overlap contraction does not care about order);
//   * augmentation-sphere tables of every site (indices, conj(p Y_lm) dV in
//     lm-major order, exp(i k.path) per k-point), built on the device in FP64;
//   * projector coefficients <p|psi> as [nk][nband][sum_sites lm] complex64.
// A (basis R, defect S) pair carries the smoothed-partial-wave projections of
// overlap_setup_real, the N_RS pair matrices, the cached pseudo overlap
// matrices and the augmentation columns of the PAW terms.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <complex>
#include <exception>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <tuple>
#include <thread>
#include <vector>

#include "host.h"
#include "kernels.h"

namespace pawpy {

using cd = std::complex<double>;

// ============================================================= state

struct SpeciesTables {
  DevBuf<double> proj_f, proj_spl, smooth_f, smooth_spl;
  SpeciesDev proj{}, smooth{};
  // (phi - phit) on the logarithmic partial-wave grid, for the all-electron real-space
  // wavefunctions; ae_rmax = the grid's last point (the radius of those spheres)
  DevBuf<double> ae_x, ae_f, ae_spl;
  AeSpeciesDev ae{};
  double ae_rmax = 0;
  int total = 0, nproj = 0;
  std::vector<int> lm_n, lm_l, lm_m;
  std::vector<double> D;  // total x total: (aeov - psov)[n_i][n_j] where (l,m) agree
};

// A CUDA event owned by the structure holding it (created on first record).
struct OwnedEvent {
  cudaEvent_t e = nullptr;
  OwnedEvent() = default;
  OwnedEvent(const OwnedEvent &) = delete;
  OwnedEvent &operator=(const OwnedEvent &) = delete;
  OwnedEvent(OwnedEvent &&o) noexcept : e(o.e) { o.e = nullptr; }
  OwnedEvent &operator=(OwnedEvent &&o) noexcept {
    if (this != &o) {
      if (e) cudaEventDestroy(e);
      e = o.e;
      o.e = nullptr;
    }
    return *this;
  }
  ~OwnedEvent() {
    if (e) cudaEventDestroy(e);
  }
  void record(cudaStream_t s) {
    if (!e) PAWPY_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    PAWPY_CUDA(cudaEventRecord(e, s));
  }
  // the stream waits for the last record (nothing when never recorded)
  void wait(cudaStream_t s) const {
    if (e) PAWPY_CUDA(cudaStreamWaitEvent(s, e, 0));
  }
};

struct SphereSet {
  int nsites = 0, Ptot = 0, max_total = 0, nkp = 0, nseg = 0;
  long long npts = 0, nvals = 0;
  std::vector<SiteDesc> host;
  std::vector<SegFill> segs;      // site-major, box-row order within a site
  std::vector<int> seg_plane;     // wrapped plane index j of each segment
  std::vector<long long> site_pt, site_val;  // first point / first table value of each site
  std::vector<int> site_npts;
  DevBuf<SiteDesc> sites;
  DevBuf<int> idx;
  DevBuf<float2> tab, phase;
  DevBuf<SpeciesDev> species;
  // idx and phase are written on the library stream; tab on the auxiliary stream of the
  // thread that built the set, which records tab_ready: readers of tab wait for it
  OwnedEvent tab_ready;
};

// Sphere tables of the all-electron real-space wavefunctions of one wavefunction on
// one grid (realspace.cu): per site the points within its partial-wave grid's last
// radius, (phi - phit)/r Y_lm there, exp(2 pi i k.(R + T)) per k-point, and the points
// grouped per grid cell for the deterministic spread.
struct AeTables {
  int N[3] = {0, 0, 0};
  std::vector<int> labels;
  std::vector<double> coords;
  long long npts = 0;
  DevBuf<int> cell;
  DevBuf<float2> val, phase;
  DevBuf<int> ucell, ent_first, ent_site, site_npts, site_total, site_pcol;
  DevBuf<long long> ent_pt, site_pt, site_val;
  AeSpread view;
  Radices r[3];
  DevBuf<float2> tw[3];
};

struct DevKpt {
  int W = 0, Wpad = 0, g1min = 0, n1 = 0;
  int g2min = 0, n2 = 0, g3min = 0, n3 = 0;  // occupied ranges of the other two axes
  int maxcnt = 0;                             // most coefficients in one plane
  std::vector<int> perm;     // sorted position -> original plane-wave index
  std::vector<int> invperm;  // original plane-wave index -> sorted position
  std::vector<int> gsorted;  // [W][3] in sorted order
  DevBuf<int> perm_d, plane_start, plane_off;
  DevBuf<int> inv_d;  // invperm on the device (host-read upload)
  DevBuf<int> gs_d;   // gsorted on the device (real-space wavefunctions)
  int off_N2 = 0, off_N3 = 0;
  size_t c_off = 0;
  double kfrac[3] = {0, 0, 0};
};

struct DevWF {
  pswf_t *wf = nullptr;
  // nband counts device bands: a noncollinear wavefunction's band b is the two
  // device bands 2b (spin-up half) and 2b+1 (spin-down half), which share the
  // G list as in onto_projector_ncl (projector.c:359-392)
  int nspin = 0, nwk = 0, nband = 0, nk = 0;
  bool ncl = false;
  int nband_host = 0;
  kpoint_t **kpts_ptr = nullptr;
  const void *cs0 = nullptr;
  double lattice[9], rec[9], vol = 0;
  std::vector<DevKpt> kp;
  DevBuf<float2> C;
  bool c_ready = false;
  // per k-point: the upload of its coefficients on the side stream (empty when
  // the upload was ordered on the library stream); band pointers of the upload
  std::vector<cudaEvent_t> c_ev;
  // ... and of each batch of kUploadChunkBands bands of it (c_chunk_ev[k][batch])
  std::vector<std::vector<cudaEvent_t>> c_chunk_ev;
  DevBuf<const float2 *> host_ptrs;
  // resident real-space wavefunctions [k][band][N1][N2][N3] (a prepared basis)
  DevBuf<float2> grid;
  bool grid_ready = false;
  // the first FFT pass of every band, issued on the auxiliary stream ahead of the sphere
  // setup when the projections are computed later: H of k-point k at hoff[k],
  // [band][n1 of k][N2][N3], complete at event h_ev[k]
  DevBuf<float2> Hall;
  std::vector<size_t> hoff;
  std::vector<cudaEvent_t> h_ev;
  bool h_ready = false;
  // projectors
  int N[3] = {0, 0, 0};
  std::vector<std::unique_ptr<SpeciesTables>> species;
  std::vector<int> labels;
  std::vector<double> coords;
  SphereSet proj;
  std::vector<int> site_lmoff;
  DevBuf<float2> P;
  bool tables_ready = false;  // element and sphere tables built (setup_projections called)
  bool p_ready = false;       // P holds <p|psi> of every band
  Radices r[3];
  DevBuf<float2> tw[3];
  std::unique_ptr<AeTables> ae;  // real-space all-electron tables (last grid asked for)
  TcSplitCache gemm_cache;       // split planes of C as operand A of the overlap contraction
  DevWF() = default;
  DevWF(const DevWF &) = delete;
  DevWF &operator=(const DevWF &) = delete;
  // the buffers are freed on the library stream: it waits for the uploads first
  ~DevWF() {
    // members are freed on the library stream: order it after the tables' auxiliary-stream fill
    proj.tab_ready.wait(stream());
    for (cudaEvent_t e : c_ev) {
      cudaStreamWaitEvent(stream(), e, 0);
      cudaEventDestroy(e);
    }
    for (auto &v : c_chunk_ev)
      for (cudaEvent_t e : v) cudaEventDestroy(e);
    for (cudaEvent_t e : h_ev) {
      cudaStreamWaitEvent(stream(), e, 0);
      cudaEventDestroy(e);
    }
  }
};

// Bands per launch of the in-place read of host coefficients (each batch has its event).
constexpr int kUploadChunkBands = 128;

// Makes the library stream wait for the upload of k-point k's coefficients;
// their device address.
static const float2 *coeffs(DevWF &d, int k) {
  if (!d.c_ev.empty()) PAWPY_CUDA(cudaStreamWaitEvent(stream(), d.c_ev[k], 0));
  return d.C.p + d.kp[k].c_off;
}

// The same for bands [b0, b0 + nb) of k-point k only; the address of band b0.
static const float2 *coeffs(DevWF &d, int k, int b0, int nb) {
  if (!d.c_chunk_ev.empty()) {
    for (int c = b0 / kUploadChunkBands; c * kUploadChunkBands < b0 + nb; c++)
      PAWPY_CUDA(cudaStreamWaitEvent(stream(), d.c_chunk_ev[k][c], 0));
  } else if (!d.c_ev.empty()) {
    PAWPY_CUDA(cudaStreamWaitEvent(stream(), d.c_ev[k], 0));
  }
  return d.C.p + d.kp[k].c_off + (size_t)b0 * d.kp[k].Wpad;
}

// The library stream waits for the uploads and the early transforms of d.
static void join_uploads(DevWF &d) {
  for (cudaEvent_t e : d.c_ev) PAWPY_CUDA(cudaStreamWaitEvent(stream(), e, 0));
  for (cudaEvent_t e : d.h_ev) PAWPY_CUDA(cudaStreamWaitEvent(stream(), e, 0));
}

struct AugKey {
  std::vector<int> lists[6];
  int flip;
  bool recip = false;  // aug_recip columns: O_M and O_N only
  bool operator==(const AugKey &o) const {
    if (flip != o.flip || recip != o.recip) return false;
    for (int i = 0; i < 6; i++)
      if (lists[i] != o.lists[i]) return false;
    return true;
  }
};

// Pinned host staging for uploads issued behind long device work: a copy from pinned memory
// returns at once, where one from pageable memory can wait for the stream's earlier launches.
// One per host thread (aug_stage), kept for the thread's life: pinning and unpinning host
// memory is slow and can wait for the device. begin() waits for the previous round's copies
// before the buffer is rewritten.
struct PinnedStage {
  void *h = nullptr;
  size_t cap = 0, used = 0;
  cudaEvent_t done = nullptr;
  PinnedStage() = default;
  PinnedStage(const PinnedStage &) = delete;
  PinnedStage &operator=(const PinnedStage &) = delete;
  ~PinnedStage() {
    if (done) {
      cudaEventSynchronize(done);
      cudaEventDestroy(done);
    }
    if (h) cudaFreeHost(h);
  }
  void begin(size_t bytes) {
    if (done) PAWPY_CUDA(cudaEventSynchronize(done));
    if (bytes > cap) {
      if (h) PAWPY_CUDA(cudaFreeHost(h));
      h = nullptr;
      PAWPY_CUDA(cudaMallocHost(&h, bytes));
      cap = bytes;
    }
    used = 0;
  }
  template <typename T>
  void upload(DevBuf<T> &d, const std::vector<T> &v) {
    const size_t bytes = v.size() * sizeof(T);
    if (!bytes) return;
    used = (used + 15) & ~size_t(15);
    PAWPY_REQUIRE(used + bytes <= cap, "pinned staging overflow");
    char *p = static_cast<char *>(h) + used;
    std::memcpy(p, v.data(), bytes);
    used += bytes;
    PAWPY_CUDA(cudaMemcpyAsync(d.p, p, bytes, cudaMemcpyHostToDevice, stream()));
  }
  void end() {
    if (!done) PAWPY_CUDA(cudaEventCreateWithFlags(&done, cudaEventDisableTiming));
    PAWPY_CUDA(cudaEventRecord(done, stream()));
  }
};

static PinnedStage &aug_stage() {
  static thread_local PinnedStage s;
  return s;
}

struct PairState {
  DevWF *R = nullptr, *S = nullptr;
  std::vector<int> N_R, N_S, N_RS_R, N_RS_S;
  SphereSet sm_NR, sm_NS;
  DevBuf<float2> WP_S, WP_R;  // [nk][nbS][sm_NR.Ptot], [nk][nbR][sm_NS.Ptot]
  std::vector<std::vector<cd>> Q;
  std::vector<double> dcoords;
  bool ready = false;
  // cached pseudo overlap matrices [nk][nbS][nbR], per flip
  DevBuf<float2> pseudo[2];
  bool pseudo_ready[2] = {false, false};
  int pseudo_prec[2] = {-1, -1};
  // augmentation columns
  bool aug_ready = false;
  AugKey aug_key;
  int Kc = 0, Kcpad = 0;
  DevBuf<double2> A64;  // [nk][nbR][Kc]   (indexed by the R k-slice)
  DevBuf<float2> A32;   // [nk][nbR][Kcpad]
  DevBuf<int> a_src, b_ptr, b_col, b_pair;
  DevBuf<double2> b_val;
  DevBuf<double2> pair_phase;  // [nk][npairs]
  DevBuf<float2> b_val32;      // [nk][entries]: b_val times the column's pair phase, FP32
  // aug_recip: set by overlap_setup_recip (the overlaps then follow that method). The
  // augmentation coefficients of R's bands on its N_R sites and of S's bands on its N_S
  // sites, [nk][nband][Wpad] in the sorted plane-wave order (empty when the list is);
  // D_S = C_S + CA_S. cross[f] = <CA_R|C_S> + <C_R|CA_S> [nk][nbS][nbR] per flip.
  bool recip = false;
  DevBuf<float2> CA_R, CA_S, D_S;
  DevBuf<float2> cross[2];
  bool cross_ready[2] = {false, false};
  int cross_prec[2] = {-1, -1};
  ~PairState() {
    // members are freed on the library stream: order it after the tables' auxiliary-stream fill
    sm_NR.tab_ready.wait(stream());
    sm_NS.tab_ready.wait(stream());
  }
};

// Overlaps are between wavefunction bands: a noncollinear band is two consecutive
// device bands (its spinor halves), so its overlap rows are twice as long.
static int host_bands(const DevWF &d) { return d.ncl ? d.nband / 2 : d.nband; }
static int spinor_factor(const DevWF &d) { return d.ncl ? 2 : 1; }

static std::recursive_mutex g_mu;
static std::map<const pswf_t *, std::unique_ptr<DevWF>> g_wfs;
static std::map<std::pair<const pswf_t *, const pswf_t *>, std::unique_ptr<PairState>> g_pairs;
// process-wide switches; serving threads read them while a caller may set them
static std::atomic<int> g_precision{PAWPY_GPU_FP32};
// sphere contraction on the tensor cores: 1 with the tensor-core precisions, 0 never, 2 always
static std::atomic<int> g_sphere_tc{1};
// picked-point rows per batch of the tensor-core sphere contraction, in bytes
constexpr long long kTcPickBatchBytes = 12LL << 30;
static bool sphere_tc_enabled() {
  const int m = g_sphere_tc.load(), prec = g_precision.load();
  return m == 2 || (m == 1 && (prec == PAWPY_GPU_BF16X3 || prec == PAWPY_GPU_TF32));
}
static std::atomic<int> g_tc_splits{0};  // K split of the tensor-core contraction, 0 = from the SM count
static std::atomic<bool> g_host_proj{true};

void release_device(pswf_t *wf) {
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  // work still queued may read the wavefunction's host arrays, which the caller frees next
  auto f = g_wfs.find(wf);
  if (f != g_wfs.end()) {
    join_uploads(*f->second);
    sync();
  }
  for (auto it = g_pairs.begin(); it != g_pairs.end();) {
    if (it->first.first == wf || it->first.second == wf)
      it = g_pairs.erase(it);
    else
      ++it;
  }
  g_wfs.erase(wf);
}

static bool fingerprint_ok(const DevWF &d, const pswf_t *wf) {
  return d.nspin == wf->nspin && d.nwk == wf->nwk && d.nband_host == wf->nband && d.kpts_ptr == wf->kpts &&
         d.ncl == (wf->is_ncl != 0) &&
         wf->kpts && wf->kpts[0] && wf->kpts[0]->bands && wf->kpts[0]->bands[0] &&
         d.cs0 == (const void *)wf->kpts[0]->bands[0]->Cs;
}

// Size of the plane-FFT intermediate H of one FFT sub-batch. Measured per
// 64-atom step on the 60^3 grid (1 MiB of H per band): 64 MiB 3.97 ms, 96 MiB
// 3.84 ms, 192 MiB 3.72 ms, 288 MiB (all 256 bands of a k-point) 3.57 ms,
// 384 MiB 3.61 ms; fewer, longer launches of the persistent kernels outweigh
// H leaving L2 between the passes.
constexpr long long kFftBatchBytes = 288LL << 20;

// Runs f(0..n-1) on the library's host worker threads (see host_parallel_for).
template <typename F>
static void parallel_for(int n, F f) {
  host_parallel_for(n, std::function<void(int)>(f));
}

// perm = plane-wave indices in (g1, g2, g3) order. The vectors are distinct
// points of a small box, so one pass over the box's cells orders them (a
// comparison sort is the fallback for a sparse box).
static void sort_gvectors(const int *G, int W, std::vector<int> &perm) {
  perm.resize(W);
  if (W == 0) return;
  int lo[3] = {G[0], G[1], G[2]}, hi[3] = {G[0], G[1], G[2]};
  for (int t = 1; t < W; t++)
    for (int a = 0; a < 3; a++) {
      lo[a] = std::min(lo[a], G[3 * t + a]);
      hi[a] = std::max(hi[a], G[3 * t + a]);
    }
  const long long s1 = hi[1] - lo[1] + 1, s2 = hi[2] - lo[2] + 1;
  const long long cells = (long long)(hi[0] - lo[0] + 1) * s1 * s2;
  std::vector<int> cell;
  bool distinct = cells <= 16LL * W + 4096;
  if (distinct) {
    cell.assign((size_t)cells, -1);
    for (int t = 0; t < W && distinct; t++) {
      long long key = ((long long)(G[3 * t] - lo[0]) * s1 + (G[3 * t + 1] - lo[1])) * s2 + (G[3 * t + 2] - lo[2]);
      if (cell[key] >= 0) distinct = false;
      cell[key] = t;
    }
  }
  if (distinct) {
    int n = 0;
    for (long long c = 0; c < cells; c++)
      if (cell[c] >= 0) perm[n++] = cell[c];
    return;
  }
  std::iota(perm.begin(), perm.end(), 0);
  std::stable_sort(perm.begin(), perm.end(), [G](int a, int b) {
    return std::tie(G[3 * a], G[3 * a + 1], G[3 * a + 2]) < std::tie(G[3 * b], G[3 * b + 1], G[3 * b + 2]);
  });
}

static DevWF &mirror(pswf_t *wf) {
  PAWPY_REQUIRE(wf != nullptr, "wavefunction pointer is NULL");
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  auto it = g_wfs.find(wf);
  if (it != g_wfs.end() && !fingerprint_ok(*it->second, wf)) {
    release_device(wf);
    it = g_wfs.end();
  }
  if (it != g_wfs.end()) return *it->second;
  HostPhase hp("mirror");
  auto d = std::make_unique<DevWF>();
  d->wf = wf;
  d->nspin = wf->nspin;
  d->nwk = wf->nwk;
  d->ncl = wf->is_ncl != 0;
  d->nband_host = wf->nband;
  d->nband = d->ncl ? 2 * wf->nband : wf->nband;
  d->nk = wf->nspin * wf->nwk;
  d->kpts_ptr = wf->kpts;
  d->cs0 = wf->kpts[0]->bands[0]->Cs;
  for (int i = 0; i < 9; i++) d->lattice[i] = wf->lattice[i];
  reciprocal(d->lattice, d->rec);
  d->vol = det3(d->lattice);
  d->kp.resize(d->nk);
  size_t off = 0;
  for (int k = 0; k < d->nk; k++) {
    kpoint_t *kp = wf->kpts[k];
    DevKpt &q = d->kp[k];
    q.W = d->ncl ? kp->num_waves / 2 : kp->num_waves;
    PAWPY_REQUIRE(!d->ncl || kp->num_waves % 2 == 0, "noncollinear k-point with an odd plane-wave count");
    q.Wpad = (q.W + 15) / 16 * 16;
    for (int a = 0; a < 3; a++) q.kfrac[a] = kp->k[a];
    q.c_off = off;
    off += (size_t)d->nband * q.Wpad;
  }
  // the plane-wave orderings of the k-points are independent: one host thread each
  parallel_for(d->nk, [&](int k) {
    DevKpt &q = d->kp[k];
    const int *G = wf->kpts[k]->Gs;
    sort_gvectors(G, q.W, q.perm);
    q.invperm.resize(q.W);
    for (int t = 0; t < q.W; t++) q.invperm[q.perm[t]] = t;
    q.gsorted.resize(3 * (size_t)q.W);
    for (int t = 0; t < q.W; t++)
      for (int a = 0; a < 3; a++) q.gsorted[3 * t + a] = G[3 * q.perm[t] + a];
    q.g1min = q.W ? q.gsorted[0] : 0;
    q.n1 = q.W ? q.gsorted[3 * (q.W - 1)] - q.g1min + 1 : 0;
  });
  DevWF &ref = *d;
  g_wfs[wf] = std::move(d);
  return ref;
}

// host coefficients of device band b at k-point k (a spinor half for noncollinear wavefunctions)
static const float2 *host_band(const DevWF &d, int k, int b) {
  const kpoint_t *kp = d.wf->kpts[k];
  if (!d.ncl) return reinterpret_cast<const float2 *>(kp->bands[b]->Cs);
  return reinterpret_cast<const float2 *>(kp->bands[b / 2]->Cs) + (size_t)(b & 1) * d.kp[k].W;
}

static int pageable_access() {
  static int v = -1;
  if (v < 0) {
    int a = 0, b = 0, dev = device();
    PAWPY_CUDA(cudaDeviceGetAttribute(&a, cudaDevAttrPageableMemoryAccess, dev));
    PAWPY_CUDA(cudaDeviceGetAttribute(&b, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev));
    v = (a && b) ? 1 : 0;
  }
  return v;
}

// Uploads the coefficients of every band into the sorted device layout. Where
// the device reads pageable host memory through the host page tables (e.g. a
// Grace-Blackwell node), a kernel reads the band arrays in place; otherwise
// each band is copied with cudaMemcpyAsync and permuted on the device.
static void ensure_coeffs(DevWF &d) {
  if (d.c_ready) return;
  HostPhase hp("upload");
  size_t total = 0;
  for (auto &q : d.kp) total += (size_t)d.nband * q.Wpad;
  d.C.alloc(total);
  int maxW = 0;
  for (auto &q : d.kp) maxW = std::max(maxW, q.W);
  if (pageable_access() && !getenv("PAWPY_GPU_NO_HOST_READ")) {
    // The uploads run on the side stream, one k-point after another, while the
    // library stream goes on with the transforms of the k-points already
    // uploaded (coeffs() orders each use after its k-point's upload). The
    // caller's arrays outlive the upload: release_device waits for it.
    std::vector<const float2 *> hp((size_t)d.nk * d.nband);
    for (int k = 0; k < d.nk; k++)
      for (int b = 0; b < d.nband; b++)
        hp[(size_t)k * d.nband + b] = host_band(d, k, b);
    d.host_ptrs.alloc(hp.size());
    d.host_ptrs.upload(hp.data(), hp.size());
    for (auto &q : d.kp) {
      q.inv_d.alloc(std::max(1, q.W));
      q.inv_d.upload(q.invperm.data(), q.W);
    }
    cudaEvent_t ready;
    PAWPY_CUDA(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
    PAWPY_CUDA(cudaEventRecord(ready, stream()));
    const cudaStream_t up = side_stream();
    PAWPY_CUDA(cudaStreamWaitEvent(up, ready, 0));
    PAWPY_CUDA(cudaEventDestroy(ready));
    d.c_ev.assign(d.nk, nullptr);
    for (auto &e : d.c_ev) PAWPY_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    const int nchunk = ceil_div(d.nband, kUploadChunkBands);
    d.c_chunk_ev.assign(d.nk, std::vector<cudaEvent_t>(nchunk, nullptr));
    {
      OnStream on(up);
      for (int k = 0; k < d.nk; k++) {
        DevKpt &q = d.kp[k];
        // in batches of bands, each with its event: the first FFT pass of a batch starts when its
        // bands have arrived
        for (int c = 0; c < nchunk; c++) {
          const int b0 = c * kUploadChunkBands, nb = std::min(kUploadChunkBands, d.nband - b0);
          launch_load_host_bands(d.host_ptrs.p + (size_t)k * d.nband + b0, q.W, q.inv_d.p,
                                 d.C.p + q.c_off + (size_t)b0 * q.Wpad, q.Wpad, nb);
          PAWPY_CUDA(cudaEventCreateWithFlags(&d.c_chunk_ev[k][c], cudaEventDisableTiming));
          PAWPY_CUDA(cudaEventRecord(d.c_chunk_ev[k][c], up));
        }
        PAWPY_CUDA(cudaEventRecord(d.c_ev[k], up));
      }
    }
    d.c_ready = true;
    return;
  }
  DevBuf<float2> raw((size_t)d.nband * maxW);
  for (int k = 0; k < d.nk; k++) {
    DevKpt &q = d.kp[k];
    for (int b = 0; b < d.nband; b++)
      PAWPY_CUDA(cudaMemcpyAsync(raw.p + (size_t)b * q.W, host_band(d, k, b), sizeof(float2) * q.W,
                                 cudaMemcpyHostToDevice, stream()));
    q.perm_d.alloc(q.W);
    q.perm_d.upload(q.perm.data(), q.W);
    launch_permute(raw.p, q.W, q.perm_d.p, d.C.p + q.c_off, q.Wpad, d.nband);
  }
  d.c_ready = true;
}

static void twiddles(int n, DevBuf<float2> &out) {
  std::vector<float2> h(n);
  for (int i = 0; i < n; i++) {
    double a = 2.0 * M_PI * i / n;
    h[i] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
  out.alloc(n);
  out.upload(h.data(), n);
}

static void set_grid(DevWF &d, const int *fftg) {
  if (d.N[0] == fftg[0] && d.N[1] == fftg[1] && d.N[2] == fftg[2]) return;
  for (int a = 0; a < 3; a++) {
    PAWPY_REQUIRE(fftg[a] >= 1 && fftg[a] <= 4096, "bad FFT grid");
    d.r[a] = make_radices(fftg[a]);
    PAWPY_REQUIRE(d.r[a].ns >= 0, "FFT grid dimensions must factor into primes <= 13");
    d.N[a] = fftg[a];
    twiddles(fftg[a], d.tw[a]);
  }
  for (auto &q : d.kp) q.off_N2 = q.off_N3 = 0;
  d.p_ready = false;
  d.tables_ready = false;
  if (d.h_ready) {
    join_uploads(d);
    d.Hall.reset();
    d.h_ready = false;
  }
}

// Plane lists of one k-point for the plane FFT: start[p] = first sorted
// coefficient of g1 plane p, off[t] = cell j * N3 + k of coefficient t within its
// plane, and the occupied ranges of the other two axes.
struct PlaneLists {
  std::vector<int> start, off;
  int g2min = 0, n2 = 0, g3min = 0, n3 = 0, maxcnt = 0;
};

static void plane_lists(const DevWF &d, const DevKpt &q, PlaneLists &pl) {
  PAWPY_REQUIRE(q.n1 <= d.N[0], "FFT grid smaller than the plane-wave sphere along the first axis");
  const int N2 = d.N[1], N3 = d.N[2];
  pl.start.assign(q.n1 + 1, 0);
  pl.off.resize(q.W);
  int lo2 = 1 << 30, hi2 = -(1 << 30), lo3 = 1 << 30, hi3 = -(1 << 30);
  for (int t = 0; t < q.W; t++) {
    const int g2 = q.gsorted[3 * t + 1], g3 = q.gsorted[3 * t + 2];
    lo2 = std::min(lo2, g2);
    hi2 = std::max(hi2, g2);
    lo3 = std::min(lo3, g3);
    hi3 = std::max(hi3, g3);
  }
  // indices inside (-N, N) wrap with one compare; others take the modulus
  const bool near = q.W == 0 || (lo2 > -N2 && hi2 < N2 && lo3 > -N3 && hi3 < N3);
  for (int t = 0; t < q.W; t++) {
    const int g1 = q.gsorted[3 * t], g2 = q.gsorted[3 * t + 1], g3 = q.gsorted[3 * t + 2];
    pl.start[g1 - q.g1min + 1]++;
    int j, kk;
    if (near) {
      j = g2 < 0 ? g2 + N2 : g2;
      kk = g3 < 0 ? g3 + N3 : g3;
    } else {
      j = ((g2 % N2) + N2) % N2;
      kk = ((g3 % N3) + N3) % N3;
    }
    pl.off[t] = j * N3 + kk;
  }
  pl.g2min = q.W ? lo2 : 0;
  pl.n2 = q.W ? hi2 - lo2 + 1 : 0;
  pl.g3min = q.W ? lo3 : 0;
  pl.n3 = q.W ? hi3 - lo3 + 1 : 0;
  for (int p = 0; p < q.n1; p++) pl.maxcnt = std::max(pl.maxcnt, pl.start[p + 1]);
  for (int p = 0; p < q.n1; p++) pl.start[p + 1] += pl.start[p];
}

static void install_planes(DevWF &d, DevKpt &q, const PlaneLists &pl) {
  q.g2min = pl.g2min;
  q.n2 = pl.n2;
  q.g3min = pl.g3min;
  q.n3 = pl.n3;
  q.maxcnt = pl.maxcnt;
  q.plane_start.alloc(q.n1 + 1);
  q.plane_start.upload(pl.start.data(), q.n1 + 1);
  q.plane_off.alloc(std::max(q.W, 1));
  q.plane_off.upload(pl.off.data(), q.W);
  q.off_N2 = d.N[1];
  q.off_N3 = d.N[2];
}

static bool planes_current(const DevWF &d, const DevKpt &q) {
  return q.off_N2 == d.N[1] && q.off_N3 == d.N[2] && q.plane_off.p;
}

static void ensure_planes(DevWF &d, DevKpt &q) {
  if (planes_current(d, q)) return;
  PlaneLists pl;
  plane_lists(d, q, pl);
  install_planes(d, q, pl);
}

// The plane lists of every k-point, computed on host threads (the device
// copies are made on the calling thread's stream).
static void ensure_all_planes(DevWF &d) {
  std::vector<int> todo;
  for (int k = 0; k < d.nk; k++)
    if (!planes_current(d, d.kp[k])) todo.push_back(k);
  if (todo.empty()) return;
  HostPhase hp("plane_lists");
  std::vector<PlaneLists> pl(todo.size());
  parallel_for((int)todo.size(), [&](int i) { plane_lists(d, d.kp[todo[i]], pl[i]); });
  for (size_t i = 0; i < todo.size(); i++) install_planes(d, d.kp[todo[i]], pl[i]);
}

// ============================================================= species / spheres

static std::unique_ptr<SpeciesTables> species_tables(const ppot_t &pp) {
  HostPhase hp("species_tables");
  auto t = std::make_unique<SpeciesTables>();
  int nd = pp.proj_gridsize, np = pp.num_projs;
  t->nproj = np;
  t->total = pp.total_projs;
  PAWPY_REQUIRE(t->total <= 32, "more than 32 projector channels per element");
  for (int k = 0; k < np; k++)
    PAWPY_REQUIRE(pp.funcs[k].l >= 0 && pp.funcs[k].l <= 3, "projector channels need 0 <= l <= 3");
  std::vector<double> pf((size_t)np * nd), ps((size_t)np * 3 * nd), sf((size_t)np * nd), ss((size_t)np * 3 * nd);
  for (int k = 0; k < np; k++) {
    const funcset_t &f = pp.funcs[k];
    for (int j = 0; j < nd; j++) {
      pf[(size_t)k * nd + j] = f.proj[j];
      sf[(size_t)k * nd + j] = f.smooth_diffwave[j];
      for (int c = 0; c < 3; c++) {
        ps[((size_t)k * 3 + c) * nd + j] = f.proj_spline[c][j];
        ss[((size_t)k * 3 + c) * nd + j] = f.smooth_diffwave_spline[c][j];
      }
    }
    for (int m = -f.l; m <= f.l; m++) {
      t->lm_n.push_back(k);
      t->lm_l.push_back(f.l);
      t->lm_m.push_back(m);
    }
  }
  t->proj_f.alloc(pf.size());
  t->proj_f.upload(pf.data(), pf.size());
  t->proj_spl.alloc(ps.size());
  t->proj_spl.upload(ps.data(), ps.size());
  t->smooth_f.alloc(sf.size());
  t->smooth_f.upload(sf.data(), sf.size());
  t->smooth_spl.alloc(ss.size());
  t->smooth_spl.upload(ss.data(), ss.size());
  for (int which = 0; which < 2; which++) {
    SpeciesDev &s = which == 0 ? t->proj : t->smooth;
    s.f = which == 0 ? t->proj_f.p : t->smooth_f.p;
    s.spl = which == 0 ? t->proj_spl.p : t->smooth_spl.p;
    s.size = nd;
    s.nfunc = np;
    s.total = t->total;
    s.rmax = which == 0 ? pp.rmax : pp.wave_rmax;
    s.grid_rmax = s.rmax;
    s.r0_size = nd;
    s.h = s.grid_rmax / nd;
    s.inv_h = nd / s.grid_rmax;
    for (int i = 0; i < t->total; i++) {
      s.lm_l[i] = t->lm_l[i];
      s.lm_m[i] = t->lm_m[i];
      s.lm_f[i] = t->lm_n[i];
      int l = t->lm_l[i], m = t->lm_m[i];
      double f1 = 1, f2 = 1;
      for (int q = 2; q <= l - m; q++) f1 *= q;
      for (int q = 2; q <= l + m; q++) f2 *= q;
      double c = std::sqrt((2 * l + 1) / (4 * M_PI) * f1 / f2);
      if (m < 0) {
        // P_l^{-a} = (-1)^a (l-a)!/(l+a)! P_l^a (utils.c:379-380)
        const int a = -m;
        double ratio = 1.0;
        for (int q = l - a + 1; q <= l + a; q++) ratio *= q;
        c = c / ratio * ((a & 1) ? -1.0 : 1.0);
      }
      s.lm_coef[i] = c;
    }
  }
  {
    const int ng = pp.wave_gridsize;
    PAWPY_REQUIRE(ng >= 2 && pp.wave_grid[0] > 0, "partial-wave grid needs two positive points");
    std::vector<double> af((size_t)np * ng), as((size_t)np * 3 * ng);
    for (int k = 0; k < np; k++) {
      const funcset_t &f = pp.funcs[k];
      PAWPY_REQUIRE(f.diffwave && f.diffwave_spline, "element without (phi - phit) splines");
      for (int j = 0; j < ng; j++) {
        af[(size_t)k * ng + j] = f.diffwave[j];
        for (int c = 0; c < 3; c++) as[((size_t)k * 3 + c) * ng + j] = f.diffwave_spline[c][j];
      }
    }
    t->ae_x.alloc(ng);
    t->ae_x.upload(pp.wave_grid, ng);
    t->ae_f.alloc(af.size());
    t->ae_f.upload(af.data(), af.size());
    t->ae_spl.alloc(as.size());
    t->ae_spl.upload(as.data(), as.size());
    AeSpeciesDev &a = t->ae;
    a.x = t->ae_x.p;
    a.f = t->ae_f.p;
    a.spl = t->ae_spl.p;
    a.size = ng;
    a.nfunc = np;
    a.total = t->total;
    a.logstep = std::log(pp.wave_grid[1] / pp.wave_grid[0]);
    for (int i = 0; i < t->total; i++) {
      a.lm_l[i] = t->proj.lm_l[i];
      a.lm_m[i] = t->proj.lm_m[i];
      a.lm_f[i] = t->proj.lm_f[i];
      a.lm_coef[i] = t->proj.lm_coef[i];
    }
    t->ae_rmax = pp.wave_grid[ng - 1];
  }
  t->D.assign((size_t)t->total * t->total, 0.0);
  for (int i = 0; i < t->total; i++)
    for (int j = 0; j < t->total; j++)
      if (t->lm_l[i] == t->lm_l[j] && t->lm_m[i] == t->lm_m[j])
        t->D[(size_t)i * t->total + j] = pp.aepw_overlap_matrix[t->lm_n[i] * np + t->lm_n[j]] -
                                         pp.pspw_overlap_matrix[t->lm_n[i] * np + t->lm_n[j]];
  return t;
}

static double vnorm(const double *v) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }

// Sphere tables of sites site_nums (indices into coords/labels) of elements
// `sp` on the grid of lattice `lat`. Follows setup_site (utils.c:590-696): the
// half box per axis (|a_j x a_k| rmax / V) N + 1, the centre round(coord N),
// the cutoff (ndata_p - 1) rmax / ndata_{labels[s]} (the reference indexes the
// denominator by the list position s). Tables carry dV V^-1/2.
// One sphere set to build (the arguments of build_spheres).
struct SphereJob {
  SphereSet *S;
  const std::vector<int> *site_nums;
  const int *labels;
  const double *coords;
  const std::vector<std::unique_ptr<SpeciesTables>> *sp;
  bool smooth;
  const double *lat;
  const int *N;
  double vol;
  const std::vector<DevKpt> *kpts;
  const double *rec;
  // between the two phases
  std::vector<SpeciesDev> sd;
  std::vector<int2> slabs;
  std::vector<int> hc;
  DevBuf<double> Ld;
  DevBuf<int> Nd, counts;
  DevBuf<int2> slabs_d;
};

// Sphere tables of several sets with one host round trip: every set's slab counts are
// launched and read back together, then every set is compacted and tabulated. The counts,
// their read-back and the index lists run on the priority stream (after the library
// stream's work so far; the library stream then waits for them), so that the host's wait
// for the counts does not last as long as a first FFT pass on the auxiliary stream.
static void build_sphere_sets_on(std::vector<SphereJob> &jobs);
static void build_sphere_sets(std::vector<SphereJob> &jobs) {
  const cudaStream_t lib = stream();
  OwnedEvent start, done;
  start.record(lib);
  {
    OnStream on(prio_stream());
    start.wait(stream());
    build_sphere_sets_on(jobs);
    // the jobs' buffers, allocated on the priority stream, are freed on the library stream
    done.record(stream());
  }
  done.wait(lib);
}

static void build_sphere_sets_on(std::vector<SphereJob> &jobs) {
  HostPhase hp("spheres");
  auto cross = [](const double *a, const double *b, double *o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
  };
  // phase 1: site descriptors and slab counts of every set
  for (SphereJob &jb : jobs) {
    SphereSet &S = *jb.S;
    S.tab_ready.wait(stream());  // the old tables are freed in the library stream's order
    S = SphereSet();
    S.nsites = (int)jb.site_nums->size();
    if (S.nsites == 0) continue;
    const double *lat = jb.lat;
    const int *N = jb.N;
    for (auto &t : *jb.sp) jb.sd.push_back(jb.smooth ? t->smooth : t->proj);
    double c23[3], c13[3], c12[3];
    cross(lat + 3, lat + 6, c23);
    cross(lat + 0, lat + 6, c13);
    cross(lat + 0, lat + 3, c12);
    S.host.resize(S.nsites);
    int lmoff = 0;
    for (int s = 0; s < S.nsites; s++) {
      int p = (*jb.site_nums)[s];
      int e = jb.labels[p];
      PAWPY_REQUIRE(e >= 0 && e < (int)jb.sp->size(), "site label out of range");
      const SpeciesDev &spd = jb.sd[e];
      SiteDesc &h = S.host[s];
      for (int a = 0; a < 3; a++) h.coord[a] = jb.coords[3 * p + a];
      h.species = e;
      double rmax = spd.rmax;
      h.g[0] = (int)(vnorm(c23) * rmax / jb.vol * N[0]) + 1;
      h.g[1] = (int)(vnorm(c13) * rmax / jb.vol * N[1]) + 1;
      h.g[2] = (int)(vnorm(c12) * rmax / jb.vol * N[2]) + 1;
      for (int a = 0; a < 3; a++) h.c[a] = (int)std::round(jb.coords[3 * p + a] * N[a]);
      int e_s = jb.labels[s];
      PAWPY_REQUIRE(e_s >= 0 && e_s < (int)jb.sp->size(), "site label out of range");
      h.R0 = (spd.size - 1) * rmax / jb.sd[e_s].size;
      h.total = spd.total;
      h.lm_off = lmoff;
      lmoff += h.total;
      S.max_total = std::max(S.max_total, h.total);
      for (int q = 0; q <= 2 * h.g[1]; q++) jb.slabs.push_back(make_int2(s, q));
    }
    S.Ptot = lmoff;
    jb.Ld.alloc(9);
    jb.Ld.upload(lat, 9);
    jb.Nd.alloc(3);
    jb.Nd.upload(N, 3);
    S.sites.alloc(S.nsites);
    S.sites.upload(S.host.data(), S.nsites);
    jb.slabs_d.alloc(jb.slabs.size());
    jb.slabs_d.upload(jb.slabs.data(), jb.slabs.size());
    jb.counts.alloc(jb.slabs.size());
    launch_slab_count(S.sites.p, jb.slabs_d.p, (int)jb.slabs.size(), jb.Ld.p, jb.Nd.p, jb.counts.p);
  }
  for (SphereJob &jb : jobs) {
    if (jb.S->nsites == 0) continue;
    jb.hc.resize(jb.slabs.size());
    jb.counts.download(jb.hc.data(), jb.hc.size());
  }
  sync();
  // phase 2: compaction and tabulation of every set
  for (SphereJob &jb : jobs) {
    SphereSet &S = *jb.S;
    if (S.nsites == 0) continue;
    const double *lat = jb.lat;
    const int *N = jb.N;
    const double vol = jb.vol;
    const std::vector<int2> &slabs = jb.slabs;
    const std::vector<int> &hc = jb.hc;
    long long pt = 0, val = 0;
    S.site_pt.assign(S.nsites, 0);
    S.site_val.assign(S.nsites, 0);
    S.site_npts.assign(S.nsites, 0);
    for (size_t q = 0; q < slabs.size(); q++) S.site_npts[slabs[q].x] += hc[q];
    for (int s = 0; s < S.nsites; s++) {
      S.site_pt[s] = pt;
      S.site_val[s] = val;
      pt += S.site_npts[s];
      val += (long long)S.site_npts[s] * S.host[s].total;
    }
    pt = 0;
    for (size_t q = 0; q < slabs.size(); q++) {
      if (hc[q] == 0) continue;
      int s = slabs[q].x;
      SegFill f;
      f.site = s;
      f.jb = slabs[q].y;
      f.pt_off = pt;
      f.npts = hc[q];
      f.site_pt = S.site_pt[s];
      f.site_npts = S.site_npts[s];
      f.site_val = S.site_val[s];
      S.segs.push_back(f);
      int j = f.jb - S.host[s].g[1] + S.host[s].c[1];
      S.seg_plane.push_back(((j % N[1]) + N[1]) % N[1]);
      pt += hc[q];
    }
    S.nseg = (int)S.segs.size();
    S.npts = pt;
    S.nvals = val;
    S.species.alloc(jb.sd.size());
    S.species.upload(jb.sd.data(), jb.sd.size());
    S.nkp = (int)jb.kpts->size();
    std::vector<double> kc(3 * (size_t)S.nkp);
    for (int q = 0; q < S.nkp; q++)
      for (int a = 0; a < 3; a++)
        kc[3 * q + a] = (*jb.kpts)[q].kfrac[0] * jb.rec[a] + (*jb.kpts)[q].kfrac[1] * jb.rec[3 + a] +
                        (*jb.kpts)[q].kfrac[2] * jb.rec[6 + a];
    DevBuf<double> kcd(kc.size());
    kcd.upload(kc.data(), kc.size());
    S.idx.alloc(std::max(1LL, pt));
    S.tab.alloc(std::max(1LL, val));
    S.phase.alloc(std::max(1LL, pt * S.nkp));
    DevBuf<SegFill> segs_d(std::max(1, S.nseg));
    segs_d.upload(S.segs.data(), S.nseg);
    double wscale = vol / N[0] / N[1] / N[2] * std::pow(vol, -0.5);
    // half the smallest lattice-plane spacing: a point nearer its site than this has the
    // unwrapped box displacement as its unique minimum image
    double hmin = 1e300;
    for (int a = 0; a < 3; a++) {
      const double *u = lat + 3 * ((a + 1) % 3), *v = lat + 3 * ((a + 2) % 3);
      double c[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]};
      hmin = std::min(hmin, 0.5 * std::fabs(vol) / std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]));
    }
    // the points' indices and phases (what the pick needs) on the library stream; the table
    // values (needed only by the contraction, after the pick) on the auxiliary stream
    launch_seg_fill(S.sites.p, segs_d.p, S.nseg, S.species.p, jb.Ld.p, jb.Nd.p, wscale, hmin, kcd.p, S.nkp, pt,
                    S.idx.p, S.tab.p, S.phase.p, 1);
    OwnedEvent inputs;
    inputs.record(stream());
    {
      OnStream on(aux_stream());
      inputs.wait(stream());
      launch_seg_fill(S.sites.p, segs_d.p, S.nseg, S.species.p, jb.Ld.p, jb.Nd.p, wscale, hmin, kcd.p, S.nkp, pt,
                      S.idx.p, S.tab.p, S.phase.p, 2);
      S.tab_ready.record(stream());
      // the fills' inputs, released in the auxiliary stream's order (after both fills)
      DevBuf<double> kcd_done = std::move(kcd), L_done = std::move(jb.Ld);
      DevBuf<SegFill> segs_done = std::move(segs_d);
      DevBuf<int> N_done = std::move(jb.Nd);
    }
  }
}

static SphereJob sphere_job(SphereSet &S, const std::vector<int> &site_nums, const int *labels, const double *coords,
                            const std::vector<std::unique_ptr<SpeciesTables>> &sp, bool smooth, const double *lat,
                            const int *N, double vol, const std::vector<DevKpt> &kpts, const double *rec) {
  SphereJob jb;
  jb.S = &S;
  jb.site_nums = &site_nums;
  jb.labels = labels;
  jb.coords = coords;
  jb.sp = &sp;
  jb.smooth = smooth;
  jb.lat = lat;
  jb.N = N;
  jb.vol = vol;
  jb.kpts = &kpts;
  jb.rec = rec;
  return jb;
}

// Sphere tables of one set (setup_site, utils.c:590-696, for every site).
static void build_spheres(SphereSet &S, const std::vector<int> &site_nums, const int *labels,
                          const double *coords, const std::vector<std::unique_ptr<SpeciesTables>> &sp,
                          bool smooth, const double *lat, const int *N, double vol,
                          const std::vector<DevKpt> &kpts, const double *rec) {
  std::vector<SphereJob> jobs;
  jobs.push_back(sphere_job(S, site_nums, labels, coords, sp, smooth, lat, N, vol, kpts, rec));
  build_sphere_sets(jobs);
}

// One FFT pass over every band of wavefunction d, gathering onto several
// sphere sets at once. outs[i] receives [nk][nband][sets[i]->Ptot].
// PAWPY_GPU_FFT=generic selects the shared-memory FFT kernels for every grid
// (the register kernels are otherwise used for the lengths they are compiled for).
static bool generic_fft_forced() {
  const char *e = getenv("PAWPY_GPU_FFT");
  return e && strcmp(e, "generic") == 0;
}

// Geometry of k-point k for the plane FFT; true when the register kernels cover it.
static bool plane_geom(DevWF &d, int k, PlaneGeom &g) {
  DevKpt &q = d.kp[k];
  ensure_planes(d, q);
  g = PlaneGeom{d.N[0], d.N[1], d.N[2], q.g1min, q.n1};
  g.g2min = q.g2min;
  g.n2 = q.n2;
  g.g3min = q.g3min;
  g.n3 = q.n3;
  g.maxcnt = q.maxcnt;
  return q.n2 <= d.N[1] && q.n3 <= d.N[2] && fft_fast_supported(g) && !generic_fft_forced();
}

// Largest H of all k-points that the early first FFT pass may hold.
constexpr long long kEarlyPlanesBytes = 8LL << 30;
// Bands per launch of the early first pass.
constexpr int kEarlyChunkBands = 128;

static long long l2_bytes() {
  static long long v = -1;
  if (v < 0) {
    int b = 0;
    PAWPY_CUDA(cudaDeviceGetAttribute(&b, cudaDevAttrL2CacheSize, device()));
    v = b;
  }
  return v;
}

// Issues the first FFT pass of every band and k-point on the auxiliary stream
// (each k-point after its coefficient upload), so that it runs while the host
// builds the sphere tables; project_bands then runs the second pass from Hall.
// Only for grids of the register kernels, an H of at most kEarlyPlanesBytes,
// and k-points whose H exceeds the L2 cache anyway (measured: at 36x45x50 a
// k-point's 77 MB of H stays in L2 between the passes of the interleaved form,
// and the early form made the second pass 2.4 times slower). Threads on a
// stream of their own (the serving form) interleave requests instead: with
// several requests in flight the device has work, and the early form only added
// memory (measured: 9.7 -> 8.4 M pairs/s with 4 slots).
// PAWPY_GPU_EARLY_FFT=1 uses the early form whatever the size (0: never).
static void transform_planes_early(DevWF &d) {
  if (d.h_ready || d.grid_ready || d.nk == 0 || thread_has_stream()) return;
  const char *sw = getenv("PAWPY_GPU_EARLY_FFT");
  if (sw && sw[0] == '0') return;
  const bool force = sw && sw[0] == '1';
  std::vector<PlaneGeom> geo(d.nk);
  std::vector<size_t> off(d.nk);
  size_t total = 0, kmax = 0;
  for (int k = 0; k < d.nk; k++) {
    if (!plane_geom(d, k, geo[k])) return;
    off[k] = total;
    const size_t hk = (size_t)d.nband * d.kp[k].n1 * d.N[1] * d.N[2];
    total += hk;
    kmax = std::max(kmax, hk);
  }
  if ((long long)(total * sizeof(float2)) > kEarlyPlanesBytes) return;
  if (!force && (long long)(kmax * sizeof(float2)) <= l2_bytes()) return;
  HostPhase hp("early_planes");
  if (d.Hall.n < total || d.Hall.n == 0) d.Hall.alloc(std::max<size_t>(total, 1));
  d.hoff = off;
  if ((int)d.h_ev.size() != d.nk) {
    for (cudaEvent_t e : d.h_ev) PAWPY_CUDA(cudaEventDestroy(e));
    d.h_ev.assign(d.nk, nullptr);
    for (auto &e : d.h_ev) PAWPY_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  // the auxiliary stream starts after the allocation and the plane lists
  cudaEvent_t ready;
  PAWPY_CUDA(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
  PAWPY_CUDA(cudaEventRecord(ready, stream()));
  const cudaStream_t xs = aux_stream();
  PAWPY_CUDA(cudaStreamWaitEvent(xs, ready, 0));
  PAWPY_CUDA(cudaEventDestroy(ready));
  {
    OnStream on(xs);
    for (int k = 0; k < d.nk; k++) {
      DevKpt &q = d.kp[k];
      // in launches of kEarlyChunkBands bands: the launches on the priority stream (sphere
      // counts and index lists) are dispatched when a launch's blocks retire
      const size_t hb = (size_t)q.n1 * d.N[1] * d.N[2];
      for (int b0 = 0; b0 < d.nband; b0 += kEarlyChunkBands) {
        const int nb = std::min(kEarlyChunkBands, d.nband - b0);
        launch_fft_planes_fast(coeffs(d, k, b0, nb), q.Wpad, q.plane_start.p, q.plane_off.p, geo[k],
                               d.Hall.p + off[k] + b0 * hb, nb);
      }
      PAWPY_CUDA(cudaEventRecord(d.h_ev[k], xs));
    }
  }
  d.h_ready = true;
}

// the k-point is Gamma: its Bloch phases are all exactly 1
static bool kpoint_is_gamma(const DevKpt &q) { return q.kfrac[0] == 0.0 && q.kfrac[1] == 0.0 && q.kfrac[2] == 0.0; }

// values per k-point of the resident real-space wavefunctions (bands in tiles of 16)
static size_t grid_kstride(const DevWF &d) {
  return (size_t)ceil_div(d.nband, 16) * 16 * d.N[0] * d.N[1] * d.N[2];
}

static void project_bands(DevWF &d, const std::vector<const SphereSet *> &sets,
                          const std::vector<float2 *> &outs) {
  HostPhase hp("project_bands");
  ensure_coeffs(d);
  // merged point space (X) over the sets; segments sorted by plane for the pick
  std::vector<GatherSeg> segs;
  std::vector<int> plane_of;
  std::vector<ChunkContract> chunks;
  struct SetMaps {
    std::vector<int> col_site, col_lm, site_ptr, chunk_off;
  };
  std::vector<SetMaps> maps(sets.size());
  long long xtot = 0;
  int ptot = 0, max_total = 0;
  const int CHUNK = CHUNK_PTS;
  // The tensor-core form reads K blocks of 16 points per site: there every site of the merged
  // point space starts on a multiple of 16 (the gaps are zero in the picked rows).
  int set_max_total = 0;
  for (const SphereSet *S : sets) set_max_total = std::max(set_max_total, S->max_total);
  const bool tc = sphere_tc_enabled() && set_max_total > 0;
  std::vector<std::vector<long long>> site_x(sets.size());  // first point of each site
  for (size_t i = 0; i < sets.size(); i++) {
    const SphereSet &S = *sets[i];
    site_x[i].resize(S.nsites);
    for (int s = 0; s < S.nsites; s++) {
      if (tc) {
        site_x[i][s] = xtot;
        xtot += (S.site_npts[s] + 15) / 16 * 16;
      } else {
        site_x[i][s] = xtot + S.site_pt[s];
      }
    }
    if (!tc) xtot += S.npts;
  }
  const long long xspace = xtot;
  xtot = 0;
  for (size_t i = 0; i < sets.size(); i++) {
    const SphereSet &S = *sets[i];
    for (int q = 0; q < S.nseg; q++) {
      const SegFill &f = S.segs[q];
      GatherSeg g;
      g.idx = S.idx.p + f.pt_off;
      g.phase = S.phase.p + f.pt_off;
      g.phase_stride = S.npts;
      g.x_off = site_x[i][f.site] + (f.pt_off - f.site_pt);
      g.npts = f.npts;
      segs.push_back(g);
      plane_of.push_back(S.seg_plane[q]);
    }
    SetMaps &m = maps[i];
    m.col_site.resize(S.Ptot);
    m.col_lm.resize(S.Ptot);
    m.site_ptr.assign(S.nsites + 1, 0);
    for (int s = 0; s < S.nsites; s++) {
      int T = S.host[s].total;
      for (int t = 0; t < T; t++) {
        m.col_site[S.host[s].lm_off + t] = s;
        m.col_lm[S.host[s].lm_off + t] = t;
      }
      int n = S.site_npts[s];
      int nch = std::max(1, (n + CHUNK - 1) / CHUNK);
      for (int c = 0; c < nch; c++) {
        ChunkContract cc;
        int p0 = (int)((long long)n * c / nch), p1 = (int)((long long)n * (c + 1) / nch);
        cc.tab = S.tab.p + S.site_val[s] + p0;
        cc.x_off = xtot + S.site_pt[s] + p0;
        cc.site_npts = n;
        cc.npts = p1 - p0;
        cc.total = T;
        cc.part_off = ptot;
        m.chunk_off.push_back(ptot);
        ptot += T;
        chunks.push_back(cc);
      }
      m.site_ptr[s + 1] = (int)m.chunk_off.size();
      max_total = std::max(max_total, T);
    }
    xtot += S.npts;
  }
  xtot = xspace;
  std::vector<int> order(segs.size());
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return plane_of[a] < plane_of[b]; });
  std::vector<GatherSeg> sorted(segs.size());
  std::vector<int> pstart(d.N[1] + 1, 0);
  for (size_t q = 0; q < order.size(); q++) {
    sorted[q] = segs[order[q]];
    pstart[plane_of[order[q]] + 1]++;
  }
  for (int j = 0; j < d.N[1]; j++) pstart[j + 1] += pstart[j];
  DevBuf<GatherSeg> segs_d(std::max<size_t>(1, sorted.size()));
  segs_d.upload(sorted.data(), sorted.size());
  // the same points as one list in plane order, for the register FFT's pick
  std::vector<int> seg_base(std::max<size_t>(1, sorted.size()), 0), plane_first(d.N[1] + 1, 0);
  int max_plane_pts = 0;
  {
    int acc = 0;
    for (int j = 0; j < d.N[1]; j++) {
      plane_first[j] = acc;
      for (int q = pstart[j]; q < pstart[j + 1]; q++) {
        seg_base[q] = acc;
        acc += sorted[q].npts;
      }
      max_plane_pts = std::max(max_plane_pts, acc - plane_first[j]);
    }
    plane_first[d.N[1]] = acc;
  }
  DevBuf<int> seg_base_d(seg_base.size()), plane_first_d(plane_first.size());
  seg_base_d.upload(seg_base.data(), seg_base.size());
  plane_first_d.upload(plane_first.data(), plane_first.size());
  const long long npick = plane_first[d.N[1]];
  DevBuf<uint2> pick_ent(std::max(1LL, npick));
  DevBuf<float2> pick_phase(std::max(1LL, npick * d.nk));
  PickList plist;
  plist.plane_first = plane_first_d.p;
  plist.ent = pick_ent.p;
  plist.phase = pick_phase.p;
  plist.npts = npick;
  plist.max_plane_pts = max_plane_pts;
  for (size_t i = 0; i < sets.size(); i++)
    PAWPY_REQUIRE(sets[i]->nkp == d.nk, "sphere tables and wavefunction differ in k-points");
  DevBuf<int> pstart_d(pstart.size());
  pstart_d.upload(pstart.data(), pstart.size());
  DevBuf<ChunkContract> ch_d(std::max<size_t>(1, chunks.size()));
  ch_d.upload(chunks.data(), chunks.size());
  // per output column: first partial, chunk count and chunk stride of its site
  std::vector<DevBuf<int4>> mdev(sets.size());
  for (size_t i = 0; i < sets.size(); i++) {
    const SetMaps &m = maps[i];
    std::vector<int4> col(std::max<size_t>(1, m.col_site.size()));
    for (size_t o = 0; o < m.col_site.size(); o++) {
      const int s = m.col_site[o], e0 = m.site_ptr[s], ne = m.site_ptr[s + 1] - e0;
      const int stride = ne > 1 ? m.chunk_off[e0 + 1] - m.chunk_off[e0] : 0;
      col[o] = make_int4(m.chunk_off[e0] + m.col_lm[o], ne, stride, 0);
    }
    mdev[i].alloc(col.size());
    mdev[i].upload(col.data(), col.size());
  }
  // tensor-core form: one site per z, table planes built once per call
  std::vector<TcSite> tsites;
  std::vector<TcTable> ttabs;
  int tc_bn = 0, tc_brows = 0, tc_maxkb = 0;
  long long tc_lb = 0;
  DevBuf<TcSite> tsites_d;
  DevBuf<unsigned char> tc_planes;
  OwnedEvent planes_ready;
  if (tc) {
    tc_bn = tc_sphere_width(max_total);
    for (size_t i = 0; i < sets.size(); i++) {
      const SphereSet &S = *sets[i];
      for (int s = 0; s < S.nsites; s++) {
        const long long x_off = site_x[i][s];  // a multiple of 16
        const int lead = 0, n = S.site_npts[s];
        TcSite ts;
        ts.a_x = x_off;
        ts.nkb = (n + 15) / 16;
        ts.b_row = (int)tsites.size() * tc_bn;
        ts.total = S.host[s].total;
        ts.ld = S.Ptot;
        ts.out = outs[i] + S.host[s].lm_off;
        TcTable tt;
        tt.tab = S.tab.p + S.site_val[s];
        tt.npts = n;
        tt.lead = lead;
        tt.total = ts.total;
        tt.nkb = ts.nkb;
        tt.b_row = ts.b_row;
        tc_maxkb = std::max(tc_maxkb, ts.nkb);
        tsites.push_back(ts);
        ttabs.push_back(tt);
      }
    }
    tc_brows = (int)tsites.size() * tc_bn;
    tc_lb = (long long)std::max(1, tc_maxkb) * 32;
    tsites_d.alloc(std::max<size_t>(1, tsites.size()));
    tsites_d.upload(tsites.data(), tsites.size());
    // the table planes follow the sets' table values on the auxiliary stream, beside the pick
    OnStream on(aux_stream());
    for (const SphereSet *S : sets) S->tab_ready.wait(stream());
    tc_planes.alloc((size_t)2 * tc_brows * tc_lb * 2);
    DevBuf<TcTable> ttabs_d(std::max<size_t>(1, ttabs.size()));
    ttabs_d.upload(ttabs.data(), ttabs.size());
    launch_tc_tables(ttabs_d.p, (int)ttabs.size(), tc_maxkb, tc_bn, tc_brows, tc_lb, tc_planes.p);
    planes_ready.record(stream());
  }
  int maxn1 = 0;
  for (auto &q : d.kp) maxn1 = std::max(maxn1, q.n1);
  // FFT sub-batch: the plane-FFT intermediate H of a sub-batch stays within L2
  // between the two passes (PAWPY_GPU_FFT_BATCH_MB overrides the size)
  long long hband = (long long)maxn1 * d.N[1] * d.N[2] * (long long)sizeof(float2);
  long long hcap = kFftBatchBytes;
  if (const char *e = getenv("PAWPY_GPU_FFT_BATCH_MB")) hcap = std::max(1LL, atoll(e)) << 20;
  int fbatch = (int)std::max(1LL, std::min<long long>(d.nband, hcap / std::max(1LL, hband)));
  // Contraction batch: rows are (k-point, band) pairs, k-major, so that one
  // launch covers several k-points (the tables do not depend on k; the Bloch
  // phase is applied at the pick); picked points and partial sums of up to 2 GiB.
  // A wavefunction held in real space skips X: the contraction gathers its grid values.
  std::vector<PlaneGeom> geo(d.nk);
  std::vector<char> fast(d.nk);
  bool all_fast = true;
  for (int k = 0; k < d.nk; k++) {
    fast[k] = plane_geom(d, k, geo[k]);
    all_fast = all_fast && fast[k];
  }
  // The tensor-core form of a wavefunction not held in real space picks the sphere points into
  // rows in pass B; with PAWPY_GPU_DEFECT_GRID=1 pass B writes the real-space grids of the batch
  // instead (band-tiled, as a prepared basis holds them) and the contraction gathers from them.
  const char *dg_env = getenv("PAWPY_GPU_DEFECT_GRID");
  const bool dgrid_mode = tc && !d.grid_ready && all_fast && !generic_fft_forced() && dg_env && dg_env[0] == '1';
  const bool gather = d.grid_ready || dgrid_mode;
  const long long xstride = (xtot + 3) / 4 * 4;
  const long long per_row = ((gather ? 0 : xstride) + (tc ? 0 : ptot)) * (long long)sizeof(float2);
  const long long rows = (long long)d.nk * d.nband;
  // (the tensor-core form keeps no partial sums and reads the rows once: a larger batch, fewer launches)
  const long long xcap = tc ? kTcPickBatchBytes : (2LL << 30);
  long long cbatch = std::min({rows, 32768LL, std::max<long long>(fbatch, xcap / std::max(1LL, per_row))});
  // the gathered tensor-core form reads whole tiles of 16 bands: batches start on a k-point
  if (tc && gather) cbatch = std::min(rows, std::max(1LL, 32768LL / d.nband) * d.nband);
  const bool split_x = tc && !gather;  // pass B writes the split BF16 rows the tensor cores read
  const bool early = d.h_ready && !d.grid_ready;
  DevBuf<float2> H(d.grid_ready || early ? 0 : (size_t)fbatch * maxn1 * d.N[1] * d.N[2]);
  DevBuf<float2> dgrid;
  if (dgrid_mode && xtot > 0) {
    dgrid.alloc((size_t)d.nk * grid_kstride(d));
    for (int k = 0; k < d.nk; k++) {
      DevKpt &q = d.kp[k];
      float2 *gk = dgrid.p + (size_t)k * grid_kstride(d);
      if (early) {
        PAWPY_CUDA(cudaStreamWaitEvent(stream(), d.h_ev[k], 0));
        launch_fft_x_grid(d.Hall.p + d.hoff[k], geo[k], gk, 0, d.nband);
        continue;
      }
      for (int b0 = 0; b0 < d.nband; b0 += fbatch) {
        const int nb = std::min(fbatch, d.nband - b0);
        launch_fft_planes_fast(coeffs(d, k) + (size_t)b0 * q.Wpad, q.Wpad, q.plane_start.p, q.plane_off.p, geo[k],
                               H.p, nb);
        launch_fft_x_grid(H.p, geo[k], gk, b0, nb);
      }
    }
  }
  const float2 *grid_src = dgrid_mode ? dgrid.p : d.grid.p;
  DevBuf<float2> X(gather ? 1 : (size_t)cbatch * std::max(1LL, xstride));
  ContractSource src;
  DevBuf<int> gcell, seg_j_d;
  DevBuf<float2> gphase;
  if (gather) {
    // global cell and Bloch phase of every point of the merged point space
    std::vector<int> seg_j(std::max<size_t>(1, sorted.size()));
    for (size_t q = 0; q < order.size(); q++) seg_j[q] = plane_of[order[q]];
    seg_j_d.alloc(seg_j.size());
    seg_j_d.upload(seg_j.data(), seg_j.size());
    gcell.alloc(std::max(1LL, xtot));
    gphase.alloc(std::max(1LL, xtot * d.nk));
    // gaps of the aligned point space: no cell and a zero phase
    PAWPY_CUDA(cudaMemsetAsync(gcell.p, 0xFF, sizeof(int) * std::max(1LL, xtot), stream()));
    PAWPY_CUDA(cudaMemsetAsync(gphase.p, 0, sizeof(float2) * std::max(1LL, xtot * d.nk), stream()));
    launch_point_index(segs_d.p, seg_j_d.p, (int)sorted.size(), d.N[1], d.N[2], d.nk, xtot, gcell.p, gphase.p);
    src.grid = grid_src;
    src.n3d = (long long)d.N[0] * d.N[1] * d.N[2];
    src.gstride = (long long)grid_kstride(d);
    src.npts = xtot;
    src.nband = d.nband;
    src.gamma = true;
    for (auto &q : d.kp) src.gamma = src.gamma && kpoint_is_gamma(q);
    src.gcell = gcell.p;
    src.gphase = gphase.p;
  } else {
    src.X = X.p;
    src.xstride = xstride;
    src.xrows = split_x ? cbatch : 0;
  }
  // split rows: K blocks of 16 points, cbatch rows each (bf16split.cuh); the last block of a site
  // whose point count is not a multiple of 16 is zeroed before each batch's pick
  const long long lo_words = split_x ? cbatch * xstride : 0;
  const long long pick_stride = split_x ? cbatch * 16 : xstride;
  DevBuf<long long> tail_blocks;
  int ntail = 0;
  if (split_x) {
    std::vector<long long> tb;
    for (const TcSite &ts : tsites)
      if (ts.nkb > 0) tb.push_back(ts.a_x / 16 + ts.nkb - 1);
    ntail = (int)tb.size();
    tail_blocks.alloc(std::max<size_t>(1, tb.size()));
    tail_blocks.upload(tb.data(), tb.size());
  }
  DevBuf<float2> partial(tc ? 1 : (size_t)cbatch * std::max(1, ptot));
  if (xtot == 0) return;
  // the pick entries carry the offsets of the values in a band's row (32-bit)
  PAWPY_REQUIRE(!split_x || ((xtot + 15) / 16) * pick_stride < (1LL << 32), "picked rows too large for 32-bit offsets");
  if (!gather) launch_flatten_pick(segs_d.p, seg_base_d.p, (int)sorted.size(), d.nk, d.N[2], split_x ? pick_stride : 0,
                                   plist);
  for (long long r0 = 0; r0 < rows; r0 += cbatch) {
    const long long r1 = std::min(rows, r0 + cbatch);
    if (split_x) launch_zero_picked_blocks(X.p, tail_blocks.p, ntail, cbatch * 16, (int)(r1 - r0), lo_words);
    for (int k = (int)(r0 / d.nband); (long long)k * d.nband < r1; k++) {
      DevKpt &q = d.kp[k];
      const PlaneGeom &g = geo[k];
      const int blo = (int)(std::max(r0, (long long)k * d.nband) - (long long)k * d.nband);
      const int bhi = (int)(std::min(r1, (long long)(k + 1) * d.nband) - (long long)k * d.nband);
      // with the first pass done early, one second-pass launch per k-point
      const int step = early ? std::max(1, bhi - blo) : fbatch;
      for (int b0 = blo; b0 < bhi; b0 += step) {
        const int nb = std::min(step, bhi - b0);
        // first row of the sub-batch (in 32-bit words of the hi plane for the split rows)
        const long long roff = (long long)k * d.nband + b0 - r0;
        float2 *xb = gather   ? nullptr
                     : split_x ? reinterpret_cast<float2 *>(reinterpret_cast<uint32_t *>(X.p) + roff * 16)
                               : X.p + roff * xstride;
        if (gather) {
          // real-space wavefunctions (resident, or written above): the contraction reads them
        } else if (early) {
          PAWPY_CUDA(cudaStreamWaitEvent(stream(), d.h_ev[k], 0));
          launch_fft_x_pick_fast(d.Hall.p + d.hoff[k] + (size_t)b0 * q.n1 * d.N[1] * d.N[2], g, plist, k, xb,
                                 pick_stride, nb, lo_words, kpoint_is_gamma(q));
        } else if (fast[k]) {
          launch_fft_planes_fast(coeffs(d, k) + (size_t)b0 * q.Wpad, q.Wpad, q.plane_start.p, q.plane_off.p, g,
                                 H.p, nb);
          launch_fft_x_pick_fast(H.p, g, plist, k, xb, pick_stride, nb, lo_words, kpoint_is_gamma(q));
        } else {
          launch_fft_planes(coeffs(d, k) + (size_t)b0 * q.Wpad, q.Wpad, q.plane_start.p, q.plane_off.p, g,
                            d.r[1], d.r[2], d.tw[1].p, d.tw[2].p, H.p, nb);
          launch_fft_x_pick(H.p, g, d.r[0], d.tw[0].p, segs_d.p, pstart_d.p, k, xb, pick_stride, nb, lo_words,
                            plist.npts);
        }
      }
    }
    const int cn = (int)(r1 - r0);
    src.r0 = r0;
    if (tc) {
      planes_ready.wait(stream());
      launch_tc_sphere(tsites_d.p, (int)tsites.size(), tc_bn, tc_planes.p, tc_brows, tc_lb, src, cn, xtot, xtot);
      continue;
    }
    for (const SphereSet *S : sets) S->tab_ready.wait(stream());
    launch_contract_staged(ch_d.p, (int)chunks.size(), max_total, src, partial.p, ptot, cn, xtot);
    for (size_t i = 0; i < sets.size(); i++) {
      const SphereSet &S = *sets[i];
      if (S.nsites == 0) continue;
      launch_chunk_reduce(partial.p, ptot, mdev[i].p, outs[i], S.Ptot, cn, r0);
    }
  }
  if (early) {
    // consumed; the buffer stays with the wavefunction for its next first pass (a fresh
    // allocation of several GB from the stream-ordered pool was measured to block the host
    // for 2.6 ms); released with the wavefunction
    d.h_ready = false;
  }
}

// Real-space wavefunctions of every band, kept on the device (grid sizes with
// register kernels only); returns whether they were built.
static bool build_grids(DevWF &d) {
  HostPhase hp("build_grids");
  ensure_coeffs(d);
  const size_t n3d = (size_t)d.N[0] * d.N[1] * d.N[2];
  std::vector<PlaneGeom> geo(d.nk);
  int maxn1 = 0;
  for (int k = 0; k < d.nk; k++) {
    DevKpt &q = d.kp[k];
    ensure_planes(d, q);
    PlaneGeom g{d.N[0], d.N[1], d.N[2], q.g1min, q.n1};
    g.g2min = q.g2min;
    g.n2 = q.n2;
    g.g3min = q.g3min;
    g.n3 = q.n3;
    g.maxcnt = q.maxcnt;
    if (!(q.n2 <= d.N[1] && q.n3 <= d.N[2] && fft_fast_supported(g)) || generic_fft_forced()) return false;
    geo[k] = g;
    maxn1 = std::max(maxn1, q.n1);
  }
  d.grid.alloc((size_t)d.nk * grid_kstride(d));
  const long long hband = (long long)maxn1 * d.N[1] * d.N[2] * (long long)sizeof(float2);
  const int fbatch = (int)std::max(1LL, std::min<long long>(d.nband, kFftBatchBytes / std::max(1LL, hband)));
  DevBuf<float2> H((size_t)fbatch * maxn1 * d.N[1] * d.N[2]);
  for (int k = 0; k < d.nk; k++) {
    DevKpt &q = d.kp[k];
    for (int b0 = 0; b0 < d.nband; b0 += fbatch) {
      const int nb = std::min(fbatch, d.nband - b0);
      launch_fft_planes_fast(coeffs(d, k) + (size_t)b0 * q.Wpad, q.Wpad, q.plane_start.p, q.plane_off.p, geo[k],
                             H.p, nb);
      launch_fft_x_grid(H.p, geo[k], d.grid.p + (size_t)k * grid_kstride(d), b0, nb);
    }
  }
  d.grid_ready = true;
  return true;
}

// ============================================================= host projection_t output

static void fill_projection_list(projection_t *pl, const std::vector<int> &site_totals, const std::vector<int> &offs,
                                 const SpeciesTables *const *sp, const float2 *vals) {
  for (size_t s = 0; s < site_totals.size(); s++) {
    int T = site_totals[s];
    projection_t &p = pl[s];
    p.num_projs = sp[s]->nproj;
    p.total_projs = T;
    p.ns = static_cast<int *>(std::malloc(sizeof(int) * T));
    p.ls = static_cast<int *>(std::malloc(sizeof(int) * T));
    p.ms = static_cast<int *>(std::malloc(sizeof(int) * T));
    p.overlaps = static_cast<pawpy_c128 *>(std::malloc(sizeof(pawpy_c128) * T));
    if (!p.ns || !p.ls || !p.ms || !p.overlaps) throw std::bad_alloc();
    for (int i = 0; i < T; i++) {
      p.ns[i] = sp[s]->lm_n[i];
      p.ls[i] = sp[s]->lm_l[i];
      p.ms[i] = sp[s]->lm_m[i];
      float2 v = vals[offs[s] + i];
      p.overlaps[i] = pawpy_c128(v.x, v.y);
    }
  }
}

// ============================================================= setup_projections

static void do_setup_projections(pswf_t *wf, ppot_t *pps, int num_elems, int num_sites, const int *fftg,
                                 const int *labels, const double *coords) {
  PAWPY_REQUIRE(wf && pps && fftg && labels && coords, "setup_projections: NULL argument");
  PAWPY_REQUIRE(num_elems > 0 && num_sites > 0, "setup_projections: empty structure");
  DevWF &d = mirror(wf);
  // the coefficient upload (on the side stream, where the device reads host memory) runs during the
  // host's table and sphere work below
  ensure_coeffs(d);
  // attach as the reference does (projector.c:563-571); the wavefunction owns pps from now on
  if (wf->pps && wf->pps != pps) free_ppot_array(wf->pps, wf->num_elems);
  if (!wf->fftg) {
    wf->fftg = static_cast<int *>(std::malloc(3 * sizeof(int)));
    if (!wf->fftg) throw std::bad_alloc();
  }
  for (int a = 0; a < 3; a++) wf->fftg[a] = fftg[a];
  wf->num_elems = num_elems;
  wf->num_sites = num_sites;
  wf->pps = pps;
  for (int e = 0; e < num_elems; e++) pps[e].num_cart_gridpts = cart_gridpts_bound(pps[e], wf->lattice, fftg);
  set_grid(d, fftg);
  ensure_all_planes(d);
  // with the projections deferred to overlap_setup_real, the first FFT pass runs from here on,
  // beside the table, sphere and pair work (its launches of 128 bands let the sphere counts on the
  // priority stream through within one launch)
  if (!g_host_proj) transform_planes_early(d);
  d.species.clear();
  for (int e = 0; e < num_elems; e++) d.species.push_back(species_tables(pps[e]));
  d.labels.assign(labels, labels + num_sites);
  d.coords.assign(coords, coords + 3 * num_sites);
  std::vector<int> all(num_sites);
  std::iota(all.begin(), all.end(), 0);
  build_spheres(d.proj, all, d.labels.data(), d.coords.data(), d.species, false, d.lattice, d.N, d.vol, d.kp,
                d.rec);
  d.site_lmoff.resize(num_sites);
  for (int s = 0; s < num_sites; s++) d.site_lmoff[s] = d.proj.host[s].lm_off;
  d.P.alloc((size_t)d.nk * d.nband * d.proj.Ptot);
  d.tables_ready = true;
  d.p_ready = false;
  // With host projections off the transform is deferred, so that overlap_setup_real can gather the
  // smoothed partial waves in the same FFT pass (the reference transforms every band twice).
  if (g_host_proj) {
    project_bands(d, {&d.proj}, {d.P.p});
    d.p_ready = true;
  }
  {
    // results of earlier pairs involving this wavefunction are stale now
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    for (auto it = g_pairs.begin(); it != g_pairs.end();) {
      if (it->first.first == wf || it->first.second == wf)
        it = g_pairs.erase(it);
      else
        ++it;
    }
  }
  if (g_host_proj) {
    std::vector<float2> h((size_t)d.nk * d.nband * d.proj.Ptot);
    d.P.download(h.data(), h.size());
    sync();
    std::vector<int> tot(num_sites), off(num_sites);
    std::vector<const SpeciesTables *> sp(num_sites);
    for (int s = 0; s < num_sites; s++) {
      tot[s] = d.proj.host[s].total;
      off[s] = d.proj.host[s].lm_off;
      sp[s] = d.species[labels[s]].get();
    }
    for (int k = 0; k < d.nk; k++)
      for (int b = 0; b < d.nband; b++) {
        // noncollinear: device band 2b -> up_projections, 2b+1 -> down_projections of band b
        band_t *bd = wf->kpts[k]->bands[d.ncl ? b / 2 : b];
        projection_t *&slot = !d.ncl ? bd->projections : (b & 1) ? bd->down_projections : bd->up_projections;
        if (slot) {
          for (int s = 0; s < num_sites; s++) {
            std::free(slot[s].ns);
            std::free(slot[s].ls);
            std::free(slot[s].ms);
            std::free(slot[s].overlaps);
          }
          std::free(slot);
        }
        slot = static_cast<projection_t *>(std::calloc(num_sites, sizeof(projection_t)));
        if (!slot) throw std::bad_alloc();
        fill_projection_list(slot, tot, off, sp.data(),
                             h.data() + ((size_t)k * d.nband + b) * d.proj.Ptot);
      }
  }
  // Without host outputs the results stay on the device and the call returns with
  // its work queued: the next call's host preparation overlaps it (a kernel error
  // surfaces at that call's synchronisation).
  if (g_host_proj) sync();
}

// ============================================================= overlap_setup_real

static PairState &pair_state(pswf_t *R, pswf_t *S) {
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  auto key = std::make_pair((const pswf_t *)R, (const pswf_t *)S);
  auto &ptr = g_pairs[key];
  if (!ptr) {
    DevWF &r = mirror(R), &s = mirror(S);
    // a noncollinear wavefunction overlaps only with another one (spinor against spinor)
    if (r.ncl != s.ncl) {
      g_pairs.erase(key);
      throw Error(ERR_UNSUPPORTED, "overlaps between a noncollinear and a collinear wavefunction are not defined");
    }
    ptr = std::make_unique<PairState>();
    ptr->R = &r;
    ptr->S = &s;
  }
  return *ptr;
}

// N_RS pair matrices (projector.c:682-719, 816-843): radial integrals on the device,
// assembly on the host worker pool; the minimum-image displacements of the pairs.
static void pair_matrices(PairState &ps, pswf_t *wf_R, pswf_t *wf_S, const int *labels_R, const int *labels_S,
                          const double *coords_R, const double *coords_S) {
  const int nNRS = (int)ps.N_RS_R.size();
  ps.Q.assign(nNRS, {});
  HostPhase hp_pairs("pair_matrices");
  ps.dcoords.assign(3 * (size_t)nNRS, 0.0);
  {
    std::vector<int> eR(nNRS), eS(nNRS);
    std::vector<double> Rs(nNRS);
    for (int i = 0; i < nNRS; i++) {
      int s1 = ps.N_RS_R[i], s2 = ps.N_RS_S[i];
      double r;
      min_image_path(coords_S + 3 * s2, coords_R + 3 * s1, wf_R->lattice, ps.dcoords.data() + 3 * i, &r);
      eR[i] = labels_R[s1];
      eS[i] = labels_S[s2];
      Rs[i] = pair_distance(ps.dcoords.data() + 3 * i);
    }
    std::vector<std::vector<double>> I;
    std::vector<int> Lmax;
    offsite_radial_integrals(wf_R->pps, wf_S->pps, eR, eS, Rs, I, Lmax);
    for (int i = 0; i < nNRS; i++) {
      const ppot_t *p1 = wf_R->pps + eR[i];
      const ppot_t *p2 = wf_S->pps + eS[i];
      ps.Q[i].assign((size_t)p1->total_projs * p2->total_projs, 0.0);
    }
    // pairs are independent: the host worker pool assembles them in parallel
    host_parallel_for(nNRS, [&](int i) {
      offsite_pair_matrix(wf_R->pps + eR[i], wf_S->pps + eS[i], ps.dcoords.data() + 3 * i, I[i].data(), Lmax[i],
                          reinterpret_cast<pawpy_c128 *>(ps.Q[i].data()));
    });
  }
}

// The pair matrices and displacements as host-visible results with the reference's
// ownership (wf_S->overlaps / dcoords, freed by free_pswf).
static void publish_pair_matrices(PairState &ps, pswf_t *wf_R, pswf_t *wf_S) {
  const int nNRS = (int)ps.N_RS_R.size();
  if (wf_S->overlaps) {
    for (int i = 0; i < wf_S->num_aug_overlap_sites; i++) std::free(wf_S->overlaps[i]);
    std::free(wf_S->overlaps);
    wf_S->overlaps = nullptr;
  }
  std::free(wf_S->dcoords);
  wf_S->dcoords = nullptr;
  if (nNRS > 0) {
    wf_S->overlaps = static_cast<pawpy_c128 **>(std::malloc(sizeof(pawpy_c128 *) * nNRS));
    wf_S->dcoords = static_cast<double *>(std::malloc(sizeof(double) * 3 * nNRS));
    if (!wf_S->overlaps || !wf_S->dcoords) throw std::bad_alloc();
    for (int i = 0; i < nNRS; i++) {
      wf_S->overlaps[i] = static_cast<pawpy_c128 *>(std::malloc(sizeof(pawpy_c128) * ps.Q[i].size()));
      if (!wf_S->overlaps[i]) throw std::bad_alloc();
      std::memcpy(wf_S->overlaps[i], ps.Q[i].data(), sizeof(pawpy_c128) * ps.Q[i].size());
    }
    std::memcpy(wf_S->dcoords, ps.dcoords.data(), sizeof(double) * 3 * nNRS);
  }
  wf_S->num_aug_overlap_sites = nNRS;
  wf_R->num_aug_overlap_sites = nNRS;
}

static void do_overlap_setup_real(pswf_t *wf_R, pswf_t *wf_S, const int *labels_R, const int *labels_S,
                                  const double *coords_R, const double *coords_S, const int *N_R, const int *N_S,
                                  const int *N_RS_R, const int *N_RS_S, int nNR, int nNS, int nNRS) {
  PAWPY_REQUIRE(wf_R && wf_S, "overlap_setup_real: NULL wavefunction");
  DevWF &R = mirror(wf_R);
  DevWF &S = mirror(wf_S);
  PAWPY_REQUIRE(R.tables_ready && S.tables_ready, "overlap_setup_real needs setup_projections on both wavefunctions");
  PAWPY_REQUIRE(R.nk == S.nk, "basis and defect differ in k-points");
  PairState &ps = pair_state(wf_R, wf_S);
  ps.N_R.assign(N_R, N_R + (N_R ? nNR : 0));
  ps.N_S.assign(N_S, N_S + (N_S ? nNS : 0));
  ps.N_RS_R.assign(N_RS_R, N_RS_R + (N_RS_R ? nNRS : 0));
  ps.N_RS_S.assign(N_RS_S, N_RS_S + (N_RS_S ? nNRS : 0));
  PAWPY_REQUIRE((int)ps.N_R.size() == nNR && (int)ps.N_S.size() == nNS && (int)ps.N_RS_R.size() == nNRS &&
                    (int)ps.N_RS_S.size() == nNRS,
                "overlap_setup_real: NULL site list with a nonzero length");
  ps.aug_ready = false;
  ps.pseudo_ready[0] = ps.pseudo_ready[1] = false;
  ps.recip = false;
  ps.cross_ready[0] = ps.cross_ready[1] = false;
  // The N_RS pair matrices depend only on the species and positions: a host thread computes them
  // (radial integrals on this thread's high-priority upload stream, which is idle by then,
  // assembly on the host pool)
  // while this thread builds the sphere tables and issues the projections.
  const cudaStream_t aux = side_stream();
  const int dev = device();
  std::exception_ptr pair_err;
  std::thread pair_thread([&, aux, dev] {
    try {
      PAWPY_CUDA(cudaSetDevice(dev));
      OnStream on(aux);
      pair_matrices(ps, wf_R, wf_S, labels_R, labels_S, coords_R, coords_S);
    } catch (...) {
      pair_err = std::current_exception();
    }
  });
  struct Joiner {
    std::thread &t;
    ~Joiner() {
      if (t.joinable()) t.join();
    }
  } joiner{pair_thread};
  // smoothed partial waves of R's N_R sites on S's grid, and of S's N_S sites on R's grid
  {
    std::vector<SphereJob> jobs;
    jobs.push_back(sphere_job(ps.sm_NR, ps.N_R, labels_R, coords_R, R.species, true, S.lattice, S.N, S.vol, S.kp,
                              S.rec));
    jobs.push_back(sphere_job(ps.sm_NS, ps.N_S, labels_S, coords_S, S.species, true, R.lattice, R.N, R.vol, R.kp,
                              R.rec));
    build_sphere_sets(jobs);
  }
  ps.WP_S.alloc(std::max<size_t>(1, (size_t)S.nk * S.nband * ps.sm_NR.Ptot));
  ps.WP_R.alloc(std::max<size_t>(1, (size_t)R.nk * R.nband * ps.sm_NS.Ptot));
  // one FFT pass per wavefunction: pending <p|psi> and the smoothed-partial-wave projections together
  for (int side = 0; side < 2; side++) {
    DevWF &W = side == 0 ? S : R;
    const SphereSet *sm = side == 0 ? &ps.sm_NR : &ps.sm_NS;
    float2 *wp = side == 0 ? ps.WP_S.p : ps.WP_R.p;
    std::vector<const SphereSet *> sets;
    std::vector<float2 *> outs;
    if (!W.p_ready) {
      sets.push_back(&W.proj);
      outs.push_back(W.P.p);
    }
    if (sm->nsites > 0) {
      sets.push_back(sm);
      outs.push_back(wp);
    }
    if (!sets.empty()) project_bands(W, sets, outs);
    if (!W.p_ready) W.p_ready = true;  // a prepared, shared basis is only read
  }
  pair_thread.join();
  if (pair_err) std::rethrow_exception(pair_err);
  publish_pair_matrices(ps, wf_R, wf_S);
  free_wave_projections(wf_R);
  free_wave_projections(wf_S);
  wf_R->wp_num = nNS;
  wf_S->wp_num = nNR;
  // host wave_projections have the reference's collinear layout (none for spinor bands)
  if (g_host_proj && !R.ncl) {
    for (int side = 0; side < 2; side++) {
      DevWF &W = side == 0 ? S : R;
      SphereSet &sm = side == 0 ? ps.sm_NR : ps.sm_NS;
      DevBuf<float2> &wp = side == 0 ? ps.WP_S : ps.WP_R;
      const std::vector<int> &lst = side == 0 ? ps.N_R : ps.N_S;
      const int *lab = side == 0 ? labels_R : labels_S;
      DevWF &owner = side == 0 ? R : S;
      if (lst.empty()) continue;
      std::vector<float2> h((size_t)W.nk * W.nband * sm.Ptot);
      wp.download(h.data(), h.size());
      sync();
      std::vector<int> tot(lst.size()), off(lst.size());
      std::vector<const SpeciesTables *> sp(lst.size());
      for (size_t s = 0; s < lst.size(); s++) {
        tot[s] = sm.host[s].total;
        off[s] = sm.host[s].lm_off;
        sp[s] = owner.species[lab[lst[s]]].get();
      }
      for (int k = 0; k < W.nk; k++)
        for (int b = 0; b < W.nband; b++) {
          band_t *bd = W.wf->kpts[k]->bands[b];
          bd->wave_projections = static_cast<projection_t *>(std::calloc(lst.size(), sizeof(projection_t)));
          if (!bd->wave_projections) throw std::bad_alloc();
          fill_projection_list(bd->wave_projections, tot, off, sp.data(),
                               h.data() + ((size_t)k * W.nband + b) * sm.Ptot);
        }
    }
  }
  ps.ready = true;
  if (g_host_proj) sync();  // without host outputs the work stays queued (see do_setup_projections)
}


// ============================================================= overlap_setup_recip

static void ensure_projections(DevWF &d);

// Device copy of a RecipSpread (the sphere points of a set per grid cell, see kernels.h).
struct RecipSpreadDev {
  DevBuf<int> cell_first, ucell, ent_first, ent_site, site_npts, site_total, site_pcol;
  DevBuf<long long> ent_pt, site_pt, site_val;
  RecipSpread view;
};

// Groups the points of sphere set S (sites site_nums of W, tables on W's grid) per grid
// cell of each plane j, entries of a cell in site order (the order of the sums in
// get_aug_freqs_helper, projector.c:305-329).
static void build_recip_spread(const SphereSet &S, const DevWF &W, const std::vector<int> &site_nums,
                               RecipSpreadDev &out) {
  HostPhase hp("recip_spread_lists");
  const int N2 = W.N[1];
  std::vector<int> idx(std::max<long long>(1, S.npts));
  S.idx.download(idx.data(), S.npts);
  sync();
  // entries per plane, site-major as the segments are
  std::vector<std::vector<std::pair<int, long long>>> per_plane(N2);  // (cell, point)
  std::vector<std::vector<int>> per_plane_site(N2);
  for (int q = 0; q < S.nseg; q++) {
    const SegFill &f = S.segs[q];
    const int j = S.seg_plane[q];
    for (int t = 0; t < f.npts; t++) {
      per_plane[j].emplace_back(idx[f.pt_off + t], f.pt_off + t);
      per_plane_site[j].push_back(f.site);
    }
  }
  std::vector<int> cell_first(N2 + 1, 0), ucell, ent_first(1, 0), ent_site;
  std::vector<long long> ent_pt;
  for (int j = 0; j < N2; j++) {
    auto &v = per_plane[j];
    std::vector<int> ord(v.size());
    std::iota(ord.begin(), ord.end(), 0);
    // by cell; equal cells keep their site-major order
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return v[a].first < v[b].first; });
    for (size_t e = 0; e < ord.size(); e++) {
      const int o = ord[e];
      if (e == 0 || v[o].first != v[ord[e - 1]].first) {
        if (e > 0) ent_first.push_back((int)ent_pt.size());
        ucell.push_back(v[o].first);
      }
      ent_pt.push_back(v[o].second);
      ent_site.push_back(per_plane_site[j][o]);
    }
    if (!ord.empty()) ent_first.push_back((int)ent_pt.size());
    cell_first[j + 1] = (int)ucell.size();
  }
  PAWPY_REQUIRE(ent_first.size() == ucell.size() + 1, "aug_recip: spread lists are inconsistent");
  std::vector<int> npts(S.nsites), tot(S.nsites), pcol(S.nsites);
  for (int s = 0; s < S.nsites; s++) {
    npts[s] = S.site_npts[s];
    tot[s] = S.host[s].total;
    pcol[s] = W.site_lmoff[site_nums[s]];
  }
  auto up_i = [](DevBuf<int> &d, const std::vector<int> &h) {
    d.alloc(std::max<size_t>(1, h.size()));
    d.upload(h.data(), h.size());
  };
  auto up_l = [](DevBuf<long long> &d, const std::vector<long long> &h) {
    d.alloc(std::max<size_t>(1, h.size()));
    d.upload(h.data(), h.size());
  };
  up_i(out.cell_first, cell_first);
  up_i(out.ucell, ucell);
  up_i(out.ent_first, ent_first);
  up_i(out.ent_site, ent_site);
  up_l(out.ent_pt, ent_pt);
  up_l(out.site_pt, S.site_pt);
  up_l(out.site_val, S.site_val);
  up_i(out.site_npts, npts);
  up_i(out.site_total, tot);
  up_i(out.site_pcol, pcol);
  RecipSpread &c = out.view;
  c.cell_first = out.cell_first.p;
  c.ucell = out.ucell.p;
  c.ent_first = out.ent_first.p;
  c.ent_site = out.ent_site.p;
  c.ent_pt = out.ent_pt.p;
  c.site_pt = out.site_pt.p;
  c.site_val = out.site_val.p;
  c.site_npts = out.site_npts.p;
  c.site_total = out.site_total.p;
  c.site_pcol = out.site_pcol.p;
  c.tab = S.tab.p;
  c.phase = S.phase.p;
  c.npts = S.npts;
  // the kernels that read these tables are ordered after their values
  S.tab_ready.wait(stream());
}

// CA[k][band][Wpad] of every band of W (get_aug_freqs for the sites site_nums of W whose
// smoothed tables on W's own grid are sm), in the sorted plane-wave order; with D given
// also D = C + CA. Needs W's projector coefficients.
static void recip_coefficients(DevWF &W, const SphereSet &sm, const std::vector<int> &site_nums,
                               DevBuf<float2> &CA, DevBuf<float2> *D) {
  HostPhase hp("recip_coefficients");
  ensure_coeffs(W);
  const size_t total = W.C.n;
  CA.alloc(std::max<size_t>(1, total));
  CA.zero();
  if (D) {
    D->alloc(std::max<size_t>(1, total));
    D->zero();
  }
  if (sm.nsites == 0) return;
  RecipSpreadDev sp;
  build_recip_spread(sm, W, site_nums, sp);
  int maxn1 = 0;
  for (auto &q : W.kp) maxn1 = std::max(maxn1, q.n1);
  const long long hband = (long long)maxn1 * W.N[1] * W.N[2] * (long long)sizeof(float2);
  const int fbatch = (int)std::max(1LL, std::min<long long>(W.nband, kFftBatchBytes / std::max(1LL, hband)));
  DevBuf<float2> H((size_t)fbatch * maxn1 * W.N[1] * W.N[2]);
  const int Pt = W.proj.Ptot;
  for (int k = 0; k < W.nk; k++) {
    PlaneGeom g;
    plane_geom(W, k, g);
    DevKpt &q = W.kp[k];
    const float2 *Ck = coeffs(W, k);
    for (int b0 = 0; b0 < W.nband; b0 += fbatch) {
      const int nb = std::min(fbatch, W.nband - b0);
      launch_recip_xspread(sp.view, W.P.p + ((size_t)k * W.nband + b0) * Pt, Pt, W.nk, k, g, W.r[0], W.tw[0].p,
                           H.p, nb);
      const size_t off = q.c_off + (size_t)b0 * q.Wpad;
      launch_recip_planes_pick(H.p, g, q.plane_start.p, q.plane_off.p, W.r[1], W.r[2], W.tw[1].p, W.tw[2].p,
                               Ck + (size_t)b0 * q.Wpad, q.Wpad, CA.p + off, D ? D->p + off : nullptr, nb);
    }
  }
}

// band->CAs of every band of W (malloc'd complex64 in the file's plane-wave order), as
// get_aug_freqs leaves them (projector.c:445-446).
static void publish_recip_coefficients(DevWF &W, const DevBuf<float2> &CA) {
  std::vector<float2> h(W.C.n);
  CA.download(h.data(), h.size());
  sync();
  for (int k = 0; k < W.nk; k++) {
    const DevKpt &q = W.kp[k];
    for (int b = 0; b < W.nband; b++) {
      band_t *bd = W.wf->kpts[k]->bands[b];
      std::free(bd->CAs);
      bd->CAs = static_cast<pawpy_c64 *>(std::calloc(std::max(1, q.W), sizeof(pawpy_c64)));
      if (!bd->CAs) throw std::bad_alloc();
      const float2 *src = h.data() + q.c_off + (size_t)b * q.Wpad;
      for (int t = 0; t < q.W; t++) bd->CAs[q.perm[t]] = pawpy_c64(src[t].x, src[t].y);
    }
  }
}

static void do_overlap_setup_recip(pswf_t *wf_R, pswf_t *wf_S, const int *labels_R, const int *labels_S,
                                   const double *coords_R, const double *coords_S, const int *N_R, const int *N_S,
                                   const int *N_RS_R, const int *N_RS_S, int nNR, int nNS, int nNRS) {
  PAWPY_REQUIRE(wf_R && wf_S, "overlap_setup_recip: NULL wavefunction");
  DevWF &R = mirror(wf_R);
  DevWF &S = mirror(wf_S);
  PAWPY_REQUIRE(R.tables_ready && S.tables_ready, "overlap_setup_recip needs setup_projections on both wavefunctions");
  PAWPY_REQUIRE(R.nk == S.nk, "basis and defect differ in k-points");
  PairState &ps = pair_state(wf_R, wf_S);
  ps.N_R.assign(N_R, N_R + (N_R ? nNR : 0));
  ps.N_S.assign(N_S, N_S + (N_S ? nNS : 0));
  ps.N_RS_R.assign(N_RS_R, N_RS_R + (N_RS_R ? nNRS : 0));
  ps.N_RS_S.assign(N_RS_S, N_RS_S + (N_RS_S ? nNRS : 0));
  PAWPY_REQUIRE((int)ps.N_R.size() == nNR && (int)ps.N_S.size() == nNS && (int)ps.N_RS_R.size() == nNRS &&
                    (int)ps.N_RS_S.size() == nNRS,
                "overlap_setup_recip: NULL site list with a nonzero length");
  ps.aug_ready = false;
  ps.pseudo_ready[0] = ps.pseudo_ready[1] = false;
  ps.cross_ready[0] = ps.cross_ready[1] = false;
  ps.recip = true;
  // smoothed partial waves of R's N_R sites on R's grid and of S's N_S sites on S's grid
  // (overlap_setup_recip, projector.c:746-789); no real-space smoothed-wave projections
  build_spheres(ps.sm_NR, ps.N_R, labels_R, coords_R, R.species, true, R.lattice, R.N, R.vol, R.kp, R.rec);
  build_spheres(ps.sm_NS, ps.N_S, labels_S, coords_S, S.species, true, S.lattice, S.N, S.vol, S.kp, S.rec);
  ps.WP_S.alloc(1);
  ps.WP_R.alloc(1);
  ensure_projections(R);
  ensure_projections(S);
  recip_coefficients(R, ps.sm_NR, ps.N_R, ps.CA_R, nullptr);
  recip_coefficients(S, ps.sm_NS, ps.N_S, ps.CA_S, &ps.D_S);
  pair_matrices(ps, wf_R, wf_S, labels_R, labels_S, coords_R, coords_S);
  publish_pair_matrices(ps, wf_R, wf_S);
  free_wave_projections(wf_R);
  free_wave_projections(wf_S);
  wf_R->wp_num = nNS;
  wf_S->wp_num = nNR;
  if (g_host_proj && !R.ncl) {
    if (!ps.N_R.empty()) publish_recip_coefficients(R, ps.CA_R);
    if (!ps.N_S.empty()) publish_recip_coefficients(S, ps.CA_S);
  }
  ps.ready = true;
  if (g_host_proj) sync();
}


// ============================================================= all-electron real-space wavefunctions

// The real-space sphere tables of d's sites on grid N (built once per grid and site list).
static AeTables &ae_tables(DevWF &d, const int *N, const int *labels, const double *coords) {
  PAWPY_REQUIRE(d.tables_ready, "real-space wavefunctions need setup_projections first");
  const int ns = (int)d.labels.size();
  std::vector<int> lab(labels, labels + ns);
  std::vector<double> crd(coords, coords + 3 * (size_t)ns);
  if (d.ae && d.ae->N[0] == N[0] && d.ae->N[1] == N[1] && d.ae->N[2] == N[2] && d.ae->labels == lab &&
      d.ae->coords == crd)
    return *d.ae;
  HostPhase hp("ae_tables");
  auto t = std::make_unique<AeTables>();
  for (int a = 0; a < 3; a++) {
    PAWPY_REQUIRE(N[a] >= 1 && N[a] <= 4096, "bad FFT grid");
    t->N[a] = N[a];
    t->r[a] = make_radices(N[a]);
    PAWPY_REQUIRE(t->r[a].ns >= 0, "FFT grid dimensions must factor into primes <= 13");
    twiddles(N[a], t->tw[a]);
  }
  PAWPY_REQUIRE(3 * (size_t)std::max({N[0], N[1], N[2]}) * sizeof(float2) <= 227 * 1024,
                "real-space grid lines do not fit in shared memory");
  t->labels = lab;
  t->coords = crd;
  const double *lat = d.lattice;
  auto cross = [](const double *a, const double *b, double *o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
  };
  double c23[3], c13[3], c12[3];
  cross(lat + 3, lat + 6, c23);
  cross(lat + 0, lat + 6, c13);
  cross(lat + 0, lat + 3, c12);
  // boxes and cutoffs of realspace_state (density.c:269-287): half box (|a_j x a_k| rmax / V) N + 1
  // around round(coord N), rmax the last point of the element's partial-wave grid
  std::vector<SiteDesc> host(ns);
  std::vector<int2> slabs;
  std::vector<AeSpeciesDev> sd;
  for (auto &sp : d.species) sd.push_back(sp->ae);
  for (int s = 0; s < ns; s++) {
    const int e = lab[s];
    PAWPY_REQUIRE(e >= 0 && e < (int)d.species.size(), "site label out of range");
    const double rmax = d.species[e]->ae_rmax;
    SiteDesc &h = host[s];
    for (int a = 0; a < 3; a++) h.coord[a] = crd[3 * s + a];
    h.species = e;
    h.g[0] = (int)(vnorm(c23) * rmax / d.vol * N[0]) + 1;
    h.g[1] = (int)(vnorm(c13) * rmax / d.vol * N[1]) + 1;
    h.g[2] = (int)(vnorm(c12) * rmax / d.vol * N[2]) + 1;
    for (int a = 0; a < 3; a++) h.c[a] = (int)std::round(crd[3 * s + a] * N[a]);
    h.R0 = rmax;
    h.total = d.species[e]->total;
    h.lm_off = d.site_lmoff[s];
    for (int jb = 0; jb <= 2 * h.g[1]; jb++) slabs.push_back(make_int2(s, jb));
  }
  DevBuf<double> Ld(9);
  Ld.upload(lat, 9);
  DevBuf<int> Nd(3);
  Nd.upload(N, 3);
  DevBuf<SiteDesc> sites(std::max(1, ns));
  sites.upload(host.data(), ns);
  DevBuf<int2> slabs_d(std::max<size_t>(1, slabs.size()));
  slabs_d.upload(slabs.data(), slabs.size());
  DevBuf<int> counts(std::max<size_t>(1, slabs.size()));
  launch_ae_count(sites.p, slabs_d.p, (int)slabs.size(), Ld.p, Nd.p, counts.p);
  std::vector<int> hc(slabs.size());
  counts.download(hc.data(), hc.size());
  sync();
  std::vector<long long> site_pt(ns, 0), site_val(ns, 0);
  std::vector<int> site_npts(ns, 0), site_total(ns), site_pcol(ns);
  for (size_t q = 0; q < slabs.size(); q++) site_npts[slabs[q].x] += hc[q];
  long long pt = 0, val = 0;
  for (int s = 0; s < ns; s++) {
    site_pt[s] = pt;
    site_val[s] = val;
    site_total[s] = host[s].total;
    site_pcol[s] = host[s].lm_off;
    pt += site_npts[s];
    val += (long long)site_npts[s] * host[s].total;
  }
  std::vector<SegFill> segs;
  pt = 0;
  for (size_t q = 0; q < slabs.size(); q++) {
    if (hc[q] == 0) continue;
    SegFill f;
    f.site = slabs[q].x;
    f.jb = slabs[q].y;
    f.pt_off = pt;
    f.npts = hc[q];
    f.site_pt = site_pt[f.site];
    f.site_npts = site_npts[f.site];
    f.site_val = site_val[f.site];
    segs.push_back(f);
    pt += hc[q];
  }
  t->npts = pt;
  std::vector<double> kf(3 * (size_t)d.nk);
  for (int k = 0; k < d.nk; k++)
    for (int a = 0; a < 3; a++) kf[3 * k + a] = d.kp[k].kfrac[a];
  DevBuf<double> kfd(kf.size());
  kfd.upload(kf.data(), kf.size());
  DevBuf<AeSpeciesDev> spd(sd.size());
  spd.upload(sd.data(), sd.size());
  DevBuf<SegFill> segs_d(std::max<size_t>(1, segs.size()));
  segs_d.upload(segs.data(), segs.size());
  t->cell.alloc(std::max(1LL, pt));
  t->val.alloc(std::max(1LL, val));
  t->phase.alloc(std::max(1LL, pt * d.nk));
  launch_ae_fill(sites.p, segs_d.p, (int)segs.size(), spd.p, Ld.p, Nd.p, kfd.p, d.nk, pt, t->cell.p, t->val.p,
                 t->phase.p);
  // the points of every cell, sites in order (segments are site-major)
  std::vector<int> cell(std::max(1LL, pt));
  t->cell.download(cell.data(), pt);
  sync();
  std::vector<int> site_of(std::max(1LL, pt));
  for (const SegFill &f : segs)
    for (int q = 0; q < f.npts; q++) site_of[f.pt_off + q] = f.site;
  std::vector<long long> ord(pt);
  std::iota(ord.begin(), ord.end(), 0LL);
  std::stable_sort(ord.begin(), ord.end(), [&](long long a, long long b) { return cell[a] < cell[b]; });
  std::vector<int> ucell, ent_first(1, 0), ent_site;
  std::vector<long long> ent_pt;
  for (size_t e = 0; e < ord.size(); e++) {
    const long long o = ord[e];
    if (e > 0 && cell[o] != cell[ord[e - 1]]) ent_first.push_back((int)e);
    if (e == 0 || cell[o] != cell[ord[e - 1]]) ucell.push_back(cell[o]);
    ent_pt.push_back(o);
    ent_site.push_back(site_of[o]);
  }
  if (pt > 0) ent_first.push_back((int)pt);
  auto up_i = [](DevBuf<int> &b, const std::vector<int> &h) {
    b.alloc(std::max<size_t>(1, h.size()));
    b.upload(h.data(), h.size());
  };
  auto up_l = [](DevBuf<long long> &b, const std::vector<long long> &h) {
    b.alloc(std::max<size_t>(1, h.size()));
    b.upload(h.data(), h.size());
  };
  up_i(t->ucell, ucell);
  up_i(t->ent_first, ent_first);
  up_i(t->ent_site, ent_site);
  up_l(t->ent_pt, ent_pt);
  up_l(t->site_pt, site_pt);
  up_l(t->site_val, site_val);
  up_i(t->site_npts, site_npts);
  up_i(t->site_total, site_total);
  up_i(t->site_pcol, site_pcol);
  AeSpread &v = t->view;
  v.ncell = (int)ucell.size();
  v.ucell = t->ucell.p;
  v.ent_first = t->ent_first.p;
  v.ent_site = t->ent_site.p;
  v.ent_pt = t->ent_pt.p;
  v.site_pt = t->site_pt.p;
  v.site_val = t->site_val.p;
  v.site_npts = t->site_npts.p;
  v.site_total = t->site_total.p;
  v.site_pcol = t->site_pcol.p;
  v.val = t->val.p;
  v.phase = t->phase.p;
  v.npts = pt;
  d.ae = std::move(t);
  return *d.ae;
}

// All-electron real-space wavefunctions of bands [b0, b0 + nb) of k-point kq on the grid of t:
// grid[b][N1][N2][N3] (realspace_state, density.c:245-310).
static void ae_grids(DevWF &d, AeTables &t, int kq, int b0, int nb, float2 *grid) {
  ensure_projections(d);
  DevKpt &q = d.kp[kq];
  const float2 *C = coeffs(d, kq);
  if (!q.gs_d.p) {
    q.gs_d.alloc(std::max<size_t>(3, q.gsorted.size()));
    q.gs_d.upload(q.gsorted.data(), q.gsorted.size());
  }
  const int *N = t.N;
  const long long n3d = (long long)N[0] * N[1] * N[2];
  launch_scatter_bands(C + (size_t)b0 * q.Wpad, q.Wpad, q.gs_d.p, q.W, N[0], N[1], N[2], grid, nb);
  for (int a = 2; a >= 0; a--) launch_fft_axis(grid, nb, N[0], N[1], N[2], a, t.r[a], t.tw[a].p);
  launch_bloch(grid, N[0], N[1], N[2], q.kfrac, std::pow(d.vol, -0.5), nb);
  const int Pt = d.proj.Ptot;
  launch_ae_add(t.view, d.P.p + ((size_t)kq * d.nband + b0) * Pt, Pt, kq, grid, n3d, nb);
}

// Bands per batch of real-space grids (about 1 GiB of grids).
static int ae_batch(const AeTables &t) {
  const long long n3d = (long long)t.N[0] * t.N[1] * t.N[2];
  return (int)std::max(1LL, (1LL << 30) / (n3d * (long long)sizeof(float2)));
}

// ============================================================= overlap matrices

static int flip_k(const DevWF &R, int k, int flip) {
  if (R.nspin == 2 && flip) return k < R.nwk ? k + R.nwk : k - R.nwk;
  return k;
}

static int choose_splits(int M, int N, int nz, int maxK) {
  int tiles = ceil_div(M, 64) * ceil_div(N, 64) * nz;
  int chunks = maxK / 16;
  int s = std::max(1, ceil_div(2 * sm_count(), tiles));
  s = std::min(s, std::max(1, chunks / 32));
  return std::min(s, 64);
}

// What an overlap contraction sums, per k-point (kR = k with the spins swapped under flip):
//   kPseudo:    <C_R|C_S>
//   kAugmented: aug_real  <C_R|C_S> + [augmentation columns A32 | B32]
//               aug_recip <C_R|C_S + CA_S> + <CA_R|C_S> + [A32 | B32] (the M and N_RS columns)
//   kCross:     aug_recip cross terms only, <CA_R|C_S> + <C_R|CA_S>
// into S[k][bS][bR]; each is one grouped launch with up to three K segments.
enum class Contraction { kPseudo, kAugmented, kCross };

static void overlap_gemm(PairState &ps, int flip, const float2 *B32, float2 *out, int prec,
                         Contraction what = Contraction::kAugmented) {
  HostPhase hp("overlap_gemm");
  DevWF &R = *ps.R, &S = *ps.S;
  ensure_coeffs(R);
  ensure_coeffs(S);
  PAWPY_REQUIRE(R.nk == S.nk, "basis and defect differ in k-points");
  int nk = S.nk;
  std::vector<GemmBatch> hb(nk);
  int maxK = 0;
  const bool recip = ps.recip && what != Contraction::kPseudo;
  const int NR = host_bands(R), NS = host_bands(S);
  const bool haveCA_R = recip && !ps.N_R.empty(), haveCA_S = recip && !ps.N_S.empty();
  for (int k = 0; k < nk; k++) {
    int kR = flip_k(R, k, flip);
    const DevKpt &qR = R.kp[kR], &qS = S.kp[k];
    PAWPY_REQUIRE(qR.W == qS.W && qR.gsorted == qS.gsorted,
                  "basis and defect plane-wave sets differ at a k-point (lattice, ENCUT or k mismatch)");
    struct Seg {
      const float2 *A, *B;
      long long lda, ldb;
      int K;
    };
    std::vector<Seg> segs;
    const float2 *CR = coeffs(R, kR), *CS = coeffs(S, k);
    // a noncollinear band's two spinor halves are consecutive rows: one row of twice the length
    const int f = spinor_factor(R);
    const long long w = (long long)f * qR.Wpad, kc = (long long)f * ps.Kcpad;
    const int K = f * qR.Wpad;
    if (what == Contraction::kCross) {
      if (haveCA_R) segs.push_back({ps.CA_R.p + qR.c_off, CS, w, w, K});
      if (haveCA_S) segs.push_back({CR, ps.CA_S.p + qS.c_off, w, w, K});
    } else {
      segs.push_back({CR, haveCA_S ? ps.D_S.p + qS.c_off : CS, w, w, K});
      if (haveCA_R) segs.push_back({ps.CA_R.p + qR.c_off, CS, w, w, K});
      if (B32 && what == Contraction::kAugmented)
        segs.push_back({ps.A32.p + (size_t)kR * R.nband * ps.Kcpad, B32 + (size_t)k * S.nband * ps.Kcpad, kc, kc,
                        (int)kc});
    }
    GemmBatch &g = hb[k];
    g.A1 = g.B1 = g.A2 = g.B2 = nullptr;
    g.lda1 = g.ldb1 = g.lda2 = g.ldb2 = 0;
    g.K1 = g.K2 = 0;
    if (segs.size() > 0) {
      g.A1 = segs[0].A, g.B1 = segs[0].B, g.lda1 = segs[0].lda, g.ldb1 = segs[0].ldb, g.K1 = segs[0].K;
    }
    if (segs.size() > 1) {
      g.A2 = segs[1].A, g.B2 = segs[1].B, g.lda2 = segs[1].lda, g.ldb2 = segs[1].ldb, g.K2 = segs[1].K;
    }
    if (segs.size() > 2) {
      g.A3 = segs[2].A, g.B3 = segs[2].B, g.lda3 = segs[2].lda, g.ldb3 = segs[2].ldb, g.K3 = segs[2].K;
    }
    g.out = out + (size_t)k * NS * NR;
    maxK = std::max(maxK, g.K1 + g.K2 + g.K3);
  }
  if (maxK == 0) {
    PAWPY_CUDA(cudaMemsetAsync(out, 0, sizeof(float2) * (size_t)nk * NS * NR, stream()));
    return;
  }
  DevBuf<GemmBatch> db(nk);
  db.upload(hb.data(), nk);
  double flops = 0;  // useful flops: 8 per complex multiply-add of every K segment
  for (const GemmBatch &g : hb) flops += 8.0 * NR * NS * (double)(g.K1 + g.K2 + g.K3);
  note_work(prec == PAWPY_GPU_BF16X3 ? "gemm_bf16x3" : prec == PAWPY_GPU_TF32 ? "gemm_tf32" : "gemm_f32", flops);
  if (prec == PAWPY_GPU_BF16X3 || prec == PAWPY_GPU_TF32) {
    // the basis's coefficient planes are split once and kept with it (operand A's first segment
    // is C_R except in the cross terms)
    launch_zgemm_tc(db.p, hb, NR, NS, prec == PAWPY_GPU_TF32, g_tc_splits, nullptr,
                    what == Contraction::kCross ? nullptr : &R.gemm_cache);
    return;
  }
  int splits = choose_splits(NR, NS, nk, maxK);
  DevBuf<float2> ws;
  if (splits > 1) ws.alloc((size_t)splits * nk * NS * NR);
  launch_zgemm_f32(db.p, nk, NR, NS, splits, ws.p);
}

static void ensure_pseudo(PairState &ps, int flip) {
  int f = flip ? 1 : 0;
  const int prec = g_precision.load();
  if (ps.pseudo_ready[f] && ps.pseudo_prec[f] == prec) return;
  DevWF &R = *ps.R, &S = *ps.S;
  ps.pseudo[f].alloc((size_t)S.nk * host_bands(S) * host_bands(R));
  overlap_gemm(ps, f, nullptr, ps.pseudo[f].p, prec, Contraction::kPseudo);
  ps.pseudo_ready[f] = true;
  ps.pseudo_prec[f] = prec;
}

// aug_recip cross terms <CA_R|C_S> + <C_R|CA_S> of every band pair, cached per flip.
static void ensure_cross(PairState &ps, int flip) {
  int f = flip ? 1 : 0;
  const int prec = g_precision.load();
  if (ps.cross_ready[f] && ps.cross_prec[f] == prec) return;
  DevWF &R = *ps.R, &S = *ps.S;
  ps.cross[f].alloc((size_t)S.nk * host_bands(S) * host_bands(R));
  overlap_gemm(ps, f, nullptr, ps.cross[f].p, prec, Contraction::kCross);
  ps.cross_ready[f] = true;
  ps.cross_prec[f] = prec;
}

// Column maps of the augmentation (see aug.cu) for the given site lists.
static void ensure_projections(DevWF &d) {
  PAWPY_REQUIRE(d.tables_ready, "setup_projections has not been called for this wavefunction");
  if (d.p_ready) return;
  project_bands(d, {&d.proj}, {d.P.p});
  d.p_ready = true;
}

static void ensure_aug(PairState &ps, const std::vector<int> lists[6], int flip) {
  ensure_projections(*ps.R);
  ensure_projections(*ps.S);
  AugKey key;
  for (int i = 0; i < 6; i++) key.lists[i] = lists[i];
  key.flip = flip ? 1 : 0;
  key.recip = ps.recip;
  if (ps.aug_ready && ps.aug_key == key) return;
  HostPhase hp("aug_setup");
  PAWPY_REQUIRE(ps.ready, "overlap_setup_real has not been called for this basis/defect pair");
  PAWPY_REQUIRE(lists[2] == ps.N_R && lists[3] == ps.N_S && lists[4] == ps.N_RS_R && lists[5] == ps.N_RS_S,
                "site lists differ from the ones given to overlap_setup_real");
  PAWPY_REQUIRE(lists[0].size() == lists[1].size(), "M_R and M_S differ in length");
  DevWF &R = *ps.R, &S = *ps.S;
  const int PtR = R.proj.Ptot, PtS = S.proj.Ptot;
  std::vector<int> a_src, b_ptr(1, 0), b_col, b_pair;
  std::vector<double2> b_val;
  auto add_b = [&](int pair) {
    b_ptr.push_back((int)b_col.size());
    b_pair.push_back(pair);
  };
  auto nsites_R = (int)R.labels.size(), nsites_S = (int)S.labels.size();
  // O_M
  for (size_t s = 0; s < lists[0].size(); s++) {
    int s1 = lists[0][s], s2 = lists[1][s];
    PAWPY_REQUIRE(s1 >= 0 && s1 < nsites_R && s2 >= 0 && s2 < nsites_S, "M site index out of range");
    const SpeciesTables &t = *R.species[R.labels[s1]];
    PAWPY_REQUIRE(S.species[S.labels[s2]]->total == t.total, "matched sites carry different projector sets");
    for (int i = 0; i < t.total; i++) {
      a_src.push_back(R.site_lmoff[s1] + i);
      for (int j = 0; j < t.total; j++) {
        double v = t.D[(size_t)i * t.total + j];
        if (v != 0.0) {
          b_col.push_back(S.site_lmoff[s2] + j);
          b_val.push_back(make_double2(v, 0.0));
        }
      }
      add_b(-1);
    }
  }
  // O_R: basis projectors on N_R sites against <smooth (phi-phit)_R | psi_S> (aug_recip has
  // these terms as <CA_R|C_S> and <C_R|CA_S> instead, compensation_terms_recip projector.c:1000-1016)
  for (size_t si = 0; si < (ps.recip ? 0 : ps.N_R.size()); si++) {
    int s = ps.N_R[si];
    const SiteDesc &h = ps.sm_NR.host[si];
    for (int i = 0; i < h.total; i++) {
      a_src.push_back(R.site_lmoff[s] + i);
      b_col.push_back(PtS + h.lm_off + i);
      b_val.push_back(make_double2(1.0, 0.0));
      add_b(-1);
    }
  }
  // O_S: <smooth (phi-phit)_S | psi_R> against defect projectors on N_S sites
  for (size_t si = 0; si < (ps.recip ? 0 : ps.N_S.size()); si++) {
    int s = ps.N_S[si];
    const SiteDesc &h = ps.sm_NS.host[si];
    for (int i = 0; i < h.total; i++) {
      a_src.push_back(PtR + h.lm_off + i);
      b_col.push_back(S.site_lmoff[s] + i);
      b_val.push_back(make_double2(1.0, 0.0));
      add_b(-1);
    }
  }
  // O_N: Q P_S exp(2 pi i k.d) per overlapping pair
  for (size_t p = 0; p < ps.N_RS_R.size(); p++) {
    int s1 = ps.N_RS_R[p], s2 = ps.N_RS_S[p];
    int T1 = R.species[R.labels[s1]]->total, T2 = S.species[S.labels[s2]]->total;
    PAWPY_REQUIRE(ps.Q[p].size() == (size_t)T1 * T2, "pair matrix size mismatch");
    for (int i = 0; i < T1; i++) {
      a_src.push_back(R.site_lmoff[s1] + i);
      for (int j = 0; j < T2; j++) {
        cd q = ps.Q[p][(size_t)i * T2 + j];
        b_col.push_back(S.site_lmoff[s2] + j);
        b_val.push_back(make_double2(q.real(), q.imag()));
      }
      add_b((int)p);
    }
  }
  ps.Kc = (int)a_src.size();
  ps.Kcpad = (ps.Kc + 15) / 16 * 16;
  int npairs = (int)ps.N_RS_R.size();
  std::vector<double2> ph((size_t)S.nk * std::max(1, npairs));
  for (int k = 0; k < S.nk; k++) {
    int kR = flip_k(R, k, flip);
    for (int p = 0; p < npairs; p++) {
      const double *dc = ps.dcoords.data() + 3 * p;
      const double *kv = R.kp[kR].kfrac;
      double a = 2 * M_PI * (kv[0] * dc[0] + kv[1] * dc[1] + kv[2] * dc[2]);
      ph[(size_t)k * npairs + p] = make_double2(std::cos(a), std::sin(a));
    }
  }
  // FP32 entries with the pair phase of their column folded in, per k-point (on the device)
  const size_t ne = std::max<size_t>(1, b_val.size());
  std::vector<int> e_pair(ne, -1);
  for (size_t c = 0; c + 1 < b_ptr.size(); c++)
    for (int e = b_ptr[c]; e < b_ptr[c + 1]; e++) e_pair[e] = b_pair[c];
  // the lists go up through pinned staging: the host does not wait for the projections queued
  // before them
  aug_stage().begin(16 * 8 + sizeof(int) * (a_src.size() + b_ptr.size() + b_col.size() + b_pair.size() + ne) +
                     sizeof(double2) * (b_val.size() + ph.size()));
  ps.a_src.alloc(std::max(1, ps.Kc));
  aug_stage().upload(ps.a_src, a_src);
  ps.b_ptr.alloc(b_ptr.size());
  aug_stage().upload(ps.b_ptr, b_ptr);
  ps.b_col.alloc(std::max<size_t>(1, b_col.size()));
  aug_stage().upload(ps.b_col, b_col);
  ps.b_val.alloc(std::max<size_t>(1, b_val.size()));
  aug_stage().upload(ps.b_val, b_val);
  ps.b_pair.alloc(std::max<size_t>(1, b_pair.size()));
  aug_stage().upload(ps.b_pair, b_pair);
  ps.pair_phase.alloc(ph.size());
  aug_stage().upload(ps.pair_phase, ph);
  {
    DevBuf<int> e_pair_d(ne);
    aug_stage().upload(e_pair_d, e_pair);
    aug_stage().end();
    ps.b_val32.alloc((size_t)S.nk * ne);
    launch_aug_val32(ps.b_val.p, e_pair_d.p, (int)b_val.size(), (int)ne, ps.pair_phase.p, std::max(1, npairs), S.nk,
                     ps.b_val32.p);
  }
  // basis-side columns for every k-slice of R
  ps.A64.alloc(std::max<size_t>(1, (size_t)R.nk * R.nband * ps.Kc));
  ps.A32.alloc(std::max<size_t>(1, (size_t)R.nk * R.nband * ps.Kcpad));
  launch_aug_a(R.P.p, PtR, ps.WP_R.p, ps.sm_NS.Ptot, R.nband, R.nk, ps.a_src.p, ps.Kc, ps.Kcpad, ps.A64.p,
               ps.A32.p);
  ps.aug_key = key;
  ps.aug_ready = true;
}

static void gather_lists(std::vector<int> lists[6], int num_M, int nNR, int nNS, int nNRS, const int *M_R,
                         const int *M_S, const int *N_R, const int *N_S, const int *N_RS_R, const int *N_RS_S) {
  const int *ptrs[6] = {M_R, M_S, N_R, N_S, N_RS_R, N_RS_S};
  int lens[6] = {num_M, num_M, nNR, nNS, nNRS, nNRS};
  for (int i = 0; i < 6; i++) {
    PAWPY_REQUIRE(lens[i] >= 0, "negative site-list length");
    PAWPY_REQUIRE(lens[i] == 0 || ptrs[i] != nullptr, "NULL site list with a nonzero length");
    lists[i].assign(ptrs[i], ptrs[i] + (ptrs[i] ? lens[i] : 0));
  }
}

// ============================================================= single-band helpers

static void onto_projector_one(kpoint_t *kpt, int band_num, real_proj_site_t *sites, int num_sites,
                               double *lattice, double *reclattice, int *fftg);

}  // namespace pawpy

using namespace pawpy;

extern "C" {

void pawpy_gpu_set_precision(int precision) {
  if (precision == PAWPY_GPU_FP32 || precision == PAWPY_GPU_BF16X3 || precision == PAWPY_GPU_TF32)
    g_precision = precision;
}
int pawpy_gpu_get_precision(void) { return g_precision; }
void pawpy_gpu_set_tc_splits(int splits) { g_tc_splits = splits < 0 ? 0 : splits; }
void pawpy_gpu_set_element_cache(int on) { set_projector_list_cache(on != 0); }
void pawpy_gpu_set_tc_tile(int bn) { set_tc_tile(bn); }
void pawpy_gpu_set_sphere_contraction(int mode) { g_sphere_tc = (mode >= 0 && mode <= 2) ? mode : 1; }

int pawpy_gpu_overlap_matrix(const pawpy_c64 *A, const pawpy_c64 *B, int M, int N, int nz, const int *K,
                             pawpy_c64 *out, int precision) {
  PAWPY_API_BEGIN
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  PAWPY_REQUIRE(A && B && K && out, "pawpy_gpu_overlap_matrix: NULL argument");
  PAWPY_REQUIRE(M > 0 && N > 0 && nz > 0, "pawpy_gpu_overlap_matrix: empty shape");
  PAWPY_REQUIRE(precision == PAWPY_GPU_FP32 || precision == PAWPY_GPU_BF16X3 || precision == PAWPY_GPU_TF32,
                "pawpy_gpu_overlap_matrix: unknown precision");
  // rows padded to a multiple of 16 elements with zeros (the GEMM's K granule)
  std::vector<size_t> offA(nz), offB(nz);
  std::vector<int> Kp(nz);
  size_t na = 0, nb = 0;
  int maxK = 0;
  for (int z = 0; z < nz; z++) {
    PAWPY_REQUIRE(K[z] >= 0, "pawpy_gpu_overlap_matrix: negative K");
    Kp[z] = std::max(16, (K[z] + 15) / 16 * 16);
    offA[z] = na;
    offB[z] = nb;
    na += (size_t)M * Kp[z];
    nb += (size_t)N * Kp[z];
    maxK = std::max(maxK, Kp[z]);
  }
  DevBuf<float2> dA(na), dB(nb), dO((size_t)nz * N * M);
  dA.zero();
  dB.zero();
  const float2 *hA = reinterpret_cast<const float2 *>(A), *hB = reinterpret_cast<const float2 *>(B);
  size_t ia = 0, ib = 0;
  std::vector<GemmBatch> hb(nz);
  for (int z = 0; z < nz; z++) {
    if (K[z] > 0) {
      PAWPY_CUDA(cudaMemcpy2DAsync(dA.p + offA[z], Kp[z] * sizeof(float2), hA + ia, K[z] * sizeof(float2),
                                   K[z] * sizeof(float2), M, cudaMemcpyHostToDevice, stream()));
      PAWPY_CUDA(cudaMemcpy2DAsync(dB.p + offB[z], Kp[z] * sizeof(float2), hB + ib, K[z] * sizeof(float2),
                                   K[z] * sizeof(float2), N, cudaMemcpyHostToDevice, stream()));
    }
    ia += (size_t)M * K[z];
    ib += (size_t)N * K[z];
    GemmBatch &g = hb[z];
    g.A1 = dA.p + offA[z];
    g.B1 = dB.p + offB[z];
    g.A2 = g.B2 = nullptr;
    g.lda1 = g.ldb1 = Kp[z];
    g.lda2 = g.ldb2 = 0;
    g.K1 = Kp[z];
    g.K2 = 0;
    g.out = dO.p + (size_t)z * N * M;
  }
  DevBuf<GemmBatch> db(nz);
  db.upload(hb.data(), nz);
  if (precision == PAWPY_GPU_FP32) {
    int splits = choose_splits(M, N, nz, maxK);
    DevBuf<float2> ws;
    if (splits > 1) ws.alloc((size_t)splits * nz * N * M);
    launch_zgemm_f32(db.p, nz, M, N, splits, ws.p);
  } else {
    launch_zgemm_tc(db.p, hb, M, N, precision == PAWPY_GPU_TF32, g_tc_splits, nullptr);
  }
  dO.download(reinterpret_cast<float2 *>(out), dO.n);
  sync();
  return 0;
  PAWPY_API_END(-1)
}
void pawpy_gpu_set_host_projections(int on) { g_host_proj = on != 0; }

int pawpy_gpu_prepare_basis(pswf_t *wf, int keep_real_space) {
  PAWPY_API_BEGIN
  HostPhase hp_api("prepare_basis");
  DevWF &d = mirror(wf);
  PAWPY_REQUIRE(d.tables_ready, "pawpy_gpu_prepare_basis: setup_projections has not been called");
  ensure_coeffs(d);
  for (auto &q : d.kp) ensure_planes(d, q);
  ensure_projections(d);
  int kept = 0;
  if (keep_real_space && !d.grid_ready) kept = build_grids(d) ? 1 : 0;
  join_uploads(d);
  sync();
  return d.grid_ready ? 1 : kept;
  PAWPY_API_END(-1)
}

void pawpy_gpu_release(pswf_t *wf) {
  PAWPY_API_BEGIN
  release_device(wf);
  PAWPY_API_END()
}

int pawpy_gpu_upload(pswf_t *wf) {
  PAWPY_API_BEGIN
  DevWF &d = mirror(wf);
  ensure_coeffs(d);
  join_uploads(d);
  sync();
  return 0;
  PAWPY_API_END(pawpy_gpu_last_error())
}

ppot_t *get_projector_list(int num_els, int *labels, int *ls, double *wave_grids, double *projectors,
                           double *aewaves, double *pswaves, double *rmaxs, double grid_encut) {
  PAWPY_API_BEGIN
  HostPhase hp_api("get_projector_list");
  return cached_projector_list(num_els, labels, ls, wave_grids, projectors, aewaves, pswaves, rmaxs, grid_encut);
  PAWPY_API_END(nullptr)
}

void setup_projections(pswf_t *wf, ppot_t *pps, int num_elems, int num_sites, int *fftg, int *labels,
                       double *coords) {
  PAWPY_API_BEGIN
  HostPhase hp_api("setup_projections");
  do_setup_projections(wf, pps, num_elems, num_sites, fftg, labels, coords);
  PAWPY_API_END()
}

void overlap_setup_real(pswf_t *wf_R, pswf_t *wf_S, int *labels_R, int *labels_S, double *coords_R,
                        double *coords_S, int *N_R, int *N_S, int *N_RS_R, int *N_RS_S, int num_N_R, int num_N_S,
                        int num_N_RS) {
  PAWPY_API_BEGIN
  HostPhase hp_api("overlap_setup_real");
  do_overlap_setup_real(wf_R, wf_S, labels_R, labels_S, coords_R, coords_S, N_R, N_S, N_RS_R, N_RS_S, num_N_R,
                        num_N_S, num_N_RS);
  PAWPY_API_END()
}

void pseudoprojection(pawpy_c128 *projections, pswf_t *wf_ref, pswf_t *wf_proj, int BAND_NUM, int flip_spin) {
  PAWPY_API_BEGIN
  PAWPY_REQUIRE(projections && wf_ref && wf_proj, "pseudoprojection: NULL argument");
  PAWPY_REQUIRE(BAND_NUM >= 0 && BAND_NUM < wf_proj->nband, "pseudoprojection: band index out of range");
  PairState &ps = pair_state(wf_ref, wf_proj);
  ensure_pseudo(ps, flip_spin);
  DevWF &R = *ps.R, &S = *ps.S;
  int f = flip_spin ? 1 : 0;
  DevBuf<double2> col((size_t)host_bands(R) * S.nk);
  launch_extract_band(ps.pseudo[f].p, S.nk, host_bands(S), host_bands(R), BAND_NUM, col.p);
  col.download(reinterpret_cast<double2 *>(projections), col.n);
  sync();
  PAWPY_API_END()
}

}  // extern "C"

// compensation_terms / compensation_terms_recip of one defect band: the PAW terms in FP64 from
// the augmentation columns, plus (aug_recip) the cross terms <CA_R|C_S> + <C_R|CA_S>.
static void do_compensation_terms(pawpy_c128 *overlap, int BAND_NUM, pswf_t *wf_S, pswf_t *wf_R, int num_M,
                                  int num_N_R, int num_N_S, int num_N_RS, int *M_R, int *M_S, int *N_R, int *N_S,
                                  int *N_RS_R, int *N_RS_S, int flip_spin, bool recip) {
  const char *name = recip ? "compensation_terms_recip" : "compensation_terms";
  PAWPY_REQUIRE(overlap && wf_S && wf_R, std::string(name) + ": NULL argument");
  PAWPY_REQUIRE(BAND_NUM >= 0 && BAND_NUM < wf_S->nband, std::string(name) + ": band index out of range");
  PairState &ps = pair_state(wf_R, wf_S);
  PAWPY_REQUIRE(!ps.ready || ps.recip == recip,
                recip ? "compensation_terms_recip needs overlap_setup_recip (overlap_setup_real was run)"
                      : "compensation_terms needs overlap_setup_real (overlap_setup_recip was run)");
  std::vector<int> lists[6];
  gather_lists(lists, num_M, num_N_R, num_N_S, num_N_RS, M_R, M_S, N_R, N_S, N_RS_R, N_RS_S);
  ensure_aug(ps, lists, flip_spin);
  DevWF &R = *ps.R, &S = *ps.S;
  int nk = S.nk, npairs = (int)ps.N_RS_R.size();
  // a noncollinear band's two spinor halves are consecutive device bands: their columns form
  // one row of f Kc values (the PAW terms summed over both components)
  const int f = spinor_factor(S), NR = host_bands(R), NS = host_bands(S), kc = f * ps.Kc;
  DevBuf<double2> B64((size_t)nk * std::max(1, kc));
  launch_aug_b(S.P.p, S.proj.Ptot, ps.WP_S.p, ps.sm_NR.Ptot, S.nband, f * BAND_NUM, f, nk, ps.b_ptr.p, ps.b_col.p,
               ps.b_val.p, ps.b_pair.p, ps.pair_phase.p, std::max(1, npairs), ps.Kc, ps.Kc, B64.p, nullptr);
  DevBuf<double2> acc((size_t)nk * NR);
  acc.zero();
  for (int k = 0; k < nk; k++) {
    int kR = flip_k(R, k, flip_spin);
    if (ps.Kc > 0)
      launch_zgemv_f64(ps.A64.p + (size_t)kR * R.nband * ps.Kc, kc, NR, kc, B64.p + (size_t)k * kc,
                       acc.p + (size_t)k * NR);
  }
  std::vector<double2> h(acc.n), hx;
  acc.download(h.data(), h.size());
  if (recip) {
    // cross terms of this band, col[bR][k]
    ensure_cross(ps, flip_spin);
    DevBuf<double2> col((size_t)NR * nk);
    launch_extract_band(ps.cross[flip_spin ? 1 : 0].p, nk, NS, NR, BAND_NUM, col.p);
    hx.resize(col.n);
    col.download(hx.data(), hx.size());
  }
  sync();
  for (int b = 0; b < NR; b++)
    for (int k = 0; k < nk; k++) {
      double2 v = h[(size_t)k * NR + b];
      overlap[(size_t)b * nk + k] += pawpy_c128(v.x, v.y);
      if (recip) {
        double2 x = hx[(size_t)b * nk + k];
        overlap[(size_t)b * nk + k] += pawpy_c128(x.x, x.y);
      }
    }
}

extern "C" {

void compensation_terms(pawpy_c128 *overlap, int BAND_NUM, pswf_t *wf_S, pswf_t *wf_R, int num_M, int num_N_R,
                        int num_N_S, int num_N_RS, int *M_R, int *M_S, int *N_R, int *N_S, int *N_RS_R,
                        int *N_RS_S, int *proj_labels, double *proj_coords, int *ref_labels, double *ref_coords,
                        int *fft_grid, int flip_spin) {
  PAWPY_API_BEGIN
  (void)proj_labels;
  (void)proj_coords;
  (void)ref_labels;
  (void)ref_coords;
  (void)fft_grid;
  do_compensation_terms(overlap, BAND_NUM, wf_S, wf_R, num_M, num_N_R, num_N_S, num_N_RS, M_R, M_S, N_R, N_S,
                        N_RS_R, N_RS_S, flip_spin, false);
  PAWPY_API_END()
}

void compensation_terms_recip(pawpy_c128 *overlap, int BAND_NUM, pswf_t *wf_S, pswf_t *wf_R, int num_M,
                              int num_N_R, int num_N_S, int num_N_RS, int *M_R, int *M_S, int *N_R, int *N_S,
                              int *N_RS_R, int *N_RS_S, int *proj_labels, double *proj_coords, int *ref_labels,
                              double *ref_coords, int *fft_grid, int flip_spin) {
  PAWPY_API_BEGIN
  HostPhase hp_api("compensation_terms_recip");
  (void)proj_labels;
  (void)proj_coords;
  (void)ref_labels;
  (void)ref_coords;
  (void)fft_grid;
  do_compensation_terms(overlap, BAND_NUM, wf_S, wf_R, num_M, num_N_R, num_N_S, num_N_RS, M_R, M_S, N_R, N_S,
                        N_RS_R, N_RS_S, flip_spin, true);
  PAWPY_API_END()
}

void overlap_setup_recip(pswf_t *wf_R, pswf_t *wf_S, int *labels_R, int *labels_S, double *coords_R,
                         double *coords_S, int *N_R, int *N_S, int *N_RS_R, int *N_RS_S, int num_N_R, int num_N_S,
                         int num_N_RS) {
  PAWPY_API_BEGIN
  HostPhase hp_api("overlap_setup_recip");
  do_overlap_setup_recip(wf_R, wf_S, labels_R, labels_S, coords_R, coords_S, N_R, N_S, N_RS_R, N_RS_S, num_N_R,
                         num_N_S, num_N_RS);
  PAWPY_API_END()
}

// The full overlap matrix <psi_R|psi_S> of every band pair on the device,
// Smat[k][bS][bR] = pseudo overlap + PAW terms (one contraction over the
// augmented columns).
static void full_overlap(PairState &ps, const std::vector<int> lists[6], int flip_spin, DevBuf<float2> &Smat) {
  ensure_aug(ps, lists, flip_spin);
  DevWF &R = *ps.R, &S = *ps.S;
  int nk = S.nk, npairs = (int)ps.N_RS_R.size();
  DevBuf<float2> B32((size_t)nk * S.nband * std::max(16, ps.Kcpad));
  (void)npairs;
  launch_aug_b32(S.P.p, S.proj.Ptot, ps.WP_S.p, ps.sm_NR.Ptot, S.nband, S.nband, nk, ps.b_ptr.p, ps.b_col.p,
                 ps.b_val32.p, (int)(ps.b_val32.n / std::max(1, nk)), ps.Kc, ps.Kcpad, B32.p);
  Smat.alloc((size_t)nk * host_bands(S) * host_bands(R));
  overlap_gemm(ps, flip_spin, ps.Kcpad > 0 ? B32.p : nullptr, Smat.p, g_precision.load());
}

int pawpy_gpu_project_all(pawpy_c128 *out, pswf_t *wf_R, pswf_t *wf_S, int num_M, int num_N_R, int num_N_S,
                          int num_N_RS, int *M_R, int *M_S, int *N_R, int *N_S, int *N_RS_R, int *N_RS_S,
                          int flip_spin) {
  PAWPY_API_BEGIN
  HostPhase hp_api("pawpy_gpu_project_all");
  PAWPY_REQUIRE(out && wf_R && wf_S, "pawpy_gpu_project_all: NULL argument");
  PairState &ps = pair_state(wf_R, wf_S);
  std::vector<int> lists[6];
  gather_lists(lists, num_M, num_N_R, num_N_S, num_N_RS, M_R, M_S, N_R, N_S, N_RS_R, N_RS_S);
  DevBuf<float2> Smat;
  full_overlap(ps, lists, flip_spin, Smat);
  DevWF &R = *ps.R, &S = *ps.S;
  const int nk = S.nk;
  if (pageable_access()) {
    // the device writes the caller's (pageable) array through the host page tables
    launch_to_host_layout(Smat.p, nk, host_bands(S), host_bands(R), reinterpret_cast<double2 *>(out));
  } else {
    DevBuf<double2> o64(Smat.n);
    launch_to_host_layout(Smat.p, nk, host_bands(S), host_bands(R), o64.p);
    o64.download(reinterpret_cast<double2 *>(out), o64.n);
  }
  sync();
  return 0;
  PAWPY_API_END(pawpy_gpu_last_error())
}

int pawpy_gpu_band_character(double *v, double *c, pswf_t *wf_R, pswf_t *wf_S, int num_M, int num_N_R,
                             int num_N_S, int num_N_RS, int *M_R, int *M_S, int *N_R, int *N_S, int *N_RS_R,
                             int *N_RS_S, const double *w_v, const double *w_c, int nch, int flip_spin) {
  PAWPY_API_BEGIN
  HostPhase hp_api("pawpy_gpu_band_character");
  PAWPY_REQUIRE(v && c && wf_R && wf_S && w_v && w_c, "pawpy_gpu_band_character: NULL argument");
  PairState &ps = pair_state(wf_R, wf_S);
  std::vector<int> lists[6];
  gather_lists(lists, num_M, num_N_R, num_N_S, num_N_RS, M_R, M_S, N_R, N_S, N_RS_R, N_RS_S);
  DevBuf<float2> Smat;
  full_overlap(ps, lists, flip_spin, Smat);
  DevWF &R = *ps.R, &S = *ps.S;
  const int nk = S.nk, nw = (int)((size_t)host_bands(R) * nk);
  DevBuf<double> wv(nw), wc(nw), dv((size_t)host_bands(S) * nch), dc((size_t)host_bands(S) * nch);
  wv.upload(w_v, nw);
  wc.upload(w_c, nw);
  launch_band_character(Smat.p, nk, host_bands(S), host_bands(R), wv.p, wc.p, S.nwk, nch, dv.p, dc.p);
  dv.download(v, dv.n);
  dc.download(c, dc.n);
  sync();
  return 0;
  PAWPY_API_END(pawpy_gpu_last_error())
}

}  // extern "C"

// out[n][m] = sum_k conj(A[m][k]) B[n][k] over K (a multiple of 16), in the overlap precision.
static void grid_overlaps(const float2 *A, int M, const float2 *B, int N, long long K, float2 *out) {
  PAWPY_REQUIRE(K % 16 == 0 && K < (1LL << 31), "grid contraction length");
  std::vector<GemmBatch> hb(1);
  GemmBatch &g = hb[0];
  g.A1 = A;
  g.B1 = B;
  g.lda1 = g.ldb1 = K;
  g.K1 = (int)K;
  g.A2 = g.B2 = nullptr;
  g.lda2 = g.ldb2 = 0;
  g.K2 = 0;
  g.out = out;
  DevBuf<GemmBatch> db(1);
  db.upload(hb.data(), 1);
  const int prec = g_precision.load();
  if (prec == PAWPY_GPU_BF16X3 || prec == PAWPY_GPU_TF32) {
    launch_zgemm_tc(db.p, hb, M, N, prec == PAWPY_GPU_TF32, g_tc_splits, nullptr);
    return;
  }
  int splits = choose_splits(M, N, 1, (int)K);
  DevBuf<float2> ws;
  if (splits > 1) ws.alloc((size_t)splits * M * N);
  launch_zgemm_f32(db.p, 1, M, N, splits, ws.p);
}

// Real-space grids of bands [b0, b0 + nb) at k-point kq, rows of ld >= n3d values (zero past n3d).
static void ae_grid_rows(DevWF &d, AeTables &t, int kq, int b0, int nb, float2 *rows, long long ld) {
  const long long n3d = (long long)t.N[0] * t.N[1] * t.N[2];
  if (ld == n3d) {
    ae_grids(d, t, kq, b0, nb, rows);
    return;
  }
  DevBuf<float2> tmp((size_t)nb * n3d);
  ae_grids(d, t, kq, b0, nb, tmp.p);
  PAWPY_CUDA(cudaMemsetAsync(rows, 0, sizeof(float2) * (size_t)nb * ld, stream()));
  PAWPY_CUDA(cudaMemcpy2DAsync(rows, sizeof(float2) * ld, tmp.p, sizeof(float2) * n3d, sizeof(float2) * n3d, nb,
                               cudaMemcpyDeviceToDevice, stream()));
}

// <psi_R,bR,k|psi_S,bS,k> of the all-electron real-space wavefunctions on grid fftg for the
// defect bands [s0, s0 + ns): out[(bS - s0)][bR * nk + k] (project_realspace_state,
// density.c:206-243: the grid sum times V / N^3).
static void realspace_overlaps(pswf_t *wf_S, pswf_t *wf_R, const int *fftg, const int *labels, const double *coords,
                               const int *labels_R, const double *coords_R, int s0, int ns, pawpy_c128 *out) {
  DevWF &S = mirror(wf_S);
  DevWF &R = mirror(wf_R);
  if (S.ncl || R.ncl)
    throw Error(ERR_UNSUPPORTED, "real-space projections of noncollinear wavefunctions are not part of this library");
  PAWPY_REQUIRE(S.nk == R.nk, "basis and defect differ in k-points");
  PAWPY_REQUIRE(s0 >= 0 && ns >= 1 && s0 + ns <= S.nband, "band index out of range");
  AeTables &tS = ae_tables(S, fftg, labels, coords);
  AeTables &tR = ae_tables(R, fftg, labels_R, coords_R);
  const long long n3d = (long long)fftg[0] * fftg[1] * fftg[2], ld = (n3d + 15) / 16 * 16;
  const int nk = S.nk, nbR = R.nband;
  const double scale = S.vol / (double)n3d;
  DevBuf<float2> gS((size_t)ns * ld), gR((size_t)nbR * ld), o((size_t)ns * nbR);
  std::vector<float2> h((size_t)ns * nbR);
  for (int k = 0; k < nk; k++) {
    ae_grid_rows(S, tS, k, s0, ns, gS.p, ld);
    const int bb = ae_batch(tR);
    for (int b0 = 0; b0 < nbR; b0 += bb)
      ae_grid_rows(R, tR, k, b0, std::min(bb, nbR - b0), gR.p + (size_t)b0 * ld, ld);
    grid_overlaps(gR.p, nbR, gS.p, ns, ld, o.p);
    o.download(h.data(), h.size());
    sync();
    for (int b = 0; b < ns; b++)
      for (int r = 0; r < nbR; r++) {
        const float2 v = h[(size_t)b * nbR + r];
        out[(size_t)b * nbR * nk + (size_t)r * nk + k] = pawpy_c128(v.x * scale, v.y * scale);
      }
  }
}

extern "C" {

void realspace_state(pawpy_c128 *x, int BAND_NUM, int KPOINT_NUM, pswf_t *wf, int *fftg, int *labels,
                     double *coords) {
  PAWPY_API_BEGIN
  HostPhase hp_api("realspace_state");
  PAWPY_REQUIRE(x && wf && fftg && labels && coords, "realspace_state: NULL argument");
  DevWF &d = mirror(wf);
  if (d.ncl) throw Error(ERR_UNSUPPORTED, "realspace_state: a noncollinear wavefunction (use the ncl_ functions)");
  PAWPY_REQUIRE(BAND_NUM >= 0 && BAND_NUM < d.nband && KPOINT_NUM >= 0 && KPOINT_NUM < d.nk,
                "realspace_state: band or k-point index out of range");
  AeTables &t = ae_tables(d, fftg, labels, coords);
  const long long n3d = (long long)fftg[0] * fftg[1] * fftg[2];
  DevBuf<float2> g(n3d);
  ae_grids(d, t, KPOINT_NUM, BAND_NUM, 1, g.p);
  DevBuf<double2> o(n3d);
  launch_scale_to_c128(g.p, n3d, 1.0, o.p);
  o.download(reinterpret_cast<double2 *>(x), n3d);
  sync();
  PAWPY_API_END()
}

void remove_phase(pawpy_c128 *x, int KPOINT_NUM, pswf_t *wf, int *fftg) {
  PAWPY_API_BEGIN
  PAWPY_REQUIRE(x && wf && fftg, "remove_phase: NULL argument");
  DevWF &d = mirror(wf);
  PAWPY_REQUIRE(KPOINT_NUM >= 0 && KPOINT_NUM < d.nk, "remove_phase: k-point index out of range");
  const long long n3d = (long long)fftg[0] * fftg[1] * fftg[2];
  DevBuf<double2> g(n3d);
  g.upload(reinterpret_cast<const double2 *>(x), n3d);
  launch_remove_phase(g.p, fftg[0], fftg[1], fftg[2], d.kp[KPOINT_NUM].kfrac);
  g.download(reinterpret_cast<double2 *>(x), n3d);
  sync();
  PAWPY_API_END()
}

void ae_state_density(double *P, int BAND_NUM, int KPOINT_NUM, pswf_t *wf, int *fftg, int *labels,
                      double *coords) {
  PAWPY_API_BEGIN
  HostPhase hp_api("ae_state_density");
  PAWPY_REQUIRE(P && wf && fftg && labels && coords, "ae_state_density: NULL argument");
  DevWF &d = mirror(wf);
  if (d.ncl) throw Error(ERR_UNSUPPORTED, "ae_state_density: a noncollinear wavefunction (use the ncl_ functions)");
  PAWPY_REQUIRE(BAND_NUM >= 0 && BAND_NUM < d.nband && KPOINT_NUM >= 0 && KPOINT_NUM < d.nk,
                "ae_state_density: band or k-point index out of range");
  AeTables &t = ae_tables(d, fftg, labels, coords);
  const long long n3d = (long long)fftg[0] * fftg[1] * fftg[2];
  DevBuf<float2> g(n3d);
  ae_grids(d, t, KPOINT_NUM, BAND_NUM, 1, g.p);
  DevBuf<double> rho(n3d), w(1);
  const double one = 1.0;
  w.upload(&one, 1);
  rho.upload(P, n3d);
  launch_density(g.p, w.p, 1, n3d, rho.p);
  rho.download(P, n3d);
  sync();
  PAWPY_API_END()
}

void ae_chg_density(double *P, pswf_t *wf, int *fftg, int *labels, double *coords) {
  PAWPY_API_BEGIN
  HostPhase hp_api("ae_chg_density");
  PAWPY_REQUIRE(P && wf && fftg && labels && coords, "ae_chg_density: NULL argument");
  DevWF &d = mirror(wf);
  if (d.ncl) throw Error(ERR_UNSUPPORTED, "ae_chg_density: a noncollinear wavefunction (use ncl_ae_chg_density)");
  AeTables &t = ae_tables(d, fftg, labels, coords);
  const long long n3d = (long long)fftg[0] * fftg[1] * fftg[2];
  const int bb = ae_batch(t);
  DevBuf<float2> g((size_t)std::min(bb, d.nband) * n3d);
  DevBuf<double> rho(n3d), w((size_t)d.nband);
  rho.upload(P, n3d);
  // occupied bands of every k-point, weight x occupation x 2 / nspin (density.c:158-178)
  const double spin_mult = 2.0 / d.nspin;
  for (int k = 0; k < d.nk; k++) {
    std::vector<int> occ;
    std::vector<double> wk;
    for (int b = 0; b < d.nband; b++) {
      const band_t *bd = wf->kpts[k]->bands[b];
      if (bd->occ > 0) {
        occ.push_back(b);
        wk.push_back(wf->kpts[k]->weight * bd->occ * spin_mult);
      }
    }
    // runs of consecutive occupied bands in batches
    size_t i = 0;
    while (i < occ.size()) {
      size_t j = i + 1;
      while (j < occ.size() && occ[j] == occ[j - 1] + 1 && (int)(j - i) < bb) j++;
      const int nb = (int)(j - i);
      ae_grids(d, t, k, occ[i], nb, g.p);
      w.upload(wk.data() + i, nb);
      launch_density(g.p, w.p, nb, n3d, rho.p);
      i = j;
    }
  }
  rho.download(P, n3d);
  sync();
  PAWPY_API_END()
}

// Noncollinear: the spinor halves of band b are device bands 2b and 2b + 1, each transformed and
// completed with its own projections (up_projections, down_projections) as a collinear band.
void ncl_realspace_state(pawpy_c128 *x, int BAND_NUM, int KPOINT_NUM, pswf_t *wf, int *fftg, int *labels,
                         double *coords) {
  PAWPY_API_BEGIN
  HostPhase hp_api("ncl_realspace_state");
  PAWPY_REQUIRE(x && wf && fftg && labels && coords, "ncl_realspace_state: NULL argument");
  DevWF &d = mirror(wf);
  PAWPY_REQUIRE(d.ncl, "ncl_realspace_state: a collinear wavefunction (use realspace_state)");
  PAWPY_REQUIRE(BAND_NUM >= 0 && 2 * BAND_NUM < d.nband && KPOINT_NUM >= 0 && KPOINT_NUM < d.nk,
                "ncl_realspace_state: band or k-point index out of range");
  AeTables &t = ae_tables(d, fftg, labels, coords);
  const long long n3d = (long long)fftg[0] * fftg[1] * fftg[2];
  DevBuf<float2> g(2 * n3d);
  ae_grids(d, t, KPOINT_NUM, 2 * BAND_NUM, 2, g.p);
  DevBuf<double2> o(2 * n3d);
  launch_scale_to_c128(g.p, 2 * n3d, 1.0, o.p);
  o.download(reinterpret_cast<double2 *>(x), 2 * n3d);
  sync();
  PAWPY_API_END()
}

// sum over occupied bands of (|psi_up|^2 + |psi_down|^2) weight occupation (density.c:181-204)
void ncl_ae_chg_density(double *P, pswf_t *wf, int *fftg, int *labels, double *coords) {
  PAWPY_API_BEGIN
  HostPhase hp_api("ncl_ae_chg_density");
  PAWPY_REQUIRE(P && wf && fftg && labels && coords, "ncl_ae_chg_density: NULL argument");
  DevWF &d = mirror(wf);
  PAWPY_REQUIRE(d.ncl, "ncl_ae_chg_density: a collinear wavefunction (use ae_chg_density)");
  AeTables &t = ae_tables(d, fftg, labels, coords);
  const long long n3d = (long long)fftg[0] * fftg[1] * fftg[2];
  const int bb = std::max(2, ae_batch(t) / 2 * 2);
  DevBuf<float2> g((size_t)std::min(bb, d.nband) * n3d);
  DevBuf<double> rho(n3d), w((size_t)d.nband);
  rho.upload(P, n3d);
  for (int k = 0; k < d.nk; k++) {
    // both halves of every occupied band, weight x occupation (no spin factor)
    std::vector<int> occ;
    std::vector<double> wk;
    for (int b = 0; b < d.nband / 2; b++) {
      const band_t *bd = wf->kpts[k]->bands[b];
      if (bd->occ > 0)
        for (int h = 0; h < 2; h++) {
          occ.push_back(2 * b + h);
          wk.push_back(wf->kpts[k]->weight * bd->occ);
        }
    }
    size_t i = 0;
    while (i < occ.size()) {
      size_t j = i + 1;
      while (j < occ.size() && occ[j] == occ[j - 1] + 1 && (int)(j - i) < bb) j++;
      const int nb = (int)(j - i);
      ae_grids(d, t, k, occ[i], nb, g.p);
      w.upload(wk.data() + i, nb);
      launch_density(g.p, w.p, nb, n3d, rho.p);
      i = j;
    }
  }
  rho.download(P, n3d);
  sync();
  PAWPY_API_END()
}

void project_realspace_state(pawpy_c128 *projs, int BAND_NUM, pswf_t *wf, pswf_t *wf_R, int *fftg, int *labels,
                             double *coords, int *labels_R, double *coords_R) {
  PAWPY_API_BEGIN
  HostPhase hp_api("project_realspace_state");
  PAWPY_REQUIRE(projs && wf && wf_R && fftg && labels && coords && labels_R && coords_R,
                "project_realspace_state: NULL argument");
  realspace_overlaps(wf, wf_R, fftg, labels, coords, labels_R, coords_R, BAND_NUM, 1, projs);
  PAWPY_API_END()
}

int pawpy_gpu_project_realspace_all(pawpy_c128 *out, pswf_t *wf, pswf_t *wf_R, int *fftg, int *labels,
                                    double *coords, int *labels_R, double *coords_R) {
  PAWPY_API_BEGIN
  HostPhase hp_api("pawpy_gpu_project_realspace_all");
  PAWPY_REQUIRE(out && wf && wf_R && fftg && labels && coords && labels_R && coords_R,
                "pawpy_gpu_project_realspace_all: NULL argument");
  DevWF &S = mirror(wf);
  realspace_overlaps(wf, wf_R, fftg, labels, coords, labels_R, coords_R, 0, S.nband, out);
  return 0;
  PAWPY_API_END(pawpy_gpu_last_error())
}

void fft3d(pawpy_c128 *x, int *G_bounds, double *lattice, double *kpt, int *Gs, pawpy_c64 *Cs, int num_waves,
           int *fftg) {
  PAWPY_API_BEGIN
  (void)G_bounds;
  (void)kpt;
  PAWPY_REQUIRE(x && lattice && Gs && Cs && fftg && num_waves >= 0, "fft3d: NULL argument");
  int N[3] = {fftg[0], fftg[1], fftg[2]};
  Radices r[3];
  DevBuf<float2> tw[3];
  for (int a = 0; a < 3; a++) {
    r[a] = make_radices(N[a]);
    PAWPY_REQUIRE(r[a].ns >= 0, "FFT grid dimensions must factor into primes <= 13");
    twiddles(N[a], tw[a]);
  }
  long long grid = (long long)N[0] * N[1] * N[2];
  DevBuf<int> g(3 * (size_t)std::max(1, num_waves));
  g.upload(Gs, 3 * (size_t)num_waves);
  DevBuf<float2> c(std::max(1, num_waves));
  c.upload(reinterpret_cast<const float2 *>(Cs), num_waves);
  DevBuf<float2> u(grid);
  launch_scatter_grid(g.p, c.p, num_waves, N[0], N[1], N[2], u.p);
  for (int a = 2; a >= 0; a--) launch_fft_axis(u.p, 1, N[0], N[1], N[2], a, r[a], tw[a].p);
  DevBuf<double2> o(grid);
  launch_scale_to_c128(u.p, grid, std::pow(det3(lattice), -0.5), o.p);
  o.download(reinterpret_cast<double2 *>(x), grid);
  sync();
  PAWPY_API_END()
}

void onto_projector(kpoint_t *kpt, int band_num, real_proj_site_t *sites, int num_sites, int *G_bounds,
                    double *lattice, double *reclattice, int num_cart_gridpts, int *fftg) {
  PAWPY_API_BEGIN
  (void)G_bounds;
  (void)num_cart_gridpts;
  PAWPY_REQUIRE(kpt && sites && lattice && reclattice && fftg, "onto_projector: NULL argument");
  PAWPY_REQUIRE(band_num >= 0 && band_num < kpt->num_bands, "onto_projector: band index out of range");
  onto_projector_one(kpt, band_num, sites, num_sites, lattice, reclattice, fftg);
  PAWPY_API_END()
}

}  // extern "C"

namespace pawpy {

// FP64 gather of one band from host real_proj_site_t tables (projector.c:223-274).
__global__ void k_gather_one(const float2 *__restrict__ u, const int *__restrict__ idx,
                             const double *__restrict__ paths, const double2 *__restrict__ vals, int npts, int total,
                             double kx, double ky, double kz, double dv, double2 *__restrict__ out) {
  int p = blockIdx.x;  // channel
  double re = 0, im = 0;
  for (int i = threadIdx.x; i < npts; i += blockDim.x) {
    float2 x = u[idx[i]];
    double kr = kx * paths[3 * i] + ky * paths[3 * i + 1] + kz * paths[3 * i + 2];
    double s, c;
    sincos(kr, &s, &c);
    double xr = (x.x * c - x.y * s) * dv, xi = (x.x * s + x.y * c) * dv;
    double2 v = vals[(long long)p * npts + i];
    re += v.x * xr + v.y * xi;
    im += v.x * xi - v.y * xr;
  }
  __shared__ double sr[256], si[256];
  sr[threadIdx.x] = re;
  si[threadIdx.x] = im;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      sr[threadIdx.x] += sr[threadIdx.x + o];
      si[threadIdx.x] += si[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) out[p] = make_double2(sr[0], si[0]);
}

static void onto_projector_one(kpoint_t *kpt, int band_num, real_proj_site_t *sites, int num_sites,
                               double *lattice, double *reclattice, int *fftg) {
  int N[3] = {fftg[0], fftg[1], fftg[2]};
  Radices r[3];
  DevBuf<float2> tw[3];
  for (int a = 0; a < 3; a++) {
    r[a] = make_radices(N[a]);
    PAWPY_REQUIRE(r[a].ns >= 0, "FFT grid dimensions must factor into primes <= 13");
    twiddles(N[a], tw[a]);
  }
  long long grid = (long long)N[0] * N[1] * N[2];
  int nw = kpt->num_waves;
  DevBuf<int> g(3 * (size_t)std::max(1, nw));
  g.upload(kpt->Gs, 3 * (size_t)nw);
  DevBuf<float2> c(std::max(1, nw));
  c.upload(reinterpret_cast<const float2 *>(kpt->bands[band_num]->Cs), nw);
  DevBuf<float2> u(grid);
  launch_scatter_grid(g.p, c.p, nw, N[0], N[1], N[2], u.p);
  for (int a = 2; a >= 0; a--) launch_fft_axis(u.p, 1, N[0], N[1], N[2], a, r[a], tw[a].p);
  double vol = det3(lattice);
  float s = (float)std::pow(vol, -0.5);
  // scale in place through the double conversion kernel's float path: fold into dv instead
  double dv = vol / N[0] / N[1] / N[2] * s;
  double kc[3];
  for (int a = 0; a < 3; a++)
    kc[a] = kpt->k[0] * reclattice[a] + kpt->k[1] * reclattice[3 + a] + kpt->k[2] * reclattice[6 + a];
  band_t *band = kpt->bands[band_num];
  projection_t *pl = static_cast<projection_t *>(std::calloc(num_sites, sizeof(projection_t)));
  if (!pl) throw std::bad_alloc();
  for (int si = 0; si < num_sites; si++) {
    real_proj_site_t &st = sites[si];
    int T = st.total_projs, n = st.num_indices;
    projection_t &p = pl[si];
    p.num_projs = st.num_projs;
    p.total_projs = T;
    p.ns = static_cast<int *>(std::malloc(sizeof(int) * T));
    p.ls = static_cast<int *>(std::malloc(sizeof(int) * T));
    p.ms = static_cast<int *>(std::malloc(sizeof(int) * T));
    p.overlaps = static_cast<pawpy_c128 *>(std::calloc(T, sizeof(pawpy_c128)));
    for (int q = 0; q < T; q++) {
      p.ns[q] = st.projs[q].func_num;
      p.ls[q] = st.projs[q].l;
      p.ms[q] = st.projs[q].m;
    }
    if (n == 0 || T == 0) continue;
    DevBuf<int> idx(n);
    idx.upload(st.indices, n);
    DevBuf<double> pth(3 * (size_t)n);
    pth.upload(st.paths, 3 * (size_t)n);
    DevBuf<double2> vals((size_t)T * n);
    for (int q = 0; q < T; q++) vals.upload(reinterpret_cast<const double2 *>(st.projs[q].values), n, (size_t)q * n);
    DevBuf<double2> o(T);
    PAWPY_LAUNCH("gather_one", k_gather_one<<<T, 256, 0, stream()>>>(u.p, idx.p, pth.p, vals.p, n, T, kc[0], kc[1],
                                                                      kc[2], dv, o.p));
    o.download(reinterpret_cast<double2 *>(p.overlaps), T);
    sync();
  }
  band->projections = pl;
}

}  // namespace pawpy
