// Dispatch and tuning of pass B of the band FFT (k_xpick_pipe).
#include "fft_fast.cuh"

namespace pawpy {

namespace {

using PickFn = void (*)(const float2 *, int, PlaneGeom, const int *, const uint2 *, const float2 *, int, float2 *,
                       long long, long long);

using DirectFn = void (*)(const float2 *, int, PlaneGeom, const int *, const uint2 *, const float2 *, float2 *,
                         long long, long long);

PickFn find_pick(int n1, int n3) {
#define X(a, b) \
  if (n1 == a && n3 == b) return k_xpick_pipe<a, b>;
  PAWPY_FFT_PAIRS(X)
#undef X
  return nullptr;
}

// the direct kernel; stile: the transformed tile is held split (Gamma point, split rows)
DirectFn find_direct(int n1, int n3, bool stile, int *bpc) {
#define X(a, b)                                                         \
  if (n1 == a && n3 == b) {                                             \
    *bpc = direct_bands(a, b);                                          \
    if (stile) return k_xpick_direct<a, b, direct_lanes(a), true>;      \
    return k_xpick_direct<a, b, direct_lanes(a), false>;                \
  }
  PAWPY_FFT_PAIRS(X)
#undef X
  return nullptr;
}

}  // namespace

using GridFn = void (*)(const float2 *, int, PlaneGeom, float2 *, int);

GridFn find_xgrid(int n1, int n3, int *bpc) {
#define X(a, b)                                 \
  if (n1 == a && n3 == b) {                     \
    *bpc = direct_bands(a, b);                  \
    return k_xgrid<a, b, direct_lanes(a)>;      \
  }
  PAWPY_FFT_PAIRS(X)
#undef X
  return nullptr;
}

bool fft_planes_fast_supported(int n2, int n3);

bool fft_fast_supported(const PlaneGeom &g) {
  return fft_planes_fast_supported(g.N2, g.N3) && find_pick(g.N1, g.N3) && g.n2 > 0 && g.n3 > 0 &&
         fftfast::planes_smem(g) <= fftfast::kSmemCap && fftfast::xpick_smem(g) <= fftfast::kSmemCap;
}

void launch_fft_x_pick_fast(const float2 *H, const PlaneGeom &g, const PickList &pl, int kq, float2 *X,
                            long long xstride, int nb, long long lo_words, bool gamma) {
  using namespace fftfast;
  if (nb <= 0) return;
  PickFn fn = find_pick(g.N1, g.N3);
  PAWPY_REQUIRE(fn, "no register FFT for this grid");
  // stage the pick lists when they fit; planes with more points read them from global memory
  const int cap = xpick_smem(g, pl.max_plane_pts) <= kSmemCap ? pl.max_plane_pts : 0;
  const size_t smem = xpick_smem(g, cap);
  allow_smem((const void *)fn, smem);
  const int waves = resident_ctas((const void *)fn, smem);
  // at Gamma every Bloch phase is 1: no phase list
  const float2 *ph = gamma ? nullptr : pl.phase + (long long)kq * pl.npts;
  int bpc = 1;
  const bool stile = lo_words && gamma;
  DirectFn dfn = find_direct(g.N1, g.N3, stile, &bpc);
  const size_t dsmem = xpick_direct_smem(g, bpc);
  allow_smem((const void *)dfn, dsmem);
  // candidates: 1, 2, 4 band groups per plane of the pipelined kernel; 0 the direct kernel. The
  // tensor-core form (Gamma point, split rows) runs only where PAWPY_GPU_XPICK_TC=1 asks for it:
  // slower than the register transform at the measured shapes, and a persistent kernel holding
  // every SM's TMEM and shared memory, which stalls concurrent requests' launches.
  const char *tc_env = getenv("PAWPY_GPU_XPICK_TC");
  const bool tc = stile && xpick_tc_supported(g) && tc_env && tc_env[0] == '1';
  auto run = [&](int mult) {
    if (mult < 0) {
      launch_xpick_tc(H, g, pl, X, nb, lo_words);
      return;
    }
    if (mult == 0) {
      dim3 grid(ceil_div(nb, bpc), g.N2);
      PAWPY_LAUNCH("fft_x_pick", dfn<<<grid, FT, dsmem, stream()>>>(H, nb, g, pl.plane_first, pl.ent, ph, X, xstride,
                                                                    lo_words));
      return;
    }
    const int G = std::max(1, std::min(nb, ceil_div((long long)waves * mult, g.N2)));
    dim3 grid(g.N2, G);
    PAWPY_LAUNCH("fft_x_pick", fn<<<grid, FT, smem, stream()>>>(H, nb, g, pl.plane_first, pl.ent, ph, cap, X, xstride,
                                                                lo_words));
  };
  // tuned per form and per density of the pick (picked points per grid point, up to 3): a
  // pass dominated by its transform and one dominated by its pick tune apart
  const int density = (int)std::min<long long>(3, pl.npts / std::max(1, g.N1 * g.N2 * g.N3));
  if (tc) {
    run(-1);
    note_work("fft_x_pick", 8.0 * ((double)g.n1 * g.N2 * g.N3 + (double)pl.npts) * nb);
    return;
  }
  std::vector<int> cands = {0, 1, 2, 4};
  int mult = tune(std::make_tuple((lo_words ? 3 : 1) + (gamma ? 4 : 0) + 8 * density, g.N1, g.N2, g.N3), cands, run);
  run(mult);
  // algorithmic bytes: the occupied planes of H read, 8 bytes per picked value written
  note_work("fft_x_pick", 8.0 * ((double)g.n1 * g.N2 * g.N3 + (double)pl.npts) * nb);
}

void launch_fft_x_grid(const float2 *H, const PlaneGeom &g, float2 *grid, int b0, int nb) {
  if (nb <= 0) return;
  int bpc = 1;
  GridFn fn = find_xgrid(g.N1, g.N3, &bpc);
  PAWPY_REQUIRE(fn, "no register FFT for this grid");
  dim3 grd(ceil_div(nb, bpc), g.N2);
  PAWPY_LAUNCH("fft_x_grid", fn<<<grd, FT, 0, stream()>>>(H, nb, g, grid, b0));
  // algorithmic bytes: the occupied planes of H read, the whole grid written
  note_work("fft_x_grid", 8.0 * ((double)g.n1 + g.N1) * g.N2 * g.N3 * nb);
}

// One CTA per segment: its points go to positions base[si] + p of the flat list, with the
// point's offset in the transformed plane's shared tile (row i, column k: i LD + k, LD the
// padded row length) in place of its cell i N3 + k, and the offset of its value in a band's
// picked row.
__global__ void k_flatten_pick(const GatherSeg *__restrict__ segs, const int *__restrict__ base, int nkp,
                               long long Q, int N3, int LD, long long kb_words, uint2 *__restrict__ ent,
                               float2 *__restrict__ phase) {
  const GatherSeg sg = segs[blockIdx.x];
  const int q0 = base[blockIdx.x];
  for (int p = threadIdx.x; p < sg.npts; p += blockDim.x) {
    const int c = sg.idx[p], i = c / N3;
    const long long pos = sg.x_off + p;
    const long long off = kb_words ? (pos >> 4) * kb_words + (pos & 15) : pos;
    ent[q0 + p] = make_uint2((unsigned)(i * LD + (c - i * N3)), (unsigned)off);
    for (int k = 0; k < nkp; k++) phase[k * Q + q0 + p] = sg.phase[k * sg.phase_stride + p];
  }
}

void launch_flatten_pick(const GatherSeg *segs, const int *base, int nsegs, int nkp, int N3, long long kb_words,
                         PickList &pl) {
  if (nsegs <= 0) return;
  PAWPY_LAUNCH("pick_list", k_flatten_pick<<<nsegs, 128, 0, stream()>>>(segs, base, nkp, pl.npts, N3, padded(N3),
                                                                         kb_words, pl.ent, pl.phase));
}

}  // namespace pawpy
