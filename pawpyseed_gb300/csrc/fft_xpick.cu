// Dispatch and tile tuning of pass B of the band FFT (k_xpick_reg).
#include "fft_fast.cuh"

namespace pawpy {

namespace {

using PickFn = void (*)(const float2 *, PlaneGeom, const GatherSeg *, const int *, int, float2 *, long long);

template <int N1, int N3>
PickFn pick_fn(int jj) {
  switch (jj) {
    case 1: return k_xpick_reg<N1, N3, 1>;
    case 2: return k_xpick_reg<N1, N3, 2>;
    default: return k_xpick_reg<N1, N3, 4>;
  }
}

PickFn find_pick(int n1, int n3, int jj) {
#define X(a, b) \
  if (n1 == a && n3 == b) return pick_fn<a, b>(jj);
  PAWPY_FFT_PAIRS(X)
#undef X
  return nullptr;
}

}  // namespace

bool fft_planes_fast_supported(int n2, int n3);

bool fft_fast_supported(const PlaneGeom &g) {
  return fft_planes_fast_supported(g.N2, g.N3) && find_pick(g.N1, g.N3, 1) && g.n2 > 0 && g.n3 > 0;
}

void launch_fft_x_pick_fast(const float2 *H, const PlaneGeom &g, const GatherSeg *segs, const int *plane_start,
                            int kq, float2 *X, long long xstride, int nb) {
  using namespace fftfast;
  if (nb <= 0) return;
  auto run = [&](int jj) {
    PickFn fn = find_pick(g.N1, g.N3, jj);
    PAWPY_REQUIRE(fn, "no register FFT for this grid");
    size_t smem = tile_bytes(jj, g.N1, g.N3);
    allow_smem((const void *)fn, smem);
    dim3 grid(ceil_div(g.N2, jj), nb);
    PAWPY_LAUNCH("fft_x_pick", fn<<<grid, FT, smem, stream()>>>(H, g, segs, plane_start, kq, X, xstride));
  };
  std::vector<int> cands;
  for (int jj : {1, 2, 4})
    if (tile_bytes(jj, g.N1, g.N3) <= kSmemCap) cands.push_back(jj);
  int jj = tune(std::make_tuple(1, g.N1, g.N2, g.N3), cands, run);
  run(jj);
}

}  // namespace pawpy
