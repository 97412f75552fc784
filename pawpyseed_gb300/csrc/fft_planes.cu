// Dispatch and tile tuning of pass A of the band FFT (k_planes_reg).
#include "fft_fast.cuh"

namespace pawpy {

namespace {

using PlanesFn = void (*)(const float2 *, int, const int *, const int *, PlaneGeom, float2 *);

template <int N2, int N3>
PlanesFn planes_fn(int pp) {
  switch (pp) {
    case 1: return k_planes_reg<N2, N3, 1>;
    case 2: return k_planes_reg<N2, N3, 2>;
    default: return k_planes_reg<N2, N3, 4>;
  }
}

}  // namespace

PlanesFn find_planes_fn(int n2, int n3, int pp) {
#define X(a, b) \
  if (n2 == a && n3 == b) return planes_fn<a, b>(pp);
  PAWPY_FFT_PAIRS(X)
#undef X
  return nullptr;
}

bool fft_planes_fast_supported(int n2, int n3) { return find_planes_fn(n2, n3, 1) != nullptr; }

void launch_fft_planes_fast(const float2 *C, int Wpad, const int *plane_start, const int *plane_off,
                            const PlaneGeom &g, float2 *H, int nb) {
  using namespace fftfast;
  if (nb <= 0 || g.n1 <= 0) return;
  auto run = [&](int pp) {
    PlanesFn fn = find_planes_fn(g.N2, g.N3, pp);
    PAWPY_REQUIRE(fn, "no register FFT for this grid");
    size_t smem = tile_bytes(pp, g.N2, g.N3);
    allow_smem((const void *)fn, smem);
    dim3 grid(ceil_div(g.n1, pp), nb);
    PAWPY_LAUNCH("fft_planes", fn<<<grid, FT, smem, stream()>>>(C, Wpad, plane_start, plane_off, g, H));
  };
  std::vector<int> cands;
  for (int pp : {1, 2, 4})
    if (tile_bytes(pp, g.N2, g.N3) <= kSmemCap) cands.push_back(pp);
  int pp = tune(std::make_tuple(0, g.N1, g.N2, g.N3), cands, run);
  run(pp);
}

}  // namespace pawpy
