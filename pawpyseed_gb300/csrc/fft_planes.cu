// Dispatch and tuning of pass A of the band FFT (k_planes_pipe).
#include "fft_fast.cuh"

namespace pawpy {

namespace {

using PlanesFn = void (*)(const float2 *, int, int, const int *, const int *, PlaneGeom, float2 *);

PlanesFn find_planes_fn(int n2, int n3) {
#define X(a, b) \
  if (n2 == a && n3 == b) return k_planes_pipe<a, b>;
  PAWPY_FFT_PAIRS(X)
#undef X
  return nullptr;
}

PlanesFn find_planes_direct(int n2, int n3, int *bpc, bool *inplace) {
#define X(a, b)                                                          \
  if (n2 == a && n3 == b) {                                              \
    *bpc = planes_direct_bands(a, b);                                    \
    *inplace = direct_lanes(b) == 1;                                     \
    return k_planes_direct<a, b, direct_lanes(a), direct_lanes(b)>;      \
  }
  PAWPY_FFT_PAIRS(X)
#undef X
  return nullptr;
}

}  // namespace

bool fft_planes_fast_supported(int n2, int n3) { return find_planes_fn(n2, n3) != nullptr; }

void launch_fft_planes_fast(const float2 *C, int Wpad, const int *plane_start, const int *plane_off,
                            const PlaneGeom &g, float2 *H, int nb) {
  using namespace fftfast;
  if (nb <= 0 || g.n1 <= 0) return;
  PlanesFn fn = find_planes_fn(g.N2, g.N3);
  PAWPY_REQUIRE(fn, "no register FFT for this grid");
  const size_t smem = planes_smem(g);
  PAWPY_REQUIRE(smem <= kSmemCap, "FFT plane tiles do not fit in shared memory");
  allow_smem((const void *)fn, smem);
  const int waves = resident_ctas((const void *)fn, smem);
  int bpc = 1;
  bool inplace = false;
  PlanesFn dfn = find_planes_direct(g.N2, g.N3, &bpc, &inplace);
  const size_t dsmem = planes_direct_smem(g, bpc, inplace);
  allow_smem((const void *)dfn, dsmem);
  // candidates: 1, 2, 4 band groups per plane of the pipelined kernel; 0 the direct kernel
  auto run = [&](int mult) {
    if (mult == 0) {
      dim3 grid(g.n1, ceil_div(nb, bpc));
      PAWPY_LAUNCH("fft_planes", dfn<<<grid, FT, dsmem, stream()>>>(C, Wpad, nb, plane_start, plane_off, g, H));
      return;
    }
    const int G = std::max(1, std::min(nb, ceil_div((long long)waves * mult, g.n1)));
    dim3 grid(g.n1, G);
    PAWPY_LAUNCH("fft_planes", fn<<<grid, FT, smem, stream()>>>(C, Wpad, nb, plane_start, plane_off, g, H));
  };
  int mult = tune(std::make_tuple(0, g.N1, g.N2, g.N3), {0, 1, 2, 4}, run);
  run(mult);
  // algorithmic bytes: the coefficients read, the occupied planes of H written
  note_work("fft_planes", 8.0 * ((double)Wpad + (double)g.n1 * g.N2 * g.N3) * nb);
}

}  // namespace pawpy
