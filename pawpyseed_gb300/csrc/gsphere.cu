// Plane-wave spheres of the k-points of a WAVECAR on the device: the cutoff test
// of the reader's G loop (reader.c:230-271) for every point of the box
// 0 <= i3 <= 2 nb3, 0 <= i2 <= 2 nb2, 0 <= i1 <= 2 nb1 (VASP order: i3 outer,
// i1 inner), g = i > nb ? (int)(i - 2 nb - 1) : i, kept when
// |(k + g) B|^2 / c <= ENCUT.
//
// The products and sums are the reference's, in its order and without fused
// multiply-adds. The reference then takes pow(pow(|s|^2, 0.5), 2.0) / c; the
// device compares |s|^2 / c, which differs from it by a few ulps at most, so a
// point within a relative 1e-12 of ENCUT is flagged undecided and the host
// decides it with the reference's expression (gsphere_keep). The flags come back
// to the host, which compacts them in box order, one k-point per host thread.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "host.h"
#include "kernels.h"

namespace pawpy {

namespace {

struct GsphereBox {
  double rec[9];  // reciprocal lattice rows b1, b2, b3 (with 2 pi)
  double nb[3];   // nb{1,2,3}max (double, as the reader keeps them)
  int n[3];       // box extents floor(2 nb) + 1
  double c;       // hbar^2 / 2m in eV A^2
  double encut;
};

// flags[k][i3][i2][i1]: 0 outside, 1 inside, 2 undecided (within the margin of ENCUT)
__global__ void k_gsphere_flags(GsphereBox b, const double *__restrict__ kpts, unsigned char *__restrict__ flags) {
  const long long n12 = (long long)b.n[0] * b.n[1], box = n12 * b.n[2];
  const long long L = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (L >= box) return;
  const int kp = blockIdx.y;
  const int i3 = (int)(L / n12), r = (int)(L - (long long)i3 * n12), i2 = r / b.n[0], i1 = r - i2 * b.n[0];
  const int g1 = i1 > b.nb[0] ? (int)(i1 - 2 * b.nb[0] - 1) : i1;
  const int g2 = i2 > b.nb[1] ? (int)(i2 - 2 * b.nb[1] - 1) : i2;
  const int g3 = i3 > b.nb[2] ? (int)(i3 - 2 * b.nb[2] - 1) : i3;
  const double a1 = __dadd_rn(kpts[3 * kp], (double)g1), a2 = __dadd_rn(kpts[3 * kp + 1], (double)g2),
               a3 = __dadd_rn(kpts[3 * kp + 2], (double)g3);
  double s[3];
#pragma unroll
  for (int j = 0; j < 3; j++)
    s[j] = __dadd_rn(__dadd_rn(__dmul_rn(a1, b.rec[j]), __dmul_rn(a2, b.rec[3 + j])), __dmul_rn(a3, b.rec[6 + j]));
  const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(s[0], s[0]), __dmul_rn(s[1], s[1])), __dmul_rn(s[2], s[2]));
  const double v = __ddiv_rn(d2, b.c);
  const double m = 1e-12 * b.encut;
  flags[(long long)kp * box + L] = v < b.encut - m ? 1 : (v > b.encut + m ? 0 : 2);
}

}  // namespace

static std::vector<std::vector<int>> device_gsphere_lists(const double *rec, double encut, const double *kpts,
                                                          int nk, const double nb[3]) {
  GsphereBox b;
  for (int i = 0; i < 9; i++) b.rec[i] = rec[i];
  for (int a = 0; a < 3; a++) {
    b.nb[a] = nb[a];
    b.n[a] = (int)std::floor(2 * nb[a]) + 1;
  }
  b.c = kGsphereC;
  b.encut = encut;
  const long long box = (long long)b.n[0] * b.n[1] * b.n[2];
  PAWPY_REQUIRE(box > 0 && box < (1LL << 31) && nk > 0 && nk <= 65535, "plane-wave box out of range");
  DevBuf<double> dk(3 * (size_t)nk);
  dk.upload(kpts, 3 * (size_t)nk);
  DevBuf<unsigned char> flags((size_t)nk * box);
  PAWPY_LAUNCH("gsphere",
               k_gsphere_flags<<<dim3(ceil_div(box, 256), nk), 256, 0, stream()>>>(b, dk.p, flags.p));
  std::vector<unsigned char> hf((size_t)nk * box);
  flags.download(hf.data(), hf.size());
  sync();
  std::vector<std::vector<int>> out(nk);
  host_parallel_for(nk, [&](int k) {
    const unsigned char *f = hf.data() + (size_t)k * box;
    const double *kv = kpts + 3 * k;
    std::vector<int> &g = out[k];
    long long cnt = 0;
    for (long long L = 0; L < box; L++) cnt += f[L] != 0;
    g.reserve(3 * cnt);
    const long long n12 = (long long)b.n[0] * b.n[1];
    for (long long L = 0; L < box; L++) {
      if (!f[L]) continue;
      const int i3 = (int)(L / n12), r = (int)(L - i3 * n12), i2 = r / b.n[0], i1 = r - i2 * b.n[0];
      const int g1 = i1 > nb[0] ? (int)(i1 - 2 * nb[0] - 1) : i1;
      const int g2 = i2 > nb[1] ? (int)(i2 - 2 * nb[1] - 1) : i2;
      const int g3 = i3 > nb[2] ? (int)(i3 - 2 * nb[2] - 1) : i3;
      if (f[L] == 2 && !gsphere_keep(rec, kv, g1, g2, g3, encut)) continue;
      g.push_back(g1);
      g.push_back(g2);
      g.push_back(g3);
    }
  });
  return out;
}

std::vector<std::vector<int>> gsphere_lists(const double *rec, double encut, const double *kpts, int nk) {
  double nb[3];
  gsphere_bounds(rec, encut, nb);
  if (device_present()) return device_gsphere_lists(rec, encut, kpts, nk, nb);
  std::vector<std::vector<int>> out(nk);
  host_parallel_for(nk, [&](int k) { out[k] = enumerate_gvectors(rec, kpts + 3 * k, encut); });
  return out;
}

}  // namespace pawpy

using namespace pawpy;

extern "C" int pawpy_gpu_gvectors(const double *lattice, const double *kpt, double encut, int *out, int cap) {
  PAWPY_API_BEGIN
  PAWPY_REQUIRE(lattice && kpt && encut > 0, "bad plane-wave sphere arguments");
  PAWPY_REQUIRE(device_present(), "no CUDA device: the plane-wave sphere is enumerated on the device");
  double rec[9], nb[3];
  reciprocal(lattice, rec);
  gsphere_bounds(rec, encut, nb);
  std::vector<int> g = device_gsphere_lists(rec, encut, kpt, 1, nb)[0];
  const int n = (int)(g.size() / 3);
  if (out) {
    PAWPY_REQUIRE(cap >= n, "output capacity below the plane-wave count");
    std::copy(g.begin(), g.end(), out);
  }
  return n;
  PAWPY_API_END(-1)
}
