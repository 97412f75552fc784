// Pass B of the band FFT on the tensor cores, fused with the sphere pick (Gamma point, split
// rows): for band b and plane j the transform along the first axis is the product
//   out[x][z] = sum_p W[x][p] H[b][p][j][z],  W[x][p] = exp(+2 pi i x (g1min + p) / N1)
// over the n1 occupied planes p, computed as one interleaved-real GEMM per (b, j) item:
//   D[z][2x + c] = sum_k A[z][k] B[2x + c][k],  k = 2p + c',
//   A[z][2p] = Re H, A[z][2p + 1] = Im H; B rows 2x = (Wr, -Wi), 2x + 1 = (Wi, Wr) per p,
// so D[z][2x] = Re out and D[z][2x + 1] = Im out (M = 128 rows z, N = NB >= 2 N1, K = 2P with
// P = n1 rounded up to 16), in split BF16 (hi*hi + hi*lo + lo*hi) with FP32 accumulation.
// The output is split into BF16 hi and lo words into the plane tile [N1][LD] and picked as in
// k_xpick_direct (pick_plane_split): the same values and layout as the register transform,
// to the split form's rounding.
//
// One persistent CTA per SM over the items (j-major, band fastest); warp roles:
//   0: TMA of the DFT operand B (both planes, every K block) once;
//   1: TMEM allocation and the MMA issue (one elected lane), two accumulator sets;
//   XT_CONV converter warps: the item's occupied planes of H (FP32) into the split A stage
//         (K-major, 64-byte swizzle), loads of the next item issued before its stage frees;
//   XT_DRAIN = 4 drain warps: TMEM rows (lane quarter = warp % 4) to the split plane tile;
//   XT_PICK pick warps: the plane's entries from the tile to the picked rows.
// Stages: one A stage, two TMEM accumulators, one tile; every wait is bounded (4 s) and a
// wait that runs out writes the status word and stops every role; the MMAs and the B copy
// are waited for before the TMEM is freed and the CTA ends.
#include "fft_fast.cuh"
#include "tc_ptx.cuh"

namespace pawpy {

using namespace tcx;

namespace {

constexpr int XT_CONV = 4, XT_DRAIN = 4, XT_PICK = 10;
constexpr int XT_THREADS = 32 * (2 + XT_CONV + XT_DRAIN + XT_PICK);
constexpr int XT_M = 128;        // rows z of an MMA tile
constexpr int XT_KB_BYTES = 64;  // bytes of a K-block row (32 BF16 = 16 complex)

struct XtGeom {
  int N1, N2, N3, n1, nb;
  int NB;  // MMA N: 2 N1 rounded up to 16
  int KB;  // K blocks of 16 planes
  int LD;  // tile row length
  long long lo_words;
};

// kind::f16 with BF16 inputs, FP32 accumulation, both operands K-major, M = 128, N = n
__host__ __device__ constexpr uint32_t xt_idesc(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(n >> 3) << 17) |
         (static_cast<uint32_t>(XT_M >> 4) << 24);
}

__device__ __forceinline__ void xt_fence_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// The DFT operand B: [2 planes][NB rows][2P BF16], row 2x + c, column 2p + c'.
__global__ void k_dft_operand(int N1, int g1min, int n1, int NB, int K, __nv_bfloat16 *__restrict__ w) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= NB * K) return;
  const int n = e / K, k = e - n * K, x = n >> 1, c = n & 1, p = k >> 1, cp = k & 1;
  float v = 0.f;
  if (x < N1 && p < n1) {
    // exp(2 pi i x g / N1) with the product reduced exactly modulo N1
    long long m = ((long long)x * (g1min + p)) % N1;
    if (m < 0) m += N1;
    double sn, cs;
    sincospi(2.0 * (double)m / (double)N1, &sn, &cs);
    const double d = c == 0 ? (cp == 0 ? cs : -sn) : (cp == 0 ? sn : cs);
    v = (float)d;
  }
  const __nv_bfloat16 hi = __float2bfloat16_rn(v);
  const __nv_bfloat16 lo = __float2bfloat16_rn(v - __bfloat162float(hi));
  w[e] = hi;
  w[(long long)NB * K + e] = lo;
}

__global__ void __launch_bounds__(XT_THREADS, 1)
    k_xpick_tc(const __grid_constant__ CUtensorMap tmW, const float2 *__restrict__ H, XtGeom g,
               const int *__restrict__ plane_first, const uint2 *__restrict__ ent, float2 *__restrict__ X,
               int *__restrict__ status) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) unsigned long long w_full, a_full, a_empty, acc_full[2], acc_empty[2], tile_full,
      tile_empty, mma_done;
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int abort_flag;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long nitems = (long long)g.nb * g.N2;
  const int nmine = blockIdx.x < nitems ? (int)((nitems - 1 - blockIdx.x) / gridDim.x + 1) : 0;
  const int w_plane = g.KB * g.NB * XT_KB_BYTES, a_plane = g.KB * XT_M * XT_KB_BYTES;

  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t sbase = (raw + 1023u) & ~1023u;
  const uint32_t w_base = sbase, a_base = sbase + 2 * w_plane, t_base = a_base + 2 * a_plane;
  uint32_t *thi = reinterpret_cast<uint32_t *>(smem_raw + (t_base - raw));
  uint32_t *tlo = thi + g.N1 * g.LD;

  // the A stage starts zeroed: rows z >= N3 and planes p >= n1 stay zero
  for (int e = threadIdx.x; e < 2 * a_plane / 16; e += blockDim.x)
    reinterpret_cast<uint4 *>(smem_raw + (a_base - raw))[e] = make_uint4(0u, 0u, 0u, 0u);
  if (threadIdx.x == 0) {
    abort_flag = 0;
    mbar_init(smem_u32(&w_full), 1);
    mbar_init(smem_u32(&a_full), 32 * XT_CONV);
    mbar_init(smem_u32(&a_empty), 1);
    for (int s = 0; s < 2; s++) {
      mbar_init(smem_u32(&acc_full[s]), 1);
      mbar_init(smem_u32(&acc_empty[s]), 32 * XT_DRAIN);
    }
    mbar_init(smem_u32(&tile_full), 32 * XT_DRAIN);
    mbar_init(smem_u32(&tile_empty), 32 * XT_PICK);
    mbar_init(smem_u32(&mma_done), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  xt_fence_async();  // the zeroed A stage, before the first MMA reads it
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;

  auto fail = [&](int code) {
    abort_flag = 1;
    atomicExch(status, code);
  };
  bool w_issued = false;

  if (warp == 0) {
    if (lane == 0 && nmine > 0) {
      // the DFT operand: plane pl, K block kb -> NB rows of 64 bytes
      mbar_expect_tx(smem_u32(&w_full), 2 * w_plane);
      for (int pl = 0; pl < 2; pl++)
        for (int kb = 0; kb < g.KB; kb++)
          tma_load_2d(w_base + pl * w_plane + kb * g.NB * XT_KB_BYTES, &tmW, smem_u32(&w_full), kb * 32, pl * g.NB);
      w_issued = true;
    }
  } else if (warp == 1) {
    if (lane == 0 && nmine > 0) {
      const uint32_t id = xt_idesc(g.NB);
      if (!mbar_wait(smem_u32(&w_full), 0, &abort_flag)) {
        if (!abort_flag) fail(31);
      }
      for (int i = 0; i < nmine && !abort_flag; i++) {
        const int set = i & 1, u = i >> 1;
        if (!mbar_wait(smem_u32(&a_full), i & 1, &abort_flag) ||
            (u > 0 && !mbar_wait(smem_u32(&acc_empty[set]), (u - 1) & 1, &abort_flag))) {
          if (!abort_flag) fail(32);
          break;
        }
        tc_fence_after();
        const uint32_t dset = tmem + set * g.NB;
        bool first = true;
        for (int kb = 0; kb < g.KB; kb++)
#pragma unroll
          for (int h = 0; h < 2; h++)
#pragma unroll
            for (int t = 0; t < 3; t++) {
              // hi*hi, hi*lo, lo*hi
              const int pa = t == 2 ? 1 : 0, pb = t == 1 ? 1 : 0;
              const uint64_t ad = sdesc_sw64(a_base + pa * a_plane + kb * XT_M * XT_KB_BYTES + h * 32);
              const uint64_t bd = sdesc_sw64(w_base + pb * w_plane + kb * g.NB * XT_KB_BYTES + h * 32);
              umma<false>(dset, ad, bd, id, first ? 0u : 1u);
              first = false;
            }
        umma_commit(smem_u32(&a_empty));
        umma_commit(smem_u32(&acc_full[set]));
      }
      umma_commit(smem_u32(&mma_done));
    }
  } else if (warp < 2 + XT_CONV) {
    // converters: unit (plane group pg of 4 planes, row z); consecutive threads, consecutive z
    constexpr int NCT = 32 * XT_CONV, BATCH = 5;
    const int ct = threadIdx.x - 64;
    const int ngroups = (g.n1 + 3) / 4, nunits = ngroups * g.N3;
    uint32_t *ahi = reinterpret_cast<uint32_t *>(smem_raw + (a_base - raw));
    for (int i = 0; i < nmine && !abort_flag; i++) {
      const long long item = blockIdx.x + (long long)i * gridDim.x;
      const int j = (int)(item / g.nb), b = (int)(item - (long long)j * g.nb);
      const float2 *hb = H + ((long long)b * g.n1 * g.N2 + j) * g.N3;
      const long long pstride = (long long)g.N2 * g.N3;
      bool ok = true;
      for (int u0 = ct; u0 < nunits && ok; u0 += NCT * BATCH) {
        float2 v[BATCH][4];
#pragma unroll
        for (int q = 0; q < BATCH; q++) {
          const int u = u0 + q * NCT;
          const int pg = u / g.N3, z = u - pg * g.N3;
#pragma unroll
          for (int e = 0; e < 4; e++) {
            const int p = 4 * pg + e;
            v[q][e] = (u < nunits && p < g.n1) ? __ldg(hb + p * pstride + z) : make_float2(0.f, 0.f);
          }
        }
        if (u0 == ct && i > 0 && !mbar_wait(smem_u32(&a_empty), (i - 1) & 1, &abort_flag)) {
          // the MMAs of the previous item have read the stage
          if (!abort_flag) fail(33);
          ok = false;
          break;
        }
#pragma unroll
        for (int q = 0; q < BATCH; q++) {
          const int u = u0 + q * NCT;
          if (u < nunits) {
            const int pg = u / g.N3, z = u - pg * g.N3;
            uint32_t h[4], l[4];
#pragma unroll
            for (int e = 0; e < 4; e++) split_bf16x2(v[q][e], h[e], l[e]);
            const uint32_t off = (pg >> 2) * XT_M * XT_KB_BYTES + sw64_offset(z, pg & 3);
            *reinterpret_cast<uint4 *>(reinterpret_cast<unsigned char *>(ahi) + off) = make_uint4(h[0], h[1], h[2], h[3]);
            *reinterpret_cast<uint4 *>(reinterpret_cast<unsigned char *>(ahi) + a_plane + off) =
                make_uint4(l[0], l[1], l[2], l[3]);
          }
        }
      }
      if (ok && nunits <= ct && i > 0 && !mbar_wait(smem_u32(&a_empty), (i - 1) & 1, &abort_flag)) {
        // (a thread without units still orders its arrival after the stage is free)
        if (!abort_flag) fail(33);
        ok = false;
      }
      if (!ok || abort_flag) break;
      xt_fence_async();
      mbar_arrive(smem_u32(&a_full));
    }
  } else if (warp < 2 + XT_CONV + XT_DRAIN) {
    // drain: TMEM lane quarter (warp % 4) = rows z, NB columns (x, re/im) per item
    const int quarter = warp & 3, z = 32 * quarter + lane;
    for (int i = 0; i < nmine && !abort_flag; i++) {
      const int set = i & 1, u = i >> 1;
      bool ok = mbar_wait(smem_u32(&acc_full[set]), u & 1, &abort_flag);
      if (ok && i > 0) ok = mbar_wait(smem_u32(&tile_empty), (i - 1) & 1, &abort_flag);
      if (!ok && !abort_flag) fail(34);
      if (!__all_sync(0xffffffffu, ok && !abort_flag)) break;
      tc_fence_after();
      const uint32_t base = tmem + (static_cast<uint32_t>(32 * quarter) << 16) + set * g.NB;
      for (int c0 = 0; c0 < g.NB; c0 += 16) {
        float w[16];
        tmem_ld16(base + c0, w);
        tmem_ld_wait();
        if (z < g.N3) {
#pragma unroll
          for (int t = 0; t < 8; t++) {
            const int x = (c0 >> 1) + t;
            if (x < g.N1) split_bf16x2(make_float2(w[2 * t], w[2 * t + 1]), thi[x * g.LD + z], tlo[x * g.LD + z]);
          }
        }
      }
      tc_fence_before();
      mbar_arrive(smem_u32(&acc_empty[set]));
      mbar_arrive(smem_u32(&tile_full));
    }
  } else {
    // pick: the plane's entries from the tile to band b's picked row
    const int pt = threadIdx.x - 32 * (2 + XT_CONV + XT_DRAIN);
    uint32_t *X32 = reinterpret_cast<uint32_t *>(X);
    for (int i = 0; i < nmine && !abort_flag; i++) {
      const long long item = blockIdx.x + (long long)i * gridDim.x;
      const int j = (int)(item / g.nb), b = (int)(item - (long long)j * g.nb);
      bool ok = mbar_wait(smem_u32(&tile_full), i & 1, &abort_flag);
      if (!ok && !abort_flag) fail(35);
      if (!ok || abort_flag) break;
      const int pf = plane_first[j], npj = plane_first[j + 1] - pf;
      pick_plane_split<16>(thi, tlo, ent + pf, npj, pt, 32 * XT_PICK, X32 + (long long)b * 16, g.lo_words);
      mbar_arrive(smem_u32(&tile_empty));
    }
  }

  // the B copy has landed and no MMA still writes TMEM before the memory is released
  if (threadIdx.x == 0 && w_issued && !mbar_wait(smem_u32(&w_full), 0)) fail(36);
  if (nmine > 0 && !mbar_wait(smem_u32(&mma_done), 0)) fail(37);
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
  }
}

}  // namespace

bool xpick_tc_supported(const PlaneGeom &g) {
  const int NB = (2 * g.N1 + 15) / 16 * 16, KB = (g.n1 + 15) / 16;
  const size_t smem = 2 * (size_t)KB * NB * XT_KB_BYTES + 2 * (size_t)KB * XT_M * XT_KB_BYTES +
                      2 * (size_t)g.N1 * padded(g.N3) * 4 + 1024;
  return g.n1 >= 1 && KB <= 4 && NB <= 256 && g.N3 <= XT_M && smem <= 227 * 1024 - 256;
}

void launch_xpick_tc(const float2 *H, const PlaneGeom &geo, const PickList &pl, float2 *X, int nb,
                     long long lo_words) {
  if (nb <= 0) return;
  PAWPY_REQUIRE(xpick_tc_supported(geo) && lo_words > 0, "tensor-core pass B: unsupported grid");
  XtGeom g;
  g.N1 = geo.N1;
  g.N2 = geo.N2;
  g.N3 = geo.N3;
  g.n1 = geo.n1;
  g.nb = nb;
  g.NB = (2 * geo.N1 + 15) / 16 * 16;
  g.KB = (geo.n1 + 15) / 16;
  g.LD = padded(geo.N3);
  g.lo_words = lo_words;
  const int K = 32 * g.KB;
  DevBuf<__nv_bfloat16> w((size_t)2 * g.NB * K);
  PAWPY_LAUNCH("fft_x_pick", k_dft_operand<<<ceil_div((long long)g.NB * K, 256), 256, 0, stream()>>>(
                                 geo.N1, geo.g1min, geo.n1, g.NB, K, w.p));
  const CUtensorMap tmW = tensor_map_2d(w.p, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, K, 2LL * g.NB, (long long)K * 2, 32,
                                        g.NB, CU_TENSOR_MAP_SWIZZLE_64B);
  const size_t smem = 2 * (size_t)g.KB * g.NB * XT_KB_BYTES + 2 * (size_t)g.KB * XT_M * XT_KB_BYTES +
                      2 * (size_t)g.N1 * g.LD * 4 + 1024;
  allow_dynamic_smem((const void *)k_xpick_tc, smem);
  int *st = device_status();
  const long long items = (long long)nb * g.N2;
  const int grid = (int)std::min<long long>(sm_count(), items);
  PAWPY_LAUNCH("fft_x_pick", k_xpick_tc<<<grid, XT_THREADS, smem, stream()>>>(tmW, H, g, pl.plane_first, pl.ent, X,
                                                                           st));
  status_readback(st, "tensor-core pass B");
}

}  // namespace pawpy
