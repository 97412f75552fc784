// Sphere contraction on the 5th-generation tensor cores (split-BF16): the
// projections <p_{s,c}|psi_row> of onto_projector_helper (projector.c:223-274)
// for every site s, channel c and row (k-point, band) of a batch,
//
//   P[row][c] = sum_{points x of s} T_s[c][x] * A[row][x],
//
// where A[row][x] is the band's value at sphere point x (the picked-point rows
// X of pass B, Bloch phase applied, or the resident real-space grid read at the
// point's cell times its Bloch phase) and T_s the site's table (sphere.cu).
//
// One CTA computes 128 rows of one site. Complex numbers are handled as
// interleaved real pairs: a K block is 16 points = 32 reals (64 bytes of BF16),
// A rows hold (re, im) of each point, and the site's table holds two rows per
// channel, (Tr, -Ti) giving the real part and (Ti, Tr) the imaginary part of
// the product, so one real MMA of N = 2 x channels yields both. Every operand
// is split into BF16 hi and lo planes (x = hi + lo) and the products
// hi*hi + hi*lo + lo*hi are accumulated in FP32 in TMEM, drained every FLUSH K
// blocks into FP32 running sums (as in tc_gemm.cu).
//
// Warp roles: warp 0 issues TMA copies (table planes; with picked rows also the
// FP32 rows into a staging ring), warp 1 the MMAs, CONV converter warps write
// the A planes (split to BF16, 64-byte swizzle) from the staging ring or from
// the gathered grid values, and 4 warps drain the accumulators. Every wait is
// bounded; a wait that runs out records a status word and the CTA winds down.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "kernels.h"
#include "tc_ptx.cuh"

namespace pawpy {

using namespace tcx;

namespace {

constexpr int STM = 128;     // rows per tile (TMEM lanes)
constexpr int KPTS = 16;     // points per K block
constexpr int KELEM = 32;    // BF16 elements per K block row (64 bytes)
constexpr int STAGES = 4;    // A/B plane stages
constexpr int STG = 4;       // FP32 staging stages (picked rows)
constexpr int FLUSH = 4;     // K blocks per accumulation interval
constexpr int DRAIN = 4;     // drain warps

template <int BN, bool GATHER>
struct SphCfg {
  static constexpr int CONV = GATHER ? 8 : 4;  // converter warps
  static constexpr int NTHREADS = 32 * (2 + CONV + DRAIN);
  static constexpr int RPW = STM / CONV;       // rows per converter warp
  static constexpr int A_PLANE = STM * 64;     // 8 KB
  static constexpr int B_PLANE = BN * 64;
  static constexpr int STAGE = 2 * A_PLANE + 2 * B_PLANE;
  static constexpr int STG_BYTES = STM * KPTS * 8;  // 16 KB of FP32 (re, im) pairs
  static constexpr int SMEM = STAGES * STAGE + (GATHER ? 0 : STG * STG_BYTES) + 1024;
  static constexpr int TMEM_COLS = 2 * BN <= 64 ? 64 : 128;  // two accumulator sets
  static constexpr int SETC = TMEM_COLS / 2;                      // columns between the sets
};

// kind::f16 with BF16 inputs, FP32 accumulation, both operands K-major, M = 128, N = bn
__host__ __device__ constexpr uint32_t idesc_bf16(int bn) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(bn >> 3) << 17) |
         (static_cast<uint32_t>(STM >> 4) << 24);
}

__device__ __forceinline__ uint32_t pack_bf16(__nv_bfloat16 a, __nv_bfloat16 b) {
  return (uint32_t)__bfloat16_as_ushort(a) | ((uint32_t)__bfloat16_as_ushort(b) << 16);
}

__device__ __forceinline__ void split2(float2 v, uint32_t &hi, uint32_t &lo) {
  const __nv_bfloat16 hr = __float2bfloat16_rn(v.x), hi_ = __float2bfloat16_rn(v.y);
  const __nv_bfloat16 lr = __float2bfloat16_rn(v.x - __bfloat162float(hr));
  const __nv_bfloat16 li = __float2bfloat16_rn(v.y - __bfloat162float(hi_));
  hi = pack_bf16(hr, hi_);
  lo = pack_bf16(lr, li);
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

}  // namespace

// grid (row tiles, sites); see the file comment. With GATHER, a row tile never
// crosses a k-point (the Bloch phase of a point depends on the k-point).
template <int BN, bool GATHER>
__global__ void __launch_bounds__(SphCfg<BN, GATHER>::NTHREADS, 1)
    k_tc_sphere(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int brows,
                const TcSite *__restrict__ sites, ContractSource src, int nb, int *__restrict__ status) {
  using C = SphCfg<BN, GATHER>;
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) unsigned long long b_full[STAGES], conv_full[STAGES], mma_empty[STAGES];
  __shared__ __align__(8) unsigned long long stg_full[STG], stg_empty[STG];
  __shared__ __align__(8) unsigned long long bar_accf[2], bar_acce[2], bar_drain;
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int abort_flag;

  const TcSite st = sites[blockIdx.y];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // rows [row0, row0 + nrows) of the batch
  int row0, nrows;
  long long kq = 0;
  if (GATHER) {
    const int bpk = (src.nband + STM - 1) / STM;
    kq = src.r0 / src.nband + blockIdx.x / bpk;
    const long long lo = kq * src.nband + (long long)(blockIdx.x % bpk) * STM;
    const long long hi = min(min(lo + STM, (kq + 1) * src.nband), src.r0 + nb);
    row0 = (int)(max(lo, src.r0) - src.r0);
    nrows = (int)(hi - src.r0) - row0;
  } else {
    row0 = blockIdx.x * STM;
    nrows = min(STM, nb - row0);
  }
  if (nrows <= 0) return;  // uniform over the CTA, before any barrier or TMEM use
  const int nkb = st.nkb;
  const int nq = (nkb + FLUSH - 1) / FLUSH;

  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t sbase = (raw + 1023u) & ~1023u;
  const uint32_t stg_base = sbase + STAGES * C::STAGE;
  auto a_plane = [&](int s, int p) { return sbase + s * C::STAGE + p * C::A_PLANE; };
  auto b_plane = [&](int s, int p) { return sbase + s * C::STAGE + 2 * C::A_PLANE + p * C::B_PLANE; };

  if (threadIdx.x == 0) {
    abort_flag = 0;
    for (int s = 0; s < STAGES; s++) {
      mbar_init(smem_u32(&b_full[s]), 1);
      mbar_init(smem_u32(&conv_full[s]), 32 * C::CONV);
      mbar_init(smem_u32(&mma_empty[s]), 1);
    }
    for (int s = 0; s < STG; s++) {
      mbar_init(smem_u32(&stg_full[s]), 1);
      mbar_init(smem_u32(&stg_empty[s]), 32 * C::CONV);
    }
    for (int s = 0; s < 2; s++) {
      mbar_init(smem_u32(&bar_accf[s]), 1);
      mbar_init(smem_u32(&bar_acce[s]), DRAIN);
    }
    mbar_init(smem_u32(&bar_drain), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(C::TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;

  auto fail = [&](int code) {
    abort_flag = 1;
    atomicExch(status, code);
  };

  if (warp == 0) {
    if (lane == 0 && nkb > 0) {
      int last_b[STAGES], last_a[STG];
#pragma unroll
      for (int s = 0; s < STAGES; s++) last_b[s] = -1;
#pragma unroll
      for (int s = 0; s < STG; s++) last_a[s] = -1;
      for (int i = 0; i < nkb; i++) {
        const int s = i % STAGES, r = i / STAGES;
        if (r > 0 && !mbar_wait(smem_u32(&mma_empty[s]), (r - 1) & 1, &abort_flag)) {
          if (!abort_flag) fail(11);
          break;
        }
        if (abort_flag) break;
        const uint32_t bf = smem_u32(&b_full[s]);
        mbar_expect_tx(bf, 2 * C::B_PLANE);
        tma_load_2d(b_plane(s, 0), &tmB, bf, i * KELEM, st.b_row);
        tma_load_2d(b_plane(s, 1), &tmB, bf, i * KELEM, brows + st.b_row);
        last_b[s] = r;
        if (!GATHER) {
          const int t = i % STG, u = i / STG;
          if (u > 0 && !mbar_wait(smem_u32(&stg_empty[t]), (u - 1) & 1, &abort_flag)) {
            if (!abort_flag) fail(12);
            break;
          }
          if (abort_flag) break;
          const uint32_t af = smem_u32(&stg_full[t]);
          mbar_expect_tx(af, C::STG_BYTES);
          tma_load_2d(stg_base + t * C::STG_BYTES, &tmA, af, (int)(2 * (st.a_x + (long long)i * KPTS)), row0);
          last_a[t] = u;
        }
      }
      if (abort_flag) {
        // let the copies already issued land before the CTA's memory is released
        for (int s = 0; s < STAGES; s++)
          if (last_b[s] >= 0) mbar_wait(smem_u32(&b_full[s]), last_b[s] & 1);
        for (int s = 0; s < STG; s++)
          if (last_a[s] >= 0) mbar_wait(smem_u32(&stg_full[s]), last_a[s] & 1);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t id = idesc_bf16(BN);
      int i = 0;
      bool stop = false;
      for (int q = 0; q < nq && !stop; q++) {
        const int set = q & 1, u = q >> 1;
        if (u > 0 && !mbar_wait(smem_u32(&bar_acce[set]), (u - 1) & 1, &abort_flag)) {
          if (!abort_flag) fail(13);
          break;
        }
        const uint32_t dset = tmem + set * C::SETC;
        bool first = true;
        const int iend = min(nkb, (q + 1) * FLUSH);
        for (; i < iend; i++) {
          const int s = i % STAGES, r = i / STAGES;
          if (!mbar_wait(smem_u32(&b_full[s]), r & 1, &abort_flag) ||
              !mbar_wait(smem_u32(&conv_full[s]), r & 1, &abort_flag)) {
            if (!abort_flag) fail(14);
            stop = true;
            break;
          }
          tc_fence_after();
#pragma unroll
          for (int j = 0; j < 2; j++) {
#pragma unroll
            for (int t = 0; t < 3; t++) {
              // hi*hi, hi*lo, lo*hi
              const int pa = t == 2 ? 1 : 0, pb = t == 1 ? 1 : 0;
              const uint64_t ad = sdesc_sw64(a_plane(s, pa) + j * 32);
              const uint64_t bd = sdesc_sw64(b_plane(s, pb) + j * 32);
              umma<false>(dset, ad, bd, id, first ? 0u : 1u);
              first = false;
            }
          }
          umma_commit(smem_u32(&mma_empty[s]));
        }
        if (!stop) umma_commit(smem_u32(&bar_accf[set]));
      }
      umma_commit(smem_u32(&bar_drain));
    }
  } else if (warp < 2 + C::CONV) {
    // converters: rows [cw RPW, (cw + 1) RPW); lane -> (row parity half, point p)
    const int cw = warp - 2, half = lane >> 4, p = lane & 15;
    for (int i = 0; i < nkb; i++) {
      const int s = i % STAGES, r = i / STAGES;
      if (r > 0 && !mbar_wait(smem_u32(&mma_empty[s]), (r - 1) & 1, &abort_flag)) {
        if (!abort_flag) fail(15);
        break;
      }
      float2 v[C::RPW / 2];
      if (GATHER) {
        const long long x = st.a_x + (long long)i * KPTS + p;
        int cell = -1;
        float2 ph = make_float2(0.f, 0.f);
        if (x < src.npts) {
          cell = __ldg(src.gcell + x);
          ph = __ldg(src.gphase + kq * src.npts + x);
        }
#pragma unroll
        for (int it = 0; it < C::RPW / 2; it++) {
          const int row = cw * C::RPW + 2 * it + half;
          float2 g = make_float2(0.f, 0.f);
          if (cell >= 0 && row < nrows) g = __ldg(src.grid + (src.r0 + row0 + row) * src.n3d + cell);
          v[it] = make_float2(g.x * ph.x - g.y * ph.y, g.x * ph.y + g.y * ph.x);
        }
      } else {
        const int t = i % STG, u = i / STG;
        if (!mbar_wait(smem_u32(&stg_full[t]), u & 1, &abort_flag)) {
          if (!abort_flag) fail(16);
          break;
        }
        const float2 *sg = reinterpret_cast<const float2 *>(smem_raw + (stg_base + t * C::STG_BYTES - raw));
#pragma unroll
        for (int it = 0; it < C::RPW / 2; it++) v[it] = sg[(cw * C::RPW + 2 * it + half) * KPTS + p];
        mbar_arrive(smem_u32(&stg_empty[t]));
      }
      unsigned char *ah = smem_raw + (a_plane(s, 0) - raw), *al = smem_raw + (a_plane(s, 1) - raw);
#pragma unroll
      for (int it = 0; it < C::RPW / 2; it++) {
        const int row = cw * C::RPW + 2 * it + half;
        uint32_t h, l;
        split2(v[it], h, l);
        const uint32_t off = sw64_offset(row, p >> 2) + 4 * (p & 3);
        *reinterpret_cast<uint32_t *>(ah + off) = h;
        *reinterpret_cast<uint32_t *>(al + off) = l;
      }
      fence_async_smem();
      mbar_arrive(smem_u32(&conv_full[s]));
    }
  } else {
    // drain warps: TMEM lane quarter (warp % 4), all BN columns
    const int quarter = warp & 3;
    float acc[BN];
#pragma unroll
    for (int j = 0; j < BN; j++) acc[j] = 0.f;
    bool good = true;
    for (int q = 0; q < nq; q++) {
      const int set = q & 1, u = q >> 1;
      bool ok = mbar_wait(smem_u32(&bar_accf[set]), u & 1, &abort_flag);
      if (!ok && !abort_flag) fail(17);
      if (!__all_sync(0xffffffffu, ok && !abort_flag)) {
        good = false;
        break;
      }
      tc_fence_after();
      const uint32_t base = tmem + (static_cast<uint32_t>(32 * quarter) << 16) + set * C::SETC;
#pragma unroll
      for (int c = 0; c < BN; c += 16) {
        float w[16];
        tmem_ld16(base + c, w);
        tmem_ld_wait();
#pragma unroll
        for (int j = 0; j < 16; j++) acc[c + j] += w[j];
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_u32(&bar_acce[set]));
    }
    const int m = 32 * quarter + lane;
    if (good && m < nrows) {
      float2 *o = st.out + (src.r0 + row0 + m) * (long long)st.ld;
#pragma unroll
      for (int c = 0; c < BN / 2; c++)
        if (c < st.total) o[c] = make_float2(acc[2 * c], acc[2 * c + 1]);
    }
  }

  // no MMA may still write TMEM when it is freed
  if (nkb > 0 && !mbar_wait(smem_u32(&bar_drain), 0)) fail(18);
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(C::TMEM_COLS));
  }
}

// Table planes of the sites: rows [b_row, b_row + bn) of site s, row 2c = (Tr, -Ti) and
// row 2c + 1 = (Ti, Tr) of channel c at each local point j (point j - lead of the site's
// table; zero outside the site and for c >= total), split into BF16 hi (plane 0) and lo
// (plane 1) planes of brows rows of lb elements. Grid (point blocks, bn, sites).
__global__ void k_tc_tables(const TcTable *__restrict__ tabs, int brows, long long lb,
                            __nv_bfloat16 *__restrict__ planes) {
  const TcTable t = tabs[blockIdx.z];
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= t.nkb * KPTS) return;
  const int n = blockIdx.y, c = n >> 1, p = j - t.lead;
  float2 v = make_float2(0.f, 0.f);
  if (c < t.total && p >= 0 && p < t.npts) v = __ldg(t.tab + (long long)c * t.npts + p);
  const float2 e = (n & 1) ? make_float2(v.y, v.x) : make_float2(v.x, -v.y);
  uint32_t h, l;
  split2(e, h, l);
  const long long off = (long long)(t.b_row + n) * lb + 2LL * j;
  *reinterpret_cast<uint32_t *>(planes + off) = h;
  *reinterpret_cast<uint32_t *>(planes + (long long)brows * lb + off) = l;
}

int tc_sphere_width(int max_total) {
  if (max_total > 32) throw Error(ERR_UNSUPPORTED, "more than 32 projector channels on one site");
  return max_total <= 16 ? 32 : max_total <= 24 ? 48 : 64;
}

void launch_tc_tables(const TcTable *tabs_dev, int nsites, int max_nkb, int bn, int brows, long long lb,
                      void *planes) {
  if (nsites <= 0 || max_nkb <= 0) return;
  PAWPY_REQUIRE(lb % KELEM == 0 && lb >= (long long)max_nkb * KELEM, "table planes too short");
  dim3 grid(ceil_div(max_nkb * KPTS, 128), bn, nsites);
  PAWPY_LAUNCH("tc_tables", k_tc_tables<<<grid, 128, 0, stream()>>>(tabs_dev, brows, lb,
                                                                   static_cast<__nv_bfloat16 *>(planes)));
}

namespace {

template <int BN, bool GATHER>
void tc_sphere(const CUtensorMap &ma, const CUtensorMap &mb, int brows, const TcSite *sites, int nsites,
               const ContractSource &src, int nb, int *st) {
  using C = SphCfg<BN, GATHER>;
  allow_dynamic_smem((const void *)k_tc_sphere<BN, GATHER>, C::SMEM);
  int tiles = ceil_div(nb, STM);
  if (GATHER) {
    const long long k0 = src.r0 / src.nband, k1 = (src.r0 + nb - 1) / src.nband;
    tiles = (int)(k1 - k0 + 1) * ceil_div(src.nband, STM);
  }
  dim3 grid(tiles, nsites);
  PAWPY_LAUNCH("sphere_contract_tc", (k_tc_sphere<BN, GATHER><<<grid, C::NTHREADS, C::SMEM, stream()>>>(
                                         ma, mb, brows, sites, src, nb, st)));
}

}  // namespace

void launch_tc_sphere(const TcSite *sites_dev, int nsites, int bn, const void *planes, int brows, long long lb,
                      const ContractSource &src, int nb, long long npts, long long xtot) {
  if (nsites <= 0 || nb <= 0) return;
  note_work("sphere_contract_tc", 8.0 * (double)npts * nb);
  const bool gather = src.grid != nullptr;
  PAWPY_REQUIRE(gather || src.X, "contraction without a source");
  PAWPY_REQUIRE(!gather || src.nband > 0, "contraction source without a band count");
  PAWPY_REQUIRE(gather || src.xstride % 4 == 0, "picked-point rows must be 32-byte aligned");
  PAWPY_REQUIRE(bn == 32 || bn == 48 || bn == 64, "tensor-core contraction: table width must be 32, 48 or 64");
  const CUtensorMap mb = tensor_map_2d(const_cast<void *>(planes), CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, lb,
                                       2LL * brows, lb * 2, KELEM, bn, CU_TENSOR_MAP_SWIZZLE_64B);
  // picked rows as FP32 (re, im) pairs; points from xtot on read as zero
  CUtensorMap ma = mb;
  if (!gather)
    ma = tensor_map_2d(const_cast<float2 *>(src.X), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, 2 * std::max(1LL, xtot), nb,
                       src.xstride * 8, 2 * KPTS, STM, CU_TENSOR_MAP_SWIZZLE_NONE);
  int *st = device_status();
#define PAWPY_TC_SPHERE(W)                                                 \
  (gather ? tc_sphere<W, true>(ma, mb, brows, sites_dev, nsites, src, nb, st) \
          : tc_sphere<W, false>(ma, mb, brows, sites_dev, nsites, src, nb, st))
  if (bn == 32)
    PAWPY_TC_SPHERE(32);
  else if (bn == 48)
    PAWPY_TC_SPHERE(48);
  else
    PAWPY_TC_SPHERE(64);
#undef PAWPY_TC_SPHERE
  status_readback(st, "tensor-core sphere contraction: a pipeline wait timed out");
}

}  // namespace pawpy
