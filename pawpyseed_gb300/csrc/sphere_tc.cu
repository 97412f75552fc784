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
// Warp roles: warp 0 issues TMA copies (table planes; with picked rows, which
// pass B writes already split, also the A planes), warp 1 the MMAs, and 4 warps
// drain the accumulators; for grid values, 8 converter warps gather them with
// cp.async into a staging ring, apply the Bloch phase, split them and write the
// A planes (64-byte swizzle). Every mbarrier wait is bounded; a wait that runs
// out records a status word and the CTA winds down.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "bf16split.cuh"
#include "kernels.h"
#include "tc_ptx.cuh"

namespace pawpy {

using namespace tcx;

namespace {

constexpr int STM = 128;     // rows per tile (TMEM lanes)
constexpr int KPTS = 16;     // points per K block
constexpr int KELEM = 32;    // BF16 elements per K block row (64 bytes)
constexpr int FLUSH = 4;     // K blocks per accumulation interval
constexpr int DRAIN = 4;     // drain warps

// GATHER = false: the picked rows are already split (bf16split.cuh), so a K block of A is
// two TMA boxes and the pipeline is TMA -> MMA only (4-5 stages, two CTAs per SM).
// GATHER = true: CONV converter warps gather the grid values with cp.async into a ring of
// STG FP32 staging slots (STG - 1 K blocks in flight), apply the Bloch phase, split and
// write the A planes of an MMA stage.
template <int BN, bool GATHER>
struct SphCfg {
  static constexpr int CONV = GATHER ? 8 : 0;
  static constexpr int NTHREADS = 32 * (2 + CONV + DRAIN);
  static constexpr int STAGES = GATHER ? 4 : (BN <= 48 ? 5 : 4);  // picked rows: two CTAs per SM
  static constexpr int STG = GATHER ? 6 : 0;
  static constexpr int A_PLANE = STM * 64;  // 8 KB
  static constexpr int B_PLANE = BN * 64;
  static constexpr int STAGE = 2 * A_PLANE + 2 * B_PLANE;
  static constexpr int STG_BYTES = STM * KPTS * 8;  // 16 KB of FP32 (re, im) pairs
  static constexpr int PH_BYTES = KPTS * 8;         // the slot's Bloch phases
  static constexpr int SMEM = STAGES * STAGE + STG * (STG_BYTES + PH_BYTES) + 1024;
  static constexpr int TMEM_COLS = 2 * BN <= 64 ? 64 : 128;  // two accumulator sets
  static constexpr int SETC = TMEM_COLS / 2;                  // columns between the sets
  static constexpr int MIN_CTAS = GATHER ? 1 : 2;
};

// kind::f16 with BF16 inputs, FP32 accumulation, both operands K-major, M = 128, N = bn
__host__ __device__ constexpr uint32_t idesc_bf16(int bn) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(bn >> 3) << 17) |
         (static_cast<uint32_t>(STM >> 4) << 24);
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 8- and 16-byte cp.async; src_bytes 0 fills the destination with zeros
__device__ __forceinline__ void cpa8z(uint32_t dst, const void *src, int src_bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cpa16z(uint32_t dst, const void *src, int src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cpa_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cpa_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ void conv_barrier(int nthreads) {
  asm volatile("bar.sync 1, %0;" ::"r"(nthreads) : "memory");
}

}  // namespace

// grid (row tiles, sites); see the file comment. With GATHER, a row tile never
// crosses a k-point (the Bloch phase of a point depends on the k-point).
// tmA (picked rows): 64-byte rows of one K block and one row each, K block b and row r at
// row b arows + r of the hi plane and aplane + b arows + r of the lo plane. Sites start on
// a multiple of 16 points.
template <int BN, bool GATHER>
__global__ void __launch_bounds__(SphCfg<BN, GATHER>::NTHREADS, SphCfg<BN, GATHER>::MIN_CTAS)
    k_tc_sphere(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int arows,
                int aplane, int brows, const TcSite *__restrict__ sites, ContractSource src, int nb,
                int *__restrict__ status) {
  using C = SphCfg<BN, GATHER>;
  constexpr int STAGES = C::STAGES;
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) unsigned long long full[STAGES], conv_full[STAGES], mma_empty[STAGES];
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
  const uint32_t ph_base = stg_base + C::STG * C::STG_BYTES;
  auto a_plane = [&](int s, int p) { return sbase + s * C::STAGE + p * C::A_PLANE; };
  auto b_plane = [&](int s, int p) { return sbase + s * C::STAGE + 2 * C::A_PLANE + p * C::B_PLANE; };

  if (threadIdx.x == 0) {
    abort_flag = 0;
    for (int s = 0; s < STAGES; s++) {
      mbar_init(smem_u32(&full[s]), 1);
      mbar_init(smem_u32(&conv_full[s]), GATHER ? 32 * C::CONV : 1);
      mbar_init(smem_u32(&mma_empty[s]), 1);
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
      // TMA producer: table planes (and, for picked rows, the A planes) of each K block
      int last[STAGES];
#pragma unroll
      for (int s = 0; s < STAGES; s++) last[s] = -1;
      for (int i = 0; i < nkb; i++) {
        const int s = i % STAGES, r = i / STAGES;
        if (r > 0 && !mbar_wait(smem_u32(&mma_empty[s]), (r - 1) & 1, &abort_flag)) {
          if (!abort_flag) fail(11);
          break;
        }
        if (abort_flag) break;
        const uint32_t bf = smem_u32(&full[s]);
        mbar_expect_tx(bf, 2 * C::B_PLANE + (GATHER ? 0 : 2 * C::A_PLANE));
        tma_load_2d(b_plane(s, 0), &tmB, bf, i * KELEM, st.b_row);
        tma_load_2d(b_plane(s, 1), &tmB, bf, i * KELEM, brows + st.b_row);
        if (!GATHER) {
          // K block (a_x / 16 + i): rows [row0, row0 + 128) of the block, hi then lo plane
          const int y = (int)((st.a_x / KPTS + i) * (long long)arows) + row0;
          tma_load_2d(a_plane(s, 0), &tmA, bf, 0, y);
          tma_load_2d(a_plane(s, 1), &tmA, bf, 0, aplane + y);
        }
        last[s] = r;
      }
      if (abort_flag) {
        // let the copies already issued land before the CTA's memory is released
        for (int s = 0; s < STAGES; s++)
          if (last[s] >= 0) mbar_wait(smem_u32(&full[s]), last[s] & 1);
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
          if (!mbar_wait(smem_u32(&full[s]), r & 1, &abort_flag) ||
              (GATHER && !mbar_wait(smem_u32(&conv_full[s]), r & 1, &abort_flag))) {
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
  } else if (GATHER && warp < 2 + C::CONV) {
    // converters. Copies: thread ct -> rows 2 (ct % 64) and 2 (ct % 64) + 1 (bands b0 + row,
    // 16 contiguous bytes of the band-tiled grid) and points [4 (ct / 64), +4) of each K block:
    // a warp's copies read 32 bands of one grid cell (two 128-byte lines) into the slot's
    // [point][row] staging layout. Conversion: thread ct -> row ct % 128 and points
    // [8 (ct / 128), +8): its 16-byte operand stores of 8 consecutive rows hit distinct banks of
    // the swizzled tile. Every converter thread runs every iteration (the named barriers need
    // all of them); after an abort the waits return at once and the conversions are skipped.
    static_assert(!GATHER || C::CONV * 32 == 2 * STM, "two converter threads per row");
    constexpr int NCT = 32 * C::CONV, STG = C::STG, D = STG - 1, PPT = KPTS / 2, CPT = KPTS / 4;
    const int ct = threadIdx.x - 64, row = ct & (STM - 1), pbase = (ct / STM) * PPT;
    const int crow = 2 * (ct & 63), cbase = (ct >> 6) * CPT;
    // rows are bands b0 + row of k-point kq (a tile never crosses a k-point and starts on a
    // multiple of 16 bands): the pair of rows at cell c starts at growp + 16 c (grid_value_index
    // with the band part hoisted)
    const int b0 = (int)(src.r0 + row0 - kq * src.nband);
    const float2 *growp = src.grid + kq * src.gstride + grid_value_index(b0 + crow, 0, src.n3d);
    int cell_next[CPT];
    auto load_cells = [&](int i) {
      const long long x = st.a_x + (long long)i * KPTS + cbase;
      if (i < nkb && x + CPT <= src.npts) {
        const int4 v = __ldg(reinterpret_cast<const int4 *>(src.gcell + x));
        cell_next[0] = v.x, cell_next[1] = v.y, cell_next[2] = v.z, cell_next[3] = v.w;
      } else {
#pragma unroll
        for (int pp = 0; pp < CPT; pp++) cell_next[pp] = (i < nkb && x + pp < src.npts) ? __ldg(src.gcell + x + pp) : -1;
      }
    };
    load_cells(0);
    auto issue = [&](int i) {
      if (i < nkb) {
        const int t = i % STG;
        int cell[CPT];
#pragma unroll
        for (int pp = 0; pp < CPT; pp++) cell[pp] = cell_next[pp];
        load_cells(i + 1);
        const uint32_t slot = stg_base + t * C::STG_BYTES;
#pragma unroll
        for (int pp = 0; pp < CPT; pp++) {
          const int p = cbase + pp;
          const bool ok = cell[pp] >= 0 && crow < nrows;
          const float2 *g = ok ? growp + 16 * cell[pp] : src.grid;
          cpa16z(slot + (p * STM + crow) * 8, g, ok ? 16 : 0);
        }
        if (row == 0 && !src.gamma) {
          // the points' Bloch phases (a gap's value is zero: any finite phase will do)
#pragma unroll
          for (int pp = 0; pp < PPT; pp++) {
            const int p = pbase + pp;
            const long long x = st.a_x + (long long)i * KPTS + p;
            const bool ok = x < src.npts;
            cpa8z(ph_base + (t * KPTS + p) * 8, ok ? src.gphase + kq * src.npts + x : src.gphase, ok ? 8 : 0);
          }
        }
      }
      cpa_commit();
    };
    for (int i = 0; i < D; i++) issue(i);
    for (int i = 0; i < nkb; i++) {
      const int s = i % STAGES, r = i / STAGES, t = i % STG;
      issue(i + D);
      cpa_wait<D>();
      conv_barrier(NCT);  // block i's values are in slot t for every converter thread
      bool ok = !abort_flag;
      if (ok && r > 0 && !mbar_wait(smem_u32(&mma_empty[s]), (r - 1) & 1, &abort_flag)) {
        if (!abort_flag) fail(15);
        ok = false;
      }
      if (ok) {
        const float2 *sg = reinterpret_cast<const float2 *>(smem_raw + (stg_base + t * C::STG_BYTES - raw));
        const float2 *phs = reinterpret_cast<const float2 *>(smem_raw + (ph_base - raw)) + t * KPTS;
        unsigned char *ah = smem_raw + (a_plane(s, 0) - raw), *al = smem_raw + (a_plane(s, 1) - raw);
#pragma unroll
        for (int c = 0; c < PPT / 4; c++) {
          uint32_t h[4], l[4];
#pragma unroll
          for (int e = 0; e < 4; e++) {
            const int p = pbase + 4 * c + e;
            const float2 g = sg[p * STM + row];
            if (src.gamma) {
              // Gamma: every Bloch phase is 1 (a gap's value is zero: its copy was zero-filled)
              split_bf16x2(g, h[e], l[e]);
            } else {
              const float2 ph = phs[p];
              split_bf16x2(make_float2(g.x * ph.x - g.y * ph.y, g.x * ph.y + g.y * ph.x), h[e], l[e]);
            }
          }
          const uint32_t off = sw64_offset(row, (pbase >> 2) + c);
          *reinterpret_cast<uint4 *>(ah + off) = make_uint4(h[0], h[1], h[2], h[3]);
          *reinterpret_cast<uint4 *>(al + off) = make_uint4(l[0], l[1], l[2], l[3]);
        }
        fence_async_smem();
        mbar_arrive(smem_u32(&conv_full[s]));
      }
      conv_barrier(NCT);  // slot t is read by every converter thread before it is refilled
    }
    cpa_wait<0>();
  } else if (warp >= 2 + C::CONV) {
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
// (plane 1) planes of brows rows of lb elements. Grid (point blocks, sites): a thread
// writes every row of its point (consecutive threads, consecutive words of a row).
__global__ void k_tc_tables(const TcTable *__restrict__ tabs, int bn, int brows, long long lb,
                            __nv_bfloat16 *__restrict__ planes) {
  const TcTable t = tabs[blockIdx.y];
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= t.nkb * KPTS) return;
  const int p = j - t.lead;
  const bool in = p >= 0 && p < t.npts;
  uint32_t *hi = reinterpret_cast<uint32_t *>(planes + (long long)t.b_row * lb + 2LL * j);
  uint32_t *lo = reinterpret_cast<uint32_t *>(planes + ((long long)brows + t.b_row) * lb + 2LL * j);
  const long long rw = lb / 2;  // 32-bit words from one row to the next
  for (int c = 0; c < bn / 2; c++) {
    float2 v = make_float2(0.f, 0.f);
    if (c < t.total && in) v = __ldg(t.tab + (long long)c * t.npts + p);
    uint32_t h0, l0, h1, l1;
    split_bf16x2(make_float2(v.x, -v.y), h0, l0);
    split_bf16x2(make_float2(v.y, v.x), h1, l1);
    hi[(2 * c) * rw] = h0;
    lo[(2 * c) * rw] = l0;
    hi[(2 * c + 1) * rw] = h1;
    lo[(2 * c + 1) * rw] = l1;
  }
}

__global__ void k_zero_picked_blocks(uint32_t *__restrict__ X, const long long *__restrict__ blocks,
                                     long long kb_words, int nb, long long lo_words) {
  uint32_t *w = X + blocks[blockIdx.x] * kb_words;
  for (int e = threadIdx.x; e < nb * 16; e += blockDim.x) {
    w[e] = 0u;
    w[lo_words + e] = 0u;
  }
}

void launch_zero_picked_blocks(float2 *X, const long long *blocks, int nblocks, long long kb_words, int nb,
                               long long lo_words) {
  if (nblocks <= 0 || nb <= 0) return;
  PAWPY_LAUNCH("pick_list", k_zero_picked_blocks<<<nblocks, 256, 0, stream()>>>(reinterpret_cast<uint32_t *>(X),
                                                                              blocks, kb_words, nb, lo_words));
}

int tc_sphere_width(int max_total) {
  if (max_total > 32) throw Error(ERR_UNSUPPORTED, "more than 32 projector channels on one site");
  return max_total <= 16 ? 32 : max_total <= 24 ? 48 : 64;
}

void launch_tc_tables(const TcTable *tabs_dev, int nsites, int max_nkb, int bn, int brows, long long lb,
                      void *planes) {
  if (nsites <= 0 || max_nkb <= 0) return;
  PAWPY_REQUIRE(lb % KELEM == 0 && lb >= (long long)max_nkb * KELEM, "table planes too short");
  dim3 grid(ceil_div(max_nkb * KPTS, 128), nsites);
  PAWPY_LAUNCH("tc_tables", k_tc_tables<<<grid, 128, 0, stream()>>>(tabs_dev, bn, brows, lb,
                                                                   static_cast<__nv_bfloat16 *>(planes)));
}

namespace {

template <int BN, bool GATHER>
void tc_sphere(const CUtensorMap &ma, const CUtensorMap &mb, int arows, int aplane, int brows, const TcSite *sites,
               int nsites, const ContractSource &src, int nb, int *st) {
  using C = SphCfg<BN, GATHER>;
  allow_dynamic_smem((const void *)k_tc_sphere<BN, GATHER>, C::SMEM);
  int tiles = ceil_div(nb, STM);
  if (GATHER) {
    const long long k0 = src.r0 / src.nband, k1 = (src.r0 + nb - 1) / src.nband;
    tiles = (int)(k1 - k0 + 1) * ceil_div(src.nband, STM);
  }
  dim3 grid(tiles, nsites);
  PAWPY_LAUNCH("sphere_contract_tc", (k_tc_sphere<BN, GATHER><<<grid, C::NTHREADS, C::SMEM, stream()>>>(
                                         ma, mb, arows, aplane, brows, sites, src, nb, st)));
}

}  // namespace

void launch_tc_sphere(const TcSite *sites_dev, int nsites, int bn, const void *planes, int brows, long long lb,
                      const ContractSource &src, int nb, long long npts, long long xtot) {
  if (nsites <= 0 || nb <= 0) return;
  PAWPY_REQUIRE(src.grid == nullptr || src.r0 % src.nband == 0, "gathered contraction batch not on a k-point");
  note_work("sphere_contract_tc", 8.0 * (double)npts * nb);
  const bool gather = src.grid != nullptr;
  PAWPY_REQUIRE(gather || src.X, "contraction without a source");
  PAWPY_REQUIRE(!gather || src.nband > 0, "contraction source without a band count");
  PAWPY_REQUIRE(gather || src.xstride % 4 == 0, "picked-point rows must be 32-byte aligned");
  PAWPY_REQUIRE(bn == 32 || bn == 48 || bn == 64, "tensor-core contraction: table width must be 32, 48 or 64");
  const CUtensorMap mb = tensor_map_2d(const_cast<void *>(planes), CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, lb,
                                       2LL * brows, lb * 2, KELEM, bn, CU_TENSOR_MAP_SWIZZLE_64B);
  // picked rows in the split form, K blocks of 16 points (bf16split.cuh): xrows rows per block,
  // xtot / 16 blocks per plane; blocks from xtot / 16 on read as zero
  CUtensorMap ma = mb;
  long long aplane = 0;
  if (gather) {
    PAWPY_REQUIRE(src.gstride > 0, "resident grid without a k-point stride");
  } else {
    PAWPY_REQUIRE(src.xrows >= nb && xtot % KPTS == 0, "picked-point blocks do not match the batch");
    aplane = xtot / KPTS * src.xrows;
    PAWPY_REQUIRE(2 * aplane < (1LL << 31), "picked-point planes too large for 32-bit box coordinates");
    ma = tensor_map_2d(const_cast<float2 *>(src.X), CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, KELEM, 2 * aplane, 64, KELEM,
                       STM, CU_TENSOR_MAP_SWIZZLE_64B);
  }
  const int arows = (int)src.xrows;
  int *st = device_status();
#define PAWPY_TC_SPHERE(W)                                                        \
  (gather ? tc_sphere<W, true>(ma, mb, arows, (int)aplane, brows, sites_dev, nsites, src, nb, st) \
          : tc_sphere<W, false>(ma, mb, arows, (int)aplane, brows, sites_dev, nsites, src, nb, st))
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
