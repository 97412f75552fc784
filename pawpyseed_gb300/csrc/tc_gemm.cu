// Overlap contraction on the 5th-generation tensor cores: the split-BF16
// (3-term) and TF32 forms of pseudoprojection (pseudoprojector.c:63-90)
// batched over every band pair and k-point, plus the augmentation columns of
// the PAW terms appended to K.
//
//   out[z][n][m] = sum_k conj(A[m][k]) B[n][k]
//               = sum_k (ar br + ai bi) + i (ar bi - ai br)
//
// Operands are first split into planes, each K-major with K contiguous:
//   split-BF16: hi_re, hi_im, lo_re, lo_im with x = hi + lo, hi = bf16(x),
//               lo = bf16(x - hi); products hi*hi + hi*lo + lo*hi (lo*lo,
//               about 2^-18 of |a||b|, is dropped), FP32 accumulation;
//   TF32:       re, im in FP32 read as TF32 by the tensor core.
// One CTA computes a 128 (basis bands) x BN (defect bands, BN = 128 or 64) tile
// of one k-point over a K range (split-K); the tile width and the split count
// are chosen per problem shape by timing the candidates once (run_tc). A single thread issues TMA copies of
// 64-byte-wide K blocks (64-byte swizzle) into a ring of shared-memory stages,
// a second issues tcgen05.mma from them into TMEM, and eight warps drain the
// accumulators into registers (see k_tc_zgemm). Partial sums over K ranges
// are reduced in a fixed order by k_split_reduce, so results do not depend on
// scheduling.
//
// Every mbarrier wait is bounded (kWaitNs); a wait that runs out records a
// status word, stops issuing work, waits (bounded) for the copies and MMAs
// already issued, frees its TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <atomic>
#include <map>
#include <mutex>
#include <string>
#include <tuple>

#include "kernels.h"
#include "tc_ptx.cuh"

namespace pawpy {

using namespace tcx;

namespace {

constexpr int TM = 128;          // basis bands per tile (TMEM lanes)
constexpr int BN_MAX = 128;      // widest defect-band tile; operand B rows are padded to it
constexpr int ROWB = 64;         // bytes of one K block row (64-byte swizzle span)
constexpr int DRAIN_WARPS = 8;   // warps 2..9
constexpr int NTHREADS = 32 * (2 + DRAIN_WARPS);
constexpr int FLUSH = 4;         // K blocks per accumulation interval

// BN defect bands per tile (TMEM columns per accumulator): 128, or 64 with two CTAs per SM
// (half the TMEM columns and fewer stages, so that two fit in TMEM and shared memory).
template <bool TF32, int BN>
struct Prec {
  static constexpr int NPL = TF32 ? 2 : 4;            // planes per operand
  static constexpr int ESZ = TF32 ? 4 : 2;            // bytes per element
  static constexpr int KB = ROWB / ESZ;               // elements per K block
  static constexpr int KSTEPS = 2;                    // 32-byte MMA K steps per block
  static constexpr int A_PLANE = TM * ROWB;           // 8 KB
  static constexpr int B_PLANE = BN * ROWB;           // 8 or 4 KB
  static constexpr int STAGE = NPL * (A_PLANE + B_PLANE);
  static constexpr int STAGES = BN == 128 ? (TF32 ? 6 : 3) : (TF32 ? 4 : 2);
  static constexpr int SMEM = STAGES * STAGE + 1024;  // + alignment slack
  static constexpr int NTERMS = TF32 ? 4 : 12;
  static constexpr int TMEM_COLS = 4 * BN;            // two sets of (re, im)
};

// Products of one K step: A plane | B plane << 4 | accumulator (0 re, 1 im)
// << 8 | negate A << 12. Split-BF16 planes are 0 hi_re, 1 hi_im, 2 lo_re,
// 3 lo_im; TF32 planes 0 re, 1 im.
template <bool TF32>
__host__ __device__ constexpr uint32_t term(int t) {
  constexpr uint32_t bf16[12] = {0x0000, 0x0020, 0x0002, 0x0011, 0x0031, 0x0013,
                                 0x0110, 0x0130, 0x0112, 0x1101, 0x1121, 0x1103};
  constexpr uint32_t tf32[4] = {0x0000, 0x0011, 0x0110, 0x1101};
  return TF32 ? tf32[t & 3] : bf16[t];
}

// Instruction descriptor of kind::f16 (BF16 inputs) or kind::tf32, FP32
// accumulation, both operands K-major, M = TM (128), N = bn.
__host__ __device__ constexpr uint32_t idesc(bool tf32, bool negA, int bn) {
  return (1u << 4) | ((tf32 ? 2u : 1u) << 7) | ((tf32 ? 2u : 1u) << 10) | ((negA ? 1u : 0u) << 13) |
         (static_cast<uint32_t>(bn >> 3) << 17) | (static_cast<uint32_t>(TM >> 4) << 24);
}

}  // namespace

// grid (M tiles, N tiles, nz * splits), NTHREADS threads. kblocks[z]: K
// blocks of batch z (zero-filled beyond its K); the planes are
// [plane][z][rows_pad][Kc].
//
// Warp 0 issues the TMA copies, warp 1 the MMAs; warps 2..9 drain the
// accumulators. The MMAs of FLUSH consecutive K blocks go into one of two TMEM
// accumulator sets (re and im, 128 columns each), starting from zero; the
// drain warps then add that set to FP32 running sums in registers (rounded to
// nearest) while the MMAs fill the other set. The tensor core truncates its
// FP32 accumulator at every instruction, an error biased towards zero that
// grows with the magnitude it accumulates; draining keeps that magnitude to a
// few K blocks, so the bias stays near 6 FLUSH 2^-24 |S| whatever K is.
template <bool TF32, int BN>
__global__ void __launch_bounds__(NTHREADS, (BN == 128 ? 1 : 2))  // CTAs per SM
    k_tc_zgemm(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmA2, int kbs,
               const __grid_constant__ CUtensorMap tmB, const GemmBatch *__restrict__ batches,
               const int *__restrict__ kblocks, int M, int N, int Mpad, int Npad, int nz, int splits,
               float2 *__restrict__ ws, int *__restrict__ status) {
  using P = Prec<TF32, BN>;
  constexpr int TN = BN;
  constexpr int TMEM_COLS = P::TMEM_COLS;
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) unsigned long long bar_full[P::STAGES], bar_empty[P::STAGES];
  __shared__ __align__(8) unsigned long long bar_accf[2], bar_acce[2], bar_drain;
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int abort_flag;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int z = blockIdx.z / splits, sp = blockIdx.z % splits;
  const int m0 = blockIdx.x * TM, n0 = blockIdx.y * TN;
  const int nkb = kblocks[z];
  const int kb0 = (int)((long long)nkb * sp / splits), kb1 = (int)((long long)nkb * (sp + 1) / splits);
  const int nloc = kb1 - kb0;
  const int nq = (nloc + FLUSH - 1) / FLUSH;  // accumulation intervals

  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t sbase = (raw + 1023u) & ~1023u;

  if (threadIdx.x == 0) {
    abort_flag = 0;
    for (int s = 0; s < P::STAGES; s++) {
      mbar_init(smem_u32(&bar_full[s]), 1);
      mbar_init(smem_u32(&bar_empty[s]), 1);
    }
    for (int s = 0; s < 2; s++) {
      mbar_init(smem_u32(&bar_accf[s]), 1);
      mbar_init(smem_u32(&bar_acce[s]), DRAIN_WARPS);
    }
    mbar_init(smem_u32(&bar_drain), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(TMEM_COLS));
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
    if (lane == 0 && nloc > 0) {
      // TMA producer
      const int rowsA = nz * Mpad, rowsB = nz * Npad;
      int last_round[P::STAGES];
#pragma unroll
      for (int s = 0; s < P::STAGES; s++) last_round[s] = -1;
      for (int i = 0; i < nloc; i++) {
        const int s = i % P::STAGES, r = i / P::STAGES;
        if (r > 0 && !mbar_wait(smem_u32(&bar_empty[s]), (r - 1) & 1)) {
          fail(1);
          break;
        }
        if (abort_flag) break;
        const uint32_t full = smem_u32(&bar_full[s]);
        const uint32_t st = sbase + s * P::STAGE;
        mbar_expect_tx(full, P::STAGE);
        const int kb = kb0 + i, x = kb * P::KB;
        // operand A: K blocks below kbs from tmA, the rest from tmA2 (planes of the columns
        // from kbs KB on)
        const CUtensorMap *ma = kb < kbs ? &tmA : &tmA2;
        const int xa = kb < kbs ? x : (kb - kbs) * P::KB;
#pragma unroll
        for (int p = 0; p < P::NPL; p++) {
          tma_load_2d(st + p * P::A_PLANE, ma, full, xa, p * rowsA + z * Mpad + m0);
          tma_load_2d(st + P::NPL * P::A_PLANE + p * P::B_PLANE, &tmB, full, x, p * rowsB + z * Npad + n0);
        }
        last_round[s] = r;
      }
      if (abort_flag) {
        // let the copies already issued land before the CTA's memory is released
        for (int s = 0; s < P::STAGES; s++)
          if (last_round[s] >= 0) mbar_wait(smem_u32(&bar_full[s]), last_round[s] & 1);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // MMA issuer
      const uint32_t id_pos = idesc(TF32, false, BN), id_neg = idesc(TF32, true, BN);
      int i = 0;
      bool stop = false;
      for (int q = 0; q < nq && !stop; q++) {
        const int set = q & 1, u = q >> 1;
        if (u > 0 && !mbar_wait(smem_u32(&bar_acce[set]), (u - 1) & 1)) {
          fail(2);
          break;
        }
        const uint32_t dset = tmem + set * (2 * TN);
        bool first[2] = {true, true};
        const int iend = min(nloc, (q + 1) * FLUSH);
        for (; i < iend; i++) {
          const int s = i % P::STAGES, r = i / P::STAGES;
          if (!mbar_wait(smem_u32(&bar_full[s]), r & 1)) {
            fail(3);
            stop = true;
            break;
          }
          if (abort_flag) {
            stop = true;
            break;
          }
          tc_fence_after();
          const uint32_t st = sbase + s * P::STAGE;
#pragma unroll
          for (int j = 0; j < P::KSTEPS; j++) {
#pragma unroll
            for (int t = 0; t < P::NTERMS; t++) {
              const uint32_t tt = term<TF32>(t);
              const uint32_t pa = tt & 15u, pb = (tt >> 4) & 15u, acc = (tt >> 8) & 15u;
              const uint64_t ad = sdesc_sw64(st + pa * P::A_PLANE + j * 32);
              const uint64_t bd = sdesc_sw64(st + P::NPL * P::A_PLANE + pb * P::B_PLANE + j * 32);
              umma<TF32>(dset + acc * TN, ad, bd, (tt >> 12) ? id_neg : id_pos, first[acc] ? 0u : 1u);
              first[acc] = false;
            }
          }
          umma_commit(smem_u32(&bar_empty[s]));
        }
        if (!stop) umma_commit(smem_u32(&bar_accf[set]));
      }
      umma_commit(smem_u32(&bar_drain));
    }
  } else {
    // drain warps: TMEM lane quarter (warp % 4), column half h
    const int quarter = warp & 3, h = (warp - 2) >> 2;
    float sr[TN / 2], si[TN / 2];
#pragma unroll
    for (int j = 0; j < TN / 2; j++) sr[j] = si[j] = 0.f;
    bool good = true;
    for (int q = 0; q < nq; q++) {
      const int set = q & 1, u = q >> 1;
      bool ok = mbar_wait(smem_u32(&bar_accf[set]), u & 1, &abort_flag);
      if (!ok && !abort_flag) fail(4);
      if (!__all_sync(0xffffffffu, ok && !abort_flag)) {
        good = false;
        break;
      }
      tc_fence_after();
      const uint32_t base = tmem + (static_cast<uint32_t>(32 * quarter) << 16) + set * (2 * TN) + h * (TN / 2);
#pragma unroll
      for (int c = 0; c < TN / 2; c += 16) {
        float re[16], im[16];
        tmem_ld16(base + c, re);
        tmem_ld16(base + TN + c, im);
        tmem_ld_wait();
#pragma unroll
        for (int j = 0; j < 16; j++) {
          sr[c + j] += re[j];
          si[c + j] += im[j];
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_u32(&bar_acce[set]));
    }
    if (good) {
      const int m = m0 + 32 * quarter + lane;
      float2 *dst = splits == 1 ? batches[z].out : ws + ((long long)sp * nz + z) * (long long)N * M;
      if (m < M) {
#pragma unroll
        for (int j = 0; j < TN / 2; j++) {
          const int n = n0 + h * (TN / 2) + j;
          if (n < N) dst[(long long)n * M + m] = make_float2(sr[j], si[j]);
        }
      }
    }
  }

  // no MMA may still write TMEM when it is freed
  if (nloc > 0 && !mbar_wait(smem_u32(&bar_drain), 0)) fail(5);
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
  }
}

// Splits columns [k_off, k_off + Kc) of one operand into planes [plane][z][rows_pad][Kc]:
// element (z, row, k) is column c = k_off + k, A1[row][c] (c < K1), A2[row][c - K1]
// (c < K1 + K2), A3[row][c - K1 - K2] (c < K1 + K2 + K3) or zero; rows >= rows are zero.
// side 0 takes the A pointers of the batch, side 1 the B pointers.
template <bool TF32>
__global__ void k_split_planes(const GemmBatch *__restrict__ batches, int side, int rows, int rows_pad, int Kc,
                               int k_off, int nz, void *__restrict__ planes) {
  const int z = blockIdx.z, row = blockIdx.y;
  const int k0 = (blockIdx.x * blockDim.x + threadIdx.x) * 4;
  if (k0 >= Kc) return;
  const GemmBatch &bt = batches[z];
  const float2 *s1 = side ? bt.B1 : bt.A1;
  const float2 *s2 = side ? bt.B2 : bt.A2;
  const float2 *s3 = side ? bt.B3 : bt.A3;
  const long long ld1 = side ? bt.ldb1 : bt.lda1, ld2 = side ? bt.ldb2 : bt.lda2;
  const long long ld3 = side ? bt.ldb3 : bt.lda3;
  float2 v[4];
#pragma unroll
  for (int e = 0; e < 4; e++) {
    const int k = k_off + k0 + e;
    v[e] = make_float2(0.f, 0.f);
    if (row < rows) {
      if (k < bt.K1)
        v[e] = s1[row * ld1 + k];
      else if (k < bt.K1 + bt.K2)
        v[e] = s2[row * ld2 + (k - bt.K1)];
      else if (k < bt.K1 + bt.K2 + bt.K3)
        v[e] = s3[row * ld3 + (k - bt.K1 - bt.K2)];
    }
  }
  const size_t plane = (size_t)nz * rows_pad * Kc;
  const size_t off = ((size_t)z * rows_pad + row) * Kc + k0;
  if constexpr (TF32) {
    float *o = static_cast<float *>(planes);
    *reinterpret_cast<float4 *>(o + off) = make_float4(v[0].x, v[1].x, v[2].x, v[3].x);
    *reinterpret_cast<float4 *>(o + plane + off) = make_float4(v[0].y, v[1].y, v[2].y, v[3].y);
  } else {
    __nv_bfloat16 *o = static_cast<__nv_bfloat16 *>(planes);
    __nv_bfloat16 h[2][4], l[2][4];
#pragma unroll
    for (int e = 0; e < 4; e++) {
      const float x[2] = {v[e].x, v[e].y};
#pragma unroll
      for (int c = 0; c < 2; c++) {
        h[c][e] = __float2bfloat16_rn(x[c]);
        l[c][e] = __float2bfloat16_rn(x[c] - __bfloat162float(h[c][e]));
      }
    }
    __nv_bfloat16 *dst[4] = {o + off, o + plane + off, o + 2 * plane + off, o + 3 * plane + off};
    const __nv_bfloat16 *src[4] = {h[0], h[1], l[0], l[1]};
#pragma unroll
    for (int p = 0; p < 4; p++) {
      uint2 u;
      u.x = (uint32_t)__bfloat16_as_ushort(src[p][0]) | ((uint32_t)__bfloat16_as_ushort(src[p][1]) << 16);
      u.y = (uint32_t)__bfloat16_as_ushort(src[p][2]) | ((uint32_t)__bfloat16_as_ushort(src[p][3]) << 16);
      *reinterpret_cast<uint2 *>(dst[p]) = u;
    }
  }
}

// ------------------------------------------------------------------ host side

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    PAWPY_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
    if (q != cudaDriverEntryPointSuccess || !p)
      throw Error(ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

CUtensorMap tensor_map_2d(void *base, CUtensorMapDataType type, int esz, long long inner, long long rows,
                          long long pitch_bytes, int box_inner, int box_rows, CUtensorMapSwizzle swizzle) {
  CUtensorMap m;
  cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)pitch_bytes};
  cuuint32_t box[2] = {(cuuint32_t)box_inner, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  (void)esz;
  CUresult r = encode_fn()(&m, type, 2, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw Error(ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  return m;
}

int sm_count() {
  static int n = 0;
  if (!n) PAWPY_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device()));
  return n;
}

namespace {

CUtensorMap plane_map(void *base, bool tf32, long long Kc, long long rows, int box_rows) {
  const int esz = tf32 ? 4 : 2;
  return tensor_map_2d(base, tf32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, esz, Kc,
                       rows, Kc * esz, ROWB / esz, box_rows, CU_TENSOR_MAP_SWIZZLE_64B);
}


// One launch of the contraction with tiles of bn defect bands and the given K split (plus
// the fixed-order reduction of the split partial sums).
template <bool TF32, int BN>
void launch_tile(const CUtensorMap &ma, const CUtensorMap &ma2, int kbs, const void *pb, int Kc,
                 const GemmBatch *batches_dev, const int *kb_dev, int M, int N, int Mpad, int Npad, int nz, int splits,
                 float2 *ws, int *st) {
  using P = Prec<TF32, BN>;
  const CUtensorMap mb = plane_map(const_cast<void *>(pb), TF32, Kc, (long long)P::NPL * nz * Npad, BN);
  allow_dynamic_smem((const void *)k_tc_zgemm<TF32, BN>, P::SMEM);
  dim3 grid(Mpad / TM, ceil_div(N, BN), nz * splits);
  PAWPY_LAUNCH(TF32 ? "gemm_tf32" : "gemm_bf16x3",
               (k_tc_zgemm<TF32, BN><<<grid, NTHREADS, P::SMEM, stream()>>>(ma, ma2, kbs, mb, batches_dev, kb_dev, M,
                                                                           N, Mpad, Npad, nz, splits, ws, st)));
  if (splits > 1) {
    dim3 g2(ceil_div((long long)M * N, 256 * 4), nz);
    PAWPY_LAUNCH("gemm_reduce", k_split_reduce<<<g2, 256, 0, stream()>>>(batches_dev, ws, M, N, splits, nz));
  }
}

// Tile width and K split per problem shape, chosen once per process by timing the candidates
// (PAWPY_GPU_TUNE_VERBOSE=1 prints each decision with the candidates' times). The key is the
// precision (and a forced width), the basis band count, the defect band count in steps of 64,
// the batch count and the K length in steps of 4096.
struct TcChoice {
  int bn = 128, splits = 1;
};
std::atomic<int> g_tc_tile{0};  // 0: tuned; 64 or 128: that tile width only
std::mutex &tc_tune_mutex() {
  static std::mutex m;
  return m;
}
std::map<std::tuple<int, int, int, int, int>, TcChoice> &tc_tuned() {
  static std::map<std::tuple<int, int, int, int, int>, TcChoice> m;
  return m;
}

template <bool TF32>
void run_tc(const GemmBatch *batches_dev, const std::vector<GemmBatch> &hb, int M, int N, int splits_hint,
            TcGemmInfo *info, TcSplitCache *cacheA) {
  using P = Prec<TF32, BN_MAX>;
  HostPhase hp("tc_gemm");
  const int nz = (int)hb.size();
  int maxK = 0, minkb = 1 << 30;
  std::vector<int> kbl(nz);
  for (int z = 0; z < nz; z++) {
    const int K = hb[z].K1 + hb[z].K2 + hb[z].K3;
    maxK = std::max(maxK, K);
    kbl[z] = ceil_div(K, P::KB);
    minkb = std::min(minkb, kbl[z]);
  }
  const int Kc = ceil_div(std::max(maxK, 1), P::KB) * P::KB;
  const int Mpad = ceil_div(M, TM) * TM, Npad = ceil_div(N, BN_MAX) * BN_MAX;
  // K split for a tile width: enough CTAs for the SMs, at least 4 K blocks per split
  auto splits_for = [&](int bn) {
    const int tiles = (Mpad / TM) * ceil_div(N, bn) * nz;
    int sp = splits_hint > 0 ? splits_hint : std::max(1, sm_count() * (bn == 128 ? 1 : 2) / tiles);
    return std::max(1, std::min(sp, std::max(1, minkb / 4)));
  };
  std::vector<TcChoice> cands;
  auto add = [&](int bn, int sp) {
    sp = std::max(1, std::min(sp, std::max(1, minkb / 4)));
    for (auto &c : cands)
      if (c.bn == bn && c.splits == sp) return;
    cands.push_back({bn, sp});
  };
  const int forced = g_tc_tile.load();
  if (splits_hint > 0) {
    add(forced == 64 ? 64 : 128, splits_for(forced == 64 ? 64 : 128));
  } else {
    for (int bn : {128, 64}) {
      if (forced && bn != forced) continue;
      const int s0 = splits_for(bn);
      add(bn, s0);
      add(bn, 2 * s0);
      add(bn, s0 / 2);
    }
  }
  int max_splits = 1;
  for (auto &c : cands) max_splits = std::max(max_splits, c.splits);

  // operand A's first segment from the cache when every batch's first segment is the cached one
  // (same arrays, a whole number of K blocks): only columns [K1, Kc) are split per call
  int K1 = hb[0].K1;
  bool cached = cacheA && K1 > 0 && K1 % P::KB == 0 && K1 < Kc;
  for (int z = 0; z < nz && cached; z++) cached = hb[z].K1 == K1;
  if (cached) {
    std::lock_guard<std::mutex> lk(cacheA->mu);
    if (!cacheA->built) {
      cacheA->planes.alloc((size_t)P::NPL * nz * Mpad * K1 * P::ESZ);
      dim3 g(ceil_div(K1 / 4, 256), Mpad, nz);
      PAWPY_LAUNCH("tc_split", k_split_planes<TF32><<<g, 256, 0, stream()>>>(batches_dev, 0, M, Mpad, K1, 0, nz,
                                                                               cacheA->planes.p));
      if (!cacheA->ready) PAWPY_CUDA(cudaEventCreateWithFlags(&cacheA->ready, cudaEventDisableTiming));
      PAWPY_CUDA(cudaEventRecord(cacheA->ready, stream()));
      cacheA->built = true;
      cacheA->tf32 = TF32;
      cacheA->nz = nz;
      cacheA->Mpad = Mpad;
      cacheA->K1 = K1;
      cacheA->src.resize(nz);
      for (int z = 0; z < nz; z++) cacheA->src[z] = hb[z].A1;
    }
    cached = cacheA->tf32 == TF32 && cacheA->nz == nz && cacheA->Mpad == Mpad && cacheA->K1 == K1;
    for (int z = 0; z < nz && cached; z++) cached = cacheA->src[z] == hb[z].A1;
    if (cached) PAWPY_CUDA(cudaStreamWaitEvent(stream(), cacheA->ready, 0));
  }
  const int Ka = cached ? Kc - K1 : Kc;  // columns of the per-call planes of A
  DevBuf<unsigned char> pa((size_t)P::NPL * nz * Mpad * Ka * P::ESZ);
  DevBuf<unsigned char> pb((size_t)P::NPL * nz * Npad * Kc * P::ESZ);
  DevBuf<int> kb_dev(nz);
  kb_dev.upload(kbl.data(), nz);
  {
    dim3 g(ceil_div(Ka / 4, 256), Mpad, nz);
    PAWPY_LAUNCH("tc_split", k_split_planes<TF32><<<g, 256, 0, stream()>>>(batches_dev, 0, M, Mpad, Ka,
                                                                             cached ? K1 : 0, nz, pa.p));
    dim3 g2(ceil_div(Kc / 4, 256), Npad, nz);
    PAWPY_LAUNCH("tc_split", k_split_planes<TF32><<<g2, 256, 0, stream()>>>(batches_dev, 1, N, Npad, Kc, 0, nz, pb.p));
  }
  const CUtensorMap ma = cached ? plane_map(cacheA->planes.p, TF32, K1, (long long)P::NPL * nz * Mpad, TM)
                                : plane_map(pa.p, TF32, Kc, (long long)P::NPL * nz * Mpad, TM);
  const CUtensorMap ma2 = cached ? plane_map(pa.p, TF32, Ka, (long long)P::NPL * nz * Mpad, TM) : ma;
  const int kbs = cached ? K1 / P::KB : Kc / P::KB;
  DevBuf<float2> ws;
  if (max_splits > 1) ws.alloc((size_t)max_splits * nz * N * M);
  int *st = device_status();
  auto run = [&](const TcChoice &c) {
    if (c.bn == 128)
      launch_tile<TF32, 128>(ma, ma2, kbs, pb.p, Kc, batches_dev, kb_dev.p, M, N, Mpad, Npad, nz, c.splits, ws.p, st);
    else
      launch_tile<TF32, 64>(ma, ma2, kbs, pb.p, Kc, batches_dev, kb_dev.p, M, N, Mpad, Npad, nz, c.splits, ws.p, st);
  };
  TcChoice choice = cands[0];
  if (cands.size() > 1) {
    const auto key = std::make_tuple((TF32 ? 1 : 0) + 2 * forced, M, ceil_div(N, 64), nz, ceil_div(Kc, 4096));
    bool have = false;
    {
      std::lock_guard<std::mutex> lk(tc_tune_mutex());
      auto it = tc_tuned().find(key);
      if (it != tc_tuned().end()) {
        choice = it->second;
        have = true;
      }
    }
    if (!have) {
      // every candidate computes the full result; the chosen one runs again below
      std::vector<cudaEvent_t> ev(cands.size() + 1);
      for (auto &e : ev) PAWPY_CUDA(cudaEventCreate(&e));
      PAWPY_CUDA(cudaEventRecord(ev[0], stream()));
      for (size_t i = 0; i < cands.size(); i++) {
        run(cands[i]);
        PAWPY_CUDA(cudaEventRecord(ev[i + 1], stream()));
      }
      PAWPY_CUDA(cudaEventSynchronize(ev.back()));
      float best = 1e30f;
      std::string log;
      for (size_t i = 0; i < cands.size(); i++) {
        float ms = 0;
        PAWPY_CUDA(cudaEventElapsedTime(&ms, ev[i], ev[i + 1]));
        char buf[64];
        snprintf(buf, sizeof buf, " (%d,%d):%.4f", cands[i].bn, cands[i].splits, ms);
        log += buf;
        if (ms < best) {
          best = ms;
          choice = cands[i];
        }
      }
      for (auto &e : ev) cudaEventDestroy(e);
      status_readback(st, "tensor-core overlap: a pipeline wait timed out");
      if (const char *v = getenv("PAWPY_GPU_TUNE_VERBOSE"))
        if (v[0] == '1')
          fprintf(stderr, "[pawpy tune] tc_gemm %s M=%d N=%d nz=%d Kc=%d (tile width, splits):ms%s -> (%d,%d)\n",
                  TF32 ? "tf32" : "bf16x3", M, N, nz, Kc, log.c_str(), choice.bn, choice.splits);
      std::lock_guard<std::mutex> lk(tc_tune_mutex());
      tc_tuned()[key] = choice;
    }
  }
  run(choice);
  status_readback(st, "tensor-core overlap: a pipeline wait timed out");
  if (info) {
    info->splits = choice.splits;
    info->Kc = Kc;
    info->ctas = (Mpad / TM) * ceil_div(N, choice.bn) * nz * choice.splits;
    info->bn = choice.bn;
  }
}

}  // namespace

void set_tc_tile(int bn) { g_tc_tile = (bn == 64 || bn == 128) ? bn : 0; }

void launch_zgemm_tc(const GemmBatch *batches_dev, const std::vector<GemmBatch> &hb, int M, int N, bool tf32,
                     int splits_hint, TcGemmInfo *info, TcSplitCache *cacheA) {
  if (hb.empty() || M <= 0 || N <= 0) return;
  if (tf32)
    run_tc<true>(batches_dev, hb, M, N, splits_hint, info, cacheA);
  else
    run_tc<false>(batches_dev, hb, M, N, splits_hint, info, cacheA);
}

}  // namespace pawpy
