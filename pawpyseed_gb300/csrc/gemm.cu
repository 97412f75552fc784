// Complex overlap contraction on the CUDA cores (FP32), the "plain FP32 GPU
// form" of pseudoprojection (pseudoprojector.c:63-90) batched over every
// defect band: out[n][m] = sum_k conj(A[m][k]) B[n][k] per k-point, with the
// K range made of two segments (plane-wave coefficients, then the augmentation
// columns of the PAW terms), split over CTAs and reduced in a fixed order.
#include <cuda_runtime.h>

#include "kernels.h"

namespace pawpy {

namespace {
constexpr int BM = 64, BN = 64, BK = 16, NT = 256;
}

// One 64 x 64 output tile of batch z over split sp of its K range (the body of
// both kernels below; bt is the batch's descriptor in registers).
__device__ __forceinline__ void zgemm_f32_tile(const GemmBatch &bt, int z, int sp, int M, int N, int splits,
                                               float2 *__restrict__ ws, int nz) {
  __shared__ float2 As[2][BK][BM + 1];
  __shared__ float2 Bs[2][BK][BN + 1];
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int K1 = bt.K1, K12 = bt.K1 + bt.K2;
  const int chunks = (K12 + bt.K3) / BK;
  const int c0 = (int)((long long)chunks * sp / splits), c1 = (int)((long long)chunks * (sp + 1) / splits);
  // loader mapping: 64 rows x 16 complex per tile, 4 complex per thread
  const int lr = tid >> 2, lk = (tid & 3) * 4;
  float acc_r[4][4], acc_i[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) acc_r[i][j] = acc_i[i][j] = 0.f;

  auto load = [&](int c, float4 &a0, float4 &a1, float4 &b0, float4 &b1) {
    int k = c * BK + lk;
    const float2 *A, *B;
    long long lda, ldb;
    if (k < K1) {
      A = bt.A1 + k;
      B = bt.B1 + k;
      lda = bt.lda1;
      ldb = bt.ldb1;
    } else if (k < K12) {
      A = bt.A2 + (k - K1);
      B = bt.B2 + (k - K1);
      lda = bt.lda2;
      ldb = bt.ldb2;
    } else {
      A = bt.A3 + (k - K12);
      B = bt.B3 + (k - K12);
      lda = bt.lda3;
      ldb = bt.ldb3;
    }
    float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    if (m0 + lr < M) {
      const float4 *p = reinterpret_cast<const float4 *>(A + (long long)(m0 + lr) * lda);
      a0 = p[0];
      a1 = p[1];
    } else {
      a0 = a1 = zero;
    }
    if (n0 + lr < N) {
      const float4 *p = reinterpret_cast<const float4 *>(B + (long long)(n0 + lr) * ldb);
      b0 = p[0];
      b1 = p[1];
    } else {
      b0 = b1 = zero;
    }
  };
  auto store = [&](int buf, const float4 &a0, const float4 &a1, const float4 &b0, const float4 &b1) {
    As[buf][lk + 0][lr] = make_float2(a0.x, a0.y);
    As[buf][lk + 1][lr] = make_float2(a0.z, a0.w);
    As[buf][lk + 2][lr] = make_float2(a1.x, a1.y);
    As[buf][lk + 3][lr] = make_float2(a1.z, a1.w);
    Bs[buf][lk + 0][lr] = make_float2(b0.x, b0.y);
    Bs[buf][lk + 1][lr] = make_float2(b0.z, b0.w);
    Bs[buf][lk + 2][lr] = make_float2(b1.x, b1.y);
    Bs[buf][lk + 3][lr] = make_float2(b1.z, b1.w);
  };
  if (c0 < c1) {
    float4 a0, a1, b0, b1;
    load(c0, a0, a1, b0, b1);
    store(0, a0, a1, b0, b1);
    __syncthreads();
    for (int c = c0; c < c1; c++) {
      int buf = (c - c0) & 1;
      bool more = c + 1 < c1;
      if (more) load(c + 1, a0, a1, b0, b1);
#pragma unroll
      for (int kk = 0; kk < BK; kk++) {
        float2 a[4], b[4];
#pragma unroll
        for (int i = 0; i < 4; i++) a[i] = As[buf][kk][tx + 16 * i];
#pragma unroll
        for (int j = 0; j < 4; j++) b[j] = Bs[buf][kk][ty + 16 * j];
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
          for (int j = 0; j < 4; j++) {
            // conj(a) * b
            acc_r[i][j] = fmaf(a[i].x, b[j].x, fmaf(a[i].y, b[j].y, acc_r[i][j]));
            acc_i[i][j] = fmaf(a[i].x, b[j].y, fmaf(-a[i].y, b[j].x, acc_i[i][j]));
          }
      }
      if (more) store(buf ^ 1, a0, a1, b0, b1);
      __syncthreads();
    }
  }
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) {
      int m = m0 + tx + 16 * i, n = n0 + ty + 16 * j;
      if (m < M && n < N) {
        float2 v = make_float2(acc_r[i][j], acc_i[i][j]);
        if (splits == 1)
          bt.out[(long long)n * M + m] = v;
        else
          ws[(((long long)sp * nz + z) * N + n) * M + m] = v;
      }
    }
}

__global__ void __launch_bounds__(NT) k_zgemm_f32(const GemmBatch *__restrict__ batches, int M, int N,
                                                  int splits, float2 *__restrict__ ws, int nz) {
  const int z = blockIdx.z / splits, sp = blockIdx.z % splits;
  const GemmBatch bt = batches[z];
  zgemm_f32_tile(bt, z, sp, M, N, splits, ws, nz);
}

__global__ void __launch_bounds__(NT) k_zgemm_f32_one(const GemmBatch bt, int M, int N, int splits,
                                                      float2 *__restrict__ ws) {
  zgemm_f32_tile(bt, 0, blockIdx.z, M, N, splits, ws, 1);
}

__global__ void k_split_reduce(const GemmBatch *__restrict__ batches, const float2 *__restrict__ ws, int M,
                               int N, int splits, int nz) {
  const int z = blockIdx.y;
  float2 *out = batches[z].out;
  long long MN = (long long)M * N;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < MN; e += (long long)gridDim.x * blockDim.x) {
    float2 s = make_float2(0.f, 0.f);
    for (int sp = 0; sp < splits; sp++) {
      float2 v = ws[((long long)sp * nz + z) * MN + e];
      s.x += v.x;
      s.y += v.y;
    }
    out[e] = s;
  }
}

__global__ void k_split_reduce_one(float2 *__restrict__ out, const float2 *__restrict__ ws, int M, int N,
                                   int splits) {
  long long MN = (long long)M * N;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < MN; e += (long long)gridDim.x * blockDim.x) {
    float2 s = make_float2(0.f, 0.f);
    for (int sp = 0; sp < splits; sp++) {
      float2 v = ws[(long long)sp * MN + e];
      s.x += v.x;
      s.y += v.y;
    }
    out[e] = s;
  }
}

void launch_zgemm_f32(const GemmBatch *batches_dev, int nz, int M, int N, int splits, float2 *workspace) {
  if (nz <= 0 || M <= 0 || N <= 0) return;
  if (splits < 1) splits = 1;
  dim3 grid(ceil_div(M, BM), ceil_div(N, BN), nz * splits);
  PAWPY_LAUNCH("gemm_f32", k_zgemm_f32<<<grid, NT, 0, stream()>>>(batches_dev, M, N, splits, workspace, nz));
  if (splits > 1) {
    dim3 g2(ceil_div((long long)M * N, 256 * 4), nz);
    PAWPY_LAUNCH("gemm_reduce", k_split_reduce<<<g2, 256, 0, stream()>>>(batches_dev, workspace, M, N, splits, nz));
  }
}

}  // namespace pawpy
