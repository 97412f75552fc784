// Allocation-free overlap contraction.
//
// Some callers of this library must not allocate device memory: code that
// runs under a fixed device-memory budget owned by another allocator (a
// framework's caching allocator, a serving process that reserved its memory
// up front), or latency-critical loops where cudaMalloc/cudaFree would
// synchronise the device. For them, pawpy_gpu_overlap_noalloc computes the
// same complex overlap contraction as the plain FP32 form of the batched
// pseudoprojection path (the k_zgemm_f32 tile with split-K and a fixed-order
// reduction) on caller-owned device buffers. Its split-K partial sums live in
// the file-scope device array below, which every GPU that loads the library
// holds (32 MiB) until the process exits; the launch descriptor travels as a
// kernel argument, so nothing but the partial sums is shared between calls.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <mutex>
#include <string>

#include "kernels.h"

namespace pawpy {

// Largest output (M*N complex values) the entry point accepts: the partial sums of at
// least one full split of such an output fit the scratch array.
constexpr long long kNoallocMaxOutput = 4LL << 20;  // 4,194,304 values = 32 MiB of float2

static __device__ __align__(256) float2 g_noalloc_scratch[kNoallocMaxOutput];

namespace {
// split-K factor: enough CTAs for two waves on the device's SMs, at least 32 K-chunks of 16 per split
int noalloc_splits(int M, int N, int K, int sms) {
  int tiles = ceil_div(M, 64) * ceil_div(N, 64);
  int s = std::max(1, ceil_div(2 * sms, tiles));
  s = std::min(s, std::max(1, K / 16 / 32));
  return std::min(s, 64);
}

struct NoallocDevice {
  void *scratch = nullptr;  // device address of g_noalloc_scratch
  int sms = 0;
};
std::mutex g_noalloc_mu;
NoallocDevice g_noalloc_dev[64];

// Set-up of device dev (the current device), once per device and process: the device
// address of the scratch array and the SM count. The address stays valid for the
// life of the CUDA context; a cudaDeviceReset invalidates it.
const NoallocDevice &noalloc_device(int dev) {
  PAWPY_REQUIRE(dev >= 0 && dev < 64, "device ordinal out of range");
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  NoallocDevice &d = g_noalloc_dev[dev];
  if (!d.scratch) {
    // host code may not use g_noalloc_scratch as a device address; take it from the runtime
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      throw Error(ERR_CUDA, std::string("cudaGetSymbolAddress of the scratch array failed: ") +
                                cudaGetErrorString(e));
    int n = 0;
    e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess || n <= 0)
      throw Error(ERR_CUDA, std::string("SM count query failed: ") + cudaGetErrorString(e));
    d.sms = n;
    d.scratch = p;
  }
  return d;
}
}  // namespace

}  // namespace pawpy

using namespace pawpy;

extern "C" int pawpy_gpu_overlap_noalloc(const pawpy_c64 *A, long long lda, const pawpy_c64 *B, long long ldb,
                                         int M, int N, int K, pawpy_c64 *out, void *stream) {
  PAWPY_API_BEGIN
  PAWPY_REQUIRE(A && B && out, "pawpy_gpu_overlap_noalloc: NULL device pointer");
  PAWPY_REQUIRE(M >= 1 && N >= 1, "pawpy_gpu_overlap_noalloc: M and N must be positive");
  PAWPY_REQUIRE(K >= 16 && K % 16 == 0, "pawpy_gpu_overlap_noalloc: K must be a positive multiple of 16");
  PAWPY_REQUIRE(lda >= K && ldb >= K && lda % 2 == 0 && ldb % 2 == 0,
                "pawpy_gpu_overlap_noalloc: lda and ldb must be even and at least K");
  PAWPY_REQUIRE(((uintptr_t)A % 16) == 0 && ((uintptr_t)B % 16) == 0,
                "pawpy_gpu_overlap_noalloc: A and B must be 16-byte aligned");
  long long mn = (long long)M * N;
  if (mn > kNoallocMaxOutput)
    throw Error(ERR_ARG, "pawpy_gpu_overlap_noalloc: output of " + std::to_string(mn) +
                             " values exceeds the scratch limit of " + std::to_string(kNoallocMaxOutput) +
                             " (M*N); use pseudoprojection or pawpy_gpu_project_all");
  int dev = 0;
  PAWPY_CUDA(cudaGetDevice(&dev));
  const NoallocDevice &nd = noalloc_device(dev);
  float2 *partial = static_cast<float2 *>(nd.scratch);
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : pawpy::stream();
  GemmBatch bt;
  bt.A1 = reinterpret_cast<const float2 *>(A);
  bt.B1 = reinterpret_cast<const float2 *>(B);
  bt.lda1 = lda;
  bt.ldb1 = ldb;
  bt.K1 = K;
  bt.A2 = bt.B2 = nullptr;
  bt.lda2 = bt.ldb2 = 0;
  bt.K2 = 0;
  bt.out = reinterpret_cast<float2 *>(out);
  int splits = noalloc_splits(M, N, K, nd.sms);
  splits = (int)std::min<long long>(splits, kNoallocMaxOutput / mn);
  if (splits < 1) splits = 1;
  // the descriptor is a kernel argument; the partials of every split are written in
  // full by this call's first kernel before its second one reduces them
  dim3 grid(ceil_div(M, 64), ceil_div(N, 64), splits);
  k_zgemm_f32_one<<<grid, 256, 0, s>>>(bt, M, N, splits, partial);
  check_launch("overlap_noalloc");
  int launches = 1;
  if (splits > 1) {
    dim3 g2(ceil_div(mn, 256 * 4), 1);
    k_split_reduce_one<<<g2, 256, 0, s>>>(bt.out, partial, M, N, splits);
    check_launch("overlap_noalloc_reduce");
    launches++;
  }
  note_launches(launches);
  return splits;
  PAWPY_API_END(-pawpy_gpu_last_error())
}
