// Internal runtime of libpawpy_gpu: error status, the library stream,
// stream-ordered device buffers and launch accounting.
#pragma once

#include <cuda_runtime.h>

#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/pawpy_gpu.h"

namespace pawpy {

// Error raised inside the library; every extern "C" entry point catches it and
// records the status instead of aborting (the reference exits on failure,
// utils.c:1100-1118).
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

enum ErrCode {
  ERR_CUDA = 1,
  ERR_ARG = 2,
  ERR_STATE = 3,
  ERR_IO = 4,
  ERR_UNSUPPORTED = 5,
  ERR_ALLOC = 6,
  ERR_DEVICE_FLAG = 7,
};

void set_error(int code, const char *msg);
void clear_error();

#define PAWPY_CUDA(call)                                                          \
  do {                                                                            \
    cudaError_t e_ = (call);                                                      \
    if (e_ != cudaSuccess)                                                        \
      throw ::pawpy::Error(::pawpy::ERR_CUDA, std::string(#call) + ": " +         \
                                                  cudaGetErrorString(e_));        \
  } while (0)

#define PAWPY_REQUIRE(cond, msg)                                                  \
  do {                                                                            \
    if (!(cond)) throw ::pawpy::Error(::pawpy::ERR_ARG, (msg));                   \
  } while (0)

// Wraps the body of an extern "C" entry point.
#define PAWPY_API_BEGIN try { ::pawpy::clear_error();
#define PAWPY_API_END(ret)                                                        \
  }                                                                               \
  catch (const ::pawpy::Error &e) {                                               \
    ::pawpy::set_error(e.code, e.what());                                         \
    return ret;                                                                   \
  }                                                                               \
  catch (const std::bad_alloc &) {                                                \
    ::pawpy::set_error(::pawpy::ERR_ALLOC, "host allocation failed");             \
    return ret;                                                                   \
  }                                                                               \
  catch (const std::exception &e) {                                               \
    ::pawpy::set_error(::pawpy::ERR_STATE, e.what());                             \
    return ret;                                                                   \
  }

// The single stream every kernel and copy of the library is ordered on.
cudaStream_t stream();
int device();
// The calling thread's upload stream (highest priority), and a scope in which
// stream() (and so every launch, copy and allocation of the library) is another
// stream. Memory allocated inside such a scope is ordered on that stream: another
// stream that uses or frees it first waits for an event recorded there after the
// allocation (and memory freed there was last used on that stream or before such
// an event).
cudaStream_t side_stream();
// The calling thread's stream for work issued ahead of the library stream's queue.
cudaStream_t aux_stream();
// The calling thread's stream above aux_stream, for short launches that the host
// waits on while long ones run on the auxiliary stream.
cudaStream_t prio_stream();
// Whether the calling thread orders its work on a stream of its own (pawpy_gpu_thread_stream).
bool thread_has_stream();
struct OnStream {
  cudaStream_t prev;
  explicit OnStream(cudaStream_t s);
  ~OnStream();
  OnStream(const OnStream &) = delete;
  OnStream &operator=(const OnStream &) = delete;
};
// Waits for the library stream; throws if a device status word read back
// since the last sync (status_readback) is nonzero.
void sync();
// A zeroed device status word (ordered on the stream) for one kernel, and the
// asynchronous read-back that the next sync() checks.
int *device_status();
void status_readback(int *dev_slot, const char *what);

// Stream-ordered device allocation (cudaMallocAsync from the device's default
// pool, whose release threshold is raised so that memory is reused between
// calls instead of returned to the driver).
void *dmalloc(size_t bytes);
// Host-to-device copy ordered on stream(); h may be reused when it returns.
// Copies of up to 1 MiB go through a pinned staging ring of the calling thread
// and never wait for the stream (a copy from pageable memory may wait for the
// stream's earlier work, which would keep the host from queueing ahead).
void upload_bytes(void *dev, const void *h, size_t bytes);
void dfree(void *p);
long long device_bytes();

template <typename T>
struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  explicit DevBuf(size_t count) { alloc(count); }
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  DevBuf(DevBuf &&o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  DevBuf &operator=(DevBuf &&o) noexcept {
    if (this != &o) { reset(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
    return *this;
  }
  ~DevBuf() { reset(); }
  void alloc(size_t count) {
    reset();
    n = count;
    if (count) p = static_cast<T *>(dmalloc(count * sizeof(T)));
  }
  void reset() {
    if (p) dfree(p);
    p = nullptr;
    n = 0;
  }
  void zero() {
    if (n) PAWPY_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), stream()));
  }
  void upload(const T *h, size_t count, size_t off = 0) {
    if (count) upload_bytes(p + off, h, count * sizeof(T));
  }
  void download(T *h, size_t count, size_t off = 0) const {
    if (count) PAWPY_CUDA(cudaMemcpyAsync(h, p + off, count * sizeof(T), cudaMemcpyDeviceToHost, stream()));
  }
  size_t bytes() const { return n * sizeof(T); }
};

// Launch accounting: every kernel launch goes through launch_begin/launch_end
// so that the count (and, when profiling, per-family device time) is known.
void launch_begin(const char *family);
void launch_end(const char *family);
// While profiling: the algorithmic work (bytes or flops, per the family's unit) of a launch of
// the family, reported beside its device time by pawpy_gpu_kernel_stats.
void note_work(const char *family, double units);
void check_launch(const char *what);
// Counts launches made outside PAWPY_LAUNCH (no events, no allocation).
void note_launches(int n);

// Host-side phases: while profiling is on, the wall time of a scope is added
// to the family "host.<name>" beside the kernel families.
bool profiling();
void host_time(const char *name, double ms);
struct HostPhase {
  const char *name;
  bool on;
  std::chrono::steady_clock::time_point t0;
  explicit HostPhase(const char *n) : name(n), on(profiling()) {
    if (on) t0 = std::chrono::steady_clock::now();
  }
  ~HostPhase() {
    if (on) host_time(name, std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count());
  }
};

// PAWPY_LAUNCH("family", kernel<<<grid, block, smem, pawpy::stream()>>>(args));
#define PAWPY_LAUNCH(family, ...)                                                 \
  do {                                                                            \
    ::pawpy::launch_begin(family);                                                \
    __VA_ARGS__;                                                                  \
    ::pawpy::check_launch(family);                                                \
    ::pawpy::launch_end(family);                                                  \
  } while (0)

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

// Runs f(0..n-1) on the library's host worker threads and the calling thread;
// returns when every index is done and rethrows the first exception. Calls of
// several threads share the workers.
void host_parallel_for(int n, const std::function<void(int)> &f);

// Raises a kernel's dynamic shared-memory limit to at least bytes (thread-safe, once per size).
void allow_dynamic_smem(const void *kernel, size_t bytes);

}  // namespace pawpy
