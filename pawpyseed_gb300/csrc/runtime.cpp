// Error status, the library stream, stream-ordered allocation, launch
// accounting and timers of libpawpy_gpu.
#include <unistd.h>

#include <algorithm>
#include <condition_variable>
#include <deque>
#include <exception>
#include <map>
#include <mutex>
#include <string>
#include <thread>

#include "common.h"

namespace pawpy {

static thread_local int g_err = 0;
static thread_local std::string g_msg;

void set_error(int code, const char *msg) {
  g_err = code;
  g_msg = msg ? msg : "";
}
void clear_error() {
  g_err = 0;
  g_msg.clear();
}

namespace {
struct Runtime {
  bool ready = false;
  int dev = 0;
  cudaStream_t s = nullptr;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  long long launches = 0;
  long long bytes = 0;
  std::map<void *, size_t> sizes;
  bool profile = false;
  // timeline origin: recorded when profiling is switched on; every launch's
  // start and end are also taken relative to it (first start, last end per family)
  cudaEvent_t origin = nullptr;
  bool has_origin = false;
  std::chrono::steady_clock::time_point host_origin;
  struct Fam {
    double ms = 0;
    long long n = 0;
    double first = -1, last = -1;
    double work = 0;  // algorithmic bytes or flops the launches declared (note_work)
  };
  std::map<std::string, Fam> fams;
  // profiled launches: family, start and end events, the stream, whether the end was recorded
  struct Pending {
    std::string family;
    cudaEvent_t a, b;
    cudaStream_t s;
    bool ended;
  };
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> event_pool;
  std::recursive_mutex mu;
};
Runtime &rt() {
  static Runtime r;
  return r;
}

void init_locked(Runtime &r) {
  if (r.ready) return;
  PAWPY_CUDA(cudaGetDevice(&r.dev));
  PAWPY_CUDA(cudaStreamCreateWithFlags(&r.s, cudaStreamNonBlocking));
  PAWPY_CUDA(cudaEventCreate(&r.t0));
  PAWPY_CUDA(cudaEventCreate(&r.t1));
  cudaMemPool_t pool;
  PAWPY_CUDA(cudaDeviceGetDefaultMemPool(&pool, r.dev));
  uint64_t thr = ~0ull;
  PAWPY_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
  r.ready = true;
}

cudaEvent_t take_event(Runtime &r) {
  if (!r.event_pool.empty()) {
    cudaEvent_t e = r.event_pool.back();
    r.event_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  PAWPY_CUDA(cudaEventCreate(&e));
  return e;
}

void drain_locked(Runtime &r) {
  for (auto &p : r.pending) {
    if (!p.ended) {
      // a launch that failed between its two records: nothing to time
      r.event_pool.push_back(p.a);
      r.event_pool.push_back(p.b);
      continue;
    }
    float ms = 0;
    PAWPY_CUDA(cudaEventSynchronize(p.b));
    PAWPY_CUDA(cudaEventElapsedTime(&ms, p.a, p.b));
    auto &f = r.fams[p.family];
    f.ms += ms;
    f.n += 1;
    if (r.has_origin) {
      float t0 = 0, t1 = 0;
      PAWPY_CUDA(cudaEventElapsedTime(&t0, r.origin, p.a));
      PAWPY_CUDA(cudaEventElapsedTime(&t1, r.origin, p.b));
      if (f.first < 0 || t0 < f.first) f.first = t0;
      if (t1 > f.last) f.last = t1;
    }
    r.event_pool.push_back(p.a);
    r.event_pool.push_back(p.b);
  }
  r.pending.clear();
}
}  // namespace

// A thread may order its work on a stream of its own (pawpy_gpu_thread_stream),
// so that several host threads keep independent work in flight on the device.
static thread_local cudaStream_t t_stream = nullptr;
// ...and a memory pool of its own: blocks freed on one thread's stream are never
// handed to another thread's stream, so the pool inserts no dependencies
// between the threads' streams (which would order their work).
static thread_local cudaMemPool_t t_pool = nullptr;

// A second stream per thread for host-to-device uploads that overlap the work
// on the thread's main stream (created on first use, at the highest priority
// so that its blocks are scheduled as soon as SM slots free up).
static thread_local cudaStream_t t_side = nullptr;
// ...and a third for work issued ahead of the main stream's queue (the first FFT
// pass of a wavefunction whose projections come later, sphere-table values).
static thread_local cudaStream_t t_aux = nullptr;
// ...and a fourth, above the third, for short work that the host waits on while
// the third is busy (the sphere point counts and index lists).
static thread_local cudaStream_t t_prio = nullptr;

cudaStream_t side_stream() {
  if (!t_side) {
    stream();
    int lo = 0, hi = 0;
    PAWPY_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    PAWPY_CUDA(cudaStreamCreateWithPriority(&t_side, cudaStreamNonBlocking, hi));
  }
  return t_side;
}

bool thread_has_stream() { return t_stream != nullptr; }

cudaStream_t aux_stream() {
  if (!t_aux) {
    stream();
    // high priority: its launches (the first FFT pass, the sphere tables' values and planes)
    // are dispatched ahead of the waiting blocks of a long launch on the library stream; one
    // level below the highest, which the sphere lists use (prio_stream)
    int lo = 0, hi = 0;
    PAWPY_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    PAWPY_CUDA(cudaStreamCreateWithPriority(&t_aux, cudaStreamNonBlocking, hi < lo ? hi + 1 : hi));
  }
  return t_aux;
}

cudaStream_t prio_stream() {
  if (!t_prio) {
    stream();
    int lo = 0, hi = 0;
    PAWPY_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    PAWPY_CUDA(cudaStreamCreateWithPriority(&t_prio, cudaStreamNonBlocking, hi));
  }
  return t_prio;
}

OnStream::OnStream(cudaStream_t s) : prev(t_stream) { t_stream = s; }
OnStream::~OnStream() { t_stream = prev; }

cudaStream_t stream() {
  if (t_stream) return t_stream;
  Runtime &r = rt();
  std::lock_guard<std::recursive_mutex> g(r.mu);
  init_locked(r);
  return r.s;
}

bool device_present() {
  static const bool present = [] {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    return n > 0;
  }();
  return present;
}

int device() {
  stream();
  return rt().dev;
}

// Device status words: a kernel that can fail without a CUDA error (a wait
// that ran out) writes a slot; the slot is copied to pinned host memory on the
// stream and checked at the next sync().
namespace {
constexpr int kSlots = 256;
struct Status {
  int *dev = nullptr, *host = nullptr;
  int next = 0;
};
// slots read back by this thread, with the stream each read-back was ordered on
struct PendingStatus {
  int slot;
  std::string what;
  cudaStream_t stream;
};
thread_local std::vector<PendingStatus> t_pending;
Status &status_state() {
  static Status s;
  return s;
}
}  // namespace

int *device_status() {
  Runtime &r = rt();
  std::lock_guard<std::recursive_mutex> g(r.mu);
  init_locked(r);
  Status &st = status_state();
  if (!st.dev) {
    PAWPY_CUDA(cudaMalloc(&st.dev, kSlots * sizeof(int)));
    PAWPY_CUDA(cudaMallocHost(&st.host, kSlots * sizeof(int)));
  }
  int slot = st.next;
  st.next = (st.next + 1) % kSlots;
  PAWPY_CUDA(cudaMemsetAsync(st.dev + slot, 0, sizeof(int), stream()));
  return st.dev + slot;
}

void status_readback(int *dev_slot, const char *what) {
  Runtime &r = rt();
  std::lock_guard<std::recursive_mutex> g(r.mu);
  Status &st = status_state();
  int slot = (int)(dev_slot - st.dev);
  PAWPY_CUDA(cudaMemcpyAsync(st.host + slot, dev_slot, sizeof(int), cudaMemcpyDeviceToHost, stream()));
  t_pending.push_back({slot, what, stream()});
}

void sync() {
  const cudaStream_t s = stream();
  PAWPY_CUDA(cudaStreamSynchronize(s));
  if (t_pending.empty()) return;
  // only the read-backs ordered on the stream just waited for have landed
  Status &st = status_state();
  std::string msg;
  std::vector<PendingStatus> rest;
  for (auto &p : t_pending) {
    if (p.stream != s) {
      rest.push_back(p);
      continue;
    }
    if (st.host[p.slot] != 0 && msg.empty()) msg = p.what + " (status " + std::to_string(st.host[p.slot]) + ")";
  }
  t_pending.swap(rest);
  if (!msg.empty()) throw Error(ERR_DEVICE_FLAG, msg);
}

namespace {
// Two halves; a half is reused once the copies out of it have completed (an
// event on each stream that copied from it, recorded when the ring left it).
constexpr size_t kRingHalf = 4u << 20;
constexpr size_t kRingMax = 1u << 20;
struct Ring {
  char *buf = nullptr;
  size_t off = 0;
  int half = 0;
  std::vector<cudaStream_t> used[2];
  std::vector<cudaEvent_t> done[2];
};
thread_local Ring t_ring;

void ring_wait(Ring &r, int h) {
  for (cudaEvent_t e : r.done[h]) {
    PAWPY_CUDA(cudaEventSynchronize(e));
    PAWPY_CUDA(cudaEventDestroy(e));
  }
  r.done[h].clear();
  r.used[h].clear();
}

void ring_free(Ring &r) {
  if (!r.buf) return;
  ring_wait(r, 0);
  ring_wait(r, 1);
  PAWPY_CUDA(cudaFreeHost(r.buf));
  r = Ring();
}
}  // namespace

void upload_bytes(void *dev, const void *h, size_t bytes) {
  cudaStream_t s = stream();
  if (bytes > kRingMax) {
    PAWPY_CUDA(cudaMemcpyAsync(dev, h, bytes, cudaMemcpyHostToDevice, s));
    return;
  }
  Ring &r = t_ring;
  if (!r.buf) PAWPY_CUDA(cudaMallocHost(reinterpret_cast<void **>(&r.buf), 2 * kRingHalf));
  const size_t need = (bytes + 255) & ~size_t(255);
  if (r.off + need > kRingHalf) {
    for (cudaStream_t u : r.used[r.half]) {
      cudaEvent_t e;
      PAWPY_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      PAWPY_CUDA(cudaEventRecord(e, u));
      r.done[r.half].push_back(e);
    }
    r.used[r.half].clear();
    r.half ^= 1;
    r.off = 0;
    ring_wait(r, r.half);
  }
  char *p = r.buf + (size_t)r.half * kRingHalf + r.off;
  std::memcpy(p, h, bytes);
  PAWPY_CUDA(cudaMemcpyAsync(dev, p, bytes, cudaMemcpyHostToDevice, s));
  auto &u = r.used[r.half];
  if (std::find(u.begin(), u.end(), s) == u.end()) u.push_back(s);
  r.off += need;
}

void *dmalloc(size_t bytes) {
  cudaStream_t s = stream();
  void *p = nullptr;
  cudaError_t e = t_pool ? cudaMallocFromPoolAsync(&p, bytes, t_pool, s) : cudaMallocAsync(&p, bytes, s);
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw Error(ERR_ALLOC, std::string("device allocation of ") + std::to_string(bytes) +
                               " bytes failed: " + cudaGetErrorString(e));
  }
  Runtime &r = rt();
  std::lock_guard<std::recursive_mutex> g(r.mu);
  r.sizes[p] = bytes;
  r.bytes += (long long)bytes;
  return p;
}

void dfree(void *p) {
  if (!p) return;
  Runtime &r = rt();
  {
    std::lock_guard<std::recursive_mutex> g(r.mu);
    auto it = r.sizes.find(p);
    if (it != r.sizes.end()) {
      r.bytes -= (long long)it->second;
      r.sizes.erase(it);
    }
  }
  cudaFreeAsync(p, stream());
}

long long device_bytes() { return rt().bytes; }

void launch_begin(const char *family) {
  Runtime &r = rt();
  std::lock_guard<std::recursive_mutex> g(r.mu);
  init_locked(r);
  r.launches++;
  if (r.profile) {
    cudaEvent_t a = take_event(r), b = take_event(r);
    const cudaStream_t s = t_stream ? t_stream : r.s;
    PAWPY_CUDA(cudaEventRecord(a, s));
    r.pending.push_back({family, a, b, s, false});
  }
}

void note_work(const char *family, double units) {
  Runtime &r = rt();
  std::lock_guard<std::recursive_mutex> g(r.mu);
  if (r.profile) r.fams[family].work += units;
}

void launch_end(const char *family) {
  Runtime &r = rt();
  std::lock_guard<std::recursive_mutex> g(r.mu);
  if (!r.profile) return;
  // the latest open launch of this family on this thread's stream (launches of other host
  // threads may have been recorded in between)
  const cudaStream_t s = t_stream ? t_stream : r.s;
  for (auto it = r.pending.rbegin(); it != r.pending.rend(); ++it)
    if (!it->ended && it->s == s && it->family == family) {
      PAWPY_CUDA(cudaEventRecord(it->b, s));
      it->ended = true;
      return;
    }
}

namespace {
// Host worker pool: threads started once (detached; the pool is never
// destroyed) that wait for jobs, so that short host loops over k-points cost
// no thread creation. Jobs of several calling threads run at once: a worker
// takes the next item of the oldest job that has items left, and each caller
// works on its own job too. A process forked from one that used the pool
// starts a pool of its own.
struct HostJob {
  const std::function<void(int)> *f = nullptr;
  int n = 0, next = 0, done = 0, users = 0;  // guarded by the pool's mutex
  std::exception_ptr err;
};

struct HostPool {
  pid_t pid = 0;
  int nthreads = 0;
  std::mutex m;
  std::condition_variable cv_work, cv_done;
  std::deque<HostJob *> jobs;  // jobs with items not yet handed out

  // Runs one item of j (m held on entry and exit).
  void run_one(HostJob *j, std::unique_lock<std::mutex> &lk) {
    const int i = j->next++;
    if (j->next >= j->n) jobs.erase(std::find(jobs.begin(), jobs.end(), j));
    j->users++;
    lk.unlock();
    std::exception_ptr e;
    try {
      (*j->f)(i);
    } catch (...) {
      e = std::current_exception();
    }
    lk.lock();
    if (e && !j->err) j->err = e;
    j->done++;
    j->users--;
    if (j->done == j->n && j->users == 0) cv_done.notify_all();
  }
  void worker() {
    std::unique_lock<std::mutex> lk(m);
    for (;;) {
      cv_work.wait(lk, [&] { return !jobs.empty(); });
      run_one(jobs.front(), lk);
    }
  }
};

HostPool *host_pool() {
  static std::mutex init;
  static HostPool *pool = nullptr;
  std::lock_guard<std::mutex> lk(init);
  if (!pool || pool->pid != getpid()) {
    pool = new HostPool();  // never destroyed: its threads outlive every caller
    pool->pid = getpid();
    const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
    pool->nthreads = std::min(hw, 16) - 1;
    for (int t = 0; t < pool->nthreads; t++) std::thread([p = pool] { p->worker(); }).detach();
  }
  return pool;
}
}  // namespace

void host_parallel_for(int n, const std::function<void(int)> &f) {
  HostPool *p = n > 1 ? host_pool() : nullptr;
  if (!p || p->nthreads == 0) {
    for (int i = 0; i < n; i++) f(i);
    return;
  }
  HostJob j;
  j.f = &f;
  j.n = n;
  std::unique_lock<std::mutex> lk(p->m);
  p->jobs.push_back(&j);
  p->cv_work.notify_all();
  while (j.next < j.n) p->run_one(&j, lk);
  // every item is handed out (j has left the queue); wait for the ones still running
  p->cv_done.wait(lk, [&] { return j.done == j.n && j.users == 0; });
  lk.unlock();
  if (j.err) std::rethrow_exception(j.err);
}

void allow_dynamic_smem(const void *kernel, size_t bytes) {
  static std::mutex m;
  static std::map<const void *, size_t> done;
  if (bytes <= 48 * 1024) return;
  std::lock_guard<std::mutex> lk(m);
  size_t &d = done[kernel];
  if (bytes > d) {
    PAWPY_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    d = bytes;
  }
}

bool profiling() {
  Runtime &r = rt();
  std::lock_guard<std::recursive_mutex> g(r.mu);
  return r.profile;
}

void host_time(const char *name, double ms) {
  Runtime &r = rt();
  const auto now = std::chrono::steady_clock::now();
  std::lock_guard<std::recursive_mutex> g(r.mu);
  auto &f = r.fams[std::string("host.") + name];
  f.ms += ms;
  f.n += 1;
  // host phases on the same timeline (the host clock when profiling was switched on stands
  // for the origin event, which the device records moments later)
  const double t1 = std::chrono::duration<double, std::milli>(now - r.host_origin).count(), t0 = t1 - ms;
  if (f.first < 0 || t0 < f.first) f.first = t0;
  if (t1 > f.last) f.last = t1;
}

void note_launches(int n) {
  Runtime &r = rt();
  std::lock_guard<std::recursive_mutex> g(r.mu);
  r.launches += n;
}

void check_launch(const char *what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    throw Error(ERR_CUDA, std::string("launch of ") + what + " failed: " + cudaGetErrorString(e));
}

}  // namespace pawpy

using namespace pawpy;

extern "C" {

int pawpy_gpu_last_error(void) { return g_err; }
const char *pawpy_gpu_error_string(void) { return g_msg.c_str(); }
void pawpy_gpu_clear_error(void) { clear_error(); }

void pawpy_gpu_timer_start(void) {
  PAWPY_API_BEGIN
  Runtime &r = rt();
  PAWPY_CUDA(cudaEventRecord(r.t0, stream()));
  PAWPY_API_END()
}

int pawpy_gpu_thread_stream(int on) {
  PAWPY_API_BEGIN
  stream();  // the device context and the shared stream exist first
  if (on && !t_stream) {
    PAWPY_CUDA(cudaStreamCreateWithFlags(&t_stream, cudaStreamNonBlocking));
    if (!t_pool) {
      cudaMemPoolProps props = {};
      props.allocType = cudaMemAllocationTypePinned;
      props.location.type = cudaMemLocationTypeDevice;
      props.location.id = device();
      PAWPY_CUDA(cudaMemPoolCreate(&t_pool, &props));
      uint64_t thr = ~0ull;
      PAWPY_CUDA(cudaMemPoolSetAttribute(t_pool, cudaMemPoolAttrReleaseThreshold, &thr));
      int no = 0;
      PAWPY_CUDA(cudaMemPoolSetAttribute(t_pool, cudaMemPoolReuseAllowInternalDependencies, &no));
    }
  } else if (!on && t_stream) {
    // the staging ring's copies were ordered on this thread's streams
    {
      Ring &r = t_ring;
      for (int h = 0; h < 2; h++) {
        for (cudaStream_t u : r.used[h]) PAWPY_CUDA(cudaStreamSynchronize(u));
        r.used[h].clear();
      }
      ring_free(r);
    }
    for (cudaStream_t *ps : {&t_side, &t_aux, &t_prio})
      if (*ps) {
        cudaStream_t u = *ps;
        *ps = nullptr;
        PAWPY_CUDA(cudaStreamSynchronize(u));
        PAWPY_CUDA(cudaStreamDestroy(u));
      }
    cudaStream_t s = t_stream;
    PAWPY_CUDA(cudaStreamSynchronize(s));
    t_stream = nullptr;
    PAWPY_CUDA(cudaStreamDestroy(s));
    if (t_pool) {
      // the pool stays (blocks may still be owned by longer-lived objects); its unused memory goes back
      PAWPY_CUDA(cudaMemPoolTrimTo(t_pool, 0));
      t_pool = nullptr;
    }
  }
  return 0;
  PAWPY_API_END(-1)
}

float pawpy_gpu_timer_stop_ms(void) {
  PAWPY_API_BEGIN
  Runtime &r = rt();
  PAWPY_CUDA(cudaEventRecord(r.t1, stream()));
  PAWPY_CUDA(cudaEventSynchronize(r.t1));
  float ms = 0;
  PAWPY_CUDA(cudaEventElapsedTime(&ms, r.t0, r.t1));
  return ms;
  PAWPY_API_END(-1.0f)
}

int pawpy_gpu_host_pool_check(int callers, int n) {
  PAWPY_API_BEGIN
  PAWPY_REQUIRE(callers >= 1 && callers <= 64 && n >= 0 && n <= (1 << 20), "host_pool_check: bad sizes");
  std::vector<std::vector<int>> hits(callers, std::vector<int>(n, 0));
  std::vector<int> bad(callers, 0);
  auto one = [&](int c) {
    host_parallel_for(n, [&](int i) { hits[c][i]++; });
    bool threw = false;
    try {
      host_parallel_for(std::max(n, 2), [&](int i) {
        if (i == 1) throw std::runtime_error("planted");
      });
    } catch (const std::runtime_error &) {
      threw = true;
    }
    for (int i = 0; i < n; i++) bad[c] += hits[c][i] != 1;
    bad[c] += !threw;
  };
  std::vector<std::thread> th;
  for (int c = 1; c < callers; c++) th.emplace_back(one, c);
  one(0);
  for (auto &t : th) t.join();
  int total = 0;
  for (int b : bad) total += b;
  return total;
  PAWPY_API_END(-1)
}

void pawpy_gpu_synchronize(void) {
  PAWPY_API_BEGIN
  // uploads and early transforms on the thread's other streams count as the library's work
  if (t_side) PAWPY_CUDA(cudaStreamSynchronize(t_side));
  if (t_aux) PAWPY_CUDA(cudaStreamSynchronize(t_aux));
  if (t_prio) PAWPY_CUDA(cudaStreamSynchronize(t_prio));
  pawpy::sync();
  PAWPY_API_END()
}

long long pawpy_gpu_launch_count(int reset) {
  Runtime &r = rt();
  std::lock_guard<std::recursive_mutex> g(r.mu);
  long long v = r.launches;
  if (reset) r.launches = 0;
  return v;
}

void pawpy_gpu_profile(int on) {
  Runtime &r = rt();
  std::lock_guard<std::recursive_mutex> g(r.mu);
  if (on && !r.profile) {
    if (!r.origin && cudaEventCreate(&r.origin) != cudaSuccess) r.origin = nullptr;
    r.has_origin = r.origin && cudaEventRecord(r.origin, stream()) == cudaSuccess;
    r.host_origin = std::chrono::steady_clock::now();
  }
  r.profile = on != 0;
}

int pawpy_gpu_kernel_stats(char *buf, int len, int reset) {
  PAWPY_API_BEGIN
  Runtime &r = rt();
  std::lock_guard<std::recursive_mutex> g(r.mu);
  drain_locked(r);
  std::string out;
  for (auto &f : r.fams) {
    char line[320];
    snprintf(line, sizeof line, "%s %.6f %lld %.6f %.6f %.6e\n", f.first.c_str(), f.second.ms, f.second.n,
             f.second.first, f.second.last, f.second.work);
    out += line;
  }
  if (reset) r.fams.clear();
  if (buf && len > 0) {
    strncpy(buf, out.c_str(), (size_t)len - 1);
    buf[len - 1] = 0;
  }
  return (int)out.size() + 1;
  PAWPY_API_END(-1)
}

long long pawpy_gpu_device_bytes(void) { return device_bytes(); }

int pawpy_gpu_pageable_memory_access(void) {
  PAWPY_API_BEGIN
  int dev = device(), a = 0, b = 0;
  PAWPY_CUDA(cudaDeviceGetAttribute(&a, cudaDevAttrPageableMemoryAccess, dev));
  PAWPY_CUDA(cudaDeviceGetAttribute(&b, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev));
  return (a ? 1 : 0) | (b ? 2 : 0);
  PAWPY_API_END(-1)
}

}  // extern "C"
