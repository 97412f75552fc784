// Projection server: continuous batching of band-projection requests against
// resident bases. Each worker thread orders its requests on a CUDA stream of
// its own, so the kernels of requests in flight overlap on the device; a
// request is admitted (first in, first out) when a worker is free and its
// estimated device memory fits the budget, and leaves the budget when it
// completes. Results do not depend on what else is in flight: every reduction
// of the path has a fixed order and requests share only read-only basis data.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "host.h"

namespace pawpy {
namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  long long id = 0;
  pawpy_gpu_request_t r{};
  int fftg[3] = {0, 0, 0};
  std::vector<int> labels, lists[6];
  std::vector<double> coords;
  long long est = 0;
  Clock::time_point t_submit, t_start, t_end;
  double phase_ms[4] = {0, 0, 0, 0};  // setup_projections, overlap_setup_real, project_all, release
  int status = 0;
  std::string msg;
  bool done = false;
};

struct Basis {
  pswf_t *wf = nullptr;
  std::vector<int> labels;
  std::vector<double> coords;
};

struct Server {
  long long budget = 0;
  int slots = 1;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request *> queue;
  std::map<long long, std::unique_ptr<Request>> reqs;
  std::vector<Basis> bases;
  std::vector<std::thread> workers;
  long long next_id = 0, in_flight = 0, peak = 0, done = 0;
  int running = 0;
  bool stop = false;
};

long long round_up(long long v, long long m) { return (v + m - 1) / m * m; }

// Device bytes a request needs at most, from its sizes: coefficients, one FFT
// sub-batch, picked points and partial sums, sphere tables, the overlap
// contraction's operand planes and outputs (25% margin). Workers run on
// streams of their own, so requests never hold the early first-pass planes.
long long estimate_bytes(const pswf_t *R, const pswf_t *S, int num_sites) {
  const long long nbS = S->nband, nbR = R->nband, nk = (long long)S->nspin * S->nwk;
  long long sumW = 0, maxW = 0;
  for (long long k = 0; k < nk; k++) {
    long long W = S->kpts[k]->num_waves;
    sumW += round_up(W, 16);
    maxW = std::max(maxW, W);
  }
  const long long pts = 1500LL * std::max(1, num_sites);  // sphere points, generous
  const long long coeff = 8 * nbS * sumW;
  // H of one FFT sub-batch; picked points and per-chunk partial sums (<= 32 channels per chunk of
  // 256 points) of every (k, band) row, at most 2 GiB
  const long long fft =
      (288LL << 20) + std::min(2LL << 30, nk * (8 * nbS * pts + 8 * nbS * 32 * (pts / 256 + num_sites)));
  const long long tables = pts * (8 * 32 + 8 * nk + 8);
  const long long Kc = round_up(maxW + 32LL * std::max(1, num_sites), 32);
  const long long gemm = 8 * (round_up(nbR, 128) + round_up(nbS, 128)) * Kc * nk + 3 * 8 * nk * nbS * nbR * 4;
  return (coeff + fft + tables + gemm) / 4 * 5;
}

bool admissible(const Server &s) {
  if (s.queue.empty()) return false;
  return s.running == 0 || s.in_flight + s.queue.front()->est <= s.budget;
}

void run_request(Server &s, Request &q) {
  pawpy_gpu_request_t &r = q.r;
  const Basis &B = s.bases[r.basis];
  auto fail = [&](const char *where) {
    q.status = pawpy_gpu_last_error();
    q.msg = std::string(where) + ": " + pawpy_gpu_error_string();
  };
  const int *L[6];
  for (int i = 0; i < 6; i++) L[i] = q.lists[i].empty() ? nullptr : q.lists[i].data();
  auto mut = [](const int *p) { return const_cast<int *>(p); };
  Clock::time_point t = Clock::now();
  auto lap = [&](int i) {
    Clock::time_point n = Clock::now();
    q.phase_ms[i] = std::chrono::duration<double, std::milli>(n - t).count();
    t = n;
  };
  setup_projections(r.wf, r.pps, r.num_elems, r.num_sites, q.fftg, q.labels.data(), q.coords.data());
  lap(0);
  if (pawpy_gpu_last_error()) {
    fail("setup_projections");
  } else {
    overlap_setup_real(B.wf, r.wf, const_cast<int *>(B.labels.data()), q.labels.data(),
                       const_cast<double *>(B.coords.data()), q.coords.data(), mut(L[2]), mut(L[3]), mut(L[4]),
                       mut(L[5]), r.num_N_R, r.num_N_S, r.num_N_RS);
    lap(1);
    if (pawpy_gpu_last_error()) {
      fail("overlap_setup_real");
    } else {
      pawpy_gpu_project_all(r.out, B.wf, r.wf, r.num_M, r.num_N_R, r.num_N_S, r.num_N_RS, mut(L[0]), mut(L[1]),
                            mut(L[2]), mut(L[3]), mut(L[4]), mut(L[5]), 0);
      lap(2);
      if (pawpy_gpu_last_error()) fail("pawpy_gpu_project_all");
    }
  }
  // the wavefunction owns pps once setup_projections attached it
  const bool attached = r.wf->pps == r.pps;
  pawpy_gpu_release(r.wf);
  pawpy_gpu_free_pswf(r.wf);
  lap(3);
  if (!attached && r.pps) free_ppot_array(r.pps, r.num_elems);
  r.wf = nullptr;
  r.pps = nullptr;
}

void worker(Server *s) {
  pawpy_gpu_thread_stream(1);
  for (;;) {
    Request *q = nullptr;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_work.wait(lk, [&] { return (s->stop && s->queue.empty()) || admissible(*s); });
      if (s->queue.empty()) break;
      q = s->queue.front();
      s->queue.pop_front();
      s->in_flight += q->est;
      s->peak = std::max(s->peak, s->in_flight);
      s->running++;
      q->t_start = Clock::now();
    }
    run_request(*s, *q);
    {
      std::lock_guard<std::mutex> lk(s->mu);
      q->t_end = Clock::now();
      q->done = true;
      s->in_flight -= q->est;
      s->running--;
      s->done++;
    }
    s->cv_done.notify_all();
    s->cv_work.notify_all();
  }
  pawpy_gpu_thread_stream(0);
}

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

}  // namespace
}  // namespace pawpy

using namespace pawpy;

extern "C" {

void *pawpy_gpu_server_create(long long hbm_budget_bytes, int slots) {
  PAWPY_API_BEGIN
  PAWPY_REQUIRE(hbm_budget_bytes > 0 && slots >= 1 && slots <= 64, "pawpy_gpu_server_create: bad budget or slots");
  auto *s = new Server();
  s->budget = hbm_budget_bytes;
  s->slots = slots;
  for (int i = 0; i < slots; i++) s->workers.emplace_back(worker, s);
  return s;
  PAWPY_API_END(nullptr)
}

int pawpy_gpu_server_add_basis(void *server, pswf_t *basis, const int *labels, const double *coords,
                               int num_sites, int keep_real_space) {
  PAWPY_API_BEGIN
  auto *s = static_cast<Server *>(server);
  PAWPY_REQUIRE(s && basis && labels && coords && num_sites > 0, "pawpy_gpu_server_add_basis: bad argument");
  if (pawpy_gpu_prepare_basis(basis, keep_real_space) < 0)
    throw Error(pawpy_gpu_last_error(), pawpy_gpu_error_string());
  Basis b;
  b.wf = basis;
  b.labels.assign(labels, labels + num_sites);
  b.coords.assign(coords, coords + 3 * num_sites);
  std::lock_guard<std::mutex> lk(s->mu);
  s->bases.push_back(std::move(b));
  return (int)s->bases.size() - 1;
  PAWPY_API_END(-1)
}

long long pawpy_gpu_server_submit(void *server, const pawpy_gpu_request_t *request) {
  PAWPY_API_BEGIN
  auto *s = static_cast<Server *>(server);
  PAWPY_REQUIRE(s && request && request->wf && request->pps && request->out && request->fftg && request->labels &&
                    request->coords && request->num_sites > 0,
                "pawpy_gpu_server_submit: bad request");
  auto q = std::make_unique<Request>();
  q->r = *request;
  for (int a = 0; a < 3; a++) q->fftg[a] = request->fftg[a];
  q->r.fftg = nullptr;
  q->labels.assign(request->labels, request->labels + request->num_sites);
  q->coords.assign(request->coords, request->coords + 3 * request->num_sites);
  const int *src[6] = {request->M_R, request->M_S, request->N_R, request->N_S, request->N_RS_R, request->N_RS_S};
  const int len[6] = {request->num_M, request->num_M, request->num_N_R, request->num_N_S, request->num_N_RS,
                      request->num_N_RS};
  for (int i = 0; i < 6; i++) {
    PAWPY_REQUIRE(len[i] == 0 || src[i], "pawpy_gpu_server_submit: NULL site list with a nonzero length");
    if (len[i] > 0) q->lists[i].assign(src[i], src[i] + len[i]);
  }
  std::lock_guard<std::mutex> lk(s->mu);
  PAWPY_REQUIRE(request->basis >= 0 && request->basis < (int)s->bases.size(), "pawpy_gpu_server_submit: no such basis");
  PAWPY_REQUIRE(!s->stop, "pawpy_gpu_server_submit: server stopping");
  q->est = estimate_bytes(s->bases[request->basis].wf, request->wf, request->num_sites);
  PAWPY_REQUIRE(q->est <= s->budget, "pawpy_gpu_server_submit: request larger than the memory budget");
  q->id = s->next_id++;
  q->t_submit = Clock::now();
  Request *raw = q.get();
  s->reqs[q->id] = std::move(q);
  s->queue.push_back(raw);
  s->cv_work.notify_all();
  return raw->id;
  PAWPY_API_END(-1)
}

int pawpy_gpu_server_wait(void *server, long long id, double *times_ms, long long *est_bytes, char *msg,
                          int msg_len) {
  PAWPY_API_BEGIN
  auto *s = static_cast<Server *>(server);
  PAWPY_REQUIRE(s, "pawpy_gpu_server_wait: NULL server");
  std::unique_ptr<Request> q;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    PAWPY_REQUIRE(it != s->reqs.end(), "pawpy_gpu_server_wait: unknown request id");
    Request *r = it->second.get();
    s->cv_done.wait(lk, [&] { return r->done; });
    q = std::move(it->second);
    s->reqs.erase(it);
  }
  if (times_ms) {
    times_ms[0] = ms_between(q->t_submit, q->t_start);
    times_ms[1] = ms_between(q->t_start, q->t_end);
    times_ms[2] = ms_between(q->t_submit, q->t_end);
    for (int i = 0; i < 4; i++) times_ms[3 + i] = q->phase_ms[i];
  }
  if (est_bytes) *est_bytes = q->est;
  if (msg && msg_len > 0) {
    std::snprintf(msg, (size_t)msg_len, "%s", q->msg.c_str());
  }
  return q->status;
  PAWPY_API_END(pawpy_gpu_last_error())
}

void pawpy_gpu_server_counts(void *server, long long *done, int *running, int *queued, long long *peak_bytes) {
  auto *s = static_cast<Server *>(server);
  if (!s) return;
  std::lock_guard<std::mutex> lk(s->mu);
  if (done) *done = s->done;
  if (running) *running = s->running;
  if (queued) *queued = (int)s->queue.size();
  if (peak_bytes) *peak_bytes = s->peak;
}

void pawpy_gpu_server_destroy(void *server) {
  auto *s = static_cast<Server *>(server);
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  for (auto &t : s->workers) t.join();
  delete s;
}

}  // extern "C"
