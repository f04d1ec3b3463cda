// Serving loop (femtc_server_* in femtc_gpu.h): continuous batching of
// matrix-free solves and operator applications.  A fixed pool of host
// workers, each with its own CUDA stream, takes requests from one queue as
// soon as a worker is free and the request fits in the HBM budget next to
// the requests already running; running requests overlap on the device.  The next request is the oldest
// (FIFO) or, by default, the one with the least estimated work less the
// time it has waited (shortest first with aging: no request waits longer
// than the estimate of the work admitted ahead of it).  Timestamps (submit,
// admit, done) are taken on one steady clock so callers get queueing and
// service latency.
#include "femtc_gpu.h"

#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

namespace femtc
{
int aux_fail(int code, const char* msg);
int solve_on_stream(const femtc_solve_request* rq, femtc_solve_result* res, cudaStream_t st);
size_t solve_bytes(int degree, int nquad, size_t ncells);
} // namespace femtc

using namespace femtc;

namespace
{
size_t storage_bytes(int dtype)
{
  return (dtype == FEMTC_F64 || dtype == FEMTC_F64E) ? 8 : 4;
}

size_t apply_geo_values(const femtc_apply_request& rq)
{
  const size_t q = (size_t)rq.nquad;
  return (rq.op == FEMTC_OP_MASS ? 1 : 6) * q * q * q;
}

// Device bytes of an operator application: its copies of u, the geometry
// and y (each allocation rounded up to 256 bytes).
size_t apply_bytes(const femtc_apply_request& rq)
{
  const size_t n = (size_t)rq.degree + 1;
  const size_t es = storage_bytes(rq.dtype);
  return rq.ncells * es * (2 * n * n * n + apply_geo_values(rq)) + 3 * 256;
}

// One operator application on `st`: device copies in, the operator, y back
// to the host; waits for the stream.
int apply_on_stream(const femtc_apply_request& rq, const void* tables, femtc_solve_result* res,
                    cudaStream_t st)
{
  const auto t0 = std::chrono::steady_clock::now();
  const size_t n = (size_t)rq.degree + 1, es = storage_bytes(rq.dtype);
  const size_t bu = rq.ncells * n * n * n * es, bg = rq.ncells * apply_geo_values(rq) * es;
  void *du = nullptr, *dg = nullptr, *dy = nullptr;
  int rc = FEMTC_OK;
  if (cudaMallocAsync(&du, bu, st) != cudaSuccess || cudaMallocAsync(&dg, bg, st) != cudaSuccess ||
      cudaMallocAsync(&dy, bu, st) != cudaSuccess)
    rc = aux_fail(FEMTC_ERR_NOMEM, "server: operator application: device allocation failed");
  if (rc == FEMTC_OK && (cudaMemcpyAsync(du, rq.u, bu, cudaMemcpyHostToDevice, st) != cudaSuccess ||
                         cudaMemcpyAsync(dg, rq.geo, bg, cudaMemcpyHostToDevice, st) != cudaSuccess))
    rc = aux_fail(FEMTC_ERR_CUDA, "server: operator application: copy in failed");
  if (rc == FEMTC_OK)
    rc = rq.op == FEMTC_OP_MASS
             ? femtc_mass_apply(rq.dtype, rq.semantics, rq.degree, rq.nquad, tables, du, dy, dg,
                                rq.ncells, st)
             : femtc_stiffness_apply(rq.dtype, rq.semantics, rq.degree, rq.nquad, tables, du, dy,
                                     dg, rq.ncells, st);
  if (rc == FEMTC_OK && cudaMemcpyAsync(rq.y, dy, bu, cudaMemcpyDeviceToHost, st) != cudaSuccess)
    rc = aux_fail(FEMTC_ERR_CUDA, "server: operator application: copy out failed");
  for (void* p : {du, dg, dy})
    if (p)
      cudaFreeAsync(p, st);
  const cudaError_t e = cudaStreamSynchronize(st);
  if (rc == FEMTC_OK && e != cudaSuccess)
    rc = aux_fail(FEMTC_ERR_CUDA, cudaGetErrorString(e));
  res->status = rc;
  res->ms_total =
      std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return rc;
}
} // namespace

struct femtc_server
{
  using clk = std::chrono::steady_clock;
  struct Job
  {
    long long ticket;
    femtc_solve_request rq;
    size_t bytes;
    double t_submit;
    double est_ms; // estimated work, in the units of the aging clock
    bool apply = false;          // an operator application (ap) instead of a solve
    femtc_apply_request ap{};
    std::vector<unsigned char> tab; // the application's tables, copied at submit
  };
  // Estimated work of a solve: DOFs times the operator's work per DOF
  // (sum factorisation: about N flops per DOF per contraction), scaled to
  // milliseconds of a solve sharing the GPU with others.
  static double estimate_ms(const femtc_solve_request& rq)
  {
    const double n = rq.degree + 1;
    return 1e-5 * (double)rq.ncells * n * n * n * n;
  }
  int policy = FEMTC_SERVE_SHORTEST_FIRST;
  size_t budget = 0;
  int device = 0;
  clk::time_point t0 = clk::now();
  std::mutex m;
  std::condition_variable cv_work, cv_done;
  std::deque<Job> queue;
  std::map<long long, femtc_solve_result> results;
  size_t in_use = 0, peak = 0;
  long long next_ticket = 1, submitted = 0, completed = 0, rejected = 0;
  int active = 0, max_conc = 0;
  bool stop = false;
  std::vector<std::thread> workers;

  double now_ms() const
  {
    return std::chrono::duration<double, std::milli>(clk::now() - t0).count();
  }

  // Queue index of the request to admit now, or -1 (caller holds m).  The
  // chosen request waits for memory rather than being passed by smaller
  // ones, so a large request is not starved.
  long pick() const
  {
    if (queue.empty())
      return -1;
    size_t best = 0;
    if (policy == FEMTC_SERVE_SHORTEST_FIRST)
    {
      const double t = now_ms();
      double key = 1e300;
      for (size_t i = 0; i < queue.size(); ++i)
      {
        const double k = queue[i].est_ms - (t - queue[i].t_submit);
        if (k < key)
        {
          key = k;
          best = i;
        }
      }
    }
    return in_use + queue[best].bytes <= budget ? (long)best : -1;
  }

  void worker()
  {
    cudaSetDevice(device);
    cudaStream_t st = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess)
      st = nullptr; // no device: solves fail with a CUDA status below
    for (;;)
    {
      Job job;
      {
        std::unique_lock<std::mutex> lk(m);
        long idx = -1;
        cv_work.wait(lk, [&] { return stop || (idx = pick()) >= 0; });
        if (stop)
          break;
        job = std::move(queue[(size_t)idx]);
        queue.erase(queue.begin() + idx);
        in_use += job.bytes;
        peak = std::max(peak, in_use);
        ++active;
        max_conc = std::max(max_conc, active);
      }
      femtc_solve_result res{};
      const double t_admit = now_ms();
      if (!st)
        res.status = aux_fail(FEMTC_ERR_CUDA, "server: no CUDA stream on this worker");
      else if (job.apply)
        apply_on_stream(job.ap, job.tab.data(), &res, st);
      else
        solve_on_stream(&job.rq, &res, st);
      {
        std::lock_guard<std::mutex> lk(m);
        res.t_submit_ms = job.t_submit;
        res.t_admit_ms = t_admit;
        res.t_done_ms = now_ms();
        results[job.ticket] = res;
        in_use -= job.bytes;
        --active;
        ++completed;
      }
      cv_done.notify_all();
      cv_work.notify_all();
    }
    if (st)
      cudaStreamDestroy(st);
  }
};

extern "C" {

int femtc_server_create(size_t hbm_budget_bytes, int max_active, femtc_server** out)
{
  if (!out || max_active < 1 || hbm_budget_bytes == 0)
    return aux_fail(FEMTC_ERR_INVALID, "server: need a budget, max_active >= 1 and an output");
  auto* s = new femtc_server();
  s->budget = hbm_budget_bytes;
  cudaGetDevice(&s->device);
  for (int i = 0; i < max_active; ++i)
    s->workers.emplace_back([s] { s->worker(); });
  *out = s;
  return FEMTC_OK;
}

int femtc_server_submit(femtc_server* s, const femtc_solve_request* rq, long long* ticket)
{
  if (!s || !rq || !ticket)
    return aux_fail(FEMTC_ERR_INVALID, "server: null argument");
  if (rq->degree < 1 || rq->degree > 7 || rq->nquad < rq->degree + 1 ||
      rq->nquad > rq->degree + 3 || rq->ncells == 0 || !rq->J || !rq->b || !rq->x)
    return aux_fail(FEMTC_ERR_INVALID, "server: malformed request");
  const size_t bytes = solve_bytes(rq->degree, rq->nquad, rq->ncells);
  std::lock_guard<std::mutex> lk(s->m);
  if (bytes > s->budget)
  {
    ++s->rejected;
    return aux_fail(FEMTC_ERR_NOMEM, "server: request exceeds the HBM budget");
  }
  *ticket = s->next_ticket++;
  s->queue.push_back(
      femtc_server::Job{*ticket, *rq, bytes, s->now_ms(), femtc_server::estimate_ms(*rq)});
  ++s->submitted;
  s->cv_work.notify_one();
  return FEMTC_OK;
}

int femtc_server_submit_apply(femtc_server* s, const femtc_apply_request* rq, long long* ticket)
{
  if (!s || !rq || !ticket)
    return aux_fail(FEMTC_ERR_INVALID, "server: null argument");
  if ((rq->op != FEMTC_OP_MASS && rq->op != FEMTC_OP_STIFFNESS) || rq->ncells == 0 ||
      !rq->tables || !rq->u || !rq->geo || !rq->y)
    return aux_fail(FEMTC_ERR_INVALID, "server: malformed operator application");
  if (femtc_supported(rq->op, rq->dtype, rq->semantics, rq->degree, rq->nquad) != 1)
    return aux_fail(FEMTC_ERR_UNSUPPORTED, "server: operator application: variant not built");
  {
    const size_t n = (size_t)rq->degree + 1;
    const size_t per_cell = storage_bytes(rq->dtype) * (2 * n * n * n + apply_geo_values(*rq));
    if (rq->ncells > (SIZE_MAX - 3 * 256) / per_cell)
      return aux_fail(FEMTC_ERR_INVALID, "server: operator application: too many cells");
  }
  const size_t bytes = apply_bytes(*rq);
  // mass reads Phi only (Q x N values), stiffness Phi then Gamma
  const size_t ntab = (rq->op == FEMTC_OP_MASS ? 1 : 2) * (size_t)(rq->degree + 1) *
                      (size_t)rq->nquad * storage_bytes(rq->dtype);
  femtc_server::Job job{};
  job.rq = femtc_solve_request{};
  job.bytes = bytes;
  job.apply = true;
  job.ap = *rq;
  job.tab.resize(ntab);
  std::memcpy(job.tab.data(), rq->tables, ntab);
  // about one operator application of a solve's several hundred
  femtc_solve_request like{};
  like.degree = rq->degree;
  like.ncells = rq->ncells;
  job.est_ms = femtc_server::estimate_ms(like) / 400.0;
  std::lock_guard<std::mutex> lk(s->m);
  if (bytes > s->budget)
  {
    ++s->rejected;
    return aux_fail(FEMTC_ERR_NOMEM, "server: request exceeds the HBM budget");
  }
  *ticket = s->next_ticket++;
  job.ticket = *ticket;
  job.t_submit = s->now_ms();
  s->queue.push_back(std::move(job));
  ++s->submitted;
  s->cv_work.notify_one();
  return FEMTC_OK;
}

int femtc_server_wait(femtc_server* s, long long ticket, double timeout_s,
                      femtc_solve_result* res)
{
  if (!s || !res)
    return aux_fail(FEMTC_ERR_INVALID, "server: null argument");
  std::unique_lock<std::mutex> lk(s->m);
  const bool ok = s->cv_done.wait_for(
      lk, std::chrono::duration<double>(timeout_s > 0 ? timeout_s : 0.0),
      [&] { return s->results.count(ticket) > 0; });
  if (!ok)
    return aux_fail(FEMTC_ERR_TIMEOUT, "server: result not ready");
  *res = s->results[ticket];
  s->results.erase(ticket);
  return res->status;
}

int femtc_server_set_policy(femtc_server* s, int policy)
{
  if (!s || (policy != FEMTC_SERVE_FIFO && policy != FEMTC_SERVE_SHORTEST_FIRST))
    return aux_fail(FEMTC_ERR_INVALID, "server: policy is FEMTC_SERVE_FIFO or "
                                       "FEMTC_SERVE_SHORTEST_FIRST");
  {
    std::lock_guard<std::mutex> lk(s->m);
    s->policy = policy;
  }
  s->cv_work.notify_all();
  return FEMTC_OK;
}

int femtc_server_get_stats(femtc_server* s, femtc_server_stats* st)
{
  if (!s || !st)
    return aux_fail(FEMTC_ERR_INVALID, "server: null argument");
  std::lock_guard<std::mutex> lk(s->m);
  st->submitted = s->submitted;
  st->completed = s->completed;
  st->rejected = s->rejected;
  st->queued = (long long)s->queue.size();
  st->active = s->active;
  st->in_use_bytes = s->in_use;
  st->peak_in_use_bytes = s->peak;
  st->max_concurrent = s->max_conc;
  return FEMTC_OK;
}

void femtc_server_destroy(femtc_server* s)
{
  if (!s)
    return;
  {
    std::lock_guard<std::mutex> lk(s->m);
    s->stop = true;
    s->queue.clear();
  }
  s->cv_work.notify_all();
  for (auto& t : s->workers)
    t.join();
  delete s;
}

} // extern "C"
