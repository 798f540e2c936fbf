// serve.cpp -- batched and served solves of independent LPs on one GPU.
//
// A server owns `workers` host threads, each with its own non-blocking CUDA
// stream.  Requests (deep copies of the submitted LPs) wait in one FIFO
// queue; a worker admits the head request when its estimated device
// footprint fits in what is left of the memory budget (a request larger than
// the whole budget is admitted alone), uploads it, solves it on its stream
// and publishes the result.  The solve path takes device memory from a
// stream-ordered pool and never synchronises the device, so the LPs in
// flight overlap on the GPU: small LPs, whose kernels fill a fraction of the
// SMs, share the machine.  Every LP's arithmetic depends on its own data
// only, so a result is bitwise the same solved alone or in any mix.
//
// No counterpart in the reference, which solves one LP per call
// (src/cupdlpx.c:174-198); each request here runs that solve.
#include <string.h>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "cupdlpx.h"
#include "pdlp_gb300.h"
#include "runtime.h"
#include "solver.cuh"

namespace {

using Clock = std::chrono::steady_clock;

double since(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double>(b - a).count();
}

// Deep copy through the public constructor (CSR input), with start values.
lp_problem_t *copy_problem(const lp_problem_t *p) {
  matrix_desc_t d{};
  d.m = p->num_constraints;
  d.n = p->num_variables;
  d.fmt = matrix_csr;
  d.zero_tolerance = 0.0;
  d.data.csr.nnz = p->constraint_matrix_num_nonzeros;
  d.data.csr.row_ptr = p->constraint_matrix_row_pointers;
  d.data.csr.col_ind = p->constraint_matrix_col_indices;
  d.data.csr.vals = p->constraint_matrix_values;
  lp_problem_t *q =
      create_lp_problem(p->objective_vector, &d, p->constraint_lower_bound,
                        p->constraint_upper_bound, p->variable_lower_bound,
                        p->variable_upper_bound, &p->objective_constant);
  if (q && (p->primal_start || p->dual_start))
    set_start_values(q, p->primal_start, p->dual_start);
  return q;
}

// Host bytes of a problem's copy (CSR and vectors).
long long host_bytes(const lp_problem_t *p) {
  return 12LL * p->constraint_matrix_num_nonzeros + 4LL * (p->num_constraints + 1) +
         8LL * (3LL * p->num_variables + 2LL * p->num_constraints);
}

struct Request {
  long long id = 0;
  lp_problem_t *prob = nullptr;
  long long bytes = 0;
  long long host = 0;  // host bytes of the queued copy
  Clock::time_point submitted, admitted, finished;
  cupdlpx_result_t *result = nullptr;
  int worker = -1;
  double upload_s = 0.0, device_s = 0.0;  // host upload call; solve on the stream
  bool done = false;
  std::string error;
};

}  // namespace

struct pdlp_server {
  pdhg_parameters_t params{};
  pdlp_options_t opts{};
  long long budget = 0;
  int device = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<std::shared_ptr<Request>> queue;
  std::map<long long, std::shared_ptr<Request>> requests;
  long long next_id = 0, in_use = 0;
  // queue bound: requests whose copies would take the waiting requests past
  // queue_limit host bytes are refused (0: no bound)
  long long queue_limit = 0, queued_host = 0, rejected = 0;
  int in_flight = 0, max_in_flight = 0;
  long long completed = 0, failed = 0, iterations = 0;
  bool stopping = false;
  Clock::time_point first_admit{}, last_finish{};
  bool any_admitted = false;
  std::vector<std::thread> threads;

  void worker_main(int w) {
    cudaSetDevice(device);
    cudaStream_t st = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) st = nullptr;
    for (;;) {
      std::shared_ptr<Request> r;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_work.wait(lk, [&] {
          if (queue.empty()) return stopping;
          const long long need = queue.front()->bytes;
          return in_use + need <= budget || in_flight == 0;
        });
        if (queue.empty()) break;  // stopping and drained
        r = queue.front();
        queue.pop_front();
        queued_host -= r->host;
        in_use += r->bytes;
        ++in_flight;
        if (in_flight > max_in_flight) max_in_flight = in_flight;
        r->admitted = Clock::now();
        r->worker = w;
        if (!any_admitted) {
          first_admit = r->admitted;
          any_admitted = true;
        }
      }
      cupdlpx_result_t *res = nullptr;
      std::string err;
      if (!st) {
        err = "no CUDA stream for this worker";
      } else {
        try {
          const auto tu = Clock::now();
          std::unique_ptr<pdlp::DevProblem> P(pdlp::upload_problem(r->prob, st));
          r->upload_s = since(tu, Clock::now());
          pdlp_solve_info_t si;
          memset(&si, 0, sizeof(si));
          res = pdlp::solve_uploaded(*P, params, opts, st, &si);
          r->device_s = si.device_seconds;
          cudaStreamSynchronize(st);
        } catch (const std::exception &e) {
          err = e.what();
          cudaGetLastError();
        }
      }
      {
        std::lock_guard<std::mutex> lk(mu);
        r->result = res;
        r->error = err;
        r->finished = Clock::now();
        r->done = true;
        lp_problem_free(r->prob);
        r->prob = nullptr;
        in_use -= r->bytes;
        --in_flight;
        ++completed;
        if (!res) ++failed;
        else iterations += res->total_count;
        last_finish = r->finished;
      }
      cv_done.notify_all();
      cv_work.notify_all();
    }
    if (st) cudaStreamDestroy(st);
  }
};

extern "C" {

long long pdlp_estimate_device_bytes(int m, int n, long long nnz, int precision) {
  if (m < 0 || n < 0 || nnz < 0) return -1;
  const long long vm = m, vn = n;
  // resident problem: A and A^T in CSR, plans, objective and bounds
  long long b = 24 * nnz + 4 * (vm + vn + 2) + 40 * vn + 16 * vm + (nnz / 512 + 64) * 56;
  // FP64 solve: scaled values, iterates and work vectors, partial sums
  b += 16 * nnz + 8 * (24 * vn + 18 * vm) + (nnz / 512 + 64) * 160 + (1 << 20);
  if (precision != PDLP_PRECISION_FP64) {
    // FP32 values, refinement workspace and the FP64 evaluator
    b += 8 * nnz + 16 * nnz + 8 * (40 * vn + 30 * vm) + (1 << 20);
  }
  return b;
}

pdlp_server_t *pdlp_server_create(const pdhg_parameters_t *params, const pdlp_options_t *opts,
                                  int workers, long long mem_budget_bytes) {
  if (workers <= 0 || workers > 256) {
    pdlp::record_error("pdlp_server_create: workers must be in 1..256.");
    return nullptr;
  }
  auto *s = new pdlp_server();
  if (!pdlp::resolve_parameters(params, s->params)) {
    delete s;
    return nullptr;
  }
  s->params.verbose = false;
  if (opts) s->opts = *opts;
  if (cudaGetDevice(&s->device) != cudaSuccess) {
    pdlp::record_error("pdlp_server_create: no CUDA device.");
    cudaGetLastError();
    delete s;
    return nullptr;
  }
  if (mem_budget_bytes <= 0) {
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
      pdlp::record_error("pdlp_server_create: cudaMemGetInfo failed.");
      cudaGetLastError();
      delete s;
      return nullptr;
    }
    mem_budget_bytes = (long long)(0.8 * (double)fr);
  }
  s->budget = mem_budget_bytes;
  for (int w = 0; w < workers; ++w) s->threads.emplace_back(&pdlp_server::worker_main, s, w);
  return s;
}

long long pdlp_server_submit(pdlp_server_t *s, const lp_problem_t *prob) {
  if (!s || !prob) return -1;
  const long long hb = host_bytes(prob);
  const auto submitted = Clock::now();
  {
    // reserve the copy's bytes in the queue, or refuse the request
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->queue_limit > 0 && !s->queue.empty() && s->queued_host + hb > s->queue_limit) {
      ++s->rejected;
      pdlp::record_error("pdlp_server_submit: queue full (host-byte limit reached)");
      return -2;
    }
    s->queued_host += hb;
  }
  lp_problem_t *q = copy_problem(prob);
  if (!q) {
    std::lock_guard<std::mutex> lk(s->mu);
    s->queued_host -= hb;
    return -1;
  }
  auto r = std::make_shared<Request>();
  r->prob = q;
  r->host = hb;
  r->bytes = pdlp_estimate_device_bytes(q->num_constraints, q->num_variables,
                                        q->constraint_matrix_num_nonzeros, s->opts.precision);
  r->submitted = submitted;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stopping) {
      s->queued_host -= hb;
      lp_problem_free(q);
      return -1;
    }
    r->id = s->next_id++;
    s->requests[r->id] = r;
    s->queue.push_back(r);
  }
  s->cv_work.notify_one();
  return r->id;
}

cupdlpx_result_t *pdlp_server_wait(pdlp_server_t *s, long long id, pdlp_request_info_t *info) {
  if (!s) return nullptr;
  std::shared_ptr<Request> r;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->requests.find(id);
    if (it == s->requests.end()) {
      pdlp::record_error("pdlp_server_wait: unknown or already collected request.");
      return nullptr;
    }
    r = it->second;
    s->cv_done.wait(lk, [&] { return r->done; });
    s->requests.erase(it);
  }
  if (info) {
    info->queued_seconds = since(r->submitted, r->admitted);
    info->solve_seconds = since(r->admitted, r->finished);
    info->latency_seconds = since(r->submitted, r->finished);
    info->worker = r->worker;
    info->device_bytes = r->bytes;
    info->upload_seconds = r->upload_s;
    info->device_seconds = r->device_s;
  }
  if (!r->result) pdlp::record_error("pdlp_server_wait: solve failed: " + r->error);
  return r->result;
}

int pdlp_server_stats(pdlp_server_t *s, pdlp_server_stats_t *out) {
  if (!s || !out) return -1;
  std::lock_guard<std::mutex> lk(s->mu);
  out->completed = s->completed;
  out->failed = s->failed;
  out->queued = (long long)s->queue.size();
  out->in_flight = s->in_flight;
  out->max_in_flight = s->max_in_flight;
  out->iterations = s->iterations;
  out->device_bytes_in_use = s->in_use;
  out->busy_seconds = s->any_admitted ? since(s->first_admit, s->last_finish) : 0.0;
  out->rejected = s->rejected;
  out->queued_host_bytes = s->queued_host;
  return 0;
}

int pdlp_server_set_queue_limit(pdlp_server_t *s, long long max_queued_host_bytes) {
  if (!s || max_queued_host_bytes < 0) return -1;
  std::lock_guard<std::mutex> lk(s->mu);
  s->queue_limit = max_queued_host_bytes;
  return 0;
}

void pdlp_server_destroy(pdlp_server_t *s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stopping = true;
  }
  s->cv_work.notify_all();
  for (auto &t : s->threads) t.join();
  for (auto &kv : s->requests) {
    if (kv.second->result) cupdlpx_result_free(kv.second->result);
    if (kv.second->prob) lp_problem_free(kv.second->prob);
  }
  delete s;
}

int pdlp_batch_solve(const lp_problem_t *const *probs, int count,
                     const pdhg_parameters_t *params, const pdlp_options_t *opts, int workers,
                     long long mem_budget_bytes, cupdlpx_result_t **results,
                     pdlp_batch_info_t *info) {
  if (count < 0 || (count > 0 && (!probs || !results))) {
    pdlp::record_error("pdlp_batch_solve: invalid arguments.");
    return -1;
  }
  for (int i = 0; i < count; ++i) results[i] = nullptr;
  if (count == 0) {
    if (info) *info = pdlp_batch_info_t{};
    return 0;
  }
  pdlp_server_t *s = pdlp_server_create(params, opts, workers, mem_budget_bytes);
  if (!s) return -2;
  auto t0 = Clock::now();
  std::vector<long long> ids(count, -1);
  for (int i = 0; i < count; ++i) ids[i] = pdlp_server_submit(s, probs[i]);
  int failed = 0;
  for (int i = 0; i < count; ++i) {
    results[i] = ids[i] >= 0 ? pdlp_server_wait(s, ids[i], nullptr) : nullptr;
    if (!results[i]) ++failed;
  }
  double wall = since(t0, Clock::now());
  pdlp_server_stats_t st{};
  pdlp_server_stats(s, &st);
  pdlp_server_destroy(s);
  if (info) {
    info->lps = count;
    info->failed = failed;
    info->wall_seconds = wall;
    info->lps_per_second = wall > 0 ? (count - failed) / wall : 0.0;
    info->iterations = st.iterations;
    info->max_concurrent = st.max_in_flight;
  }
  return failed ? -3 : 0;
}

void pdlp_release_pooled_memory(void) { pdlp::release_pooled_memory(); }

}  // extern "C"
