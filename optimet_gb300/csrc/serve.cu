// Serving and batching runtime: a fixed set of slots (device context + host
// thread + stream) on one GPU that take wavelength-solve requests in arrival
// order, admit them against a device-memory budget and run them side by side.
// No counterpart in the reference (Simulation::scan_wavelengths,
// Simulation.cpp:604-685, runs one wavelength-solve after another).
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <vector>

#include "om_internal.h"

namespace {

using clock_type = std::chrono::steady_clock;

double ms_between(clock_type::time_point a, clock_type::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Job {
  unsigned long long ticket = 0;
  om_request rq{};
  std::vector<om_sphere> spheres;
  size_t bytes = 0;        // admission estimate of the single-request path
  size_t batch_bytes = 0;  // ... and of the batched path (0: not batchable)
  clock_type::time_point submitted;
};

struct Slot {
  int index = 0;
  om_context *ctx = nullptr;
  om_problem *pr = nullptr;       // resident problem (kept for the next request of its key)
  unsigned long long key = 0;     // cluster key of the resident problem
  int n_spheres = 0, nmax = 0;
  size_t resident = 0;            // bytes reserved for the resident problem
  bool drop = false;              // release the resident problem at the next chance
  std::thread th;
  cudaEvent_t mark_prev = nullptr, mark_cur = nullptr;
};

// Device bytes of one request: the matrix (one harmonic at a time: the FF
// matrix is released before the SH assembly), the factor copy of the LU
// solves, the Krylov bases and the split-K partial sums, plus a fixed margin
// for per-sphere state and tables.
size_t estimate_bytes(const om_request &rq, int nmax) {
  const size_t P = (size_t)nmax * (nmax + 2);
  const size_t n = 2 * P * (size_t)rq.n_spheres;
  const size_t elem = rq.precision == OM_C64 ? 8 : 16;
  size_t b = n * n * elem;
  const om_solve_options &o = rq.opts;
  if(o.method == OM_SOLVE_LU)
    b += n * n * 16;
  if(o.method == OM_SOLVE_LU_MIXED)
    b += n * n * 8;
  if(o.method == OM_SOLVE_FGMRES_MIXED && rq.precision == OM_C64)
    b += n * n * 4;  // the inner GMRES's bf16 copy of the matrix
  const size_t m = (size_t)std::max(o.max_iter, 1), mi = (size_t)std::max(o.inner_iter, 1);
  b += (2 * (m + 2) + (mi + 2) + 16) * n * 16;
  b += 2 * ((n + 1023) / 1024) * n * 16;
  b += (size_t)256 << 20;
  return b;
}

}  // namespace

struct om_server {
  int device = 0;
  size_t budget = 0;
  std::vector<Slot> slots;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Job> queue;
  std::map<unsigned long long, om_result> done;
  std::set<unsigned long long> pending;   // submitted, not finished
  size_t reserved = 0;            // running + resident bytes
  unsigned long long next_ticket = 1;
  long outstanding = 0;
  long launches = 0;
  bool stop = false;
  bool has_mark = false;
  int batch_max = 0;        // > 1: slots take runs of batchable requests
  size_t batch_arena = 0;   // om_batch_solve arena per run (0: its default)
  size_t batch_limit = 0;   // batch only requests with a footprint up to this (0: any)

  bool batchable(const Job &j) const {
    return batch_max > 1 && j.batch_bytes && (!batch_limit || j.batch_bytes <= batch_limit);
  }
  std::string err;

  void run_slot(Slot &s);
  int serve(Slot &s, Job &job, om_result &res);
  void serve_batch(Slot &s, std::vector<Job> &jobs);
};

namespace {

void drop_resident(om_server *srv, Slot &s) {
  if(s.pr) {
    om_problem_destroy(s.pr);
    s.pr = nullptr;
  }
  s.key = 0;
  std::lock_guard<std::mutex> lk(srv->mu);
  srv->reserved -= s.resident;
  s.resident = 0;
  s.drop = false;
  srv->cv_work.notify_all();
}

}  // namespace

// One request on one slot: the call sequence of om_wavelength_solve_sh, with
// the problem kept resident for the next request of the same cluster.
int om_server::serve(Slot &s, Job &job, om_result &res) {
  const om_request &rq = job.rq;
  om_context *ctx = s.ctx;
  long kernels = 0;
  auto step = [&](int rc) {
    kernels += ctx->last_launches;
    return rc;
  };
  int rc = OM_OK;
  const bool reuse = s.pr && rq.cluster_key != 0 && rq.cluster_key == s.key &&
                     rq.n_spheres == s.n_spheres && job.spheres[0].nmax == s.nmax;
  if(reuse) {
    rc = step(om_problem_set_wave(s.pr, &rq.wave));
  } else {
    if(s.pr) {
      om_problem_destroy(s.pr);
      s.pr = nullptr;
    }
    rc = step(om_problem_create(ctx, job.spheres.data(), rq.n_spheres, &rq.background, &rq.wave,
                                &s.pr));
    s.key = rc ? 0 : rq.cluster_key;
    s.n_spheres = rq.n_spheres;
    s.nmax = job.spheres[0].nmax;
  }
  int conv = OM_OK;
  if(!rc) rc = step(om_source_vector(s.pr, nullptr));
  if(!rc) rc = step(om_assemble(s.pr, OM_FF, rq.precision));
  if(!rc) {
    int r = step(om_solve(s.pr, &rq.opts, &res.ff));
    if(r == OM_ERR_NOT_CONVERGED)
      conv = r;
    else
      rc = r;
  }
  if(!rc) rc = step(om_cross_sections(s.pr, res.xsec));
  if(!rc && rq.wave.sh) {
    om::release_matrix(s.pr, OM_FF);
    rc = step(om_assemble(s.pr, OM_SH, rq.precision));
    if(!rc) {
      int r = step(om_solve_sh(s.pr, &rq.opts, &res.sh));
      if(r == OM_ERR_NOT_CONVERGED)
        conv = r;
      else
        rc = r;
    }
    if(!rc) rc = step(om_sh_cross_sections(s.pr, res.xsec_sh));
  }
  if(rc) {
    std::lock_guard<std::mutex> lk(mu);
    err = "slot " + std::to_string(s.index) + ": " + ctx->err;
  }
  {
    std::lock_guard<std::mutex> lk(mu);
    launches += kernels;
  }
  return rc ? rc : conv;
}

// A run of requests on one slot through the batching form (om_batch_solve):
// size classes, one assembly launch and graph-captured lockstep solves per
// batch.
void om_server::serve_batch(Slot &s, std::vector<Job> &jobs) {
  om_context *ctx = s.ctx;
  std::vector<om_request> rq(jobs.size());
  for(size_t i = 0; i < jobs.size(); ++i) {
    rq[i] = jobs[i].rq;
    rq[i].spheres = jobs[i].spheres.data();
  }
  std::vector<om_result> res(jobs.size());
  const auto t0 = clock_type::now();
  size_t arena = batch_arena;
  if(!arena)
    for(const Job &j : jobs)
      arena += j.batch_bytes;
  int rc = om_batch_solve(ctx, rq.data(), (int)rq.size(), arena, res.data());
  const auto t1 = clock_type::now();
  std::lock_guard<std::mutex> lk(mu);
  if(rc)
    err = "slot " + std::to_string(s.index) + ": " + ctx->err;
  launches += ctx->last_launches;
  for(size_t i = 0; i < jobs.size(); ++i) {
    om_result r = res[i];
    if(rc && (r.status == OM_OK || r.status == OM_ERR_NOT_CONVERGED))
      r.status = rc;
    r.slot = s.index;
    r.device_bytes = jobs[i].batch_bytes;
    r.queue_ms = ms_between(jobs[i].submitted, t0);
    r.service_ms = ms_between(t0, t1);
    r.latency_ms = ms_between(jobs[i].submitted, t1);
    reserved -= jobs[i].batch_bytes;
    done[jobs[i].ticket] = r;
    pending.erase(jobs[i].ticket);
    --outstanding;
  }
  cv_done.notify_all();
  cv_work.notify_all();
}

void om_server::run_slot(Slot &s) {
  cudaSetDevice(device);
  for(;;) {
    Job job;
    {
      std::unique_lock<std::mutex> lk(mu);
      for(;;) {
        if(stop && queue.empty())
          break;
        if(s.drop && s.resident) {
          lk.unlock();
          drop_resident(this, s);
          lk.lock();
          continue;
        }
        if(!queue.empty()) {
          Job &head = queue.front();
          // the slot's own resident bytes are reused (same key) or released
          const size_t others = reserved - s.resident;
          // a batchable request anywhere in the queue that fits, or the head
          bool batch_ready = false;
          if(batch_max > 1)
            for(const Job &j : queue)
              if(batchable(j) && others + j.batch_bytes <= budget) {
                batch_ready = true;
                break;
              }
          if(batch_ready || (!batchable(head) && others + head.bytes <= budget))
            break;
          if(batchable(head) && others + head.bytes <= budget)
            break;
          if(head.bytes > budget) {
            // can never run: fail it here
            Job j = std::move(queue.front());
            queue.pop_front();
            om_result r{};
            r.status = OM_ERR_BUDGET;
            r.slot = s.index;
            r.device_bytes = j.bytes;
            r.latency_ms = ms_between(j.submitted, clock_type::now());
            err = "request needs " + std::to_string(j.bytes) + " bytes, budget " +
                  std::to_string(budget);
            done[j.ticket] = r;
            pending.erase(j.ticket);
            --outstanding;
            cv_done.notify_all();
            continue;
          }
          // memory pressure: every idle slot releases what it keeps resident
          bool flagged = false;
          for(auto &o : slots)
            if(&o != &s && o.resident && !o.drop) {
              o.drop = true;
              flagged = true;
            }
          if(flagged)
            cv_work.notify_all();
        }
        cv_work.wait(lk);
      }
      if(stop && queue.empty())
        break;
      const bool head_single =
          !batchable(queue.front()) && reserved - s.resident + queue.front().bytes <= budget;
      std::vector<Job> run;
      if(batch_max > 1 && !head_single) {
        // the batchable requests of the queue, in arrival order, up to
        // batch_max and within the budget (none: a batchable head that fits
        // only on the single-request path takes that path)
        size_t take = reserved - s.resident;
        for(auto it = queue.begin(); it != queue.end() && (int)run.size() < batch_max;) {
          if(batchable(*it) && take + it->batch_bytes <= budget) {
            take += it->batch_bytes;
            reserved += it->batch_bytes;
            run.push_back(std::move(*it));
            it = queue.erase(it);
          } else {
            ++it;
          }
        }
      }
      if(!run.empty()) {
        // the slot's resident problem goes first
        lk.unlock();
        if(s.resident || s.pr)
          drop_resident(this, s);
        serve_batch(s, run);
        continue;
      }
      job = std::move(queue.front());
      queue.pop_front();
      reserved -= s.resident;
      s.resident = 0;
      reserved += job.bytes;
    }
    om_result res{};
    res.slot = s.index;
    res.device_bytes = job.bytes;
    const auto t0 = clock_type::now();
    res.queue_ms = ms_between(job.submitted, t0);
    res.status = serve(s, job, res);
    if(res.status && res.status != OM_ERR_NOT_CONVERGED && s.pr) {
      om_problem_destroy(s.pr);
      s.pr = nullptr;
      s.key = 0;
    }
    const auto t1 = clock_type::now();
    res.service_ms = ms_between(t0, t1);
    res.latency_ms = ms_between(job.submitted, t1);
    {
      std::lock_guard<std::mutex> lk(mu);
      // what stays resident is at most the request's own estimate
      if(s.pr) {
        s.resident = job.bytes;
      } else {
        reserved -= job.bytes;
        s.resident = 0;
      }
      done[job.ticket] = res;
      pending.erase(job.ticket);
      --outstanding;
      cv_done.notify_all();
      cv_work.notify_all();
    }
  }
  if(s.pr) {
    om_problem_destroy(s.pr);
    s.pr = nullptr;
  }
  cudaStreamSynchronize(s.ctx->stream);
}

extern "C" {

int om_server_create(int device, size_t hbm_budget, int slots, om_server **out) {
  if(!out || slots < 1 || slots > 64)
    return OM_ERR_INVALID;
  *out = nullptr;
  om_server *srv = new(std::nothrow) om_server();
  if(!srv)
    return OM_ERR_INVALID;
  srv->device = device;
  if(hbm_budget == 0) {
    size_t free_b = 0, total_b = 0;
    cudaSetDevice(device);
    if(cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
      cudaGetLastError();
      delete srv;
      return OM_ERR_CUDA;
    }
    hbm_budget = free_b - free_b / 16;
  }
  srv->budget = hbm_budget;
  srv->slots.resize(slots);
  for(int i = 0; i < slots; ++i) {
    Slot &s = srv->slots[i];
    s.index = i;
    int rc = om_context_create(device, 0, &s.ctx);
    if(rc == OM_OK && (cudaEventCreate(&s.mark_prev) != cudaSuccess ||
                       cudaEventCreate(&s.mark_cur) != cudaSuccess))
      rc = OM_ERR_CUDA;
    if(rc) {
      for(int j = 0; j <= i; ++j) {
        if(srv->slots[j].ctx)
          om_context_destroy(srv->slots[j].ctx);
        if(srv->slots[j].mark_prev)
          cudaEventDestroy(srv->slots[j].mark_prev);
        if(srv->slots[j].mark_cur)
          cudaEventDestroy(srv->slots[j].mark_cur);
      }
      delete srv;
      return rc;
    }
  }
  if(slots > 1) {
    // side by side, the matvec kernels leave room for another slot's assembly
    // (plain matvec: the TMA one's stage buffers would fill the SM)
    const om_tuning t{4, 2, 50, 50, -1, 0, -1, -1, -1, -1, -1};
    for(auto &s : srv->slots)
      om_context_tune(s.ctx, &t);
  }
  for(auto &s : srv->slots)
    s.th = std::thread([srv, &s] { srv->run_slot(s); });
  *out = srv;
  return OM_OK;
}

int om_server_submit(om_server *srv, const om_request *rq, unsigned long long *ticket) {
  if(!srv || !rq || !rq->spheres || rq->n_spheres < 1 ||
     (rq->precision != OM_C128 && rq->precision != OM_C64))
    return OM_ERR_INVALID;
  const int nmax = rq->spheres[0].nmax;
  if(nmax < 1 || nmax > om::kMaxNmax)
    return OM_ERR_INVALID;
  Job job;
  job.rq = *rq;
  job.spheres.assign(rq->spheres, rq->spheres + rq->n_spheres);
  job.rq.spheres = nullptr;
  job.bytes = estimate_bytes(*rq, nmax);
  job.batch_bytes = om::batch_request_bytes(*rq);
  job.submitted = clock_type::now();
  std::lock_guard<std::mutex> lk(srv->mu);
  if(srv->stop)
    return OM_ERR_STATE;
  job.ticket = srv->next_ticket++;
  if(ticket)
    *ticket = job.ticket;
  srv->pending.insert(job.ticket);
  srv->queue.push_back(std::move(job));
  ++srv->outstanding;
  srv->cv_work.notify_all();
  return OM_OK;
}

int om_server_poll(om_server *srv, unsigned long long ticket, int wait, om_result *out) {
  if(!srv)
    return OM_ERR_INVALID;
  std::unique_lock<std::mutex> lk(srv->mu);
  for(;;) {
    auto it = srv->done.find(ticket);
    if(it != srv->done.end()) {
      if(out)
        *out = it->second;
      srv->done.erase(it);
      return OM_OK;
    }
    if(!srv->pending.count(ticket))
      return OM_ERR_INVALID;
    if(!wait)
      return OM_PENDING;
    srv->cv_done.wait(lk);
  }
}

int om_server_drain(om_server *srv) {
  if(!srv)
    return OM_ERR_INVALID;
  std::unique_lock<std::mutex> lk(srv->mu);
  srv->cv_done.wait(lk, [srv] { return srv->outstanding == 0; });
  return OM_OK;
}

int om_server_mark(om_server *srv, double *ms) {
  if(!srv)
    return OM_ERR_INVALID;
  cudaSetDevice(srv->device);
  for(auto &s : srv->slots)
    if(cudaEventRecord(s.mark_cur, s.ctx->stream) != cudaSuccess)
      return OM_ERR_CUDA;
  for(auto &s : srv->slots)
    if(cudaEventSynchronize(s.mark_cur) != cudaSuccess)
      return OM_ERR_CUDA;
  double t = 0.0;
  if(srv->has_mark) {
    // earliest previous event, latest current one (device timestamps)
    Slot *first = &srv->slots[0];
    for(auto &s : srv->slots) {
      float d = 0.f;
      cudaEventElapsedTime(&d, first->mark_prev, s.mark_prev);
      if(d < 0.f)
        first = &s;
    }
    for(auto &s : srv->slots) {
      float d = 0.f;
      cudaEventElapsedTime(&d, first->mark_prev, s.mark_cur);
      t = std::max(t, (double)d);
    }
  }
  for(auto &s : srv->slots)
    std::swap(s.mark_prev, s.mark_cur);
  srv->has_mark = true;
  if(ms)
    *ms = t;
  return OM_OK;
}

int om_server_batching(om_server *srv, int max_requests, size_t arena_bytes,
                       size_t max_request_bytes) {
  if(!srv || max_requests < 0)
    return OM_ERR_INVALID;
  std::lock_guard<std::mutex> lk(srv->mu);
  srv->batch_max = max_requests;
  srv->batch_arena = arena_bytes;
  srv->batch_limit = max_request_bytes;
  srv->cv_work.notify_all();
  return OM_OK;
}

int om_server_tune(om_server *srv, const om_tuning *t) {
  if(!srv || !t)
    return OM_ERR_INVALID;
  std::lock_guard<std::mutex> lk(srv->mu);
  if(srv->outstanding)
    return OM_ERR_STATE;
  for(auto &s : srv->slots) {
    int rc = om_context_tune(s.ctx, t);
    if(rc)
      return rc;
  }
  return OM_OK;
}

int om_server_autotune(om_server *srv, const om_request *rq, int count, double step,
                       om_tuning *chosen) {
  if(!srv || !rq || count < 1)
    return OM_ERR_INVALID;
  // the TMA matvec's 144 KB of stage buffers leave no room for another slot's
  // assembly on the SM, so the overlapping candidates use the plain kernel
  static const om_tuning cands[] = {{8, 8, -1, -1, -1, 1, -1, -1, -1, -1, -1}, {6, 3, 50, 50, -1, 0, -1, -1, -1, -1, -1},
                                    {4, 2, 50, 50, -1, 0, -1, -1, -1, -1, -1}, {4, 2, -1, -1, -1, 0, -1, -1, -1, -1, -1},
                                    {3, 2, 50, 50, -1, 0, -1, -1, -1, -1, -1}, {3, 2, -1, -1, -1, 0, -1, -1, -1, -1, -1},
                                    {4, 1, -1, -1, -1, 0, -1, -1, -1, -1, -1}, {5, 2, -1, -1, -1, 0, -1, -1, -1, -1, -1},
                                    {4, 3, -1, -1, -1, 0, -1, -1, -1, -1, -1}, {6, 2, -1, -1, -1, 0, -1, -1, -1, -1, -1}};
  const int nslots = (int)srv->slots.size();
  double best = 1e300;
  om_tuning pick = cands[0];
  double lambda = rq->wave.wavelength;
  for(const om_tuning &t : cands) {
    int rc = om_server_tune(srv, &t);
    if(rc)
      return rc;
    std::vector<unsigned long long> tk;
    auto run = [&](int k) -> int {
      tk.clear();
      for(int i = 0; i < k; ++i) {
        om_request r = *rq;
        r.wave.wavelength = lambda;
        lambda += step;
        unsigned long long id = 0;
        int e = om_server_submit(srv, &r, &id);
        if(e)
          return e;
        tk.push_back(id);
      }
      for(auto id : tk) {
        om_result res{};
        om_server_poll(srv, id, 1, &res);
        if(res.status && res.status != OM_ERR_NOT_CONVERGED)
          return res.status;
      }
      return OM_OK;
    };
    rc = run(nslots);
    if(rc)
      return rc;
    double ms = 0.0;
    om_server_mark(srv, nullptr);
    rc = run(count);
    if(rc)
      return rc;
    om_server_mark(srv, &ms);
    if(ms < best) {
      best = ms;
      pick = t;
    }
  }
  int rc = om_server_tune(srv, &pick);
  if(chosen)
    *chosen = pick;
  return rc;
}

long om_server_launches(om_server *srv) {
  if(!srv)
    return 0;
  std::lock_guard<std::mutex> lk(srv->mu);
  long n = srv->launches;
  srv->launches = 0;
  return n;
}

const char *om_server_last_error(om_server *srv) { return srv ? srv->err.c_str() : ""; }

void om_server_destroy(om_server *srv) {
  if(!srv)
    return;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->stop = true;
    srv->cv_work.notify_all();
  }
  for(auto &s : srv->slots)
    if(s.th.joinable())
      s.th.join();
  cudaSetDevice(srv->device);
  for(auto &s : srv->slots) {
    cudaEventDestroy(s.mark_prev);
    cudaEventDestroy(s.mark_cur);
    om_context_destroy(s.ctx);
  }
  delete srv;
}

}  // extern "C"
