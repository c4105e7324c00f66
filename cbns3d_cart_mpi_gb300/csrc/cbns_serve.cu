// cbns_serve.cu — continuous-batching request loop for independent solves.
//
// A server owns one worker thread.  Callers submit solve requests (parameters,
// grid, and either a host state or a seed for the device-side Taylor-Green
// initial condition); the worker
//   1. admits queued requests, first come first served among those that fit,
//      while their device footprint (cbns_footprint) fits the memory budget and
//      the active count is below max_active: each admitted request gets its own
//      handle, and its state is created on and stays resident on the device;
//   2. steps every admitted request together as one batch (one launch per
//      kernel over all their tiles, a batch step replayed as a CUDA graph) for
//      steps_per_round steps, each request stopping at its own t_end;
//   3. retires requests that finished (or met a non-physical state, or were
//      cancelled): reads their KE/enstrophy and, if asked, their final state,
//      frees their device memory, and admits the next ones — so requests that
//      arrive while others run join the batch at the next round.
// The batch is rebuilt only when membership changes.  A request's result is
// bitwise what stepping it alone gives: batching changes the launch grouping,
// never the arithmetic of a cell.
#include <cuda_runtime.h>

#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "cbns_internal.h"

namespace {

enum ReqState { RQ_QUEUED = 0, RQ_ACTIVE = 1, RQ_DONE = 2 };

struct Request {
  uint64_t id = 0;
  cbns_params params{};
  uint32_t IM = 0, JM = 0, KM = 0;
  std::vector<double> Q0;  // host state, or empty for the device initial condition
  std::string ckpt;        // checkpoint file read at admission, if not empty
  uint64_t seed = 0;
  double amp = 0.0;
  int nmodes = 0, kmax = 1;
  int keep_state = 0;
  std::vector<double> result;
  uint64_t footprint = 0;
  int state = RQ_QUEUED;
  int status = CBNS_OK;
  bool cancel = false;
  double t_submit = 0, t_admit = 0, t_done = 0;
  double t_final = 0, ke = 0, enstrophy = 0;
  uint32_t steps = 0;
  cbns_handle* h = nullptr;
  std::string error;
};

}  // namespace

struct cbns_server {
  cbns_server_opts opts{};
  int device = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request*> queue;
  std::map<uint64_t, std::unique_ptr<Request>> reqs;
  std::vector<Request*> active;  // worker thread only
  uint64_t next_id = 1;
  uint64_t budget = 0, used = 0;
  bool stop = false;
  std::thread worker;
  cbns_batch* batch = nullptr;  // worker thread only
  std::chrono::steady_clock::time_point t0;
  cbns_server_stats stats{};

  double now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
};

namespace {

void retire(cbns_server* sv, Request* r, int status, std::string err) {
  // Worker thread, without the lock: read results, free the solve.  A read that
  // fails retires the request with that read's status and error text instead.
  if (r->h) {
    if (status == CBNS_OK || status == CBNS_ERR_NONPHYSICAL) {
      double dt_last = 0.0;
      cbns_status st = cbns_get_time(r->h, &r->t_final, &dt_last);
      if (st == CBNS_OK && status == CBNS_OK) st = cbns_diagnostics(r->h, &r->ke, &r->enstrophy);
      if (st == CBNS_OK && status == CBNS_OK && r->keep_state) {
        try {
          r->result.resize((size_t)CBNS_NEQ * (r->IM + 2 * CBNS_NG) * (r->JM + 2 * CBNS_NG) *
                           (r->KM + 2 * CBNS_NG));
          st = cbns_download_Q(r->h, r->result.data());
        } catch (const std::bad_alloc&) {
          st = CBNS_ERR_OUT_OF_MEMORY;
          cbns::set_last_error("retire: no host memory for the final state");
        }
      }
      if (st != CBNS_OK) {
        status = st;
        err = cbns_last_error();
        std::vector<double>().swap(r->result);
      }
    }
    cbns_destroy(r->h);
    r->h = nullptr;
  }
  std::lock_guard<std::mutex> lk(sv->mu);
  sv->used -= r->footprint;
  r->status = status;
  r->error = err;
  r->state = RQ_DONE;
  r->t_done = sv->now();
  if (status == CBNS_OK) sv->stats.completed++;
  else sv->stats.failed++;
  sv->cv_done.notify_all();
}

void worker_loop(cbns_server* sv) {
  cudaSetDevice(sv->device);
  for (;;) {
    std::vector<Request*> admit;
    {
      std::unique_lock<std::mutex> lk(sv->mu);
      sv->cv_work.wait(lk, [&] { return sv->stop || !sv->queue.empty() || !sv->active.empty(); });
      if (sv->stop) break;
      // Admission by device footprint, first come first served among those that fit.
      for (auto it = sv->queue.begin(); it != sv->queue.end();) {
        Request* r = *it;
        const bool slot = sv->opts.max_active == 0 || sv->active.size() + admit.size() < sv->opts.max_active;
        if (r->cancel) {
          r->state = RQ_DONE;
          r->status = CBNS_ERR_CANCELLED;
          r->t_done = sv->now();
          sv->stats.failed++;
          it = sv->queue.erase(it);
          sv->cv_done.notify_all();
          continue;
        }
        if (slot && sv->used + r->footprint <= sv->budget) {
          sv->used += r->footprint;
          r->state = RQ_ACTIVE;
          r->t_admit = sv->now();
          admit.push_back(r);
          it = sv->queue.erase(it);
        } else {
          ++it;
        }
      }
    }
    bool changed = false;
    for (Request* r : admit) {
      cbns_status st = cbns_create(&r->params, r->IM, r->JM, r->KM, sv->opts.precision, &r->h);
      if (st == CBNS_OK) {
        if (!r->ckpt.empty())
          st = cbns_load_checkpoint(r->h, r->ckpt.c_str(), nullptr);
        else if (r->Q0.empty())
          st = cbns_init_tgv(r->h, r->seed, r->amp, r->nmodes, r->kmax, r->params.t_cur);
        else
          st = cbns_upload_Q(r->h, r->Q0.data(), r->params.t_cur);
        std::vector<double>().swap(r->Q0);
      }
      if (st != CBNS_OK) {
        retire(sv, r, st, cbns_last_error());
        continue;
      }
      sv->active.push_back(r);
      changed = true;
    }
    if (sv->active.empty()) continue;
    if (changed || !sv->batch) {
      if (sv->batch) cbns_batch_destroy(sv->batch);
      sv->batch = nullptr;
      std::vector<cbns_handle*> hs;
      for (Request* r : sv->active) hs.push_back(r->h);
      cbns_status st = cbns_batch_create(hs.data(), (int)hs.size(), &sv->batch);
      if (st == CBNS_OK && sv->opts.tile_rows) {
        cbns_launch_config cfg{sv->opts.tile_rows, sv->opts.ctas_per_sm};
        st = cbns_batch_set_config(sv->batch, &cfg);
      }
      if (st != CBNS_OK) {
        std::string err = cbns_last_error();
        for (Request* r : sv->active) retire(sv, r, st, err);
        sv->active.clear();
        continue;
      }
      std::lock_guard<std::mutex> lk(sv->mu);
      sv->stats.batch_builds++;
      if (sv->active.size() > sv->stats.peak_active) sv->stats.peak_active = (uint32_t)sv->active.size();
    }
    std::vector<uint32_t> steps(sv->active.size());
    cbns_status st = cbns_batch_run(sv->batch, sv->opts.steps_per_round, steps.data());
    if (st != CBNS_OK && st != CBNS_ERR_NONPHYSICAL) {
      std::string err = cbns_last_error();
      for (Request* r : sv->active) retire(sv, r, st, err);
      sv->active.clear();
      cbns_batch_destroy(sv->batch);
      sv->batch = nullptr;
      continue;
    }
    std::vector<Request*> still;
    uint64_t cell_steps = 0;
    for (size_t i = 0; i < sv->active.size(); ++i) {
      Request* r = sv->active[i];
      // The control block's step counter counts from the request's upload (a
      // batch's own counts restart whenever membership changes).
      const cbns::SolveCtl& c = sv->batch->h_ctl[i];
      cell_steps += (uint64_t)(c.steps - r->steps) * r->IM * r->JM * r->KM;
      r->steps = c.steps;
      bool cancel;
      {
        std::lock_guard<std::mutex> lk(sv->mu);
        cancel = r->cancel;
      }
      if (c.status & cbns::kStatusBounds)
        retire(sv, r, CBNS_ERR_BOUNDS, "a kernel index left its array (bounds-checked build)");
      else if (c.status)
        retire(sv, r, CBNS_ERR_NONPHYSICAL, "non-physical state (rho <= 0, p <= 0 or NaN)");
      else if (cancel) retire(sv, r, CBNS_ERR_CANCELLED, "cancelled");
      else if (!c.active) retire(sv, r, CBNS_OK, "");
      else still.push_back(r);
    }
    {
      std::lock_guard<std::mutex> lk(sv->mu);
      sv->stats.rounds++;
      sv->stats.cell_steps += cell_steps;
    }
    if (still.size() != sv->active.size()) {
      sv->active.swap(still);
      if (sv->batch) cbns_batch_destroy(sv->batch);
      sv->batch = nullptr;
    }
  }
  // Shutdown: cancel what is left.
  for (Request* r : sv->active) retire(sv, r, CBNS_ERR_CANCELLED, "server stopped");
  sv->active.clear();
  if (sv->batch) cbns_batch_destroy(sv->batch);
  sv->batch = nullptr;
}

cbns_status serve_fail(cbns_status st, const std::string& msg) {
  cbns::set_last_error(msg);
  return st;
}

cbns_status submit(cbns_server* sv, Request* r, uint64_t* id) {
  if (r->params.IM != r->IM || r->params.JM != r->JM || r->params.KM != r->KM) {
    delete r;
    return serve_fail(CBNS_ERR_BAD_DIMS, "cbns_server_submit: the extents must equal the grid's (p->IM, p->JM, "
                                         "p->KM): one GPU holds the whole periodic grid");
  }
  uint64_t fp = 0;
  cbns_status st = cbns_footprint(r->IM, r->JM, r->KM, sv->opts.precision, &fp);
  if (st != CBNS_OK) {
    delete r;
    return st;
  }
  r->footprint = fp;
  std::lock_guard<std::mutex> lk(sv->mu);
  if (fp > sv->budget) {
    delete r;
    return serve_fail(CBNS_ERR_OUT_OF_MEMORY, "cbns_server_submit: request needs more device memory than the budget");
  }
  r->id = sv->next_id++;
  r->t_submit = sv->now();
  sv->queue.push_back(r);
  sv->reqs.emplace(r->id, std::unique_ptr<Request>(r));
  sv->stats.submitted++;
  if (id) *id = r->id;
  sv->cv_work.notify_one();
  return CBNS_OK;
}

}  // namespace

extern "C" {

cbns_status cbns_server_create(const cbns_server_opts* opts, cbns_server** out) {
  if (!opts || !out) return serve_fail(CBNS_ERR_INVALID_ARG, "cbns_server_create: null argument");
  *out = nullptr;
  if (opts->precision != CBNS_FP64 && opts->precision != CBNS_FP32_MIXED && opts->precision != CBNS_FP64_FF)
    return serve_fail(CBNS_ERR_INVALID_ARG, "cbns_server_create: unknown precision");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return serve_fail(CBNS_ERR_NO_DEVICE, "cbns_server_create: no CUDA device");
  }
  // The calling thread's current device, unless CBNS_DEVICE names one; the
  // worker thread makes it current before it creates any solve.
  int dev = 0;
  if (const char* e = std::getenv("CBNS_DEVICE")) {
    dev = std::atoi(e);
  } else if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    dev = 0;
  }
  if (dev < 0 || dev >= ndev) return serve_fail(CBNS_ERR_NO_DEVICE, "cbns_server_create: CBNS_DEVICE out of range");
  cudaSetDevice(dev);
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess)
    return serve_fail(CBNS_ERR_CUDA, "cbns_server_create: cudaMemGetInfo failed");
  cbns_server* sv = new cbns_server();
  sv->opts = *opts;
  sv->device = dev;
  if (sv->opts.steps_per_round == 0) sv->opts.steps_per_round = 10;
  sv->budget = opts->memory_budget_bytes ? opts->memory_budget_bytes : (uint64_t)(0.8 * (double)free_b);
  if (sv->budget > free_b) sv->budget = free_b;
  sv->t0 = std::chrono::steady_clock::now();
  sv->worker = std::thread(worker_loop, sv);
  *out = sv;
  return CBNS_OK;
}

cbns_status cbns_server_destroy(cbns_server* sv) {
  if (!sv) return CBNS_OK;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->stop = true;
    for (Request* r : sv->queue) {
      r->state = RQ_DONE;
      r->status = CBNS_ERR_CANCELLED;
    }
    sv->queue.clear();
  }
  sv->cv_work.notify_all();
  if (sv->worker.joinable()) sv->worker.join();
  sv->cv_done.notify_all();
  delete sv;
  return CBNS_OK;
}

cbns_status cbns_server_submit(cbns_server* sv, const cbns_params* p, uint32_t IM, uint32_t JM, uint32_t KM,
                               const double* Q0, int keep_state, uint64_t* id) {
  if (!sv || !p) return serve_fail(CBNS_ERR_INVALID_ARG, "cbns_server_submit: null argument");
  if (!Q0) return serve_fail(CBNS_ERR_INVALID_ARG, "cbns_server_submit: null state");
  Request* r = new Request();
  r->params = *p;
  cbns_params_derive(&r->params);
  r->IM = IM;
  r->JM = JM;
  r->KM = KM;
  r->keep_state = keep_state;
  r->Q0.assign(Q0, Q0 + (size_t)CBNS_NEQ * (IM + 2 * CBNS_NG) * (JM + 2 * CBNS_NG) * (KM + 2 * CBNS_NG));
  return submit(sv, r, id);
}

cbns_status cbns_server_submit_tgv(cbns_server* sv, const cbns_params* p, uint32_t IM, uint32_t JM, uint32_t KM,
                                   uint64_t seed, double amp, int nmodes, int kmax, int keep_state, uint64_t* id) {
  if (!sv || !p) return serve_fail(CBNS_ERR_INVALID_ARG, "cbns_server_submit_tgv: null argument");
  if (nmodes < 0 || nmodes > 64 || (nmodes > 0 && kmax < 1))
    return serve_fail(CBNS_ERR_INVALID_ARG, "cbns_server_submit_tgv: nmodes in [0, 64], kmax >= 1");
  Request* r = new Request();
  r->params = *p;
  cbns_params_derive(&r->params);
  r->IM = IM;
  r->JM = JM;
  r->KM = KM;
  r->seed = seed;
  r->amp = amp;
  r->nmodes = nmodes;
  r->kmax = kmax;
  r->keep_state = keep_state;
  return submit(sv, r, id);
}

cbns_status cbns_server_submit_checkpoint(cbns_server* sv, const cbns_params* p, uint32_t IM, uint32_t JM,
                                          uint32_t KM, const char* path, int keep_state, uint64_t* id) {
  if (!sv || !p || !path) return serve_fail(CBNS_ERR_INVALID_ARG, "cbns_server_submit_checkpoint: null argument");
  Request* r = new Request();
  r->params = *p;
  cbns_params_derive(&r->params);
  r->IM = IM;
  r->JM = JM;
  r->KM = KM;
  r->ckpt = path;
  r->keep_state = keep_state;
  return submit(sv, r, id);
}

cbns_status cbns_server_cancel(cbns_server* sv, uint64_t id) {
  if (!sv) return serve_fail(CBNS_ERR_INVALID_ARG, "cbns_server_cancel: null server");
  std::lock_guard<std::mutex> lk(sv->mu);
  auto it = sv->reqs.find(id);
  if (it == sv->reqs.end()) return serve_fail(CBNS_ERR_INVALID_ARG, "cbns_server_cancel: unknown request");
  it->second->cancel = true;
  sv->cv_work.notify_one();
  return CBNS_OK;
}

cbns_status cbns_server_wait(cbns_server* sv, uint64_t id, double timeout_s, cbns_request_info* info) {
  if (!sv) return serve_fail(CBNS_ERR_INVALID_ARG, "cbns_server_wait: null server");
  std::unique_lock<std::mutex> lk(sv->mu);
  auto it = sv->reqs.find(id);
  if (it == sv->reqs.end()) return serve_fail(CBNS_ERR_INVALID_ARG, "cbns_server_wait: unknown request");
  Request* r = it->second.get();
  auto done = [&] { return r->state == RQ_DONE; };
  if (timeout_s < 0) sv->cv_done.wait(lk, done);
  else if (!sv->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), done))
    return serve_fail(CBNS_ERR_TIMEOUT, "cbns_server_wait: request not finished within the timeout");
  if (info) {
    info->status = r->status;
    info->steps = r->steps;
    info->t_final = r->t_final;
    info->ke = r->ke;
    info->enstrophy = r->enstrophy;
    info->submit_s = r->t_submit;
    info->admit_s = r->t_admit;
    info->done_s = r->t_done;
    info->device_bytes = r->footprint;
  }
  if (r->status != CBNS_OK) cbns::set_last_error(r->error);
  return (cbns_status)r->status;
}

cbns_status cbns_server_result(cbns_server* sv, uint64_t id, double* Q_out) {
  if (!sv || !Q_out) return serve_fail(CBNS_ERR_INVALID_ARG, "cbns_server_result: null argument");
  std::lock_guard<std::mutex> lk(sv->mu);
  auto it = sv->reqs.find(id);
  if (it == sv->reqs.end()) return serve_fail(CBNS_ERR_INVALID_ARG, "cbns_server_result: unknown request");
  Request* r = it->second.get();
  if (r->state != RQ_DONE || r->status != CBNS_OK || r->result.empty())
    return serve_fail(CBNS_ERR_INVALID_ARG, "cbns_server_result: no stored result (not done, failed, or keep_state 0)");
  std::memcpy(Q_out, r->result.data(), sizeof(double) * r->result.size());
  return CBNS_OK;
}

cbns_status cbns_server_release(cbns_server* sv, uint64_t id) {
  if (!sv) return serve_fail(CBNS_ERR_INVALID_ARG, "cbns_server_release: null server");
  std::lock_guard<std::mutex> lk(sv->mu);
  auto it = sv->reqs.find(id);
  if (it == sv->reqs.end() || it->second->state != RQ_DONE)
    return serve_fail(CBNS_ERR_INVALID_ARG, "cbns_server_release: unknown or unfinished request");
  sv->reqs.erase(it);
  return CBNS_OK;
}

cbns_status cbns_server_get_stats(cbns_server* sv, cbns_server_stats* out) {
  if (!sv || !out) return serve_fail(CBNS_ERR_INVALID_ARG, "cbns_server_get_stats: null argument");
  std::lock_guard<std::mutex> lk(sv->mu);
  *out = sv->stats;
  out->budget_bytes = sv->budget;
  out->used_bytes = sv->used;
  out->queued = (uint32_t)sv->queue.size();
  out->clock_s = sv->now();
  return CBNS_OK;
}

}  // extern "C"
