// fvm_serve.cpp -- continuous-batching service of steady solves on one GPU,
// in native code on top of the batch API (no counterpart in the reference,
// whose driver runs one solve per process: main.f:42-76).
//
// Callers submit solves from any thread (the block layout is built on the
// submitting thread, so several submitters prepare requests in parallel);
// one service thread owns the batch arena and loops:
//   admit   queued solves in arrival order while the arena has room (a solve
//           that does not fit an empty arena is refused with
//           FVM_ERR_CAPACITY);
//   step    every resident solve `chunk` iterations (one CUDA graph launch
//           per iteration, every mesh in each kernel);
//   checkpoint  running solves the caller asked to stop: their state is
//           read back and kept, the arena ranges freed (status
//           FVM_CHECKPOINTED); fvm_serve_resume queues a solve that starts
//           from such a state;
//   retire  solves that reached their residual drop or iteration cap
//           (main.f:42) or stopped with a status: results (and the final
//           state when asked) are kept for the caller, the arena ranges
//           freed;
// and, when asked, re-runs the autotuner every `tune_every` steps.
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/fvm_gpu.h"

namespace fvm {   // fvm_batch.cpp: admission beside a running step
int32_t batch_add_prepared_deferred(fvm_batch *b, fvm_prepared *prep, int32_t *slot_out);
int32_t batch_commit_admissions(fvm_batch *b);
}  // namespace fvm

namespace {

using Clock = std::chrono::steady_clock;

struct Ticket {
  int state = 0;                 // 0 queued, 1 running, 2 done
  fvm_prepared *prep = nullptr;
  int32_t np = 0, nmax = 0, slot = -1;
  double minres = 0.0;
  bool keep_state = false;
  Clock::time_point t_submit, t_admit, t_done;
  int32_t status = FVM_OK, niter = 0;
  double fres = 0.0, cl = 0.0, cd = 0.0;
  double cl_tail = 0.0, cd_tail = 0.0;   // means over the last kTail iterations
  std::vector<double> prim, nut;         // final or checkpointed state
  // checkpoint: asked by the caller; the kept viscosities and the
  // iteration count a resume starts from
  bool ckpt_req = false;
  std::vector<double> ck_mul, ck_mu;
  int32_t ck_iter = 0;
  // resume: the state the solve starts from, at iteration iterlast
  bool resume = false;
  int32_t iterlast = 0;
  std::vector<double> start_prim, start_nut, start_mul, start_mu;
};

constexpr int kTail = 256;
// fvm_serve_wait timeouts at or above this many seconds (about 32 years,
// and +inf) wait until the ticket is done; the bound keeps the conversion
// to clock ticks finite
constexpr double kWaitForever = 1e9;

double seconds(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double>(b - a).count();
}

}  // namespace

struct fvm_server {
  fvm_batch *b = nullptr;
  int device = 0;
  int32_t chunk = 50, tune_every = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<int64_t> queue;            // prepared, waiting for admission
  std::map<int64_t, Ticket> tickets;
  std::map<int32_t, int64_t> resident;  // slot -> ticket (service thread only)
  int64_t next_id = 1, submitted = 0, done = 0, steps = 0;
  // service-thread seconds: admitting, tuning, stepping (launch + waiting
  // for the GPU), retiring
  double t_admit = 0, t_tune = 0, t_step = 0, t_retire = 0;
  double t_admit_beside = 0;            // admission work overlapped with a step
  int32_t error = FVM_OK;               // a CUDA failure stops the service
  bool stop = false;
  std::thread worker;
  // API calls in progress (counted before the mutex is taken): destroy
  // frees the server only when none is left inside
  std::atomic<int> callers{0};
};

namespace {

// Counts an API call as in progress for its whole duration, including the
// wait for the mutex.
struct InCall {
  fvm_server *s;
  explicit InCall(fvm_server *srv) : s(srv) { s->callers.fetch_add(1); }
  ~InCall() { s->callers.fetch_sub(1); }
};

void finish(fvm_server *s, int64_t id, Ticket &t, int32_t status) {
  t.status = status;
  t.state = 2;
  t.t_done = Clock::now();
  s->done++;
  (void)id;
}

// Moves every resident solve that stopped to the done state.
int32_t retire(fvm_server *s) {
  std::vector<std::pair<int32_t, int64_t>> res(s->resident.begin(), s->resident.end());
  for (const auto &r : res) {
    int32_t active = 0, niter = 0, status = 0, bad = 0;
    double fres = 0, cl = 0, cd = 0;
    int32_t st = fvm_batch_poll(s->b, r.first, &active, &niter, &fres, &cl, &cd, &status, &bad);
    if (st) return st;
    if (active) continue;
    std::vector<double> prim, nut;
    bool keep;
    int32_t np;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      keep = s->tickets[r.second].keep_state;
      np = s->tickets[r.second].np;
    }
    if (keep) {
      prim.resize(4 * (size_t)np);
      nut.resize(np);
      std::vector<double> mul(np), mu(np), qx(4 * (size_t)np), qy(4 * (size_t)np);
      st = fvm_batch_get_state(s->b, r.first, prim.data(), nut.data(), mul.data(), mu.data(),
                               qx.data(), qy.data());
      if (st) return st;
    }
    // mean cl, cd over the last iterations (the history the device keeps)
    double clt = 0.0, cdt = 0.0;
    const int k = niter < kTail ? niter : kTail;
    if (k > 0) {
      std::vector<double> hf(k), hfi(k), hcl(k), hcd(k);
      std::vector<int32_t> hi(k);
      st = fvm_batch_history(s->b, r.first, niter - k, k, hf.data(), hi.data(), hfi.data(),
                             hcl.data(), hcd.data());
      if (st) return st;
      for (int j = 0; j < k; j++) {
        clt += hcl[j];
        cdt += hcd[j];
      }
      clt /= k;
      cdt /= k;
    }
    if ((st = fvm_batch_remove(s->b, r.first))) return st;
    s->resident.erase(r.first);
    std::lock_guard<std::mutex> lk(s->mu);
    Ticket &t = s->tickets[r.second];
    t.niter = niter;
    t.fres = fres;
    t.cl = cl;
    t.cd = cd;
    t.cl_tail = clt;
    t.cd_tail = cdt;
    t.prim.swap(prim);
    t.nut.swap(nut);
    finish(s, r.second, t, status);
  }
  return FVM_OK;
}

// Starts an admitted solve: from the freestream, or (resume) from the
// ticket's state at its iteration iterlast.
int32_t start_solve(fvm_server *s, const Ticket &t, int32_t slot, int32_t nmax, double minres) {
  if (t.resume) {
    auto ptr = [](const std::vector<double> &v) { return v.empty() ? nullptr : v.data(); };
    const int32_t st = fvm_batch_set_state(s->b, slot, t.start_prim.data(), ptr(t.start_nut),
                                           ptr(t.start_mul), ptr(t.start_mu), t.iterlast);
    if (st) return st;
  }
  return fvm_batch_start(s->b, slot, nmax, minres);
}

// Admits queued solves while the arena has room.  Deferred (a step is
// running): the uploads go beside it and the solves start at
// start_admitted, after the step.
struct Admitted {
  int64_t id;
  int32_t slot, nmax;
  double minres;
  Ticket *t;
};

int32_t admit(fvm_server *s, bool deferred, std::vector<Admitted> *staged) {
  for (;;) {
    int64_t id;
    fvm_prepared *prep;
    int32_t nmax;
    double minres;
    Ticket *tp;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      if (s->queue.empty()) return FVM_OK;
      id = s->queue.front();
      Ticket &t = s->tickets[id];
      prep = t.prep;
      nmax = t.nmax;
      minres = t.minres;
      tp = &t;   // map nodes stay put; a queued or running ticket is not released
    }
    int32_t slot = -1;
    int32_t st = deferred ? fvm::batch_add_prepared_deferred(s->b, prep, &slot)
                          : fvm_batch_add_prepared(s->b, prep, &slot);
    std::lock_guard<std::mutex> lk(s->mu);
    Ticket &t = s->tickets[id];
    if (st == FVM_ERR_CAPACITY && !s->resident.empty()) return FVM_OK;   // waits for room
    s->queue.pop_front();
    if (st) {                  // too large for an empty arena, or bad input
      fvm_prepared_free(prep);
      t.prep = nullptr;
      finish(s, id, t, st);
      s->cv_done.notify_all();
      if (st == FVM_ERR_CUDA) return st;
      continue;
    }
    t.prep = nullptr;          // taken by the batch
    t.slot = slot;
    t.state = 1;
    t.t_admit = Clock::now();
    if (deferred) {
      staged->push_back({id, slot, nmax, minres, tp});
      continue;
    }
    s->resident[slot] = id;
    if ((st = start_solve(s, *tp, slot, nmax, minres))) return st;
  }
}

// The solves admitted beside the last step join the batch and start.
int32_t start_admitted(fvm_server *s, std::vector<Admitted> &staged) {
  if (staged.empty()) return FVM_OK;
  int32_t st = fvm::batch_commit_admissions(s->b);
  for (const Admitted &a : staged) {
    s->resident[a.slot] = a.id;
    if (!st) st = start_solve(s, *a.t, a.slot, a.nmax, a.minres);
  }
  staged.clear();
  return st;
}

// Stops the running solves whose checkpoint was asked: state read back and
// kept, arena ranges freed, ticket done with FVM_CHECKPOINTED.  A solve
// that finished in the same step retires as usual.
int32_t checkpoint(fvm_server *s) {
  std::vector<std::pair<int32_t, int64_t>> want;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    for (const auto &r : s->resident)
      if (s->tickets[r.second].ckpt_req) want.push_back(r);
  }
  for (const auto &r : want) {
    int32_t active = 0, niter = 0, status = 0, bad = 0;
    double fres = 0, cl = 0, cd = 0;
    int32_t st = fvm_batch_poll(s->b, r.first, &active, &niter, &fres, &cl, &cd, &status, &bad);
    if (st) return st;
    if (!active) continue;
    int32_t np, iterlast;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      np = s->tickets[r.second].np;
      iterlast = s->tickets[r.second].iterlast;
    }
    std::vector<double> prim(4 * (size_t)np), nut(np), mul(np), mu(np);
    st = fvm_batch_get_state(s->b, r.first, prim.data(), nut.data(), mul.data(), mu.data(),
                             nullptr, nullptr);
    if (st) return st;
    if ((st = fvm_batch_remove(s->b, r.first))) return st;
    s->resident.erase(r.first);
    std::lock_guard<std::mutex> lk(s->mu);
    Ticket &t = s->tickets[r.second];
    t.niter = niter;
    t.fres = fres;
    t.cl = cl;
    t.cd = cd;
    t.prim.swap(prim);
    t.nut.swap(nut);
    t.ck_mul.swap(mul);
    t.ck_mu.swap(mu);
    t.ck_iter = iterlast + niter;
    finish(s, r.second, t, FVM_CHECKPOINTED);
  }
  return FVM_OK;
}

void service(fvm_server *s) {
  cudaSetDevice(s->device);
  int32_t st = FVM_OK;
  for (;;) {
    {
      std::unique_lock<std::mutex> lk(s->mu);
      if (s->stop) break;
      if (s->queue.empty() && s->resident.empty()) {
        s->cv_work.wait_for(lk, std::chrono::milliseconds(20));
        continue;
      }
    }
    auto sec = [](Clock::time_point a, Clock::time_point b) {
      return std::chrono::duration<double>(b - a).count();
    };
    // this pass's times, published under the lock (fvm_serve_times reads them)
    double d_admit = 0, d_tune = 0, d_step = 0, d_retire = 0, d_beside = 0;
    int64_t d_steps = 0;
    auto publish = [&]() {
      std::lock_guard<std::mutex> lk(s->mu);
      s->t_admit += d_admit;
      s->t_tune += d_tune;
      s->t_step += d_step;
      s->t_retire += d_retire;
      s->t_admit_beside += d_beside;
      s->steps += d_steps;
    };
    const Clock::time_point t0 = Clock::now();
    // with nothing resident, admit now; otherwise beside the next step
    if (s->resident.empty()) st = admit(s, false, nullptr);
    const Clock::time_point t1 = Clock::now();
    d_admit += sec(t0, t1);
    if (st || s->resident.empty()) {
      publish();
      if (st) break;
      continue;
    }
    int64_t steps_now;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      steps_now = s->steps;
    }
    if (s->tune_every > 0 && steps_now % s->tune_every == 0) {
      int32_t choice = 0;
      st = fvm_batch_tune(s->b, 10, 0, nullptr, &choice);
    }
    const Clock::time_point t2 = Clock::now();
    d_tune += sec(t1, t2);
    std::vector<Admitted> staged;
    if (!st) st = fvm_batch_step(s->b, s->chunk);
    // uploads of waiting solves while the step runs
    const Clock::time_point ta = Clock::now();
    if (!st) st = admit(s, true, &staged);
    const Clock::time_point tb = Clock::now();
    d_beside += sec(ta, tb);
    if (!st) st = fvm_batch_sync(s->b);
    const Clock::time_point t3 = Clock::now();
    d_step += sec(t2, t3);
    if (!st) st = start_admitted(s, staged);
    const Clock::time_point t4 = Clock::now();
    d_admit += sec(t3, t4);
    if (!st) {
      d_steps = 1;
      st = checkpoint(s);
    }
    if (!st) st = retire(s);
    d_retire += sec(t4, Clock::now());
    publish();
    if (st) break;
    s->cv_done.notify_all();
  }
  std::lock_guard<std::mutex> lk(s->mu);
  if (st) {                   // the service cannot continue: fail what is left
    s->error = st;
    for (auto &kv : s->tickets)
      if (kv.second.state != 2) finish(s, kv.first, kv.second, st);
  }
  s->cv_done.notify_all();
}

}  // namespace

extern "C" int32_t fvm_serve_create(int32_t precision, const fvm_batch_caps *caps,
                                    int32_t chunk, int32_t tune_every, fvm_server **out) {
  if (!caps || !out || chunk < 1 || tune_every < 0) return FVM_ERR_ARG;
  *out = nullptr;
  fvm_server *s = new (std::nothrow) fvm_server();
  if (!s) return FVM_ERR_NOMEM;
  int32_t st = fvm_batch_create(precision, caps, &s->b);
  if (st) {
    delete s;
    return st;
  }
  cudaGetDevice(&s->device);
  s->chunk = chunk;
  s->tune_every = tune_every;
  try {
    s->worker = std::thread(service, s);
  } catch (...) {
    fvm_batch_destroy(s->b);
    delete s;
    return FVM_ERR_NOMEM;
  }
  *out = s;
  return FVM_OK;
}

namespace {

// Queues a solve (a resume when prim is given).
int32_t submit(fvm_server *s, const fvm_params *p, const fvm_mesh *m, int32_t nmax,
               double minres, int32_t keep_state, const double *prim, const double *nut,
               const double *mul, const double *mu, int32_t iterlast, int64_t *ticket) {
  if (!s || !p || !m || !ticket || nmax < 1 || m->np < 1 || iterlast < 0) return FVM_ERR_ARG;
  InCall in_call(s);
  *ticket = 0;
  Ticket nt;
  if (prim) {
    const size_t np = (size_t)m->np;
    nt.resume = true;
    nt.iterlast = iterlast;
    nt.start_prim.assign(prim, prim + 4 * np);
    if (nut) nt.start_nut.assign(nut, nut + np);
    if (mul) nt.start_mul.assign(mul, mul + np);
    if (mu) nt.start_mu.assign(mu, mu + np);
  }
  fvm_prepared *prep = nullptr;
  const int32_t st = fvm_batch_prepare(p, m, &prep);   // on the caller's thread
  if (st) return st;
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stop || s->error) {
    fvm_prepared_free(prep);
    return s->error ? s->error : FVM_ERR_STATE;
  }
  const int64_t id = s->next_id++;
  Ticket &t = s->tickets[id];
  t = std::move(nt);
  t.prep = prep;
  t.np = m->np;
  t.nmax = nmax;
  t.minres = minres;
  t.keep_state = keep_state != 0;
  t.t_submit = Clock::now();
  s->queue.push_back(id);
  s->submitted++;
  s->cv_work.notify_one();
  *ticket = id;
  return FVM_OK;
}

}  // namespace

extern "C" int32_t fvm_serve_submit(fvm_server *s, const fvm_params *p, const fvm_mesh *m,
                                    int32_t nmax, double minres, int32_t keep_state,
                                    int64_t *ticket) {
  return submit(s, p, m, nmax, minres, keep_state, nullptr, nullptr, nullptr, nullptr, 0,
                ticket);
}

extern "C" int32_t fvm_serve_resume(fvm_server *s, const fvm_params *p, const fvm_mesh *m,
                                    int32_t nmax, double minres, const double *prim,
                                    const double *nut, const double *mul, const double *mu,
                                    int32_t iterlast, int32_t keep_state, int64_t *ticket) {
  if (!prim) return FVM_ERR_ARG;
  return submit(s, p, m, nmax, minres, keep_state, prim, nut, mul, mu, iterlast, ticket);
}

extern "C" int32_t fvm_serve_checkpoint(fvm_server *s, int64_t ticket) {
  if (!s) return FVM_ERR_ARG;
  InCall in_call(s);
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return FVM_ERR_ARG;
  if (it->second.state != 1) return FVM_ERR_STATE;
  it->second.ckpt_req = true;
  s->cv_work.notify_one();
  return FVM_OK;
}

extern "C" int32_t fvm_serve_checkpoint_read(fvm_server *s, int64_t ticket, double *prim,
                                             double *nut, double *mul, double *mu,
                                             int32_t *iter) {
  if (!s) return FVM_ERR_ARG;
  InCall in_call(s);
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return FVM_ERR_ARG;
  const Ticket &t = it->second;
  if (t.state != 2 || t.status != FVM_CHECKPOINTED) return FVM_ERR_STATE;
  if (prim) std::memcpy(prim, t.prim.data(), t.prim.size() * sizeof(double));
  if (nut) std::memcpy(nut, t.nut.data(), t.nut.size() * sizeof(double));
  if (mul) std::memcpy(mul, t.ck_mul.data(), t.ck_mul.size() * sizeof(double));
  if (mu) std::memcpy(mu, t.ck_mu.data(), t.ck_mu.size() * sizeof(double));
  if (iter) *iter = t.ck_iter;
  return FVM_OK;
}

extern "C" int32_t fvm_serve_poll(fvm_server *s, int64_t ticket, int32_t *state) {
  if (!s || !state) return FVM_ERR_ARG;
  InCall in_call(s);
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return FVM_ERR_ARG;
  *state = it->second.state;
  return FVM_OK;
}

extern "C" int32_t fvm_serve_wait(fvm_server *s, int64_t ticket, double timeout_s,
                                  int32_t *state) {
  if (!s || !state || std::isnan(timeout_s)) return FVM_ERR_ARG;
  InCall in_call(s);
  std::unique_lock<std::mutex> lk(s->mu);
  if (s->tickets.find(ticket) == s->tickets.end()) return FVM_ERR_ARG;
  // the ticket is looked up again after every wake-up: another thread may
  // have released it meanwhile
  auto done = [&] {
    auto it = s->tickets.find(ticket);
    return it == s->tickets.end() || it->second.state == 2;
  };
  if (timeout_s >= kWaitForever)
    s->cv_done.wait(lk, done);
  else if (timeout_s > 0)
    s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), done);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return FVM_ERR_ARG;
  *state = it->second.state;
  return FVM_OK;
}

extern "C" int32_t fvm_serve_result(fvm_server *s, int64_t ticket, int32_t *status,
                                    int32_t *niter, double *fres, double *cl, double *cd,
                                    double *tail, double *times) {
  if (!s) return FVM_ERR_ARG;
  InCall in_call(s);
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end() || it->second.state != 2) return FVM_ERR_ARG;
  const Ticket &t = it->second;
  if (status) *status = t.status;
  if (niter) *niter = t.niter;
  if (fres) *fres = t.fres;
  if (cl) *cl = t.cl;
  if (cd) *cd = t.cd;
  if (tail) {
    tail[0] = t.cl_tail;
    tail[1] = t.cd_tail;
  }
  if (times) {   // queued, resident, total (seconds)
    const bool ran = t.slot >= 0;
    times[0] = ran ? seconds(t.t_submit, t.t_admit) : seconds(t.t_submit, t.t_done);
    times[1] = ran ? seconds(t.t_admit, t.t_done) : 0.0;
    times[2] = seconds(t.t_submit, t.t_done);
  }
  return FVM_OK;
}

extern "C" int32_t fvm_serve_state(fvm_server *s, int64_t ticket, double *prim, double *nut) {
  if (!s || !prim) return FVM_ERR_ARG;
  InCall in_call(s);
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end() || it->second.state != 2 || it->second.prim.empty())
    return FVM_ERR_ARG;
  std::memcpy(prim, it->second.prim.data(), it->second.prim.size() * sizeof(double));
  if (nut) std::memcpy(nut, it->second.nut.data(), it->second.nut.size() * sizeof(double));
  return FVM_OK;
}

extern "C" int32_t fvm_serve_release(fvm_server *s, int64_t ticket) {
  if (!s) return FVM_ERR_ARG;
  InCall in_call(s);
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end() || it->second.state != 2) return FVM_ERR_ARG;
  s->tickets.erase(it);
  return FVM_OK;
}

extern "C" int32_t fvm_serve_stats(fvm_server *s, int64_t *out) {
  if (!s || !out) return FVM_ERR_ARG;
  InCall in_call(s);
  std::lock_guard<std::mutex> lk(s->mu);
  int64_t queued = 0, running = 0;
  for (const auto &kv : s->tickets) {
    queued += kv.second.state == 0;
    running += kv.second.state == 1;
  }
  out[0] = s->submitted;
  out[1] = s->done;
  out[2] = queued;
  out[3] = running;
  out[4] = s->steps;
  out[5] = s->error;
  return FVM_OK;
}

extern "C" int32_t fvm_serve_times(fvm_server *s, double *out) {
  if (!s || !out) return FVM_ERR_ARG;
  InCall in_call(s);
  std::lock_guard<std::mutex> lk(s->mu);
  out[0] = s->t_admit;
  out[1] = s->t_tune;
  out[2] = s->t_step;
  out[3] = s->t_retire;
  out[4] = s->t_admit_beside;
  return FVM_OK;
}

extern "C" int32_t fvm_serve_destroy(fvm_server *s) {
  if (!s) return FVM_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  if (s->worker.joinable()) s->worker.join();
  {
    // solves that never finished end with FVM_ERR_STATE, which wakes their
    // waiters
    std::lock_guard<std::mutex> lk(s->mu);
    for (auto &kv : s->tickets) {
      if (kv.second.prep) fvm_prepared_free(kv.second.prep);
      kv.second.prep = nullptr;
      if (kv.second.state != 2) finish(s, kv.first, kv.second, FVM_ERR_STATE);
    }
  }
  s->cv_done.notify_all();
  // calls already inside the API (waiters woken above, callers queued on
  // the mutex) leave before the server is freed
  while (s->callers.load() > 0) std::this_thread::sleep_for(std::chrono::microseconds(100));
  const int32_t st = fvm_batch_destroy(s->b);
  delete s;
  return st;
}
