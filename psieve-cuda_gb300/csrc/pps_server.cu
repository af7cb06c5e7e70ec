// pps_server.cu -- the serving loop: continuous batching over the batched form.
//
// A worker thread owns one engine.  Each turn it admits queued jobs into free
// device slots (in submission order, while the slot count and the factor-buffer
// budget allow), cuts the next p pieces of every admitted job into one wave,
// runs the wave (sieve + persistent walk + output rule, one captured graph) and
// hands each job its survivors.  A job whose last piece was in the wave is
// finished: its prime counters are read from its slot, its latency (submit to
// result ready) recorded, and its slot and reservation freed.  New jobs join at
// the next wave; nothing waits for a batch to fill.
//
// Admission by device memory: a job reserves room for its expected raw
// candidates (32 B each, twice the Mertens estimate sum_p #k #n / p, at least
// 16 KiB) in the hit buffers that every wave shares; the sum over admitted jobs
// stays within the configured budget, and a job that alone exceeds it is
// refused at submission.  Job state between waves (parameters and prime
// counters) stays in the device slots.
//
// Reference counterpart: none -- the reference runs one range per process
// (main.c:887-1266).  The per-job results are the ones pps_run_job returns.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "pps_engine_impl.h"

namespace {

using Clock = std::chrono::steady_clock;

struct JobRec {
  uint64_t id = 0;
  pps_job_params jp{};
  int state = PPS_JOB_QUEUED;
  int status = PPS_OK;
  uint32_t slot = 0;
  uint64_t cursor = 0;   // next p handed to a wave
  uint64_t reserve = 0;  // bytes of the shared hit buffers reserved
  std::vector<pps_factor> factors;
  uint64_t primes = 0, sum = 0;  // of the primes below done_p
  uint64_t done_p = 0;           // boundary of the waves completed so far
  bool cancel = false;           // asked to stop (pps_job_cancel)
  Clock::time_point t_submit, t_done;
};

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

// Estimated walk steps of the piece [lo, hi) of a job: primes ~ (hi - lo) /
// ln lo, each walked over the job's whole n range.
double piece_work(const pps_job_params& jp, uint64_t lo, uint64_t hi) {
  const double nsteps = (double)((jp.nmax - jp.nmin + jp.step - 1) / jp.step);
  return (double)(hi - lo) / log((double)std::max<uint64_t>(lo, 3)) * nsteps;
}

// Expected raw candidates of a job: sum over primes p in the range of
// #k * #n / p, with sum 1/p over [a, b) ~ ln(ln b / ln a) (Mertens).
uint64_t job_reservation(const pps_job_params& jp) {
  const double nk = (double)((jp.kmax - jp.kmin) / std::max<uint32_t>(jp.kstep, 1) + 1);
  const double nn = (double)(jp.nmax - jp.nmin);
  const double lo = std::max(3.0, (double)jp.pmin), hi = std::max(lo + 1.0, (double)jp.pmax);
  const double expect = nk * nn * log(log(hi) / log(lo));
  const double bytes = 2.0 * expect * (double)sizeof(pps_hit);
  return (uint64_t)std::max(16384.0, std::min(bytes, 1e18));
}

}  // namespace

struct pps_server {
  pps_engine* e = nullptr;
  pps_server_config cfg{};
  std::thread worker;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  bool stop = false;
  std::deque<uint64_t> queue;   // submitted, not yet admitted
  std::vector<JobRec*> active;  // admitted, in admission order
  std::unordered_map<uint64_t, std::unique_ptr<JobRec>> jobs;
  std::vector<uint32_t> free_slots;
  uint64_t reserved = 0;
  uint64_t next_id = 1;
  pps_server_stats st{};
  std::vector<double> latencies;
};

namespace {

// One turn of the worker: admit, build and run one wave, retire finished jobs.
// Returns false when the server stops.
bool serve_turn(pps_server* s, std::vector<BatchPiece>& pieces, std::vector<pps_hit>& surv) {
  std::vector<JobRec*> admitted, act;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    s->cv_work.wait(lk, [&] { return s->stop || !s->queue.empty() || !s->active.empty(); });
    if (s->stop) return false;
    while (!s->queue.empty() && !s->free_slots.empty()) {
      JobRec* j = s->jobs[s->queue.front()].get();
      if (s->reserved + j->reserve > s->cfg.factor_bytes) break;  // waits for memory to free up
      s->queue.pop_front();
      j->slot = s->free_slots.back();
      s->free_slots.pop_back();
      j->state = PPS_JOB_RUNNING;
      s->reserved += j->reserve;
      s->active.push_back(j);
      admitted.push_back(j);
      s->st.admitted++;
    }
    act = s->active;  // only this thread removes active jobs, so the pointers stay valid
    for (JobRec* j : act)
      if (j->cancel && !j->status) j->status = PPS_ERR_CANCELLED;  // no more pieces; retired below
  }
  std::vector<JobRec*> failed;
  for (JobRec* j : act)
    if (j->status == PPS_ERR_CANCELLED) failed.push_back(j);
  pps_engine* e = s->e;
  for (JobRec* j : admitted) {
    j->cursor = j->jp.pmin | 1ull;
    j->done_p = j->jp.pmin;
    const int rc = batch_set_jobs(e, j->slot, &j->jp, 1);
    if (rc) {
      j->status = rc;
      failed.push_back(j);
    }
  }
  // The wave: one piece per job first (oldest first), each at most an equal
  // share of the wave's work, then fill oldest first.  A wave holds at most
  // wave_segments segments and about wave_work walk steps, so a job that
  // arrives while it runs waits at most one such wave for its first piece.
  // Under load (more than 4 jobs running) the work per wave grows with the
  // running jobs, up to 8 times, so that the per-wave cost (host turns, the
  // last chunks' tail) stays small next to the walk.
  pieces.clear();
  const uint64_t cap = s->cfg.wave_segments;
  const double load = std::min(8.0, std::max(1.0, (double)act.size() / 4.0));
  const double work_cap = (double)s->cfg.wave_work * load;
  // a piece is at most one batch, and never more than the wave holds
  const uint64_t span = std::min<uint64_t>(batch_piece_span(e), cap * 2ull * pps::SEG_BITS);
  const uint64_t seg_span = 2ull * pps::SEG_BITS;  // p range of one segment
  uint64_t segs = 0;
  double work = 0;
  std::vector<JobRec*> in_wave, finishing;
  auto take = [&](JobRec* j, double share) -> bool {
    if (j->status || j->cursor >= j->jp.pmax) return false;
    uint64_t hi = std::min(j->jp.pmax, j->cursor + span);
    // cut to the work left in the wave (or the share), whole segments, at least one
    const double room = std::min(work_cap - work, share);
    const double w = piece_work(j->jp, j->cursor, hi);
    if (w > room) {
      if (room <= 0 && !pieces.empty()) return false;
      const double frac = std::max(room, 0.0) / w;
      uint64_t width = (uint64_t)(frac * (double)(hi - j->cursor));
      width = std::max<uint64_t>(seg_span, width / seg_span * seg_span);
      hi = std::min(hi, j->cursor + width);
    }
    const uint64_t ns = batch_piece_segments(j->cursor, hi);
    if (segs + ns > cap) return false;
    pieces.push_back(BatchPiece{j->cursor, hi, j->slot});
    segs += ns;
    work += piece_work(j->jp, j->cursor, hi);
    j->cursor = hi;
    return true;
  };
  const double first_share = act.empty() ? work_cap : work_cap / (double)act.size();
  for (JobRec* j : act)
    if (take(j, first_share)) in_wave.push_back(j);
  for (JobRec* j : act) {
    bool any = false;
    while (work < work_cap && take(j, work_cap)) any = true;
    if (any && std::find(in_wave.begin(), in_wave.end(), j) == in_wave.end()) in_wave.push_back(j);
  }
  for (JobRec* j : act)
    if (!j->status && j->cursor >= j->jp.pmax) finishing.push_back(j);

  surv.clear();
  uint64_t raw = 0;
  double fms = 0;
  int rc = PPS_OK;
  const Clock::time_point t0 = Clock::now();
  if (!pieces.empty()) rc = batch_wave(e, pieces.data(), pieces.size(), &surv, &raw, &fms);
  const double busy = ms_between(t0, Clock::now());
  if (rc) {
    // the wave failed: every job in it fails with the wave's status
    for (JobRec* j : in_wave) {
      j->status = rc;
      failed.push_back(j);
    }
    finishing.clear();
  }
  // the jobs' prime counters after the wave (one copy of their slot range)
  std::vector<uint64_t> pr, sm;
  uint32_t slot_lo = 0;
  if (!rc && !in_wave.empty()) {
    uint32_t slot_hi = 0;
    slot_lo = UINT32_MAX;
    for (JobRec* j : in_wave) {
      slot_lo = std::min(slot_lo, j->slot);
      slot_hi = std::max(slot_hi, j->slot);
    }
    pr.resize(slot_hi - slot_lo + 1);
    sm.resize(slot_hi - slot_lo + 1);
    if (int crc = batch_job_counts(e, slot_lo, pr.size(), pr.data(), sm.data())) {
      for (JobRec* j : in_wave) {
        j->status = crc;
        failed.push_back(j);
      }
      finishing.clear();
    }
  }
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (!rc && !pr.empty()) {
      // survivors to their jobs, and each job's drained boundary (its checkpoint)
      std::unordered_map<uint32_t, JobRec*> by_slot;
      for (JobRec* j : in_wave) by_slot[j->slot] = j;
      for (const pps_hit& h : surv) {
        auto it = by_slot.find(batch_hit_slot(h));
        if (it == by_slot.end()) continue;
        it->second->factors.push_back(pps_factor{h.p, h.k, h.n, batch_hit_sign(h)});
      }
      for (JobRec* j : in_wave) {
        if (j->status) continue;
        j->primes = pr[j->slot - slot_lo];
        j->sum = sm[j->slot - slot_lo];
        j->done_p = std::min(j->cursor, j->jp.pmax);
      }
    }
    if (!pieces.empty()) {
      s->st.waves++;
      s->st.busy_ms += busy;
    }
    auto retire = [&](JobRec* j, int state) {
      if (j->state == PPS_JOB_DONE || j->state == PPS_JOB_FAILED) return;
      j->state = state;
      j->t_done = Clock::now();
      s->free_slots.push_back(j->slot);
      s->reserved -= j->reserve;
      s->active.erase(std::find(s->active.begin(), s->active.end(), j));
      if (state == PPS_JOB_DONE) {
        s->st.completed++;
        s->st.primes += j->primes;
        s->st.steps += j->primes * (uint64_t)((j->jp.nmax - j->jp.nmin + j->jp.step - 1) / j->jp.step);
        s->latencies.push_back(ms_between(j->t_submit, j->t_done));
      } else {
        s->st.failed++;
      }
    };
    for (JobRec* j : failed) retire(j, PPS_JOB_FAILED);
    for (JobRec* j : finishing)
      if (!j->status) retire(j, PPS_JOB_DONE);
  }
  s->cv_done.notify_all();
  return true;
}

void serve(pps_server* s) {
  cudaSetDevice(s->e->device);
  std::vector<BatchPiece> pieces;
  std::vector<pps_hit> surv;
  while (serve_turn(s, pieces, surv)) {
  }
}

}  // namespace

extern "C" int pps_server_create(int device, const pps_server_config* cfg, pps_server** out) {
  if (!out) return set_err(PPS_ERR_INVALID_PARAM, "null output");
  *out = nullptr;
  pps_server_config c{};
  if (cfg) c = *cfg;
  if (!c.factor_bytes) c.factor_bytes = 1ull << 30;
  if (!c.max_jobs) c.max_jobs = 4096;
  if (c.max_jobs > batch_max_slots())
    return set_err(PPS_ERR_INVALID_PARAM, "max_jobs above %u", batch_max_slots());
  if (!c.wave_segments || c.wave_segments > batch_wave_segments(nullptr))
    c.wave_segments = (uint32_t)batch_wave_segments(nullptr);
  if (!c.wave_work) c.wave_work = 40000000000ull;
  pps_engine* e = nullptr;
  int rc = pps_engine_create(device, &e);
  if (rc) return rc;
  if ((rc = batch_prepare(e))) {
    pps_engine_destroy(e);
    return rc;
  }
  pps_server* s = new pps_server();
  s->e = e;
  s->cfg = c;
  for (uint32_t i = c.max_jobs; i > 0; --i) s->free_slots.push_back(i - 1);
  try {
    s->worker = std::thread(serve, s);
  } catch (...) {
    pps_engine_destroy(e);
    delete s;
    return set_err(PPS_ERR_INSUFFICIENT_RESOURCE, "worker thread");
  }
  *out = s;
  return PPS_OK;
}

extern "C" int pps_server_destroy(pps_server* s) {
  if (!s) return PPS_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  if (s->worker.joinable()) s->worker.join();
  pps_engine_destroy(s->e);
  s->cv_done.notify_all();
  delete s;
  return PPS_OK;
}

extern "C" int pps_job_submit(pps_server* s, const pps_job_params* jp, uint64_t* id) {
  if (!s || !jp || !id) return set_err(PPS_ERR_INVALID_PARAM, "null argument");
  if (jp->step < 1 || jp->step > 32 || jp->pmin <= (1ull << 32) || jp->pmax <= jp->pmin ||
      jp->nmax <= jp->nmin || jp->kmax < jp->kmin)
    return set_err(PPS_ERR_INVALID_PARAM, "job not normalized");
  auto j = std::make_unique<JobRec>();
  j->jp = *jp;
  j->reserve = job_reservation(*jp);
  j->t_submit = Clock::now();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return set_err(PPS_ERR_CANCELLED, "server stopping");
    s->st.submitted++;
    if (j->reserve > s->cfg.factor_bytes) {
      s->st.refused++;
      return set_err(PPS_ERR_INSUFFICIENT_RESOURCE,
                     "job needs %llu bytes of candidate buffers, the server's budget is %llu",
                     (unsigned long long)j->reserve, (unsigned long long)s->cfg.factor_bytes);
    }
    j->id = s->next_id++;
    *id = j->id;
    s->queue.push_back(j->id);
    s->jobs[j->id] = std::move(j);
  }
  s->cv_work.notify_one();
  return PPS_OK;
}

extern "C" int pps_job_cancel(pps_server* s, uint64_t id) {
  if (!s) return set_err(PPS_ERR_INVALID_PARAM, "null server");
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->jobs.find(id);
    if (it == s->jobs.end()) return set_err(PPS_ERR_NOT_FOUND, "no job %llu", (unsigned long long)id);
    JobRec* j = it->second.get();
    if (j->state == PPS_JOB_DONE || j->state == PPS_JOB_FAILED) return PPS_OK;
    if (j->state == PPS_JOB_QUEUED) {
      s->queue.erase(std::find(s->queue.begin(), s->queue.end(), id));
      j->state = PPS_JOB_FAILED;
      j->status = PPS_ERR_CANCELLED;
      j->t_done = Clock::now();
      s->st.failed++;
    } else {
      j->cancel = true;  // the worker retires it after the wave in flight
    }
  }
  s->cv_work.notify_one();
  s->cv_done.notify_all();
  return PPS_OK;
}

extern "C" int pps_job_poll(pps_server* s, uint64_t id, int* state) {
  if (!s || !state) return set_err(PPS_ERR_INVALID_PARAM, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end()) return set_err(PPS_ERR_NOT_FOUND, "no job %llu", (unsigned long long)id);
  *state = it->second->state;
  return PPS_OK;
}

extern "C" int pps_job_wait(pps_server* s, uint64_t id, double timeout_s, pps_factor* out, size_t cap,
                            size_t* nout, pps_job_result* res) {
  if (!s) return set_err(PPS_ERR_INVALID_PARAM, "null server");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end()) return set_err(PPS_ERR_NOT_FOUND, "no job %llu", (unsigned long long)id);
  JobRec* j = it->second.get();
  auto done = [&] { return j->state == PPS_JOB_DONE || j->state == PPS_JOB_FAILED || s->stop; };
  if (timeout_s < 0) {
    s->cv_done.wait(lk, done);
  } else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), done)) {
    return set_err(PPS_ERR_TIMEOUT, "job %llu not finished", (unsigned long long)id);
  }
  if (j->state != PPS_JOB_DONE && j->state != PPS_JOB_FAILED)
    return set_err(PPS_ERR_CANCELLED, "server stopping");
  const size_t nf = j->factors.size();
  if (nout) *nout = nf;
  if (res) {
    memset(res, 0, sizeof *res);
    res->primes = j->primes;
    res->prime_sum = j->sum;
    res->factors = nf;
    res->latency_ms = ms_between(j->t_submit, j->t_done);
    res->status = j->status;
  }
  if (!out) return PPS_OK;  // size query: the job stays for a later call
  if (nf > cap) return set_err(PPS_ERR_OVERFLOW, "%zu factors, buffer holds %zu", nf, cap);
  if (nf) memcpy(out, j->factors.data(), nf * sizeof(pps_factor));
  const int status = j->status;
  s->jobs.erase(it);
  if (status) return set_err(status, "job %llu failed", (unsigned long long)id);
  return PPS_OK;
}

extern "C" int pps_job_checkpoint(pps_server* s, uint64_t id, pps_factor* out, size_t cap, size_t* nout,
                                  pps_checkpoint* c) {
  if (!s) return set_err(PPS_ERR_INVALID_PARAM, "null server");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end()) return set_err(PPS_ERR_NOT_FOUND, "no job %llu", (unsigned long long)id);
  const JobRec* j = it->second.get();
  const size_t nf = j->factors.size();
  if (nout) *nout = nf;
  if (c) {
    memset(c, 0, sizeof *c);
    c->pmin = j->jp.pmin;
    c->p = j->state == PPS_JOB_QUEUED ? j->jp.pmin : j->done_p;
    c->count = j->primes;
    c->sum = j->sum;
    c->nmin = j->jp.nmin;
    c->nmax = j->jp.nmax;
    c->factor_count = (uint32_t)nf;
  }
  if (out) {
    if (nf > cap) return set_err(PPS_ERR_OVERFLOW, "%zu factors, buffer holds %zu", nf, cap);
    if (nf) memcpy(out, j->factors.data(), nf * sizeof(pps_factor));
  }
  return PPS_OK;
}

extern "C" int pps_server_get_stats(pps_server* s, pps_server_stats* st) {
  if (!s || !st) return set_err(PPS_ERR_INVALID_PARAM, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  *st = s->st;
  st->queued = s->queue.size();
  st->running = s->active.size();
  st->reserved_bytes = s->reserved;
  uint32_t work = 0, unroll = 0;
  batch_tuning(s->e, &work, &unroll);
  st->chunk = work;
  st->unroll = unroll;
  if (!s->latencies.empty()) {
    std::vector<double> v = s->latencies;
    std::sort(v.begin(), v.end());
    auto rank = [&](double q) {  // nearest-rank percentile
      size_t r = (size_t)ceil(q * (double)v.size());
      if (r < 1) r = 1;
      return v[std::min(r, v.size()) - 1];
    };
    st->p50_ms = rank(0.50);
    st->p99_ms = rank(0.99);
  }
  return PPS_OK;
}
