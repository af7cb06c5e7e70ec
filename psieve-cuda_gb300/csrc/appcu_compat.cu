// appcu_compat.cu -- libppsgpu_appcu.so: the reference's pps/appcu.h ABI on top
// of libppsgpu.so (declarations and contract in include/appcu_compat.h).
//
// Host side only.  Each host thread th gets its own engine and a worker thread
// that runs the walk, so check_ns() returns at once and the caller's CPU work
// overlaps the GPU exactly as with the reference (pps/app.c:1224-1250).
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <condition_variable>
#include <mutex>
#include <thread>
#include <vector>

#include "appcu_compat.h"
#include "ppsgpu.h"

// ---- symbols the reference's main.c / pps/app.c define (main.h:51-60,
// pps/app.h:85-96).  The struct layout must match pps/app.h:85-89.
extern "C" {
struct n_subsection {
  unsigned int n_subsection_start[9];
  unsigned int* first_n_subsection;
};
extern struct n_subsection* thread_subsections;
extern unsigned int nmin, nmax;
extern int search_proth;
extern uint64_t kmax, kmin;
extern int num_threads;
extern uint64_t pmin, pmax;
void bmsg(const char* msg);
void bexit(int status);
char* bmprefix();

unsigned int ld_nstep;
int ld_bbits;
uint64_t ld_r0;
}

namespace {

constexpr int kMaxThreads = 64;
constexpr unsigned kBlock = 128;  // pps/appcu.h:14 BLOCKSIZE

struct CompatThread {
  int th = 0;
  pps_engine* eng = nullptr;
  int sms = 0;
  std::vector<uint64_t> P;
  unsigned count = 0;
  std::vector<pps_hit> hits;
  size_t nhits = 0;
  int rc = PPS_OK;
  std::thread worker;
  bool running = false;
  unsigned start[9] = {};
  int nsub = 1;
};

CompatThread* g_threads[kMaxThreads];
thread_local CompatThread* t_self = nullptr;

int lg2(uint64_t v) {
  int r = 0;
  while (v >>= 1) r++;
  return r;
}

void fatal(const char* what) {
  fprintf(stderr, "%s%s: %s\n", bmprefix(), what, pps_last_error());
  bexit(EXIT_FAILURE);
}

pps_job_params job_from_globals() {
  pps_job_params jp;
  memset(&jp, 0, sizeof jp);
  jp.pmin = pmin;
  jp.pmax = pmax;
  jp.kmin = kmin;
  jp.kmax = kmax;
  jp.nmin = nmin;
  jp.nmax = nmax;
  jp.sign = search_proth == 1 ? 1 : -1;
  jp.kstep = 2;
  jp.koffset = 1;
  jp.qmax = 0;
  jp.nstep = ld_nstep;
  jp.step = ld_nstep < 32 ? ld_nstep : 32;
  return jp;
}

void run_walk(CompatThread* s) {
  const pps_job_params jp = job_from_globals();
  size_t cap = s->hits.size();
  for (;;) {
    size_t n = 0;
    s->rc = pps_check_primes_raw(s->eng, &jp, s->P.data(), s->count, s->hits.data(), cap, &n);
    if (s->rc == PPS_ERR_OVERFLOW && n > cap) {
      cap = n;
      s->hits.resize(cap);
      continue;
    }
    s->nhits = n;
    return;
  }
}

void join(CompatThread* s) {
  if (s && s->running) {
    s->worker.join();
    s->running = false;
  }
}

}  // namespace

// pps/appcu.cu:155-209: nstep clamp, the 2^(64-nstep) <= pmin rule, 32-forcing,
// nmin >= 64, and the r0 / bbits constants.
extern "C" void cuda_init(void) {
  if (ld_nstep > (nmax - nmin + 1)) ld_nstep = nmax - nmin + 1;
  if ((((uint64_t)1) << (64 - ld_nstep)) > pmin) {
    bmsg("Error: pmin is not large enough (or nmax is close to nmin).\n");
    bexit(PPS_ERR_INVALID_PARAM);
  }
  if (ld_nstep >= 32 && ld_nstep < 48 && (((uint64_t)1) << 32) <= pmin) {
    if (ld_nstep != 32) printf("nstep changed to 32\n");
    ld_nstep = 32;
  } else {
    printf("Didn't change nstep from %u\n", ld_nstep);
  }
  ld_bbits = lg2(nmin);
  if (ld_bbits < 6) {
    fprintf(stderr, "%sError: nmin too small at %d (must be at least 64).\n", bmprefix(), nmin);
    bexit(PPS_ERR_INVALID_PARAM);
  }
  ld_r0 = ((uint64_t)1) << (64 - (nmin >> (ld_bbits - 5)));
  ld_bbits = ld_bbits - 6;
}

extern "C" unsigned int cuda_app_init(int gpuno, int th, unsigned int cthread_count) {
  if (th < 0 || th >= kMaxThreads) return 0;
  if (pmin <= ((uint64_t)1) << 32) {
    bmsg("Error: PMin is too small, <= 2^32!\n");
    bexit(PPS_ERR_INVALID_PARAM);
  }
  CompatThread* s = new CompatThread();
  s->th = th;
  if (pps_engine_create(gpuno, &s->eng) != PPS_OK) {
    fprintf(stderr, "%sGPU %d not usable: %s\n", bmprefix(), gpuno, pps_last_error());
    delete s;
    return 0;
  }
  const int sms = pps_engine_sm_count(s->eng);
  s->sms = sms > 0 ? sms : 1;
  // batch size: pps/appcu.cu:257-266 (2048 threads per SM on cc >= 2, or the
  // -m value rounded to BLOCKSIZE, times the SM count)
  if (cthread_count == 0) {
    cthread_count = 2048;
  } else if (cthread_count < kBlock) {
    cthread_count *= kBlock;
  } else {
    cthread_count -= cthread_count % kBlock;
  }
  cthread_count *= (unsigned)s->sms;
  s->P.resize(cthread_count);
  s->hits.resize(1u << 16);

  // n-subsections on the nstep grid from nmin (so the CPU re-walk of each
  // subsection stops exactly at the next one's first n): at most 8 equal parts.
  unsigned* st = thread_subsections[th].n_subsection_start;
  uint64_t width = ((uint64_t)(nmax - nmin) + 7) / 8;
  width = (width + ld_nstep - 1) / ld_nstep * ld_nstep;
  if (width == 0) width = ld_nstep;
  unsigned bounds[9];
  int nb = 0;
  bounds[nb++] = nmin;
  for (int i = 1; i < 8; ++i) {
    const uint64_t b = (uint64_t)nmin + (uint64_t)i * width;
    if (b >= nmax) break;
    bounds[nb++] = (unsigned)b;
  }
  // nb subsections: bit j covers [start[j+1], start[j]); start[0] = nmax
  s->nsub = nb;
  st[0] = nmax;
  for (int j = 1; j <= 8; ++j) st[j] = j <= nb ? bounds[nb - j] : nmin;
  thread_subsections[th].first_n_subsection = &st[nb - 1];
  memcpy(s->start, st, sizeof s->start);
  g_threads[th] = s;
  t_self = s;
  return cthread_count;
}

extern "C" void check_ns(const uint64_t* P, const unsigned int cthread_count, const int th) {
  CompatThread* s = (th >= 0 && th < kMaxThreads) ? g_threads[th] : nullptr;
  if (!s) {
    bmsg("check_ns: thread not initialised\n");
    bexit(EXIT_FAILURE);
  }
  t_self = s;
  join(s);
  if (P) {
    if (s->P.size() < cthread_count) s->P.resize(cthread_count);
    memcpy(s->P.data(), P, (size_t)cthread_count * sizeof(uint64_t));
  }
  s->count = cthread_count;
  s->running = true;
  s->worker = std::thread(run_walk, s);
}

extern "C" void get_factors_found(unsigned char* factor_found, const unsigned int cthread_count,
                                  const uint64_t start_t, int* check_ns_delay) {
  (void)start_t;
  (void)check_ns_delay;
  CompatThread* s = t_self;
  if (!s) {
    bmsg("get_factors_found: no walk started on this thread\n");
    bexit(EXIT_FAILURE);
  }
  join(s);
  if (s->rc != PPS_OK) fatal("Cuda error: getting factors found");
  memset(factor_found, 0, cthread_count);
  for (size_t i = 0; i < s->nhits; ++i) {
    const pps_hit& h = s->hits[i];
    if (h.idx >= cthread_count) continue;
    for (int j = 0; j < s->nsub; ++j) {
      if (h.n >= s->start[j + 1] && h.n < s->start[j]) {
        factor_found[h.idx] |= (unsigned char)(1u << j);
        break;
      }
    }
  }
}

extern "C" void cuda_finalize(void) {
  CompatThread* s = t_self;
  if (!s) return;
  join(s);
  pps_engine_destroy(s->eng);
  g_threads[s->th] = nullptr;
  delete s;
  t_self = nullptr;
}
