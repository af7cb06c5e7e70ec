// pps_engine.cu -- host side of libppsgpu.so: the C ABI of include/ppsgpu.h.
//
// One engine = one GPU + one CUDA stream + device buffers that are grown on
// demand and reused across calls.  A job is processed in p-range batches:
//   device sieve (primes + Montgomery constants to HBM) -> walk kernel (raw
//   hits appended to a device buffer) ; after the last batch the filter kernel
//   applies the output rule and the survivors are copied to the caller.
// Reference call stack this replaces (Ken-g6/PSieve-CUDA): main.c:736-783
// (host sieve feeding batches) -> pps/app.c:1224-1250 -> pps/appcu.cu:1205-1308
// (check_ns / get_factors_found) -> pps/app.c:1197-1219 (CPU re-walk) ->
// pps/app.c:159-186 (filter) -> pps/app.c:124-148 (report).
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <vector>

#include "pps_engine_impl.h"
#include "pps_internal.h"
#include "ppsgpu.h"

using namespace pps;

// --------------------------------------------------------------- errors
static thread_local char g_err[512];

int set_err(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
  return code;
}

extern "C" const char* pps_last_error(void) { return g_err; }

// ---------------------------------------------------- fault injection
// After `skip` more device-buffer allocations succeed, the next `count` fail
// (host side only: no kernel is launched or disturbed); used to test that every
// error path leaves the engine, the batched form and the serving loop usable.
static std::mutex g_fail_mu;
static long g_fail_skip = 0, g_fail_pending = 0, g_fail_done = 0;

bool alloc_fault_injected() {
  std::lock_guard<std::mutex> lk(g_fail_mu);
  if (g_fail_pending <= 0) return false;
  if (g_fail_skip > 0) {
    --g_fail_skip;
    return false;
  }
  --g_fail_pending;
  ++g_fail_done;
  return true;
}

extern "C" int pps_debug_fail_allocs(int skip, int count) {
  std::lock_guard<std::mutex> lk(g_fail_mu);
  const long done = g_fail_done;
  g_fail_skip = skip > 0 ? skip : 0;
  g_fail_pending = count > 0 ? count : 0;
  g_fail_done = 0;
  return (int)done;
}
static std::atomic<uint32_t> g_dbg_qcap{(uint32_t)WALK_QUEUE_CAP}, g_dbg_hitcap{0};

uint32_t debug_queue_cap() { return g_dbg_qcap.load(std::memory_order_relaxed); }
uint32_t debug_first_hit_cap() { return g_dbg_hitcap.load(std::memory_order_relaxed); }

extern "C" int pps_debug_limits(int warp_queue, uint32_t first_candidates) {
  if (warp_queue > WALK_QUEUE_CAP) return set_err(PPS_ERR_INVALID_PARAM, "warp queue above %d", WALK_QUEUE_CAP);
  g_dbg_qcap = warp_queue < 0 ? (uint32_t)WALK_QUEUE_CAP : (uint32_t)warp_queue;
  g_dbg_hitcap = first_candidates;
  return PPS_OK;
}

extern "C" const char* pps_version(void) { return "ppsgpu-0.1 (sm_103a)"; }

// ------------------------------------------------------------ normalize
static int lg2u64(uint64_t v) {
  int r = 0;
  while (v >>= 1) r++;
  return r;
}

extern "C" int pps_normalize(const pps_job_spec* in, pps_job_params* o) {
  if (!in || !o) return set_err(PPS_ERR_INVALID_PARAM, "null argument");
  const uint64_t PMAX_MAX = 1ull << 62;  // main.h:43
  memset(o, 0, sizeof *o);
  uint64_t pmin = in->pmin, pmax = in->pmax, kmin = in->kmin, kmax = in->kmax;
  uint32_t nmin = in->nmin, nmax = in->nmax, qmax = in->qmax;
  int32_t sign = in->sign ? in->sign : 1;
  if (sign != 1 && sign != -1 && sign != PPS_SIGN_TWIN)
    return set_err(PPS_ERR_INVALID_PARAM, "sign must be +1, -1 or PPS_SIGN_TWIN");
  const bool twin = sign == PPS_SIGN_TWIN;
  // pps/app.c:53-58 KSTEP/KOFFSET: 6/3 in the twin (SEARCH_TWIN) build, else 2/1
  uint32_t kstep = in->kstep ? in->kstep : (twin ? 6u : 2u);
  uint32_t koffset = in->koffset ? in->koffset : (twin ? 3u : 1u);
  // main.c:916-931
  if (pmin < 3) pmin = 3;
  if (pmax > PMAX_MAX) pmax = PMAX_MAX;
  if (pmin >= pmax) {
    if (pmax == 0 && pmin < PMAX_MAX - 1000000000ull)
      pmax = pmin + 1000000000ull;
    else
      return set_err(PPS_ERR_INVALID_PARAM, "pmax must be greater than pmin");
  }
  // main.c:971-972, sieve.c:98-110
  if (qmax == 0) qmax = 1u << 31;
  if ((uint64_t)qmax * qmax > pmax) qmax = (uint32_t)sqrt((double)pmax);
  if (qmax < 61) qmax = 61;
  // pps/app.c:657-700
  if (kmin == 0 || kmax == 0)
    return set_err(PPS_ERR_INVALID_PARAM, "Please specify an input file or all of kmin, kmax, and nmax");
  if (kmin > kmax) return set_err(PPS_ERR_INVALID_PARAM, "kmin <= kmax is required");
  if (kmax >= pmin) return set_err(PPS_ERR_INVALID_PARAM, "kmax < pmin is required");
  if (kmax - kmin >= (3ull << 36)) return set_err(PPS_ERR_INVALID_PARAM, "kmax-kmin < 3*2^36 is required");
  if (nmin == 0) nmin = (uint32_t)(2 * lg2u64(pmin) - lg2u64(kmax) - 1);
  if (nmax == 0) nmax = nmin;
  if (nmin > nmax) return set_err(PPS_ERR_INVALID_PARAM, "nmin <= nmax is required");
  // pps/app.c:703-712
  kmin = (kmin / kstep) * kstep + koffset;
  kmax = (kmax / kstep) * kstep + koffset;
  uint32_t nstep = 1;
  while ((kmax << nstep) < pmin) nstep++;
  // pps/appcu.cu:158-204
  if (nstep > nmax - nmin + 1) nstep = nmax - nmin + 1;
  if ((1ull << (64 - nstep)) > pmin)
    return set_err(PPS_ERR_INVALID_PARAM, "pmin is not large enough (or nmax is close to nmin)");
  if (twin) nstep--;  // pps/appcu.cu:177-180: twin steps overlap by one n
  if (nstep >= 32 && nstep < 48 && (1ull << 32) <= pmin) nstep = 32;
  if (lg2u64(nmin) < 6) return set_err(PPS_ERR_INVALID_PARAM, "nmin too small at %u (must be at least 64)", nmin);
  // pps/appcu.cu:236-239
  if (pmin <= (1ull << 32)) return set_err(PPS_ERR_INVALID_PARAM, "PMin is too small, <= 2^32");
  o->pmin = pmin;
  o->pmax = pmax;
  o->kmin = kmin;
  o->kmax = kmax;
  o->nmin = nmin;
  o->nmax = nmax;
  o->sign = sign;
  o->kstep = kstep;
  o->koffset = koffset;
  o->qmax = qmax;
  o->nstep = nstep;
  o->step = nstep < 32 ? nstep : 32;
  return PPS_OK;
}

// ---------------------------------------------------------------- engine

static void free_engine(pps_engine* e) {
  if (!e) return;
  cudaSetDevice(e->device);
  e->base_q.release();
  e->seed_q.release();
  e->in_keys.release();
  e->bitmap.release();
  e->seg_count.release();
  e->seg_off.release();
  e->P.release();
  e->Pinv.release();
  e->totals.release();
  e->hits.release();
  e->factors.release();
  e->counters.release();
  e->small_q.release();
  e->presieve.release();
  e->sieve_res.release();
  e->probe_sink.release();
  batch_state_free(e);
  if (e->h_pinned) cudaFreeHost(e->h_pinned);
  for (auto& v : e->ev)
    if (v) cudaEventDestroy(v);
  if (e->st) cudaStreamDestroy(e->st);
  delete e;
}

extern "C" void pps_engine_destroy(pps_engine* e) { free_engine(e); }

static std::vector<uint32_t> host_odd_primes(uint32_t limit) {
  std::vector<uint8_t> comp(limit + 1, 0);
  std::vector<uint32_t> r;
  for (uint32_t i = 3; i <= limit; i += 2) {
    if (comp[i]) continue;
    r.push_back(i);
    for (uint64_t j = (uint64_t)i * i; j <= limit; j += 2ull * i) comp[j] = 1;
  }
  return r;
}

extern "C" int pps_engine_create(int device, pps_engine** out) {
  if (!out) return set_err(PPS_ERR_INVALID_PARAM, "null out");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return set_err(PPS_ERR_NO_DEVICE, "no CUDA device available");
  }
  if (device < 0) device = 0;
  if (device >= ndev) return set_err(PPS_ERR_NO_DEVICE, "device %d not present (%d devices)", device, ndev);
  pps_engine* e = new pps_engine();
  e->device = device;
  int rc = PPS_OK;
  do {
    if (cudaSetDevice(device) != cudaSuccess) { rc = set_err(PPS_ERR_CUDA, "cudaSetDevice failed"); break; }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) { rc = set_err(PPS_ERR_CUDA, "cudaGetDeviceProperties failed"); break; }
    e->num_sms = prop.multiProcessorCount;
    if (cudaStreamCreateWithFlags(&e->st, cudaStreamNonBlocking) != cudaSuccess) { rc = set_err(PPS_ERR_CUDA, "stream"); break; }
    for (auto& v : e->ev)
      if (cudaEventCreate(&v) != cudaSuccess) { rc = set_err(PPS_ERR_CUDA, "event"); break; }
    if (rc) break;
    if (cudaMallocHost(&e->h_pinned, 16 * sizeof(uint64_t)) != cudaSuccess) { rc = set_err(PPS_ERR_CUDA, "pinned"); break; }
    // odd primes 3..32749 for the output filter (pps/factor_proth.c:26-42 range)
    std::vector<uint32_t> sp = host_odd_primes(32767);
    std::vector<uint16_t> sp16(sp.begin(), sp.end());
    e->nsmall = (uint32_t)sp16.size();
    if ((rc = e->small_q.ensure(sp16.size()))) break;
    if (cudaMemcpy(e->small_q.p, sp16.data(), sp16.size() * 2, cudaMemcpyHostToDevice) != cudaSuccess) { rc = set_err(PPS_ERR_CUDA, "copy"); break; }
    {
      std::vector<uint32_t> pre(PRESIEVE_WORDS);
      presieve_table(pre.data());
      if ((rc = e->presieve.ensure(PRESIEVE_WORDS))) break;
      if (cudaMemcpy(e->presieve.p, pre.data(), PRESIEVE_WORDS * 4, cudaMemcpyHostToDevice) != cudaSuccess) { rc = set_err(PPS_ERR_CUDA, "copy"); break; }
    }
    e->host_seed = host_odd_primes(SEG_BITS - 1);
    if ((rc = e->seed_q.ensure(e->host_seed.size()))) break;
    if (cudaMemcpy(e->seed_q.p, e->host_seed.data(), e->host_seed.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess) { rc = set_err(PPS_ERR_CUDA, "copy"); break; }
    if ((rc = e->counters.ensure(8))) break;
    if ((rc = e->totals.ensure(4))) break;
  } while (0);
  if (rc) {
    free_engine(e);
    return rc;
  }
  *out = e;
  return PPS_OK;
}

extern "C" uint64_t pps_engine_device_bytes(const pps_engine* e) {
  if (!e) return 0;
  return e->base_q.bytes() + e->seed_q.bytes() + e->bitmap.bytes() + e->seg_count.bytes() +
         e->seg_off.bytes() + e->P.bytes() + e->Pinv.bytes() + e->totals.bytes() + e->hits.bytes() +
         e->factors.bytes() + e->counters.bytes() + e->small_q.bytes() + e->probe_sink.bytes() +
         e->presieve.bytes() + e->sieve_res.bytes();
}

extern "C" int pps_engine_sm_count(const pps_engine* e) { return e ? e->num_sms : 0; }

extern "C" int pps_engine_set_batch_span(pps_engine* e, uint64_t span) {
  if (!e || span < 2ull * SEG_BITS) return set_err(PPS_ERR_INVALID_PARAM, "batch span too small");
  e->batch_span = span & ~1ull;
  return PPS_OK;
}

extern "C" int pps_engine_set_variant(pps_engine* e, int v) {
  if (!e || v < -1 || v >= PPS_NUM_VARIANTS) return set_err(PPS_ERR_INVALID_PARAM, "bad variant %d", v);
  e->forced_variant = v;
  return PPS_OK;
}

extern "C" int pps_engine_set_split(pps_engine* e, int split) {
  if (!e || (split != 0 && split != 1 && split != 2 && split != 4 && split != 8))
    return set_err(PPS_ERR_INVALID_PARAM, "bad split %d (0, 1, 2, 4 or 8)", split);
  e->forced_split = split;
  return PPS_OK;
}

extern "C" uint64_t pps_engine_launches(const pps_engine* e) { return e ? e->launches : 0; }

extern "C" const char* pps_walk_variant_name(int v) { return walk_variant_name(v); }

// ----------------------------------------------------------------- sieve
uint32_t isqrt64(uint64_t x) {
  uint64_t r = (uint64_t)sqrt((double)x);
  while (r * r > x) r--;
  while ((r + 1) * (r + 1) <= x) r++;
  return (uint32_t)r;
}

static int sieve_batch(pps_engine* e, uint64_t lo, uint64_t hi, const uint32_t* dq, uint32_t nq,
                       uint32_t nq_tiny, uint32_t nq_seg, uint64_t* out64, uint64_t* pinv64,
                       uint32_t* out32) {
  SieveBatch b;
  b.lo = lo | 1ull;
  if (hi <= b.lo) return PPS_OK;
  b.nbits = (hi - b.lo + 1) / 2;
  b.nseg = (uint32_t)((b.nbits + SEG_BITS - 1) / SEG_BITS);
  int rc;
  if ((rc = e->bitmap.ensure((size_t)b.nseg * SEG_WORDS))) return rc;
  if ((rc = e->seg_count.ensure(b.nseg))) return rc;
  if ((rc = e->seg_off.ensure(b.nseg))) return rc;
  b.q = dq;
  b.nq = nq;
  b.nq_tiny = nq_tiny;
  b.nq_seg = nq_seg;
  b.bitmap = e->bitmap.p;
  b.seg_count = e->seg_count.p;
  b.seg_off = e->seg_off.p;
  b.d_total = e->totals.p;
  b.presieve = e->presieve.p;
  // residues in 32 bits need seg * (2 SEG_BITS mod q) + (lo mod q) < 2^32
  if (nq_seg > nq_tiny && b.nseg <= 8192u) {
    if ((rc = e->sieve_res.ensure(2 * (size_t)(nq_seg - nq_tiny)))) return rc;
    b.res = e->sieve_res.p;
  }
  CU(cudaMemsetAsync(e->totals.p, 0, 2 * sizeof(uint64_t), e->st));
  e->launches += launch_sieve_batch(b, out64, pinv64, out32, e->st);
  CU(cudaGetLastError());
  return PPS_OK;
}

static uint32_t count_le(const std::vector<uint32_t>& v, uint32_t x) {
  return (uint32_t)(std::upper_bound(v.begin(), v.end(), x) - v.begin());
}


// Make sure the device holds all odd primes <= limit and fill the counts.
// Returns 1 when the host-made seed table (odd primes < SEG_BITS) serves,
// 0 when the device-made table base_q does, or a negative error.
static int ensure_base(pps_engine* e, uint32_t limit, BaseTable* bt) {
  if (limit < 3) limit = 3;
  if (limit < SEG_BITS) {
    // straight from the host seed list
    uint32_t n = count_le(e->host_seed, limit);
    bt->nq = n;
    bt->nq_tiny = count_le(e->host_seed, TINY_Q_LIMIT - 1);
    if (bt->nq_tiny > n) bt->nq_tiny = n;
    bt->nq_seg = std::min(n, count_le(e->host_seed, SEG_BITS - 1));
    return 1;
  }
  if (e->base_limit < limit) {
    // odd primes in [3, limit] with seeds <= sqrt(limit) (all < 2^16)
    const uint32_t root = isqrt64(limit);
    const uint32_t ns = count_le(e->host_seed, root);
    const uint32_t ns_tiny = std::min(ns, count_le(e->host_seed, TINY_Q_LIMIT - 1));
    // capacity: pi(limit) < 1.26 limit / ln(limit)
    const size_t cap = (size_t)(1.3 * limit / log((double)limit)) + 1024;
    int rc;
    // the table is rebuilt from scratch: a failure below leaves no table
    e->base_limit = 0;
    e->base_count = 0;
    e->base_le.clear();
    if ((rc = e->base_q.ensure(cap))) return rc;
    uint64_t filled = 0;
    const uint64_t span = 1ull << 31;
    for (uint64_t a = 3; a <= limit; a += span) {
      uint64_t b = std::min<uint64_t>((uint64_t)limit + 1, a + span);
      if ((rc = sieve_batch(e, a, b, e->seed_q.p, ns, ns_tiny, ns, nullptr, nullptr,
                            e->base_q.p + filled)))
        return rc;
      CU(cudaMemcpyAsync(e->h_pinned, e->totals.p, 2 * sizeof(uint64_t), cudaMemcpyDeviceToHost, e->st));
      CU(cudaStreamSynchronize(e->st));
      filled += e->h_pinned[0];
    }
    e->base_limit = limit;
    e->base_count = (uint32_t)filled;
  }
  // counts for `limit` within the (possibly larger) table: a binary search on
  // the device values through small copies, remembered per limit until the
  // table is rebuilt
  uint32_t n = e->base_count;
  if (e->base_limit > limit) {
    auto it = e->base_le.find(limit);
    if (it != e->base_le.end()) {
      n = it->second;
    } else {
      // the first index with q > limit, by a binary search on the device
      uint32_t* d_n = (uint32_t*)(e->totals.p + 2);  // a free word of the totals
      CU(launch_count_le(e->base_q.p, e->base_count, limit, d_n, e->st));
      e->launches++;
      CU(cudaMemcpyAsync(e->h_pinned, d_n, sizeof(uint32_t), cudaMemcpyDeviceToHost, e->st));
      CU(cudaStreamSynchronize(e->st));
      n = ((uint32_t*)e->h_pinned)[0];
      e->base_le[limit] = n;
    }
  }
  bt->nq = n;
  bt->nq_tiny = std::min(n, count_le(e->host_seed, TINY_Q_LIMIT - 1));
  bt->nq_seg = std::min(n, count_le(e->host_seed, SEG_BITS - 1));
  return 0;
}

int prepare_sieving_primes(pps_engine* e, uint32_t qmax, uint64_t pmax, const uint32_t** dq,
                                  BaseTable* bt) {
  // only q with q*q < pmax can matter
  uint32_t lim = qmax;
  const uint32_t r = isqrt64(pmax - 1);
  if (r < lim) lim = r;
  int which = ensure_base(e, lim, bt);
  if (which < 0) return which;
  *dq = which == 1 ? e->seed_q.p : e->base_q.p;
  return PPS_OK;
}

extern "C" int pps_sieve_range(pps_engine* e, uint64_t lo, uint64_t hi, uint32_t qmax, uint64_t* out,
                               size_t cap, size_t* count, uint64_t* sum) {
  if (!e || hi <= lo || lo < 3) return set_err(PPS_ERR_INVALID_PARAM, "bad range");
  CU(cudaSetDevice(e->device));
  if (qmax == 0) {
    qmax = 1u << 31;
    if ((uint64_t)qmax * qmax > hi) qmax = (uint32_t)sqrt((double)hi);
  }
  const uint32_t* dq;
  BaseTable bt;
  int rc = prepare_sieving_primes(e, qmax, hi, &dq, &bt);
  if (rc) return rc;
  size_t total = 0;
  uint64_t s = 0;
  for (uint64_t a = lo | 1ull; a < hi; a += e->batch_span) {
    uint64_t b = std::min(hi, a + e->batch_span);
    const uint64_t nbits = (b - a + 1) / 2;
    if ((rc = e->P.ensure(nbits / 2 + 64))) return rc;  // density of odd primes < 1/2 above 2^5
    if ((rc = sieve_batch(e, a, b, dq, bt.nq, bt.nq_tiny, bt.nq_seg, e->P.p, nullptr, nullptr))) return rc;
    CU(cudaMemcpyAsync(e->h_pinned, e->totals.p, 2 * sizeof(uint64_t), cudaMemcpyDeviceToHost, e->st));
    CU(cudaStreamSynchronize(e->st));
    const uint64_t n = e->h_pinned[0];
    s += e->h_pinned[1];
    if (out && total < cap) {
      size_t m = std::min<size_t>(n, cap - total);
      CU(cudaMemcpy(out + total, e->P.p, m * sizeof(uint64_t), cudaMemcpyDeviceToHost));
    }
    total += n;
  }
  if (count) *count = total;
  if (sum) *sum = s;
  if (out && total > cap) return set_err(PPS_ERR_OVERFLOW, "%zu primes, buffer holds %zu", total, cap);
  return PPS_OK;
}

// ------------------------------------------------------------------- walk
// t = (lg p + kb - 1) / 2 balances P(K < 2^t) ~ 2^(t - lg p) against
// P(low t+1-kb bits zero) = 2^-(t+1-kb) (kmax < 2^kb); it stays exact while
// K < p <= 2^(t+32), so that a funnel shift sees all of K >> t.
void pps::small_p_window_of(const pps_job_params* jp, uint32_t* t_out, uint32_t* mask_out) {
  *t_out = 32;
  *mask_out = 0;
  const int kb = lg2u64(jp->kmax) + 1;
  const int lp = lg2u64(jp->pmin);
  if (lp + kb - 64 >= 0) return;
  const int B = lg2u64(jp->pmax - 1) + 1;  // every p, and so every K, is below 2^B
  int t = (lp + kb - 1) / 2;
  t = std::max(t, B - 32);
  t = std::max(t, kb);
  if (t >= 32) return;
  *t_out = (uint32_t)t;
  *mask_out = (1u << (t + 1 - kb)) - 1u;
}

static void fill_walk_args(const pps_job_params* jp, WalkArgs* a) {
  memset(a, 0, sizeof *a);
  a->kmin = jp->kmin;
  a->kmax = jp->kmax;
  a->nmin = jp->nmin;
  a->nmax = jp->nmax;
  a->step = jp->step;
  a->nsteps = (jp->nmax - jp->nmin + jp->step - 1) / jp->step;
  if (jp->nmax == jp->nmin) a->nsteps = 0;
  a->proth = jp->sign == 1 ? 1u : 0u;
  a->qcap = debug_queue_cap();
  // window pre-test parameters
  const int kb = lg2u64(jp->kmax) + 1;         // kmax < 2^kb
  const int lp = lg2u64(jp->pmin);
  int u = (lp + kb - 64) / 2;
  const int umin = kb > 32 ? kb - 32 : 0, umax = kb < 32 ? kb : 32;
  if (u < umin) u = umin;
  if (u > umax) u = umax;
  const int t = 32 + u - kb;
  a->win_hi = u >= 32 ? 0xffffffffu : ((1u << u) - 1u);
  a->win_mask = t >= 32 ? 0xffffffffu : ((1u << t) - 1u);
  a->kmax32 = jp->kmax < (1ull << 32) ? (uint32_t)jp->kmax : 0xffffffffu;
  a->bound_hi = jp->kmax < (1ull << 32) ? (uint32_t)(jp->kmax >> 1) : 0xffffffffu;
  pps::small_p_window_of(jp, &a->sh_t, &a->sh_mask);
  a->shift_ok = jp->step < 32 && ((jp->pmax - 1) >> (32 + jp->step)) == 0 ? 1u : 0u;
  {
    const int r = (int)jp->step + 1 - kb;  // a hit with i > s - kb has its low r bits zero
    a->sw_mask = r <= 0 ? 0u : (r >= 32 ? 0xffffffffu : (1u << r) - 1u);
  }
}

static int variant_ok(const pps_job_params* jp, int v) {
  const VariantTraits& t = walk_variant_traits(v);
  // the twin variants walk both sides of a twin job; every other variant one side
  const bool twin = jp->sign == PPS_SIGN_TWIN;
  if (twin != t.twin) return 0;
  if (t.lowbit && jp->kmax >= (1ull << 32)) return 0;  // low-bit test needs kmax < 2^32
  if (t.s32 && jp->step != 32) return 0;
  if (t.shifted || t.smallp || t.min_window) {
    WalkArgs a;
    fill_walk_args(jp, &a);
    if (t.shifted && !a.shift_ok) return 0;   // shifted chain: s < 32, p <= 2^(32+s)
    if (t.smallp && a.sh_t >= 32) return 0;   // small-p window
    if (t.min_window && a.win_hi != 0) return 0;  // running-minimum window: u == 0
  }
  if (t.bound) {  // single bound: kmax < 2^32, false-pass rate below 2^-12
    if (jp->kmax >= (1ull << 32)) return 0;
    if (jp->pmin / jp->kmax < (1ull << 43)) return 0;
  }
  return 1;
}

// The raw-candidate capacity of this attempt: the buffer's size, or less under
// pps_debug_limits.
static uint32_t hit_cap_now(const pps_engine* e) {
  size_t c = std::min<size_t>(e->hits.n, 0xffffffffu);
  if (e->hit_cap_limit && e->hit_cap_limit < c) c = e->hit_cap_limit;
  return (uint32_t)c;
}

static int run_walk(pps_engine* e, const pps_job_params* jp, int v, const uint64_t* dP, const uint64_t* dPinv,
                    const uint64_t* d_np, uint64_t np_max, uint32_t idx_base, uint32_t nsteps_cap,
                    uint32_t split = 1) {
  WalkArgs a;
  fill_walk_args(jp, &a);
  if (nsteps_cap && a.nsteps > nsteps_cap) a.nsteps = nsteps_cap;
  // threads per prime: queued walks only
  const VariantTraits& vt = walk_variant_traits(v);
  a.nsplit = vt.queued && split > 1 ? split : 1;
  a.P = dP;
  a.Pinv = dPinv;
  a.d_np = d_np;
  a.np = np_max;
  a.idx_base = idx_base;
  a.hits = e->hits.p;
  a.hit_count = e->counters.p;
  a.hit_cap = hit_cap_now(e);
  const int threads = walk_block_threads(v);
  int maxb = walk_max_blocks(v, threads, jp->step, e->num_sms);
  if (maxb <= 0) return set_err(PPS_ERR_CUDA, "walk variant %d unavailable", v);
  // queued walks: a warp covers 32 x per_thread primes of one n part
  const uint64_t wp = 32ull * (uint64_t)vt.per_thread;
  const uint64_t nvirt = vt.queued ? (np_max + wp - 1) / wp * 32ull * a.nsplit : np_max;
  uint64_t need = (nvirt + threads - 1) / threads;
  // The queued walks get one thread per prime (or per primes_per_thread): the block
  // scheduler then hands new primes to whichever SM has finished its blocks, so
  // every SM keeps its full complement of warps to the end (with a grid of one
  // resident wave that loops over the primes, the warps the scheduler favours
  // finish their share early and the SMs run the rest at reduced occupancy).
  // The older walks keep one resident wave (their ILP forms stride over it).
  const uint64_t cap = vt.queued ? 0x7fffffffull : (uint64_t)maxb;
  int blocks = (int)std::min<uint64_t>(cap, need ? need : 1);
  CU(launch_walk(v, a, blocks, threads, e->st));
  e->launches++;
  return PPS_OK;
}

namespace pps {
void walk_args_for_job(const pps_job_params* jp, WalkArgs* a) { fill_walk_args(jp, a); }
int walk_variant_exact(const pps_job_params* jp, int v) { return variant_ok(jp, v); }
int set_error_text(int code, const char* msg) { return set_err(code, "%s", msg); }
}  // namespace pps

// PPS_TUNE_LOG=1 in the environment prints the tuner's timings to stderr.
static bool tune_log() {
  static const bool on = [] {
    const char* v = getenv("PPS_TUNE_LOG");
    return v && *v && *v != '0';
  }();
  return on;
}

// Estimated probability that variant v's pre-test passes a random walk value
// (a false pass costs an exact re-check of the block).  Window tests pass when
// K < 2^(32+u) or its low t bits are zero; the small-p window when K < 2^sh_t
// or its low sh_t+1-kb bits are zero; the single bound when hi <= kmax/2; the
// low-bit test roughly when K < kmax 2^32.  Twin variants test two values.
static double pretest_pass_rate(const pps_job_params* jp, int v) {
  WalkArgs a;
  fill_walk_args(jp, &a);
  const VariantTraits& t = walk_variant_traits(v);
  const double p = (double)jp->pmin, kmax = (double)jp->kmax;
  const int kb = lg2u64(jp->kmax) + 1;
  double r;
  if (t.bound) {
    r = kmax * 2147483648.0 / p;
  } else if (t.lowbit) {
    r = kmax * 4294967296.0 / p;
  } else if (t.smallp) {
    r = ldexp(1.0, (int)a.sh_t) / p + ldexp(1.0, -((int)a.sh_t + 1 - kb));
  } else if (t.stepwin) {
    r = ldexp(1.0, (int)jp->step) / p + ldexp(1.0, kb - 1 - (int)jp->step);
  } else {
    const int u = a.win_hi == 0xffffffffu ? 32 : __builtin_popcount(a.win_hi);
    r = ldexp(1.0, 32 + u) / p + (a.win_mask == 0xffffffffu ? ldexp(1.0, -32) : 1.0 / ((double)a.win_mask + 1.0));
  }
  if (t.twin) r *= 2.0;
  return std::min(r, 1.0);
}

// The walk variants the tuner may pick for a job (bit v: variant v): those
// exact for it whose pre-test passes at most 1 step in 512 and, for the queued
// walks, whose expected queue load over the whole n range fits in half the
// warp queue; every exact variant where none does.
static uint64_t variant_set(const pps_job_params* jp) {
  const double nsteps_full = jp->nmax > jp->nmin ? (double)((jp->nmax - jp->nmin + jp->step - 1) / jp->step) : 0.0;
  uint64_t exact = 0, cls = 0;
  for (int v = 0; v < PPS_NUM_VARIANTS; ++v)
    if (variant_ok(jp, v)) {
      const VariantTraits& t = walk_variant_traits(v);
      exact |= 1ull << v;
      const double r = pretest_pass_rate(jp, v);
      // a warp's queue holds the flagged blocks of its 32 x per_thread primes
      const double lanes = 32.0 * t.per_thread;
      if (r <= 1.0 / 512.0 && (!t.queued || lanes * nsteps_full * r <= WALK_QUEUE_CAP / 2)) cls |= 1ull << v;
    }
  return cls ? cls : exact;
}

// Time each walk variant on the first `np` resident primes with a capped n
// range and keep the fastest for this step class.
static int autotune(pps_engine* e, const pps_job_params* jp, const uint64_t* dP, const uint64_t* dPinv,
                    uint64_t np) {
  // Candidates: the variants exact for this job whose pre-test passes at most
  // 1 step in 512 (a block of 8 then stays below 2% re-checked) and, for the
  // queued walks (variants 10 and up), whose expected flagged blocks per warp
  // over the whole n range (32 lanes x nsteps x rate) stay within half the warp
  // queue; or every exact variant where none does.  The tuner times a capped
  // n range, so without the queue bound it could pick a variant whose queue
  // overflows on the full range (each lane then re-walks its prime exactly);
  // and without the rate bound a choice timed on one job could be reused for a
  // job of the same kind at much smaller p, where its window passes most steps.
  const uint64_t cls = variant_set(jp);
  // jobs are told apart by that set (step size, side, window kind, bound test,
  // pass rates): a choice is reused only within the same set
  // a forced variant is honoured only where it is exact for this job
  if (e->forced_variant >= 0 && variant_ok(jp, e->forced_variant) &&
      walk_max_blocks(e->forced_variant, walk_block_threads(e->forced_variant), jp->step, e->num_sms) > 0)
    return e->forced_variant;
  const uint64_t sample = std::min<uint64_t>(np, (uint64_t)e->num_sms * 8 * 256);
  // long enough that per-prime setup and launch timing do not sway the comparison
  // (about 1.3 ms per timed launch at 2e12 steps/s)
  const uint32_t cap_steps = 8192;
  // a choice is reused for jobs of the same kind whose sample is not much larger
  // (a choice timed on a few primes or steps would not hold for a long job)
  const uint64_t work = sample * std::min<uint64_t>(std::max<uint32_t>(jp->nmax - jp->nmin, 1) / jp->step + 1, cap_steps);
  size_t slot = e->tuned_variant.size();
  for (size_t i = 0; i < e->tuned_variant.size(); ++i)
    if (e->tuned_variant[i].mask == cls) {
      if (work <= 4 * e->tuned_variant[i].work) return e->tuned_variant[i].variant;
      slot = i;
    }
  int best = -1;
  float best_ms = 1e30f;  // per prime of the sample
  for (int v = 0; v < PPS_NUM_VARIANTS; ++v) {
    if (!(cls & (1ull << v))) continue;
    // each variant is timed on one whole wave of its own grid (one thread per
    // prime, or per two for the two-prime walks) where the job has that many
    // primes, so that a variant with fewer resident blocks per SM is not timed
    // with a partly idle last wave
    const uint64_t wave = (uint64_t)walk_max_blocks(v, 256, jp->step, e->num_sms) * 256 *
                          (uint64_t)walk_variant_traits(v).per_thread;
    const uint64_t sv = std::min<uint64_t>(np, wave ? wave : sample);
    CU(cudaMemsetAsync(e->counters.p, 0, sizeof(uint32_t), e->st));
    int rc = run_walk(e, jp, v, dP, dPinv, nullptr, sv, 0, cap_steps);  // warm-up
    if (rc) return rc;
    CU(cudaEventRecord(e->ev[6], e->st));
    for (int r = 0; r < 3; ++r)
      if ((rc = run_walk(e, jp, v, dP, dPinv, nullptr, sv, 0, cap_steps))) return rc;
    CU(cudaEventRecord(e->ev[7], e->st));
    CU(cudaEventSynchronize(e->ev[7]));
    float ms = 0;
    CU(cudaEventElapsedTime(&ms, e->ev[6], e->ev[7]));
    const float per = ms / (float)std::max<uint64_t>(sv, 1);
    if (tune_log())
      fprintf(stderr, "pps tune: step %u variant %d (%s): %.3f ms for %llu primes (%.3f ns per prime)\n", jp->step, v,
              walk_variant_name(v), ms, (unsigned long long)sv, per * 1e6f);
    if (per < best_ms) {
      best_ms = per;
      best = v;
    }
  }
  CU(cudaMemsetAsync(e->counters.p, 0, sizeof(uint32_t), e->st));
  if (best < 0)  // a twin job with s < 32 and p above 2^(32+s)
    return set_err(PPS_ERR_NOT_IMPLEMENTED, "no walk kernel for this job on the prime-list path");
  if (slot == e->tuned_variant.size()) e->tuned_variant.push_back({});
  e->tuned_variant[slot] = {cls, best, work};
  return best;
}

static int ceil_lg(uint64_t x) {
  int r = 0;
  while ((1ull << r) < x && r < 63) r++;
  return r;
}

// Threads per prime for the queued walk v on np primes (1 where the walk is not
// a queued one).  Where the job's primes fill less than one wave of the
// walk's resident threads R, most SMs would idle for the whole walk; cutting
// each prime's n range into T parts (T np >= R, T <= 8, parts of at least 32
// blocks) fills them, at the cost of one more start value (an
// exponentiation) per part.  From one wave up, T = 1: the partial last wave
// then costs little (a lightly loaded SM runs its warps faster), and timing T
// per job cost more than it saved on a 512-job mix of distinct jobs (measured
// on the GB300: 3.2e5 primes, 1.37 waves, ran 5% faster with T = 2).
static int choose_split(pps_engine* e, const pps_job_params* jp, int v, uint64_t np) {
  const VariantTraits& vt = walk_variant_traits(v);
  if (!vt.queued || np == 0) return 1;
  if (e->forced_split > 0) return e->forced_split;
  WalkArgs a;
  fill_walk_args(jp, &a);
  const uint64_t blocks = a.nsteps / (uint32_t)vt.unroll;
  const uint64_t resident = (uint64_t)walk_max_blocks(v, 256, jp->step, e->num_sms) * 256 * vt.per_thread;
  int t = 1;
  while (t < 8 && np * (uint64_t)t < resident && blocks / (2ull * t) >= 32) t *= 2;
  return t;
}

static int ensure_hit_buffers(pps_engine* e, size_t hit_cap, size_t fac_cap) {
  int rc;
  if ((rc = e->hits.ensure(hit_cap))) return rc;
  if ((rc = e->factors.ensure(fac_cap))) return rc;
  return PPS_OK;
}

static bool factor_less(const pps_factor& x, const pps_factor& y) {
  if (x.p != y.p) return x.p < y.p;
  if (x.k != y.k) return x.k < y.k;
  if (x.n != y.n) return x.n < y.n;
  return x.c < y.c;
}

// The input file's key table for this job (built when the job's ranges change).
static int ensure_input_keys(pps_engine* e, const pps_job_params* jp) {
  if (!e->input) return PPS_OK;
  const pps_job_params& b = e->in_job;
  if (e->in_built && b.kmin == jp->kmin && b.kmax == jp->kmax && b.kstep == jp->kstep &&
      b.koffset == jp->koffset && b.nmin == jp->nmin && b.nmax == jp->nmax)
    return PPS_OK;
  e->in_built = false;  // until the new table is on the device
  std::vector<uint64_t> keys;
  uint64_t width = 0;
  int rc = input_keys_for_job(e->input, jp, &keys, &width);
  if (rc) return rc;
  if ((rc = e->in_keys.ensure(std::max<size_t>(keys.size(), 1)))) return rc;
  if (!keys.empty())
    CU(cudaMemcpy(e->in_keys.p, keys.data(), keys.size() * sizeof(uint64_t), cudaMemcpyHostToDevice));
  e->in_n = keys.size();
  e->in_width = width;
  e->in_job = *jp;
  e->in_built = true;
  return PPS_OK;
}

extern "C" int pps_engine_set_input(pps_engine* e, const pps_input* in) {
  if (!e) return set_err(PPS_ERR_INVALID_PARAM, "null engine");
  e->input = in;
  e->in_built = false;
  return PPS_OK;
}

// Filter the raw hits accumulated in e->hits and copy the factors out.
// The filter runs on the device-side count of raw hits (clamped to the
// buffer), so the two counts come back in one copy after it: a raw count
// beyond the buffer then means an overflow (the call walks again).
static int finish_job(pps_engine* e, const pps_job_params* jp, pps_factor* out, size_t cap, size_t* nout,
                      pps_job_stats* st, uint32_t* raw_hits_out, bool* overflow) {
  if (int rc = ensure_input_keys(e, jp)) return rc;
  FilterArgs f;
  f.hits = e->hits.p;
  f.d_nhits = e->counters.p;
  f.hit_cap = hit_cap_now(e);
  f.kstep = jp->kstep;
  f.koffset = jp->koffset;
  f.nmin = jp->nmin;
  f.nmax = jp->nmax;
  f.sign = jp->sign;
  f.small_q = e->small_q.p;
  f.nsmall = e->nsmall;
  f.out = e->factors.p;
  f.out_count = e->counters.p + 1;
  f.out_cap = (uint32_t)std::min<size_t>(e->factors.n, 0xffffffffu);
  if (e->input) {
    f.in_keys = e->in_keys.p;
    f.in_n = e->in_n;
    f.in_width = e->in_width;
    f.kmin = jp->kmin;
    f.kmax = jp->kmax;
  }
  CU(cudaEventRecord(e->ev[4], e->st));
  // one resident wave of CTAs (one per candidate at a time); the kernel reads
  // the count on the device
  CU(launch_filter(f, (uint32_t)e->num_sms * 8u, e->st));
  e->launches++;
  CU(cudaEventRecord(e->ev[5], e->st));
  CU(cudaMemcpyAsync(e->h_pinned, e->counters.p, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, e->st));
  CU(cudaStreamSynchronize(e->st));
  const uint32_t raw = ((uint32_t*)e->h_pinned)[0];
  *raw_hits_out = raw;
  if (raw > hit_cap_now(e)) {
    *overflow = true;
    return PPS_OK;
  }
  const uint32_t nf = ((uint32_t*)e->h_pinned)[1];
  float fms = 0;
  CU(cudaEventElapsedTime(&fms, e->ev[4], e->ev[5]));
  if (st) st->filter_ms += fms;
  if (nf > e->factors.n) {
    *overflow = true;
    return PPS_OK;
  }
  std::vector<pps_factor> tmp(nf);
  if (nf) CU(cudaMemcpy(tmp.data(), e->factors.p, nf * sizeof(pps_factor), cudaMemcpyDeviceToHost));
  std::sort(tmp.begin(), tmp.end(), factor_less);
  if (nout) *nout = nf;
  if (out) memcpy(out, tmp.data(), std::min<size_t>(nf, cap) * sizeof(pps_factor));
  if (st) st->factors = nf;
  if (out && nf > cap) return set_err(PPS_ERR_OVERFLOW, "%u factors, buffer holds %zu", nf, cap);
  if (!out && nf > 0 && cap > 0) return set_err(PPS_ERR_OVERFLOW, "null output buffer");
  return PPS_OK;
}

static int run_job_once(pps_engine* e, const pps_job_params* jp, pps_factor* out, size_t cap, size_t* nout,
                        pps_job_stats* st, bool* overflow) {
  const uint32_t* dq;
  BaseTable bt;
  int rc = prepare_sieving_primes(e, jp->qmax, jp->pmax, &dq, &bt);
  if (rc) return rc;
  CU(cudaMemsetAsync(e->counters.p, 0, 2 * sizeof(uint32_t), e->st));
  int variant = -1;
  const uint64_t span = e->batch_span;
  for (uint64_t a = jp->pmin | 1ull; a < jp->pmax; a += span) {
    const uint64_t b = std::min(jp->pmax, a + span);
    const uint64_t nbits = (b - a + 1) / 2;
    // odd primes among nbits odd candidates above 2^32: density < 2/ln(2^32) < 0.1
    const size_t pcap = (size_t)(nbits / 10) + 1024;
    if ((rc = e->P.ensure(pcap))) return rc;
    if ((rc = e->Pinv.ensure(pcap))) return rc;
    CU(cudaEventRecord(e->ev[0], e->st));
    if ((rc = sieve_batch(e, a, b, dq, bt.nq, bt.nq_tiny, bt.nq_seg, e->P.p, e->Pinv.p, nullptr))) return rc;
    CU(cudaEventRecord(e->ev[1], e->st));
    CU(cudaMemcpyAsync(e->h_pinned, e->totals.p, 2 * sizeof(uint64_t), cudaMemcpyDeviceToHost, e->st));
    CU(cudaStreamSynchronize(e->st));
    const uint64_t np = e->h_pinned[0];
    if (st) {
      st->primes += np;
      st->prime_sum += e->h_pinned[1];
      st->batches++;
    }
    if (np == 0) continue;
    if (variant < 0) {
      variant = autotune(e, jp, e->P.p, e->Pinv.p, np);
      if (variant < 0) return variant;
      if (st) st->variant = (uint32_t)variant;
    }
    const int split = choose_split(e, jp, variant, np);
    if (split < 0) return split;
    if (st) st->split = std::max<uint32_t>(st->split, (uint32_t)split);
    CU(cudaEventRecord(e->ev[2], e->st));
    if ((rc = run_walk(e, jp, variant, e->P.p, e->Pinv.p, nullptr, np, 0, 0, (uint32_t)split))) return rc;
    CU(cudaEventRecord(e->ev[3], e->st));
    if (st) {
      CU(cudaEventSynchronize(e->ev[3]));
      float ms0 = 0, ms1 = 0;
      CU(cudaEventElapsedTime(&ms0, e->ev[0], e->ev[1]));
      CU(cudaEventElapsedTime(&ms1, e->ev[2], e->ev[3]));
      st->sieve_ms += ms0;
      st->walk_ms += ms1;
      const uint64_t nsteps = jp->nmax > jp->nmin ? (jp->nmax - jp->nmin + jp->step - 1) / jp->step : 0;
      st->steps += np * nsteps;
    }
  }
  uint32_t raw = 0;
  rc = finish_job(e, jp, out, cap, nout, st, &raw, overflow);
  if (st) st->raw_hits = raw;
  return rc;
}

// A twin job walks once for both sides on the batched form (one job, one
// slot); its stats come from the batch's.
static int run_twin_job(pps_engine* e, const pps_job_params* jp, pps_factor* out, size_t cap, size_t* nout,
                        pps_job_stats* st) {
  pps_batch_stats bst;
  size_t n = 0, off[2];
  const int rc = pps_run_batch(e, jp, 1, out, cap, &n, off, &bst);
  if (nout) *nout = n;
  if (st) {
    memset(st, 0, sizeof *st);
    st->primes = bst.primes;
    st->prime_sum = bst.prime_sum;
    st->raw_hits = bst.raw_hits;
    st->factors = bst.factors;
    st->steps = bst.steps;
    st->batches = bst.waves;
    st->variant = PPS_NUM_VARIANTS;  // the batched walk
    st->total_ms = bst.total_ms;
    st->filter_ms = bst.filter_ms;
    st->walk_ms = bst.total_ms - bst.filter_ms;
  }
  return rc;
}

extern "C" int pps_run_job(pps_engine* e, const pps_job_params* jp, pps_factor* out, size_t cap,
                           size_t* nout, pps_job_stats* st) {
  if (!e || !jp) return set_err(PPS_ERR_INVALID_PARAM, "null argument");
  if (jp->step < 1 || jp->step > 32 || jp->pmin <= (1ull << 32)) return set_err(PPS_ERR_INVALID_PARAM, "job not normalized");
  if (jp->sign == PPS_SIGN_TWIN) {
    // twin jobs run on the batched walk, except with an input file: its rule
    // applies on the one-job path, whose twin kernels need 32-bit steps or
    // p <= 2^(32+s)
    if (!e->input) return run_twin_job(e, jp, out, cap, nout, st);
    bool exact = false;
    for (int v = 0; v < PPS_NUM_VARIANTS && !exact; ++v) exact = variant_ok(jp, v) != 0;
    if (!exact)
      return set_err(PPS_ERR_NOT_IMPLEMENTED, "a twin job with an input file needs 32-bit steps or p <= 2^(32+s)");
  }
  CU(cudaSetDevice(e->device));
  size_t hit_cap = 1u << 20, fac_cap = 1u << 18;
  for (int attempt = 0; attempt < 4; ++attempt) {
    int rc = ensure_hit_buffers(e, std::max(hit_cap, e->hits.n), std::max(fac_cap, e->factors.n));
    if (rc) return rc;
    e->hit_cap_limit = attempt == 0 ? debug_first_hit_cap() : 0;
    if (st) memset(st, 0, sizeof *st);
    bool overflow = false;
    cudaEventRecord(e->ev[6], e->st);
    rc = run_job_once(e, jp, out, cap, nout, st, &overflow);
    if (rc) return rc;
    if (!overflow) {
      cudaEventRecord(e->ev[7], e->st);
      cudaEventSynchronize(e->ev[7]);
      float ms = 0;
      cudaEventElapsedTime(&ms, e->ev[6], e->ev[7]);
      if (st) st->total_ms = ms;
      return PPS_OK;
    }
    // grow the buffers, unless the overflow was only the first attempt's
    // debug cap (the retry lifts it)
    const size_t grow = attempt == 0 && debug_first_hit_cap() ? 1 : 4;
    hit_cap = e->hits.n * grow;
    fac_cap = e->factors.n * grow;
  }
  return set_err(PPS_ERR_INSUFFICIENT_RESOURCE, "hit buffer overflow persisted");
}

// Walk primes already on the device; hits accumulate in e->hits.
static int walk_device_list(pps_engine* e, const pps_job_params* jp, const uint64_t* dP, size_t np,
                            pps_job_stats* st) {
  int variant = autotune(e, jp, dP, nullptr, np);
  if (variant < 0) return variant;
  if (st) st->variant = (uint32_t)variant;
  const int split = choose_split(e, jp, variant, np);
  if (split < 0) return split;
  if (st) st->split = (uint32_t)split;
  CU(cudaEventRecord(e->ev[2], e->st));
  int rc = run_walk(e, jp, variant, dP, nullptr, nullptr, np, 0, 0, (uint32_t)split);
  if (rc) return rc;
  CU(cudaEventRecord(e->ev[3], e->st));
  if (st) {
    CU(cudaEventSynchronize(e->ev[3]));
    float ms = 0;
    CU(cudaEventElapsedTime(&ms, e->ev[2], e->ev[3]));
    st->walk_ms += ms;
    st->primes += np;
    const uint64_t nsteps = jp->nmax > jp->nmin ? (jp->nmax - jp->nmin + jp->step - 1) / jp->step : 0;
    st->steps += np * nsteps;
  }
  return PPS_OK;
}

extern "C" int pps_check_primes_device(pps_engine* e, const pps_job_params* jp, const uint64_t* d_P,
                                       size_t np, pps_factor* out, size_t cap, size_t* nout,
                                       pps_job_stats* st) {
  if (!e || !jp || (!d_P && np)) return set_err(PPS_ERR_INVALID_PARAM, "null argument");
  CU(cudaSetDevice(e->device));
  size_t hit_cap = 1u << 20, fac_cap = 1u << 18;
  for (int attempt = 0; attempt < 4; ++attempt) {
    int rc = ensure_hit_buffers(e, std::max(hit_cap, e->hits.n), std::max(fac_cap, e->factors.n));
    if (rc) return rc;
    e->hit_cap_limit = attempt == 0 ? debug_first_hit_cap() : 0;
    if (st) memset(st, 0, sizeof *st);
    CU(cudaMemsetAsync(e->counters.p, 0, 2 * sizeof(uint32_t), e->st));
    if (np && (rc = walk_device_list(e, jp, d_P, np, st))) return rc;
    bool overflow = false;
    uint32_t raw = 0;
    rc = finish_job(e, jp, out, cap, nout, st, &raw, &overflow);
    if (st) st->raw_hits = raw;
    if (rc || !overflow) return rc;
    // grow the buffers, unless the overflow was only the first attempt's
    // debug cap (the retry lifts it)
    const size_t grow = attempt == 0 && debug_first_hit_cap() ? 1 : 4;
    hit_cap = e->hits.n * grow;
    fac_cap = e->factors.n * grow;
  }
  return set_err(PPS_ERR_INSUFFICIENT_RESOURCE, "hit buffer overflow persisted");
}

// The device address of a caller's host list of primes.  A page-locked
// (pinned) buffer is read in place by the walk over the host link: each prime
// is loaded once, 8 B per prime, a small fraction of the link's bandwidth at
// the walk's rate.  Any other host buffer is first copied into the engine's
// device list.
static int host_list_on_device(pps_engine* e, const uint64_t* P, size_t np, const uint64_t** dP) {
  *dP = nullptr;
  if (!np) return PPS_OK;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, P) == cudaSuccess && at.type == cudaMemoryTypeHost && at.devicePointer) {
    *dP = (const uint64_t*)at.devicePointer;
    return PPS_OK;
  }
  cudaGetLastError();  // an unregistered pointer is not an error
  int rc;
  if ((rc = e->P.ensure(np))) return rc;
  CU(cudaMemcpyAsync(e->P.p, P, np * sizeof(uint64_t), cudaMemcpyHostToDevice, e->st));
  *dP = e->P.p;
  return PPS_OK;
}

extern "C" int pps_check_primes(pps_engine* e, const pps_job_params* jp, const uint64_t* P, size_t np,
                                pps_factor* out, size_t cap, size_t* nout, pps_job_stats* st) {
  if (!e || !jp || (!P && np)) return set_err(PPS_ERR_INVALID_PARAM, "null argument");
  int rc;
  CU(cudaSetDevice(e->device));
  const uint64_t* dP;
  if ((rc = host_list_on_device(e, P, np, &dP))) return rc;
  return pps_check_primes_device(e, jp, dP, np, out, cap, nout, st);
}

static bool hit_less(const pps_hit& x, const pps_hit& y) {
  if (x.idx != y.idx) return x.idx < y.idx;
  if (x.n != y.n) return x.n < y.n;
  return x.k < y.k;
}

extern "C" int pps_check_primes_raw(pps_engine* e, const pps_job_params* jp, const uint64_t* P, size_t np,
                                    pps_hit* out, size_t cap, size_t* nout) {
  if (!e || !jp || (!P && np)) return set_err(PPS_ERR_INVALID_PARAM, "null argument");
  if (np > 0xffffffffull) return set_err(PPS_ERR_INVALID_PARAM, "too many primes for one call");
  int rc;
  CU(cudaSetDevice(e->device));
  const uint64_t* dP;
  if ((rc = host_list_on_device(e, P, np, &dP))) return rc;
  size_t hit_cap = std::max<size_t>(1u << 20, e->hits.n);
  for (int attempt = 0; attempt < 4; ++attempt) {
    if ((rc = ensure_hit_buffers(e, hit_cap, std::max<size_t>(1u << 18, e->factors.n)))) return rc;
    e->hit_cap_limit = attempt == 0 ? debug_first_hit_cap() : 0;
    CU(cudaMemsetAsync(e->counters.p, 0, 2 * sizeof(uint32_t), e->st));
    if (np && (rc = walk_device_list(e, jp, dP, np, nullptr))) return rc;
    CU(cudaMemcpyAsync(e->h_pinned, e->counters.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, e->st));
    CU(cudaStreamSynchronize(e->st));
    const uint32_t raw = ((uint32_t*)e->h_pinned)[0];
    if (raw > hit_cap_now(e)) {
      hit_cap = std::max<size_t>(hit_cap, raw > e->hits.n ? (size_t)raw * 2 : e->hits.n);
      continue;
    }
    std::vector<pps_hit> tmp(raw);
    if (raw) CU(cudaMemcpy(tmp.data(), e->hits.p, raw * sizeof(pps_hit), cudaMemcpyDeviceToHost));
    std::sort(tmp.begin(), tmp.end(), hit_less);
    if (nout) *nout = raw;
    if (out) memcpy(out, tmp.data(), std::min<size_t>(raw, cap) * sizeof(pps_hit));
    if (raw > cap) return set_err(PPS_ERR_OVERFLOW, "%u raw hits, buffer holds %zu", raw, cap);
    return PPS_OK;
  }
  return set_err(PPS_ERR_INSUFFICIENT_RESOURCE, "hit buffer overflow persisted");
}

// ------------------------------------------------------------ IMAD probe
extern "C" int pps_measure_imad_peak(pps_engine* e, double* mults_per_sec) {
  if (!e || !mults_per_sec) return set_err(PPS_ERR_INVALID_PARAM, "null argument");
  CU(cudaSetDevice(e->device));
  const int threads = 256, blocks = e->num_sms * 8;
  int rc;
  if ((rc = e->probe_sink.ensure((size_t)threads * blocks))) return rc;
  const uint32_t iters = 1u << 16;
  CU(launch_imad_probe(e->probe_sink.p, 1024, blocks, threads, e->st));  // warm-up
  e->launches++;
  CU(cudaEventRecord(e->ev[6], e->st));
  CU(launch_imad_probe(e->probe_sink.p, iters, blocks, threads, e->st));
  e->launches++;
  CU(cudaEventRecord(e->ev[7], e->st));
  CU(cudaEventSynchronize(e->ev[7]));
  float ms = 0;
  CU(cudaEventElapsedTime(&ms, e->ev[6], e->ev[7]));
  const double mults = 3.0 * 4.0 * (double)iters * threads * blocks;
  *mults_per_sec = mults / (ms * 1e-3);
  return PPS_OK;
}
