// pps_noalloc.cu -- pps_check_primes_noalloc(): the walk + output rule over
// primes already in device memory, for callers that cannot allocate memory.
//
// Who needs it: code that must not call cudaMalloc/cudaFree at all -- a host
// program whose device memory is handed out by someone else's pool or arena, a
// real-time loop that may not allocate between frames, or a plugin running
// inside a framework that owns every device allocation.  The engine API
// (pps_engine_create) grows its own buffers with cudaMalloc; this entry point
// uses none.  The caller passes the primes and the output buffer (device
// memory it already owns); the only other memory is the candidate scratch
// below, a file-scope __device__ array that every GPU which loads the library
// holds until the process exits.
//
// The scratch is shared by all calls on a device and keeps the last call's
// contents; its counters are cleared at the start of each call.  Two calls that
// overlap on the GPU (different streams or host threads at the same time) race
// on it: serialise them.
//
// Set-up: the first call on each device (with that device current) looks up
// the scratch's device address with cudaGetSymbolAddress and copies the small-
// prime table into it, on the caller's stream, and waits for that copy before
// it records the device as set up.  Make that first call before any stream
// capture.  The address is looked up once per device for the life of the
// process, so cudaDeviceReset() on a device that has been set up is not
// supported: a call that finds the table gone (its tag word no longer set)
// reports PPS_ERR_CUDA instead of returning factors.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <mutex>

#include "pps_internal.h"
#include "ppsgpu.h"

namespace {

constexpr uint32_t kTableTag = 0x50505351u;  // written with the small-prime table

struct NoallocScratch {
  uint32_t counters[4];  // [0] raw candidates, [1] factors
  uint32_t table_tag;    // kTableTag once the small-prime table is in place
  uint32_t pad[3];
  uint16_t small_q[3584];
  pps_hit hits[PPS_NOALLOC_MAX_CANDIDATES];
};

static __device__ __align__(256) NoallocScratch g_noalloc_scratch;

constexpr int kMaxDevices = 64;
std::mutex g_mu;
NoallocScratch* g_addr[kMaxDevices];
uint32_t g_nsmall = 0;
uint16_t g_small_host[3584];

// errors are reported through pps_last_error()
int fail(int code, const char* fmt, ...) {
  char msg[256];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(msg, sizeof msg, fmt, ap);
  va_end(ap);
  return pps::set_error_text(code, msg);
}

// Odd primes 3..32749 into a static host table (no heap).
void make_small_primes() {
  static unsigned char comp[32768];
  uint32_t n = 0;
  for (uint32_t i = 3; i < 32768; i += 2) {
    if (comp[i]) continue;
    g_small_host[n++] = (uint16_t)i;
    for (uint32_t j = i * i; j < 32768; j += 2 * i) comp[j] = 1;
  }
  g_nsmall = n;
}

int setup(int dev, cudaStream_t st, NoallocScratch** out) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (dev < 0 || dev >= kMaxDevices) return fail(PPS_ERR_NO_DEVICE, "device %d out of range", dev);
  if (g_addr[dev]) {
    *out = g_addr[dev];
    return PPS_OK;
  }
  if (!g_nsmall) make_small_primes();
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return fail(PPS_ERR_CUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
  NoallocScratch* s = (NoallocScratch*)p;
  // on the caller's stream, and complete before any call relies on it (a copy
  // from pageable memory may return before the device has the data)
  static const uint32_t tag = kTableTag;
  e = cudaMemcpyAsync(s->small_q, g_small_host, g_nsmall * sizeof(uint16_t), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&s->table_tag, &tag, sizeof tag, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail(PPS_ERR_CUDA, "small-prime table: %s", cudaGetErrorString(e));
  g_addr[dev] = s;
  *out = s;
  return PPS_OK;
}

}  // namespace

extern "C" int pps_check_primes_noalloc(const pps_job_params* jp, const uint64_t* d_P, size_t np,
                                        pps_factor* d_out, uint32_t out_cap, uint32_t* nout,
                                        void* stream) {
  using namespace pps;
  if (!jp || !nout || (np && !d_P) || (out_cap && !d_out))
    return fail(PPS_ERR_INVALID_PARAM, "null argument");
  if (jp->step < 1 || jp->step > 32 || jp->pmin <= (1ull << 32))
    return fail(PPS_ERR_INVALID_PARAM, "job not normalized (use pps_normalize)");
  if (jp->sign == PPS_SIGN_TWIN) return fail(PPS_ERR_NOT_IMPLEMENTED, "twin jobs run through pps_run_job");
  if (np > PPS_NOALLOC_MAX_PRIMES)
    return fail(PPS_ERR_INVALID_PARAM, "%zu primes exceed the limit of %u per call; split the list",
                np, (unsigned)PPS_NOALLOC_MAX_PRIMES);
  *nout = 0;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(PPS_ERR_NO_DEVICE, "cudaGetDevice: %s", cudaGetErrorString(e));
  cudaStream_t st = (cudaStream_t)stream;
  NoallocScratch* s = nullptr;
  int rc = setup(dev, st, &s);
  if (rc) return rc;
  e = cudaMemsetAsync(s->counters, 0, sizeof s->counters, st);
  if (e != cudaSuccess) return fail(PPS_ERR_CUDA, "clear counters: %s", cudaGetErrorString(e));

  if (np) {
    WalkArgs a;
    walk_args_for_job(jp, &a);
    a.P = d_P;
    a.Pinv = nullptr;
    a.d_np = nullptr;
    a.np = np;
    a.idx_base = 0;
    a.hits = s->hits;
    a.hit_count = &s->counters[0];
    a.hit_cap = PPS_NOALLOC_MAX_CANDIDATES;
    // queued walks first (32-bit steps: 13, 10; shorter steps: 21, 19), then the
    // plain block walks, which are exact for every job
    static const int order[] = {13, 10, 21, 19, 2, 1, 0};
    int v = -1;
    for (int c : order)
      if (walk_variant_exact(jp, c)) {
        v = c;
        break;
      }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int maxb = walk_max_blocks(v, 256, jp->step, sms > 0 ? sms : 1);
    if (v < 0 || maxb <= 0) return fail(PPS_ERR_CUDA, "no walk kernel for this job");
    // the queued walks get one thread per prime (the block scheduler keeps every
    // SM full to the end); the block walks one resident wave that strides
    const uint64_t need = (np + 255) / 256;
    const uint64_t cap = walk_variant_traits(v).queued ? 0x7fffffffull : (uint64_t)maxb;
    const int blocks = (int)(need < cap ? need : cap);
    e = launch_walk(v, a, blocks, 256, st);
    if (e != cudaSuccess) return fail(PPS_ERR_CUDA, "walk launch: %s", cudaGetErrorString(e));

    FilterArgs f;
    f.hits = s->hits;
    f.d_nhits = &s->counters[0];
    f.hit_cap = PPS_NOALLOC_MAX_CANDIDATES;
    f.kstep = jp->kstep;
    f.koffset = jp->koffset;
    f.nmin = jp->nmin;
    f.nmax = jp->nmax;
    f.sign = jp->sign;
    f.small_q = s->small_q;
    f.nsmall = g_nsmall;
    f.out = d_out;
    f.out_count = &s->counters[1];
    f.out_cap = out_cap;
    e = launch_filter(f, PPS_NOALLOC_MAX_CANDIDATES, st);
    if (e != cudaSuccess) return fail(PPS_ERR_CUDA, "filter launch: %s", cudaGetErrorString(e));
  }
  uint32_t counts[5] = {0, 0, 0, 0, 0};  // the counters and the table tag
  e = cudaMemcpyAsync(counts, s->counters, sizeof counts, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail(PPS_ERR_CUDA, "read counters: %s", cudaGetErrorString(e));
  if (counts[4] != kTableTag)
    return fail(PPS_ERR_CUDA, "the scratch's small-prime table is gone (cudaDeviceReset is not supported)");
  if (counts[0] > PPS_NOALLOC_MAX_CANDIDATES)
    return fail(PPS_ERR_OVERFLOW, "%u candidates exceed the scratch limit of %u; split the list",
                counts[0], (unsigned)PPS_NOALLOC_MAX_CANDIDATES);
  *nout = counts[1];
  if (counts[1] > out_cap)
    return fail(PPS_ERR_OVERFLOW, "%u factors, output holds %u", counts[1], out_cap);
  return PPS_OK;
}
