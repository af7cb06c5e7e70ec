/* ppsgpu.h -- C ABI of the GB300 PPSieve library (libppsgpu.so).

   The path: for every odd prime p in [pmin, pmax) walk k = -/+2^-n (mod p) over
   n in [nmin, nmax) and report every p | k*2^n+c (c = +1 Proth, -1 Riesel) with
   k in [kmin, kmax], k == koffset (mod kstep), k*2^n+c free of odd prime factors
   below 32768.  Everything runs on one GPU: a segmented sieve makes the primes,
   a walk kernel finds candidates, a filter kernel applies the output rule.

   Plain C types only; no CUDA or torch types cross this boundary.  All calls
   return PPS_OK (0) or a negative error code and never exit the process.

   Reference interfaces this library replaces (file:line in Ken-g6/PSieve-CUDA):
     - the GPU C ABI pps/appcu.h:27-37 (cuda_init, cuda_app_init, check_ns,
       get_factors_found, cuda_finalize, ld_nstep/ld_bbits/ld_r0): declared in
       include/appcu_compat.h and exported by libppsgpu_appcu.so;
     - the parameter rules of pps/app.c:649-712 and pps/appcu.cu:155-209:
       pps_normalize below;
     - check_ns + get_factors_found + the CPU re-walk pps/app.c:1037-1219 and
       the filter pps/app.c:159-186: pps_check_primes / pps_run_job below,
       which return exact (p, k, n, c) instead of per-subsection flags;
     - the host prime generator sieve.c:168-1314 feeding main.c:750-777:
       pps_sieve_range / the sieve inside pps_run_job.
*/
#ifndef PPSGPU_H
#define PPSGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The first four match pps/app.h:64-71. */
#define PPS_OK                         0
#define PPS_ERR_INVALID_PARAM       (-178)
#define PPS_ERR_INSUFFICIENT_RESOURCE (-198)
#define PPS_ERR_NOT_IMPLEMENTED     (-150)
#define PPS_ERR_FOPEN               (-108)
#define PPS_ERR_SCANF               (-140) /* bad input sieve file (pps/app.h:69) */
#define PPS_ERR_CUDA                (-300) /* a CUDA runtime call failed */
#define PPS_ERR_NO_DEVICE           (-301) /* no usable GPU */
#define PPS_ERR_OVERFLOW            (-302) /* caller's output buffer too small */
#define PPS_ERR_TIMEOUT             (-303) /* a bounded device wait expired */
#define PPS_ERR_BUSY                (-304) /* server queue / memory budget full */
#define PPS_ERR_NOT_FOUND           (-305) /* unknown job id */
#define PPS_ERR_CANCELLED           (-306)

/* sign of a twin job: both k*2^n+1 and k*2^n-1 from one walk, as the
   reference's twin build (tpsieve, -DSEARCH_TWIN: pps/app.c:1071-1107,
   pps/appcu.cu:177-180, 741-767) reports them; k == 3 (mod 6) unless -M/-s
   say otherwise.  Each factor carries its own c.  pps_run_job, pps_run_batch
   and the serving loop run twin jobs on the batched walk; pps_check_primes*,
   and pps_run_job with an input file, on the one-job twin kernels (which need
   s = 32, or p <= 2^(32+s): PPS_ERR_NOT_IMPLEMENTED otherwise; raw candidates
   of a twin job carry their side in idx bit 31).  An input file for a twin job
   is in the twin build's formats (pps_input_read).  The appcu.h layer and
   pps_check_primes_noalloc take one side only. */
#define PPS_SIGN_TWIN 2

/* A job as the user states it; zero means "not given" exactly as in the
   reference options (-p -P -k -K -n -N -R -M -s -Q). */
typedef struct {
  uint64_t pmin, pmax;
  uint64_t kmin, kmax;
  uint32_t nmin, nmax;
  int32_t  sign;      /* +1 Proth (default when 0), -1 Riesel (-R), PPS_SIGN_TWIN both */
  uint32_t kstep;     /* -M, default 2 */
  uint32_t koffset;   /* -s, default 1 */
  uint32_t qmax;      /* -Q, default sqrt(pmax) */
} pps_job_spec;

/* A job after the reference's normalisation (pps_normalize). */
typedef struct {
  uint64_t pmin, pmax;   /* primes pmin <= p < pmax */
  uint64_t kmin, kmax;   /* rounded to kstep*b+koffset (pps/app.c:705-708) */
  uint32_t nmin, nmax;   /* n in [nmin, nmax) */
  int32_t  sign;
  uint32_t kstep, koffset;
  uint32_t qmax;         /* sieving primes q <= qmax */
  uint32_t nstep;        /* the reference's ld_nstep after pps/appcu.cu:158-186 */
  uint32_t step;         /* n values per device walk step: min(nstep, 32) */
} pps_job_params;

/* One reported factor: p | k*2^n+c. */
typedef struct {
  uint64_t p;
  uint64_t k;
  uint32_t n;
  int32_t  c;
} pps_factor;

/* One raw candidate before the output filter (k in range, n < nmax). */
typedef struct {
  uint64_t p;
  uint64_t k;
  uint32_t n;
  uint32_t idx;   /* index of p in the caller's prime list, or job slot */
} pps_hit;

typedef struct {
  uint64_t primes;      /* primes walked */
  uint64_t prime_sum;   /* wrapping 64-bit sum of those primes (main.c:1232) */
  uint64_t raw_hits;    /* candidates before the output filter */
  uint64_t factors;     /* lines reported */
  uint64_t steps;       /* walk steps executed (primes x ceil((nmax-nmin)/step)) */
  uint32_t batches;     /* device batches used */
  uint32_t variant;     /* walk kernel variant used */
  double   sieve_ms, walk_ms, filter_ms, total_ms;  /* device time per phase */
  uint32_t split;       /* threads per prime of the walk (the tuner's choice, 1..8) */
  uint32_t reserved;
} pps_job_stats;

typedef struct pps_engine pps_engine;

/* Last error message of the calling thread ("" if none). */
const char *pps_last_error(void);

/* Library version string. */
const char *pps_version(void);

/* Test hook (host-side fault injection): after the next `skip` device-buffer
   allocations of any engine succeed, the `count` after them fail as if device
   memory were exhausted, so the call that needed them returns
   PPS_ERR_INSUFFICIENT_RESOURCE; count 0 clears it.  Returns the number of
   failures injected since the previous call.  No kernel is launched or
   disturbed.  Replaces nothing in the reference, whose allocation failure path
   is a retry loop, then exit (pps/appcu.cu:283-324). */
int pps_debug_fail_allocs(int skip, int count);

/* Test hook for the correctness fallbacks that only a wrong tuning choice
   reaches: warp_queue caps the flagged blocks a warp of the queued walks
   holds for its exact re-check (0..512; -1 = 512), so that warps whose queue
   overflows re-walk their primes with the exact test at every step; and
   first_candidates (0 = no cap) caps the raw-candidate buffer on the first
   attempt of every call (and of every wave of the batched form), so that the
   call finds it overflowed, grows the buffer and walks again.  Results are
   unchanged; only speed is.  Applies to every engine from the next call. */
int pps_debug_limits(int warp_queue, uint32_t first_candidates);

/* Apply the reference's option rules (main.c:916-931, main.c:971-972,
   pps/app.c:657-712, pps/appcu.cu:158-204, pps/appcu.cu:236). */
int pps_normalize(const pps_job_spec *in, pps_job_params *out);

/* Engine: one per GPU and host thread; owns streams, device buffers and the
   tuned kernel choice.  device < 0 picks device 0. */
int pps_engine_create(int device, pps_engine **out);
void pps_engine_destroy(pps_engine *e);

/* Device memory held by the engine, in bytes. */
uint64_t pps_engine_device_bytes(const pps_engine *e);

/* Streaming multiprocessors of the engine's device. */
int pps_engine_sm_count(const pps_engine *e);

/* Batch width of the p-range per device sieve batch (default 2^31).  Smaller
   batches lower memory; results do not depend on it. */
int pps_engine_set_batch_span(pps_engine *e, uint64_t span);

/* Force a walk kernel variant (0..PPS_NUM_VARIANTS-1), or -1 for the tuned one. */
#define PPS_NUM_VARIANTS 31
int pps_engine_set_variant(pps_engine *e, int variant);

/* A walk variant's short description ("queue2-min-u8": queued walk, two primes
   per thread, running-minimum window, 8-step blocks), or "?" out of range. */
const char *pps_walk_variant_name(int variant);

/* Force the threads per prime of the queued walks (1, 2, 4 or 8: each prime's
   n range is cut into that many parts walked side by side), or 0 for the
   choice per job (where a job's primes fill less than one wave of the walk's
   resident threads, the smallest number of parts that fills it).  In the batched form and the serving loop the
   same number of n parts is used for every job (tuned: long n ranges are cut
   into parts of about the tuned work per chunk). */
int pps_engine_set_split(pps_engine *e, int split);

/* Whole job: device sieve of [pmin,pmax), walk, filter.  Factors are sorted by
   (p, k, n); *nout is the total found (may exceed cap -> PPS_ERR_OVERFLOW, with
   the first cap entries written). */
int pps_run_job(pps_engine *e, const pps_job_params *jp, pps_factor *out,
                size_t cap, size_t *nout, pps_job_stats *st);

/* Walk a caller-supplied list of primes held in HOST memory.  A page-locked
   (pinned) buffer, e.g. from cudaHostAlloc, is read in place by the walk over
   the host link; any other buffer is copied to the device inside the call.  A
   list that starts in page-locked memory must lie in one page-locked
   allocation or registration (cudaHostRegister) for its whole length.  Same
   output rule and order as pps_run_job. */
int pps_check_primes(pps_engine *e, const pps_job_params *jp, const uint64_t *P,
                     size_t np, pps_factor *out, size_t cap, size_t *nout,
                     pps_job_stats *st);

/* Same walk, returning the raw candidates (before the output filter), with
   pps_hit.idx = index into P.  Used by the pps/appcu.h compatibility layer to
   build per-subsection flags. Sorted by (idx, n). */
int pps_check_primes_raw(pps_engine *e, const pps_job_params *jp, const uint64_t *P,
                         size_t np, pps_hit *out, size_t cap, size_t *nout);

/* Walk primes already resident in device memory (d_P: np uint64 values).
   Factors are written to host memory. */
int pps_check_primes_device(pps_engine *e, const pps_job_params *jp,
                            const uint64_t *d_P, size_t np, pps_factor *out,
                            size_t cap, size_t *nout, pps_job_stats *st);

/* Device sieve of odd primes in [lo, hi) with sieving primes q <= qmax
   (0 = floor(sqrt(hi-1)) rule of main.c:971-972).  Writes up to cap primes to
   out (host, may be NULL), returns count and wrapping sum. */
int pps_sieve_range(pps_engine *e, uint64_t lo, uint64_t hi, uint32_t qmax,
                    uint64_t *out, size_t cap, size_t *count, uint64_t *sum);

/* Measured throughput of the device's 32-bit multiply pipe on the walk's own
   multiply mix (one lo, one hi, one wide multiply), in multiplies per second.
   The roofline denominator for the walk kernel. */
int pps_measure_imad_peak(pps_engine *e, double *mults_per_sec);

/* Number of the engine's own kernels launched so far. */
uint64_t pps_engine_launches(const pps_engine *e);

/* ---- Input sieve files (-i; pps/app.c:190-517 read them, pps/app.c:180-183
   applies them).  A file lists the (k, n) still to be tested, in NewPGen
   format ("p0:P:x:2:c" then "k n" lines) or ABCD format ("ABCD k*2^$a+1 [n0]"
   then n deltas).  With a file the output rule is the file: a factor is
   reported iff its (k, n) is in the file (and k == koffset mod kstep, n in
   [nmin, nmax)); the small-prime filter is not applied.

   pps_input_read parses a file against the job as the user stated it.  When
   one of spec->kmin, kmax, nmin, nmax is 0 it scans the file like
   scan_input_file (pps/app.c:190-347): it detects the format, takes the sign
   from the header and fills kmin/kmax/nmin/nmax from the file's extents
   (nmax one past the largest n).  When all four are given the file is read as
   ABCD without a scan (pps/app.c:97), so a NewPGen file is refused.  Errors:
   PPS_ERR_FOPEN, PPS_ERR_SCANF.  Entries the reference would write outside its
   bitmap (an ABCD k below kmin or past kmax; n past nmax) are ignored.

   For a twin job (spec->sign == PPS_SIGN_TWIN) the file is in the formats of
   the reference's twin build (pps/app.c:208-216): NewPGen "p0:T:x:2:3" then
   "k n" lines, or ABCD "ABCD (6*$a+3)*2^n+1 & (6*$a+3)*2^n-1 [a0]" per n then
   deltas of the k index a (k = kstep a + koffset; the extents reported are k
   values).  A factor of either side is reported iff its (k, n) is in the
   file.  One-side formats are refused for a twin job and twin formats for a
   one-side job, as each reference build does. */
typedef struct pps_input pps_input;

typedef struct {
  int32_t format;          /* 1 NewPGen, 2 ABCD (the reference's FORMAT_ values) */
  int32_t sign;            /* the header's side */
  uint64_t records;        /* (k, n) entries read */
  uint64_t k0, k1;         /* smallest and largest k */
  uint32_t n0, n1;         /* smallest n, one past the largest */
} pps_input_info;

int pps_input_read(const char *path, pps_job_spec *spec, pps_input **out);
int pps_input_get_info(const pps_input *in, pps_input_info *info);
void pps_input_free(pps_input *in);

/* Use `in` as the output rule of this engine's pps_run_job and
   pps_check_primes* calls (NULL: back to the small-prime filter).  The engine
   keeps the pointer: `in` must outlive its use.  The file's table for a job is
   built at the job's first call (PPS_ERR_SCANF when a NewPGen line has
   k != koffset mod kstep, pps/app.c:385-389).  The batched form and the
   serving loop always apply the small-prime filter. */
int pps_engine_set_input(pps_engine *e, const pps_input *in);

/* ---- Batched persistent form (no single counterpart in the reference, which
   runs one range per process, main.c:887-1266).  Many normalised jobs --
   different k, n and p ranges, mixed signs -- are sieved wave by wave into one
   device prime table and walked by one persistent kernel whose warps take
   chunks of primes from a device work counter; each wave's launch sequence is
   a captured CUDA graph; the work per chunk (walk steps per lane: a job's
   chunk holds work*32/nsteps primes) and the unroll are tuned on the first
   wave and reported in `chunk` and `unroll`.  Factors come back grouped by
   job (job_offsets[j]..job_offsets[j+1]), each group sorted by (p, k, n),
   exactly as pps_run_job would return them. */
typedef struct {
  uint64_t primes, prime_sum, raw_hits, factors, steps;
  uint32_t waves, chunk, unroll;
  uint32_t primes_per_lane;  /* the tuned walk: 2 where 32-bit-step jobs walk two primes per lane */
  double total_ms, filter_ms;
  double sieve_ms, walk_ms;  /* device time of the waves' sieve parts and walks */
} pps_batch_stats;

int pps_run_batch(pps_engine *e, const pps_job_params *jobs, size_t njobs, pps_factor *out,
                  size_t cap, size_t *nout, size_t *job_offsets, pps_batch_stats *st);

/* Segments (2^18 odd candidates each) one wave of the batched form holds, at
   most and by default 16384 (2^32 odd candidates: about 7.5 GB of wave
   buffers).  Fewer hold proportionally less device memory (a profiler
   capture, a shared GPU).  Only before the engine's first batched call
   (PPS_ERR_BUSY after it). */
int pps_engine_set_wave_segments(pps_engine *e, uint32_t segments);

/* Force the batched form's walk kernel: unroll 8 or 16 steps per block, 1 or
   2 primes per lane for the 32-bit-step jobs (2: the 64-register kernel); 0, 0
   for the choice the first wave's timing makes among the two-primes-per-lane
   kernels (reported in pps_batch_stats). */
int pps_engine_set_batch_walk(pps_engine *e, int unroll, int primes_per_lane);

/* Per-job prime count and wrapping prime sum of the last pps_run_batch. */
int pps_batch_job_primes(pps_engine *e, size_t njobs, uint64_t *primes, uint64_t *sums);

/* ---- Serving loop (no counterpart in the reference, which runs one range per
   process, main.c:887-1266): continuous batching over the batched form.  A
   worker thread owns an engine on `device`; each turn it admits queued jobs,
   runs one wave over the next p pieces of every admitted job (one piece per
   job first, oldest first, then the oldest fill the wave), and finishes the
   jobs whose last piece was in it.  Jobs join at the next wave.  Admission is
   in submission order, while a job slot is free (max_jobs) and the reserved
   candidate-buffer bytes stay within factor_bytes: a job reserves twice its
   expected raw candidates (32 B each, Mertens estimate #k * #n * ln(ln pmax /
   ln pmin)), at least 16 KiB; a job whose reservation alone exceeds the budget
   is refused at submission with PPS_ERR_INSUFFICIENT_RESOURCE.  Job state
   between waves (parameters, prime counters) stays in device slots.  Each
   job's factor list is exactly what pps_run_job returns for it alone. */
typedef struct pps_server pps_server;

typedef struct {
  uint64_t factor_bytes;   /* candidate-buffer budget; 0 = 1 GiB */
  uint32_t max_jobs;       /* admitted jobs at once (device slots); 0 = 4096, at most 65536 */
  uint32_t wave_segments;  /* sieve segments (2^18 odd candidates) per wave; 0 = the maximum, 16384 */
  uint64_t wave_work;      /* walk steps per wave, estimated from each piece's p range and n
                              range (primes ~ width / ln p); 0 = 4e10 (about 15 ms of the
                              GPU); a piece is at least one segment.  A job that arrives
                              while a wave runs joins the next one, so this bounds its wait.
                              With more than 4 jobs running it grows with them, up to 8x. */
} pps_server_config;

#define PPS_JOB_QUEUED  0  /* submitted, waiting for admission */
#define PPS_JOB_RUNNING 1  /* admitted: its pieces are being walked */
#define PPS_JOB_DONE    2
#define PPS_JOB_FAILED  3

typedef struct {
  uint64_t primes, prime_sum, factors;
  double latency_ms;       /* submission to result ready */
  int32_t status;          /* PPS_OK, or the failure code of a failed job */
  int32_t pad;
} pps_job_result;

typedef struct {
  uint64_t submitted, admitted, completed, refused, failed;
  uint64_t queued, running, reserved_bytes;
  uint64_t primes, steps, waves;
  uint32_t chunk, unroll;  /* the walk tuning of the batched form */
  double busy_ms;          /* worker time inside waves */
  double p50_ms, p99_ms;   /* latency of the completed jobs (nearest rank) */
} pps_server_stats;

int pps_server_create(int device, const pps_server_config *cfg, pps_server **out);
/* Stops the worker after its current wave; unfinished jobs are dropped.  No
   other call on this server may be in progress or follow. */
int pps_server_destroy(pps_server *s);
/* jp: normalised (pps_normalize).  *id identifies the job until its result is taken. */
int pps_job_submit(pps_server *s, const pps_job_params *jp, uint64_t *id);
int pps_job_poll(pps_server *s, uint64_t id, int *state);
/* Cancels a job: a queued job at once, a running one at the end of the wave in
   flight (its slot and reservation are freed then).  The job ends FAILED with
   status PPS_ERR_CANCELLED (pps_job_wait returns that code and releases it);
   a job already finished is left as it is (PPS_OK). */
int pps_job_cancel(pps_server *s, uint64_t id);
/* Waits up to timeout_s seconds (< 0: no limit; PPS_ERR_TIMEOUT when it
   expires).  Then *nout = the factor count and res (if given) the job's
   figures.  With out == NULL the job stays (a size query); otherwise the
   sorted (p, k, n, c) list is copied (PPS_ERR_OVERFLOW, job kept, when cap is
   too small) and the job is released.  A failed job returns its failure code. */
int pps_job_wait(pps_server *s, uint64_t id, double timeout_s, pps_factor *out, size_t cap,
                 size_t *nout, pps_job_result *res);
int pps_server_get_stats(pps_server *s, pps_server_stats *st);

/* ---- Checkpoints (main.c:304-372 write_checkpoint / read_checkpoint,
   pps/app.c:1301-1352).  A job is done for every prime below p; count and sum
   are the primes done and their wrapping sum, factor_count the factors found
   so far (all with p below the boundary). */
typedef struct {
  uint64_t pmin;          /* the job's pmin */
  uint64_t p;             /* boundary: every prime below p is done */
  uint64_t count, sum;
  uint32_t nmin, nmax;
  uint32_t factor_count;
  uint32_t pad;
} pps_checkpoint;

/* The reference's checkpoint file text, two lines:
   "pmin=%llu,p=%llu,count=%llu,sum=0x%016llx,checksum=0x%016llx" (checksum =
   pmin+p+count+sum) and "nmin=%u,nmax=%u,factor_count=%u".  Returns the length
   written, or a negative code (PPS_ERR_OVERFLOW when cap is too small). */
int pps_checkpoint_format(const pps_checkpoint *c, char *buf, size_t cap);
/* Parses that text and validates it for job jp as the reference does: pmin
   equal, pmin < p < pmax, the checksum, nmin and nmax equal.  An invalid
   checkpoint is PPS_ERR_INVALID_PARAM (the reference ignores it and starts
   over). */
int pps_checkpoint_parse(const char *text, const pps_job_params *jp, pps_checkpoint *c);

/* A served job's boundary: the p below which its pieces are walked (waves are
   the unit, so the boundary is drained), with the factors found so far, sorted
   (out == NULL: counts only).  A job resumed from it -- the same parameters
   with pmin = c->p -- gives exactly the remaining factors. */
int pps_job_checkpoint(pps_server *s, uint64_t id, pps_factor *out, size_t cap, size_t *nout,
                       pps_checkpoint *c);

/* Allocation-free walk (no counterpart in the reference): the walk and the
   output rule over np primes already in device memory (d_P), factors written
   to the caller's device buffer d_out (capacity out_cap, in no particular
   order), their count to *nout (host).  For callers that cannot call
   cudaMalloc -- device memory owned by another allocator or pool, or code that
   must not allocate while it runs: this call allocates nothing; its candidate
   scratch is a fixed __device__ array that each GPU loading the library holds
   until exit.  Limits: np <= PPS_NOALLOC_MAX_PRIMES per call (larger lists are
   rejected with PPS_ERR_INVALID_PARAM), and at most PPS_NOALLOC_MAX_CANDIDATES
   raw candidates per call (beyond that PPS_ERR_OVERFLOW: split the list).
   stream: a cudaStream_t or NULL; the call returns after the work finished
   (it synchronises the stream, so it cannot be captured into a CUDA graph).
   The first call on a device sets the scratch up: it looks the scratch's
   address up and copies a small-prime table into it.  The address is kept for the life of the
   process: cudaDeviceReset() of a set-up device is not supported (a call
   that then finds the table gone returns PPS_ERR_CUDA).  All calls on a
   device share the scratch: calls that overlap on the GPU race, so serialise
   them.  Errors: pps_last_error(). */
#define PPS_NOALLOC_MAX_PRIMES (1u << 24)
#define PPS_NOALLOC_MAX_CANDIDATES (1u << 16)
int pps_check_primes_noalloc(const pps_job_params *jp, const uint64_t *d_P, size_t np,
                             pps_factor *d_out, uint32_t out_cap, uint32_t *nout,
                             void *stream);

#ifdef __cplusplus
}
#endif
#endif
