/* pps_oracle.c -- CPU restatement of PPSieve's hot path (see pps_oracle.h).

   ORACLE / TEST INFRASTRUCTURE ONLY: the shipped library never links or calls it.
   Every function cites the reference file:line it restates.  Arithmetic is plain
   unsigned __int128 math so that this file shares no code and no tricks with the
   device kernels it checks.
*/
#define _GNU_SOURCE
#include "pps_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 u128;

/* ---------------------------------------------------------------- helpers */

static int lg2_u64(uint64_t v) /* pps/app.c:641-647 lg2 */
{
  int r = 0;
  while (v >>= 1) r++;
  return r;
}

static uint64_t mulmod64(uint64_t a, uint64_t b, uint64_t m)
{
  return (uint64_t)(((u128)a * b) % m);
}

static uint64_t powmod64(uint64_t b, uint64_t e, uint64_t m)
{
  uint64_t r = 1 % m;
  b %= m;
  while (e) {
    if (e & 1) r = mulmod64(r, b, m);
    b = mulmod64(b, b, m);
    e >>= 1;
  }
  return r;
}

/* k*2^n + c mod p, for per-line verification. */
uint64_t ppo_kpow_mod(uint64_t k, uint32_t n, int32_t c, uint64_t p)
{
  uint64_t t = mulmod64(k % p, powmod64(2, n, p), p);
  if (c >= 0) return (uint64_t)(((u128)t + (uint64_t)c) % p);
  uint64_t cc = (uint64_t)(-(int64_t)c) % p;
  return t >= cc ? t - cc : t + p - cc;
}

/* Deterministic Miller-Rabin, bases 2..37 (exact for n < 3.3e24). */
int ppo_is_prime(uint64_t n)
{
  static const uint64_t bases[] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};
  if (n < 2) return 0;
  for (unsigned i = 0; i < sizeof bases / sizeof bases[0]; i++) {
    if (n == bases[i]) return 1;
    if (n % bases[i] == 0) return 0;
  }
  uint64_t d = n - 1;
  int s = 0;
  while ((d & 1) == 0) { d >>= 1; s++; }
  for (unsigned i = 0; i < sizeof bases / sizeof bases[0]; i++) {
    uint64_t x = powmod64(bases[i], d, n);
    if (x == 1 || x == n - 1) continue;
    int composite = 1;
    for (int r = 1; r < s; r++) {
      x = mulmod64(x, x, n);
      if (x == n - 1) { composite = 0; break; }
    }
    if (composite) return 0;
  }
  return 1;
}

/* ------------------------------------------------------- parameter rules */

int ppo_normalize(ppo_params *o, uint64_t pmin, uint64_t pmax, uint64_t kmin,
                  uint64_t kmax, uint32_t nmin, uint32_t nmax, int32_t c,
                  uint32_t kstep, uint32_t koffset, uint32_t qmax)
{
  const uint64_t PMAX_MAX = (uint64_t)1 << 62; /* main.h:43 */
  memset(o, 0, sizeof *o);
  if (c != 1 && c != -1 && c != PPO_TWIN) return PPO_ERR_INVALID_PARAM;
  /* pps/app.c:53-58 KSTEP/KOFFSET: 6/3 in the SEARCH_TWIN build, else 2/1 */
  if (kstep == 0) kstep = c == PPO_TWIN ? 6 : 2;
  if (koffset == 0) koffset = c == PPO_TWIN ? 3 : 1;

  /* main.c:916-931 */
  if (pmin < 3) pmin = 3;
  if (pmax > PMAX_MAX) pmax = PMAX_MAX;
  if (pmin >= pmax) {
    if (pmax == 0 && pmin < PMAX_MAX - 1000000000ULL)
      pmax = pmin + 1000000000ULL;
    else
      return PPO_ERR_INVALID_PARAM;
  }
  /* main.c:971-972 + sieve.c:98-110 */
  if (qmax == 0) qmax = 1u << 31;
  if ((uint64_t)qmax * qmax > pmax) qmax = (uint32_t)sqrt((double)pmax);
  if (qmax < 61) qmax = 61;

  /* pps/app.c:657-700 */
  if (kmin == 0 || kmax == 0) return PPO_ERR_INVALID_PARAM;
  if (kmin > kmax) return PPO_ERR_INVALID_PARAM;
  if (kmax >= pmin) return PPO_ERR_INVALID_PARAM;
  if (kmax - kmin >= ((uint64_t)3 << 36)) return PPO_ERR_INVALID_PARAM;
  if (nmin == 0) nmin = (uint32_t)(2 * lg2_u64(pmin) - lg2_u64(kmax) - 1);
  if (nmax == 0) nmax = nmin;
  if (nmin > nmax) return PPO_ERR_INVALID_PARAM;

  /* pps/app.c:703-712 */
  kmin = (kmin / kstep) * kstep + koffset;
  kmax = (kmax / kstep) * kstep + koffset;
  uint32_t nstep = 1;
  while ((kmax << nstep) < pmin) nstep++;

  /* pps/appcu.cu:158-204 */
  if (nstep > nmax - nmin + 1) nstep = nmax - nmin + 1;
  if ((((uint64_t)1) << (64 - nstep)) > pmin) return PPO_ERR_INVALID_PARAM;
  /* pps/appcu.cu:177-180: the twin walk steps one n less, so that consecutive
     steps overlap by one n (its even value is tested for i <= nstep) */
  if (c == PPO_TWIN) nstep--;
  if (nstep >= 32 && nstep < 48 && (((uint64_t)1) << 32) <= pmin) nstep = 32;
  if (lg2_u64(nmin) < 6) return PPO_ERR_INVALID_PARAM;
  /* pps/appcu.cu:236-239 */
  if (pmin <= ((uint64_t)1) << 32) return PPO_ERR_INVALID_PARAM;

  o->pmin = pmin; o->pmax = pmax;
  o->kmin = kmin; o->kmax = kmax;
  o->nmin = nmin; o->nmax = nmax;
  o->c = c; o->kstep = kstep; o->koffset = koffset;
  o->qmax = qmax; o->nstep = nstep;
  return PPO_OK;
}

/* ----------------------------------------------------------- output filter */

/* Odd primes 3 <= q < 32768 (pps/factor_proth.c:26-42 lists 11..32767; 3, 5
   and 7 are covered by the mod-15 / mod-7 tests of pps/app.c:171-172). */
static uint16_t g_small_primes[3600];
static int g_num_small;
static pthread_once_t g_small_once = PTHREAD_ONCE_INIT;

static void init_small_primes(void)
{
  static unsigned char comp[32768];
  int n = 0;
  for (int i = 3; i < 32768; i += 2) {
    if (comp[i]) continue;
    g_small_primes[n++] = (uint16_t)i;
    for (int j = i * i; j < 32768; j += 2 * i) comp[j] = 1;
  }
  g_num_small = n;
}

uint32_t ppo_small_factor(uint64_t k, uint32_t n, int32_t c)
{
  return ppo_small_factor_from(k, n, c, 3);
}

uint32_t ppo_small_factor_from(uint64_t k, uint32_t n, int32_t c, uint32_t qmin)
{
  pthread_once(&g_small_once, init_small_primes);
  for (int i = 0; i < g_num_small; i++) {
    uint32_t q = g_small_primes[i];
    if (q < qmin) continue;
    uint32_t t = (uint32_t)((k % q) * (uint64_t)powmod64(2, n, q) % q);
    t = (uint32_t)((t + (uint32_t)(c + (int32_t)q)) % q);
    if (t == 0) return q;
  }
  return 0;
}

/* pps/app.c:159-186 test_factor (bitmap == NULL branch). */
int ppo_test_factor(const ppo_params *pp, uint64_t k, uint32_t n, int32_t c)
{
  uint64_t b = k / pp->kstep;
  if (k != pp->kstep * b + pp->koffset) return 0;
  if (n < pp->nmin || n >= pp->nmax) return 0;
  if (pp->input_keys) {
    /* pps/app.c:180-183: the bit of (k, n) in the input file's bitmap */
    if (k < pp->kmin || k > pp->kmax) return 0;
    const uint64_t key = (uint64_t)(n - pp->nmin) * pp->input_width + (k - pp->kmin) / pp->kstep;
    uint64_t lo = 0, hi = pp->ninput;
    while (lo < hi) {
      const uint64_t mid = lo + (hi - lo) / 2;
      if (pp->input_keys[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo < pp->ninput && pp->input_keys[lo] == key;
  }
  return ppo_small_factor(k, n, c) == 0;
}

/* ------------------------------------------------------------------ walk */

/* -p^{-1} mod 2^64 by Newton iteration (pps/app.c:895-914 invmod2pow_ul). */
static uint64_t neg_inv64(uint64_t p)
{
  uint64_t r = p;              /* correct to 3 bits for odd p */
  for (int i = 0; i < 5; i++) r *= 2 - p * r;
  return (uint64_t)0 - r;
}

/* k * 2^-s mod p for k < p, s < 64: one Montgomery shift reduction
   (pps/app.c:963-986 shiftmod_REDC). */
static inline uint64_t shift_down(uint64_t k, uint64_t p, uint64_t ps, uint32_t s)
{
  uint64_t m = (k * ps) & ((((uint64_t)1) << s) - 1);
  uint64_t r = (uint64_t)(((u128)m * p + k) >> s);
  return r >= p ? r - p : r;
}

static void emit(ppo_factor *out, size_t cap, size_t *found, uint64_t p, uint64_t k, uint32_t n,
                 int32_t c)
{
  if (*found < cap) {
    out[*found].p = p; out[*found].k = k;
    out[*found].n = n; out[*found].c = c;
  }
  (*found)++;
}

/* The SEARCH_TWIN build of test_one_p (pps/app.c:1071-1107): one walk of
   k0 = 2^-n serves both sides, k0 itself for -1 and p - k0 for +1.  At nmin
   the odd one of the two is tested as it is; then at every step the even one,
   with i = ctz <= nstep, since the steps overlap by one n.  filter = 0 gives
   the raw candidates (k in range, n < nmax) with their sides. */
static size_t walk_twin(const ppo_params *pp, uint64_t p, ppo_factor *out, size_t cap, int filter)
{
  size_t found = 0;
  const uint64_t ps = neg_inv64(p);
  uint64_t k0 = powmod64((p + 1) / 2, pp->nmin, p);
  uint32_t n = pp->nmin;
  const uint32_t s = pp->nstep;
  uint64_t kpos = (k0 & 1) ? k0 : p - k0;
  if (kpos <= pp->kmax && kpos >= pp->kmin) {
    const int32_t c = kpos == k0 ? -1 : 1;
    if (filter ? ppo_test_factor(pp, kpos, n, c) : n < pp->nmax) emit(out, cap, &found, p, kpos, n, c);
  }
  do {
    kpos = (k0 & 1) ? p - k0 : k0;
    const int i = __builtin_ctzll(kpos);
    const uint64_t kk = kpos >> i;
    if (kk <= pp->kmax && kk >= pp->kmin && (uint32_t)i <= s) {
      const int32_t c = kpos == k0 ? -1 : 1;
      const uint32_t ni = n + (uint32_t)i;
      if (filter ? ppo_test_factor(pp, kk, ni, c) : ni < pp->nmax) emit(out, cap, &found, p, kk, ni, c);
    }
    n += s;
    k0 = shift_down(k0, p, ps, s);
  } while (n < pp->nmax);
  return found;
}

/* pps/app.c:1037-1121 test_one_p over the whole [nmin, nmax). */
size_t ppo_walk_prime(const ppo_params *pp, uint64_t p, ppo_factor *out, size_t cap)
{
  if (pp->c == PPO_TWIN) return walk_twin(pp, p, out, cap, 1);
  size_t found = 0;
  const uint64_t ps = neg_inv64(p);
  /* 2^-nmin mod p (pps/app.c:1014-1035 invpowmod_REDClr computes the same). */
  uint64_t k = powmod64((p + 1) / 2, pp->nmin, p);
  if (pp->c == 1) k = p - k; /* pps/app.c:1076 */
  uint32_t n = pp->nmin;
  const uint32_t s = pp->nstep;
  do {
    int i = __builtin_ctzll(k);
    uint64_t kk = k >> i;
    if (kk <= pp->kmax && kk >= pp->kmin && (uint32_t)i < s) {
      if (ppo_test_factor(pp, kk, n + (uint32_t)i, pp->c)) {
        if (found < cap) {
          out[found].p = p; out[found].k = kk;
          out[found].n = n + (uint32_t)i; out[found].c = pp->c;
        }
        found++;
      }
    }
    n += s;
    k = shift_down(k, p, ps, s);
  } while (n < pp->nmax);
  return found;
}

/* Raw candidates of one prime before the output filter: k in [kmin, kmax],
   nmin <= n < nmax (what sets a flag bit in pps/appcu.cu:803-1115).  Same walk
   as ppo_walk_prime; c is set to the job's sign. */
size_t ppo_walk_prime_raw(const ppo_params *pp, uint64_t p, ppo_factor *out, size_t cap)
{
  if (pp->c == PPO_TWIN) return walk_twin(pp, p, out, cap, 0);
  size_t found = 0;
  const uint64_t ps = neg_inv64(p);
  uint64_t k = powmod64((p + 1) / 2, pp->nmin, p);
  if (pp->c == 1) k = p - k;
  uint32_t n = pp->nmin;
  const uint32_t s = pp->nstep;
  do {
    int i = __builtin_ctzll(k);
    uint64_t kk = k >> i;
    if (kk <= pp->kmax && kk >= pp->kmin && (uint32_t)i < s && n + (uint32_t)i < pp->nmax) {
      if (found < cap) {
        out[found].p = p; out[found].k = kk;
        out[found].n = n + (uint32_t)i; out[found].c = pp->c;
      }
      found++;
    }
    n += s;
    k = shift_down(k, p, ps, s);
  } while (n < pp->nmax);
  return found;
}

/* ------------------------------------------------------------------ sieve */

typedef struct {
  uint32_t *q;
  size_t nq;
} base_primes;

static void make_base_primes(uint32_t qmax, base_primes *bp)
{
  /* Odd primes <= qmax by a segmented sieve seeded with primes <= sqrt(qmax). */
  uint32_t root = (uint32_t)sqrt((double)qmax) + 2;
  unsigned char *small = calloc(root + 1, 1);
  size_t cap = qmax < 100000 ? 20000 : (size_t)(1.2 * qmax / (log((double)qmax) - 1.2)) + 1000;
  bp->q = malloc(cap * sizeof(uint32_t));
  bp->nq = 0;
  uint32_t *seed = malloc((root / 2 + 2) * sizeof(uint32_t));
  size_t ns = 0;
  for (uint32_t i = 3; i <= root; i += 2) {
    if (small[i]) continue;
    seed[ns++] = i;
    for (uint64_t j = (uint64_t)i * i; j <= root; j += 2 * i) small[j] = 1;
  }
  const uint64_t SEG = 1 << 20;
  unsigned char *seg = malloc(SEG);
  for (uint64_t lo = 3; lo <= qmax; lo += 2 * SEG) {
    uint64_t hi = lo + 2 * SEG;
    if (hi > (uint64_t)qmax + 1) hi = (uint64_t)qmax + 1;
    size_t len = (hi - lo + 1) / 2;
    memset(seg, 0, len);
    for (size_t t = 0; t < ns; t++) {
      uint64_t q = seed[t];
      if (q * q >= hi) break;
      uint64_t st = q * q;
      if (st < lo) {
        st = ((lo + q - 1) / q) * q;
        if ((st & 1) == 0) st += q;
      }
      for (uint64_t m = st; m < hi; m += 2 * q) seg[(m - lo) / 2] = 1;
    }
    for (size_t j = 0; j < len; j++)
      if (!seg[j]) bp->q[bp->nq++] = (uint32_t)(lo + 2 * j);
  }
  free(seg);
  free(seed);
  free(small);
}

/* The table of odd primes up to the largest qmax asked for so far is built
   once per process and shared (read-only) by later calls and threads. */
static pthread_mutex_t g_base_mu = PTHREAD_MUTEX_INITIALIZER;
static base_primes g_base;
static uint32_t g_base_limit;

static void get_base_primes(uint32_t qmax, base_primes *view)
{
  pthread_mutex_lock(&g_base_mu);
  if (g_base.q == NULL || g_base_limit < qmax) {
    base_primes nb;
    make_base_primes(qmax, &nb);
    free(g_base.q);
    g_base = nb;
    g_base_limit = qmax;
  }
  size_t lo = 0, hi = g_base.nq; /* first index with q > qmax */
  while (lo < hi) {
    size_t mid = lo + (hi - lo) / 2;
    if (g_base.q[mid] <= qmax) lo = mid + 1; else hi = mid;
  }
  view->q = g_base.q;
  view->nq = lo;
  pthread_mutex_unlock(&g_base_mu);
}

/* Odd p in [lo, hi) with no prime factor q <= qmax other than p itself
   (sieve.c:168-608 with main.c:971-972 default qmax).  lo is rounded up to odd. */
static size_t sieve_segment(uint64_t lo, uint64_t hi, const base_primes *bp,
                            unsigned char *seg, uint64_t *out, size_t cap)
{
  lo |= 1;
  if (hi <= lo) return 0;
  size_t len = (hi - lo + 1) / 2;
  memset(seg, 0, len);
  for (size_t t = 0; t < bp->nq; t++) {
    uint64_t q = bp->q[t];
    if (q * q >= hi) break;
    uint64_t st = q * q;
    if (st < lo) {
      st = ((lo + q - 1) / q) * q;
      if ((st & 1) == 0) st += q;
    }
    for (uint64_t m = st; m < hi; m += 2 * q) seg[(m - lo) / 2] = 1;
  }
  size_t n = 0;
  for (size_t j = 0; j < len; j++) {
    if (seg[j]) continue;
    uint64_t p = lo + 2 * j;
    if (p < 3) continue;
    if (n < cap) out[n] = p;
    n++;
  }
  return n;
}

size_t ppo_sieve_range(uint64_t lo, uint64_t hi, uint32_t qmax, uint64_t *out, size_t cap)
{
  base_primes bp;
  get_base_primes(qmax, &bp);
  const uint64_t SEG = 1 << 20;
  unsigned char *seg = malloc(SEG);
  size_t total = 0;
  for (uint64_t a = lo; a < hi; a += 2 * SEG) {
    uint64_t b = a + 2 * SEG < hi ? a + 2 * SEG : hi;
    size_t room = total < cap ? cap - total : 0;
    total += sieve_segment(a, b, &bp, seg, out ? out + (total < cap ? total : 0) : NULL,
                           out ? room : 0);
  }
  free(seg);
  return total;
}

/* --------------------------------------------------------------- drivers */

typedef struct {
  const ppo_params *pp;
  const base_primes *bp;
  const uint64_t *P;   /* list mode */
  size_t np;
  uint64_t chunk;      /* range mode: range width per chunk */
  uint64_t nchunks;
  volatile uint64_t next;
  pthread_mutex_t mu;
  ppo_factor *out;
  size_t cap, nout;
  uint64_t count, sum;
} job_t;

static void job_emit(job_t *j, const ppo_factor *f, size_t nf, uint64_t cnt, uint64_t sm)
{
  pthread_mutex_lock(&j->mu);
  for (size_t i = 0; i < nf; i++) {
    if (j->nout < j->cap) j->out[j->nout] = f[i];
    j->nout++;
  }
  j->count += cnt;
  j->sum += sm;
  pthread_mutex_unlock(&j->mu);
}

static void *range_worker(void *arg)
{
  job_t *j = arg;
  const ppo_params *pp = j->pp;
  const uint64_t seg_len = j->chunk / 2 + 2;
  unsigned char *seg = malloc(seg_len);
  uint64_t *pr = malloc(seg_len * sizeof(uint64_t));
  size_t fcap = 64, nf;
  ppo_factor *f = malloc(fcap * sizeof *f);
  for (;;) {
    uint64_t ci = __atomic_fetch_add(&j->next, 1, __ATOMIC_RELAXED);
    if (ci >= j->nchunks) break;
    uint64_t lo = pp->pmin + ci * j->chunk;
    uint64_t hi = lo + j->chunk;
    if (hi > pp->pmax || hi < lo) hi = pp->pmax;
    size_t np = sieve_segment(lo, hi, j->bp, seg, pr, seg_len);
    uint64_t sm = 0;
    nf = 0;
    for (size_t i = 0; i < np; i++) {
      sm += pr[i];
      for (;;) {
        size_t got = ppo_walk_prime(pp, pr[i], f + nf, fcap - nf);
        if (nf + got <= fcap) { nf += got; break; }
        fcap *= 2;
        f = realloc(f, fcap * sizeof *f);
      }
    }
    job_emit(j, f, nf, np, sm);
  }
  free(f); free(pr); free(seg);
  return NULL;
}

static int cmp_factor(const void *a, const void *b)
{
  const ppo_factor *x = a, *y = b;
  if (x->p != y->p) return x->p < y->p ? -1 : 1;
  if (x->k != y->k) return x->k < y->k ? -1 : 1;
  if (x->n != y->n) return x->n < y->n ? -1 : 1;
  return (x->c > y->c) - (x->c < y->c);
}

static long run_threads(job_t *j, void *(*fn)(void *), int nthreads)
{
  if (nthreads < 1) nthreads = 1;
  pthread_t *t = malloc(nthreads * sizeof *t);
  for (int i = 0; i < nthreads; i++) pthread_create(&t[i], NULL, fn, j);
  for (int i = 0; i < nthreads; i++) pthread_join(t[i], NULL);
  free(t);
  size_t keep = j->nout < j->cap ? j->nout : j->cap;
  if (j->out && keep) qsort(j->out, keep, sizeof *j->out, cmp_factor);
  return (long)j->nout;
}

long ppo_run(const ppo_params *pp, int nthreads, ppo_factor *out, size_t cap,
             uint64_t *count, uint64_t *sum)
{
  base_primes bp;
  get_base_primes(pp->qmax, &bp);
  job_t j;
  memset(&j, 0, sizeof j);
  pthread_mutex_init(&j.mu, NULL);
  j.pp = pp; j.bp = &bp; j.out = out; j.cap = out ? cap : 0;
  /* at least ~8 chunks per thread, between 2^14 and 2^22 wide (even) */
  uint64_t span = pp->pmax - pp->pmin;
  uint64_t ch = span / ((uint64_t)(nthreads > 0 ? nthreads : 1) * 8);
  if (ch < ((uint64_t)1 << 14)) ch = (uint64_t)1 << 14;
  if (ch > ((uint64_t)1 << 22)) ch = (uint64_t)1 << 22;
  j.chunk = ch & ~(uint64_t)1;
  j.nchunks = (span + j.chunk - 1) / j.chunk;
  long r = run_threads(&j, range_worker, nthreads);
  if (count) *count = j.count;
  if (sum) *sum = j.sum;
  pthread_mutex_destroy(&j.mu);
  return r;
}

static void *list_worker(void *arg)
{
  job_t *j = arg;
  size_t fcap = 64;
  ppo_factor *f = malloc(fcap * sizeof *f);
  const uint64_t B = 256;
  for (;;) {
    uint64_t ci = __atomic_fetch_add(&j->next, 1, __ATOMIC_RELAXED);
    uint64_t lo = ci * B;
    if (lo >= j->np) break;
    uint64_t hi = lo + B < j->np ? lo + B : j->np;
    size_t nf = 0;
    uint64_t sm = 0;
    for (uint64_t i = lo; i < hi; i++) {
      sm += j->P[i];
      for (;;) {
        size_t got = ppo_walk_prime(j->pp, j->P[i], f + nf, fcap - nf);
        if (nf + got <= fcap) { nf += got; break; }
        fcap *= 2;
        f = realloc(f, fcap * sizeof *f);
      }
    }
    job_emit(j, f, nf, hi - lo, sm);
  }
  free(f);
  return NULL;
}

long ppo_walk_list(const ppo_params *pp, const uint64_t *P, size_t np, int nthreads,
                   ppo_factor *out, size_t cap)
{
  job_t j;
  memset(&j, 0, sizeof j);
  pthread_mutex_init(&j.mu, NULL);
  j.pp = pp; j.P = P; j.np = np; j.out = out; j.cap = out ? cap : 0;
  long r = run_threads(&j, list_worker, nthreads);
  pthread_mutex_destroy(&j.mu);
  return r;
}

/* ----------------------------------------------------- range fingerprint */

/* The count and 64-bit wrapping sum of the primes a sieve job walks, for
   ranges far too wide for ppo_sieve_range's output array: the reference's
   count=/sum= line (main.c:1232) over [lo, hi) with the sieve rule of
   sieve.c:168-608 (odd p with no prime factor q <= qmax other than p).

   Work items are chunks of up to 2^28 odd candidates, one bit each.  Sieving
   primes below WIN_BITS are marked window by window (128 KB windows, each q
   carrying its next multiple from window to window); larger ones first write
   their multiples' positions into per-window buckets, a bounded group of q at
   a time, and the buckets are then applied window by window, so that every
   bit clear lands in a cache-resident window. */
#define WIN_LOG 20
#define WIN_BITS ((uint64_t)1 << WIN_LOG)
#define BUCKET_GROUP_ENTRIES ((size_t)1 << 24)

typedef struct {
  uint64_t lo;          /* first odd candidate of the range */
  uint64_t nbits;       /* odd candidates in the range */
  uint64_t chunk_bits;  /* per work item */
  uint64_t nchunks;
  const base_primes *bp;
  volatile uint64_t next;
  pthread_mutex_t mu;
  uint64_t count, sum;
} fp_job;

typedef struct {
  uint32_t *e;
  size_t n, cap;
} bucket_t;

static void bucket_push(bucket_t *b, uint32_t v)
{
  if (b->n == b->cap) {
    b->cap = b->cap ? 2 * b->cap : 1024;
    b->e = realloc(b->e, b->cap * sizeof *b->e);
  }
  b->e[b->n++] = v;
}

/* bit index (from chunk value base, odd) of q's first odd multiple that is
   >= max(q*q, base), or UINT64_MAX when that is beyond hi */
static uint64_t first_hit(uint64_t q, uint64_t base, uint64_t hi)
{
  uint64_t st;
  if (q * q >= base) {
    st = q * q;
  } else {
    uint64_t r = base % q;
    st = r ? base + (q - r) : base;
    if ((st & 1) == 0) st += q;
  }
  if (st >= hi) return UINT64_MAX;
  return (st - base) >> 1;
}

static void fp_chunk(fp_job *j, uint64_t ci, uint64_t *bits, uint64_t *next_small, bucket_t *bk,
                     uint64_t *cnt_out, uint64_t *sum_out)
{
  const uint64_t b0 = ci * j->chunk_bits;
  const uint64_t nb = (j->nbits - b0) < j->chunk_bits ? (j->nbits - b0) : j->chunk_bits;
  const uint64_t base = j->lo + 2 * b0, hi = base + 2 * nb; /* odd values base .. hi-2 */
  const size_t nw = (size_t)((nb + 63) / 64);
  memset(bits, 0xff, nw * 8);
  if (nb & 63) bits[nw - 1] = ((uint64_t)1 << (nb & 63)) - 1;
  const base_primes *bp = j->bp;
  /* sieving primes that matter: q*q < hi */
  size_t nq = 0;
  while (nq < bp->nq && (uint64_t)bp->q[nq] * bp->q[nq] < hi) nq++;
  size_t nsmall = 0;
  while (nsmall < nq && bp->q[nsmall] < WIN_BITS) nsmall++;

  /* small q, window by window */
  for (size_t t = 0; t < nsmall; t++) next_small[t] = first_hit(bp->q[t], base, hi);
  for (uint64_t w0 = 0; w0 < nb; w0 += WIN_BITS) {
    const uint64_t w1 = w0 + WIN_BITS < nb ? w0 + WIN_BITS : nb;
    for (size_t t = 0; t < nsmall; t++) {
      const uint64_t q = bp->q[t];
      uint64_t x = next_small[t];
      for (; x < w1; x += q) bits[x >> 6] &= ~((uint64_t)1 << (x & 63));
      next_small[t] = x;
    }
  }

  /* large q through per-window buckets, a bounded group at a time */
  const size_t nwin = (size_t)((nb + WIN_BITS - 1) / WIN_BITS);
  size_t t = nsmall;
  while (t < nq) {
    size_t entries = 0;
    for (; t < nq && entries < BUCKET_GROUP_ENTRIES; t++) {
      const uint64_t q = bp->q[t];
      for (uint64_t x = first_hit(q, base, hi); x < nb; x += q) {
        bucket_push(&bk[x >> WIN_LOG], (uint32_t)(x & (WIN_BITS - 1)));
        entries++;
      }
    }
    for (size_t w = 0; w < nwin; w++) {
      uint64_t *wb = bits + ((uint64_t)w << (WIN_LOG - 6));
      for (size_t e = 0; e < bk[w].n; e++) {
        const uint32_t x = bk[w].e[e];
        wb[x >> 6] &= ~((uint64_t)1 << (x & 63));
      }
      bk[w].n = 0;
    }
  }

  uint64_t c = 0, s = 0;
  for (size_t w = 0; w < nw; w++) {
    uint64_t v = bits[w];
    while (v) {
      const int b = __builtin_ctzll(v);
      v &= v - 1;
      s += base + 2 * (64 * (uint64_t)w + (uint64_t)b);
      c++;
    }
  }
  *cnt_out = c;
  *sum_out = s;
}

static void *fp_worker(void *arg)
{
  fp_job *j = arg;
  uint64_t *bits = malloc((size_t)((j->chunk_bits + 63) / 64) * 8);
  uint64_t *next_small = malloc(sizeof(uint64_t) * (size_t)(WIN_BITS / 2 + 16));
  const size_t nwin = (size_t)((j->chunk_bits + WIN_BITS - 1) / WIN_BITS);
  bucket_t *bk = calloc(nwin, sizeof *bk);
  uint64_t c = 0, s = 0;
  for (;;) {
    const uint64_t ci = __atomic_fetch_add(&j->next, 1, __ATOMIC_RELAXED);
    if (ci >= j->nchunks) break;
    uint64_t cc, ss;
    fp_chunk(j, ci, bits, next_small, bk, &cc, &ss);
    c += cc;
    s += ss;
  }
  pthread_mutex_lock(&j->mu);
  j->count += c;
  j->sum += s;
  pthread_mutex_unlock(&j->mu);
  for (size_t w = 0; w < nwin; w++) free(bk[w].e);
  free(bk);
  free(next_small);
  free(bits);
  return NULL;
}

int ppo_sieve_fingerprint(uint64_t lo, uint64_t hi, uint32_t qmax, int nthreads, uint64_t *count,
                          uint64_t *sum)
{
  *count = 0;
  *sum = 0;
  lo |= 1;
  if (lo < 3) lo = 3;
  if (hi <= lo) return PPO_OK;
  base_primes bp;
  get_base_primes(qmax, &bp);
  fp_job j;
  memset(&j, 0, sizeof j);
  pthread_mutex_init(&j.mu, NULL);
  j.lo = lo;
  j.nbits = (hi - lo + 1) / 2;
  j.bp = &bp;
  if (nthreads < 1) nthreads = 1;
  /* about four work items per thread, 2^20 .. 2^28 candidates each */
  uint64_t cb = j.nbits / ((uint64_t)nthreads * 4) + 1;
  if (cb < WIN_BITS) cb = WIN_BITS;
  if (cb > ((uint64_t)1 << 28)) cb = (uint64_t)1 << 28;
  cb = (cb + WIN_BITS - 1) & ~(WIN_BITS - 1);
  j.chunk_bits = cb;
  j.nchunks = (j.nbits + cb - 1) / cb;
  pthread_t *th = malloc((size_t)nthreads * sizeof *th);
  for (int i = 0; i < nthreads; i++) pthread_create(&th[i], NULL, fp_worker, &j);
  for (int i = 0; i < nthreads; i++) pthread_join(th[i], NULL);
  free(th);
  *count = j.count;
  *sum = j.sum;
  pthread_mutex_destroy(&j.mu);
  return PPO_OK;
}

/* ---------------------------------------------------- per-line verification */

typedef struct {
  const ppo_params *jobs;
  const uint32_t *job_of;
  const ppo_factor *f;
  size_t n;
  uint8_t *bad;
  volatile uint64_t next;
  volatile long failures;
} vf_job;

static uint8_t verify_one(const ppo_params *pp, const ppo_factor *x)
{
  uint8_t b = 0;
  if (!ppo_is_prime(x->p)) b |= PPO_BAD_NOT_PRIME;
  if (x->p < pp->pmin || x->p >= pp->pmax) b |= PPO_BAD_P_RANGE;
  if (x->k < pp->kmin || x->k > pp->kmax || x->k != pp->kstep * (x->k / pp->kstep) + pp->koffset)
    b |= PPO_BAD_K;
  if (x->n < pp->nmin || x->n >= pp->nmax) b |= PPO_BAD_N;
  if (pp->c == PPO_TWIN ? (x->c != 1 && x->c != -1) : x->c != pp->c) b |= PPO_BAD_C;
  if ((x->c == 1 || x->c == -1) && x->p > 2 && ppo_kpow_mod(x->k, x->n, x->c, x->p) != 0)
    b |= PPO_BAD_NOT_DIVISOR;
  if (!(b & (PPO_BAD_K | PPO_BAD_N | PPO_BAD_C)) && !ppo_test_factor(pp, x->k, x->n, x->c))
    b |= PPO_BAD_RULE;
  return b;
}

static void *vf_worker(void *arg)
{
  vf_job *j = arg;
  const uint64_t B = 64;
  long bad = 0;
  for (;;) {
    const uint64_t i0 = __atomic_fetch_add(&j->next, B, __ATOMIC_RELAXED);
    if (i0 >= j->n) break;
    const uint64_t i1 = i0 + B < j->n ? i0 + B : j->n;
    for (uint64_t i = i0; i < i1; i++) {
      const ppo_params *pp = &j->jobs[j->job_of ? j->job_of[i] : 0];
      const uint8_t b = verify_one(pp, &j->f[i]);
      if (j->bad) j->bad[i] = b;
      bad += b != 0;
    }
  }
  __atomic_fetch_add(&j->failures, bad, __ATOMIC_RELAXED);
  return NULL;
}

long ppo_verify_factors(const ppo_params *jobs, const uint32_t *job_of, const ppo_factor *f, size_t n,
                        int nthreads, uint8_t *bad)
{
  vf_job j;
  memset(&j, 0, sizeof j);
  j.jobs = jobs;
  j.job_of = job_of;
  j.f = f;
  j.n = n;
  j.bad = bad;
  if (nthreads < 1) nthreads = 1;
  pthread_once(&g_small_once, init_small_primes);
  pthread_t *th = malloc((size_t)nthreads * sizeof *th);
  for (int i = 0; i < nthreads; i++) pthread_create(&th[i], NULL, vf_worker, &j);
  for (int i = 0; i < nthreads; i++) pthread_join(th[i], NULL);
  free(th);
  return j.failures;
}
