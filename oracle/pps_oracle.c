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
