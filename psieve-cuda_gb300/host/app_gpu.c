/* app_gpu.c -- the application plugin hooks (include/pps_app.h) on the GPU
   library (include/ppsgpu.h).  Links behind the reference's main.c / sieve.c in
   place of pps/app.c + pps/appcu.cu + pps/factor_proth.c.

   Per host thread th: one engine on device (-d or th); app_thread_fun hands the
   batch to a worker thread and returns, so main.c sieves the next batch while
   the GPU walks this one (the pipelining of pps/app.c:1224-1250); the factors of
   a batch are reported when the next batch arrives or in app_thread_fun1.
   Options, messages, checkpoint lines and the factor line format follow
   pps/app.c:551-617, 649-790, 1294-1398 and 124-148.
*/
#define _GNU_SOURCE
#include <inttypes.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>

#include "pps_app.h"
#include "ppsgpu.h"

/* main.c symbols (main.h:51-60) */
extern int num_threads;
extern uint64_t pmin, pmax, pstart;
extern unsigned int quiet_opt;
void bmsg(const char *msg);
void bexit(int status);
char *bmprefix();

/* PPS_TWIN builds the twin plugin (the reference's tpsieve, -DSEARCH_TWIN:
   pps/app.h:20-45, pps/app.c:53-55): both sides from one walk, k == 3 mod 6
   by default, no -R. */
#ifdef PPS_TWIN
#define PPS_APP_NAME "tpsieve"
#define FACTORS_FILENAME_DEFAULT "tpfactors.txt"
#define KSTEP_DEFAULT 6u
#define KOFFSET_DEFAULT 3u
#else
#define PPS_APP_NAME "ppsieve"
#define FACTORS_FILENAME_DEFAULT "ppfactors.txt"
#define KSTEP_DEFAULT 2u
#define KOFFSET_DEFAULT 1u
#endif
#define PPS_APP_VERSION "gb300-0.1"
#define ERR_FOPEN (-108)
#define ERR_INVALID_PARAM (-178)
#define ERR_SCANF (-140)
#define MAX_APP_THREADS 64
#define BATCH_BLOCK 128u /* pps/appcu.h:14 */

/* pps/app.h:85-96 globals */
uint64_t kmin = 0, kmax = 0;
unsigned int nmin = 0, nmax = 0;
int search_proth = 1;
struct n_subsection *thread_subsections;

static const char *input_filename = NULL;
static pps_input *input_set = NULL;  /* -i: the file as the output rule */
static const char *factors_filename = NULL;
static FILE *factors_file = NULL;
static unsigned int factor_count = 0;
static int print_factors = 1;
static int device_opt = -1;
static unsigned int user_cthread_count = 0;
static unsigned int kstep = KSTEP_DEFAULT, koffset = KOFFSET_DEFAULT;
static pps_job_params job;
static pthread_mutex_t factors_mutex = PTHREAD_MUTEX_INITIALIZER;

typedef struct {
  pps_engine *eng;
  uint64_t *P;        /* copy of the batch being walked */
  unsigned count;
  pps_factor *out;
  size_t cap, nout;
  int rc;
  pthread_t worker;
  int running;
} app_thread_t;

static app_thread_t threads[MAX_APP_THREADS];

/* Number parsing is main.c's own: putil.c:86-168 parse_uint64 / parse_uint
   (putil.h:36-39), resolved from the executable like bexit() above, so option
   values are read exactly as the reference reads them (K M G T P suffixes,
   k m g t p, eN, bN; 0 ok, -1 unparsable, -2 out of range). */
int parse_uint(unsigned int *result, const char *str, unsigned int lo, unsigned int hi);
int parse_uint64(uint64_t *result, const char *str, uint64_t lo, uint64_t hi);

/* ------------------------------------------------------------------- hooks */

void app_banner(void)
{
  printf("%s version %s (GB300 sm_103a; %s)\n", PPS_APP_NAME, PPS_APP_VERSION, pps_version());
}

/* pps/app.c:551-617 */
int app_parse_option(int opt, char *arg, const char *source)
{
  int status = 0;
  switch (opt) {
    case 'k': status = parse_uint64(&kmin, arg, 1, ((uint64_t)1 << 62) - 1); break;
    case 'K': status = parse_uint64(&kmax, arg, 1, ((uint64_t)1 << 62) - 1); break;
    case 'm': status = parse_uint(&user_cthread_count, arg, 1, 1u << 31); break;
    case 'n': status = parse_uint(&nmin, arg, 1, (1u << 31) - 1); break;
    case 'N': status = parse_uint(&nmax, arg, 1, (1u << 31) - 1); break;
    case 'i': input_filename = (source == NULL) ? arg : strdup(arg); break;
    case 'f': factors_filename = (source == NULL) ? arg : strdup(arg); break;
    case 'd': status = parse_uint((unsigned *)&device_opt, arg, 0, INT32_MAX); break;
    case 'M':
      status = parse_uint(&kstep, arg, 1, (1u << 31) - 1);
      if (koffset >= kstep) koffset = kstep / 2;
      break;
    case 's': status = parse_uint(&koffset, arg, 1, (1u << 31) - 1); break;
#ifndef PPS_TWIN
    case 'R': search_proth = -1; break;
#endif
  }
  return status;
}

void app_help(void)
{
  printf("-f --factors=FILE  Write factors to FILE (default `%s')\n", FACTORS_FILENAME_DEFAULT);
  printf("-i --input=FILE    Read initial sieve from FILE\n");
  printf("-M --modulus       (Default 2)\n");
  printf("-s --modshift      Print only k's == s mod M. Default 1, or M/2\n");
  printf("-k --kmin=K0\n");
  printf("-K --kmax=K1       Sieve for primes k*2^n+/-1 with K0 <= k <= K1\n");
  printf("-m --mthreads=M    Force M threads or blocks/multiprocessor.\n");
  printf("-n --nmin=N0\n");
  printf("-N --nmax=N1       Sieve for primes k*2^n+/-1 with N0 <= n <= N1\n");
#ifndef PPS_TWIN
  printf("-R --riesel        Sieve for primes k*2^n-1 instead of +1.\n");
#endif
  printf("-d --device=N      Use GPU N instead of 0-threads\n");
}

/* pps/app.c:649-790 (the rules themselves live in pps_normalize) */
void app_init(void)
{
  pps_job_spec spec;
  print_factors = quiet_opt ? 0 : 1;
  memset(&spec, 0, sizeof spec);
  spec.pmin = pmin;
  spec.pmax = pmax;
  spec.kmin = kmin;
  spec.kmax = kmax;
  spec.nmin = nmin;
  spec.nmax = nmax;
#ifdef PPS_TWIN
  spec.sign = PPS_SIGN_TWIN;
#else
  spec.sign = search_proth;
#endif
  spec.kstep = kstep;
  spec.koffset = koffset;
  if (input_filename != NULL) {
    /* pps/app.c:661-663 and 726-738: the file fills the bounds the command
       line left open, and becomes the output rule (the twin build reads the
       twin formats, pps/app.c:208-216) */
    const int rc = pps_input_read(input_filename, &spec, &input_set);
    if (rc == PPS_ERR_FOPEN) {
      perror(input_filename);
      bexit(ERR_FOPEN);
    }
    if (rc != PPS_OK) {
      fprintf(stderr, "%s%s\n", bmprefix(), pps_last_error());
      bexit(ERR_SCANF);
    }
#ifndef PPS_TWIN
    search_proth = spec.sign;  /* the twin build's files are twin (both sides) */
#endif
  }
  if (pps_normalize(&spec, &job) != PPS_OK) {
    char msg[600];
    snprintf(msg, sizeof msg, "%s\n", pps_last_error());
    bmsg(msg);
    bexit(ERR_INVALID_PARAM);
  }
  kmin = job.kmin;
  kmax = job.kmax;
  nmin = job.nmin;
  nmax = job.nmax;
  printf("nstart=%u, nstep=%u\n", nmin, job.nstep);
  if (factors_filename == NULL) factors_filename = FACTORS_FILENAME_DEFAULT;
  if ((factors_file = fopen(factors_filename, "a")) == NULL) {
    fprintf(stderr, "%sCannot open factors file `%s'\n", bmprefix(), factors_filename);
    bexit(ERR_FOPEN);
  }
  thread_subsections = calloc((size_t)(num_threads > 0 ? num_threads : 1), sizeof *thread_subsections);
  printf("%s initialized: %" PRIu64 " <= k <= %" PRIu64 ", %u <= n < %u\n", PPS_APP_NAME, kmin,
         kmax, nmin, nmax);
  fflush(stdout);
}

/* pps/appcu.cu:257-266 batch size rule, per pps/app.c:797-827 */
unsigned int app_thread_init(int th)
{
  app_thread_t *t;
  unsigned cnt = user_cthread_count;
  int dev = device_opt >= 0 ? device_opt : th;
  if (th < 0 || th >= MAX_APP_THREADS) return 0;
  t = &threads[th];
  memset(t, 0, sizeof *t);
  if (pps_engine_create(dev, &t->eng) != PPS_OK) {
    fprintf(stderr, "%sGPU %d not usable: %s\n", bmprefix(), dev, pps_last_error());
    return 0;
  }
  if (input_set) pps_engine_set_input(t->eng, input_set);
  if (cnt == 0) cnt = 2048;
  else if (cnt < BATCH_BLOCK) cnt *= BATCH_BLOCK;
  else cnt -= cnt % BATCH_BLOCK;
  cnt *= (unsigned)pps_engine_sm_count(t->eng);
  t->P = malloc((size_t)cnt * sizeof(uint64_t));
  t->cap = 4096;
  t->out = malloc(t->cap * sizeof(pps_factor));
  if (!t->P || !t->out) return 0;
  /* one subsection [nmin, nmax) for code that inspects thread_subsections */
  for (int j = 1; j <= 8; j++) thread_subsections[th].n_subsection_start[j] = nmin;
  thread_subsections[th].n_subsection_start[0] = nmax;
  thread_subsections[th].first_n_subsection = &thread_subsections[th].n_subsection_start[0];
  fprintf(stderr, "%sThread %d: GPU %d, %u primes per batch\n", bmprefix(), th, dev, cnt);
  return cnt;
}

/* pps/app.c:124-148 */
static void report_factor(uint64_t p, uint64_t k, unsigned n, int c)
{
  pthread_mutex_lock(&factors_mutex);
  if (factors_file != NULL && fprintf(factors_file, "%" PRIu64 " | %" PRIu64 "*2^%u%+d\n", p, k, n, c) > 0) {
    if (print_factors) printf("%" PRIu64 " | %" PRIu64 "*2^%u%+d\n", p, k, n, c);
  } else {
    fprintf(stderr, "%sUNSAVED: %" PRIu64 " | %" PRIu64 "*2^%u%+d\n", bmprefix(), p, k, n, c);
  }
  factor_count++;
  pthread_mutex_unlock(&factors_mutex);
}

static void walk_batch(app_thread_t *t)
{
  for (;;) {
    size_t n = 0;
    t->rc = pps_check_primes(t->eng, &job, t->P, t->count, t->out, t->cap, &n, NULL);
    if (t->rc == PPS_ERR_OVERFLOW && n > t->cap) {
      t->cap = n;
      t->out = realloc(t->out, t->cap * sizeof(pps_factor));
      continue;
    }
    t->nout = n;
    return;
  }
}

static void *worker_main(void *arg)
{
  walk_batch((app_thread_t *)arg);
  return NULL;
}

/* Wait for the batch in flight and report its factors. */
static void drain(app_thread_t *t)
{
  if (!t->running) return;
  pthread_join(t->worker, NULL);
  t->running = 0;
  if (t->rc != PPS_OK) {
    fprintf(stderr, "%sGPU error: %s\n", bmprefix(), pps_last_error());
    bexit(EXIT_FAILURE);
  }
  for (size_t i = 0; i < t->nout; i++)
    report_factor(t->out[i].p, t->out[i].k, t->out[i].n, t->out[i].c);
  t->nout = 0;
}

/* pps/app.c:1224-1250 */
void app_thread_fun(int th, const uint64_t *P, uint64_t *lastP, const unsigned int cthread_count)
{
  app_thread_t *t = &threads[th];
  (void)lastP;
  drain(t);
  memcpy(t->P, P, (size_t)cthread_count * sizeof(uint64_t));
  t->count = cthread_count;
  if (pthread_create(&t->worker, NULL, worker_main, t) != 0) {
    bmsg("Cannot start the batch worker thread\n");
    bexit(EXIT_FAILURE);
  }
  t->running = 1;
}

/* pps/app.c:1257-1286: the partial batch of len primes, then drain. */
void app_thread_fun1(int th, uint64_t *P, uint64_t *lastP, const unsigned int cthread_count,
                     unsigned int len)
{
  app_thread_t *t = &threads[th];
  (void)lastP;
  (void)cthread_count;
  drain(t);
  if (len > 0) {
    memcpy(t->P, P, (size_t)len * sizeof(uint64_t));
    t->count = len;
    walk_batch(t);
    if (t->rc != PPS_OK) {
      fprintf(stderr, "%sGPU error: %s\n", bmprefix(), pps_last_error());
      bexit(EXIT_FAILURE);
    }
    for (size_t i = 0; i < t->nout; i++)
      report_factor(t->out[i].p, t->out[i].k, t->out[i].n, t->out[i].c);
    t->nout = 0;
  }
}

void app_thread_fini(int th)
{
  app_thread_t *t = &threads[th];
  drain(t);
  pps_engine_destroy(t->eng);
  free(t->P);
  free(t->out);
  memset(t, 0, sizeof *t);
}

/* pps/app.c:1294-1334 */
int app_read_checkpoint(FILE *fin)
{
  unsigned n0, n1;
  if (fscanf(fin, "nmin=%u,nmax=%u,factor_count=%u", &n0, &n1, &factor_count) != 3) {
    factor_count = 0;
    return 0;
  }
  if (n0 != nmin || n1 != nmax) {
    factor_count = 0;
    return 0;
  }
  if (factor_count > 0) {
    struct stat st;
    fstat(fileno(factors_file), &st);
    if (st.st_size == 0) {
      bmsg("Factors file missing.  Restarting test.\n");
      factor_count = 0;
      return 0;
    }
  }
  return 1;
}

/* pps/app.c:1348-1352 */
void app_write_checkpoint(FILE *fout)
{
  fflush(factors_file);
  fprintf(fout, "nmin=%u,nmax=%u,factor_count=%u\n", nmin, nmax, factor_count);
}

/* pps/app.c:1356-1398 */
void app_fini(uint64_t pstop)
{
  (void)pstop;
  if (factors_file) fclose(factors_file);
  factors_file = NULL;
  printf("Found %u factor%s\n", factor_count, (factor_count == 1) ? "" : "s");
  free(thread_subsections);
  thread_subsections = NULL;
  pps_input_free(input_set);
  input_set = NULL;
}
