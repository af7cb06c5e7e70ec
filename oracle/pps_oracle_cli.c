/* pps_oracle_cli.c -- command-line front end of the CPU oracle.

   ORACLE / TEST INFRASTRUCTURE ONLY.  Prints the sorted factor lines in the
   reference's format ("%llu | %llu*2^%u%+d", pps/app.c:133) followed on stderr by
   the prime fingerprint "count=...,sum=0x..." (main.c:1232) and the elapsed time.
   Options follow main.c:380-398 and pps/app.h:47-59: -p -P -k -K -n -N -R -M -s
   -Q, plus -t (threads) and -f (output file).  Number suffixes follow
   putil.c:86-168 (K M G T P = powers of 1000, k m g t p = powers of 1024, eN, bN).
*/
#define _GNU_SOURCE
#include <errno.h>
#include <inttypes.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>

#include "pps_oracle.h"

static int parse_u64(const char *s, uint64_t *out)
{
  char *tail;
  errno = 0;
  uint64_t v = strtoull(s, &tail, 0);
  if (errno) return -1;
  unsigned e = 0;
  switch (*tail) {
    case 'P': e += 3; /* fall through */
    case 'T': e += 3; /* fall through */
    case 'G': e += 3; /* fall through */
    case 'M': e += 3; /* fall through */
    case 'K': e += 3;
      if (tail[1]) return -1;
      while (e) { v *= 1000; e -= 3; }
      break;
    case 'p': e += 10; /* fall through */
    case 't': e += 10; /* fall through */
    case 'g': e += 10; /* fall through */
    case 'm': e += 10; /* fall through */
    case 'k': e += 10;
      if (tail[1]) return -1;
      v <<= e;
      break;
    case 'e': case 'E':
      e = (unsigned)strtoul(tail + 1, &tail, 0);
      if (*tail) return -1;
      while (e--) v *= 10;
      break;
    case 'b': case 'B':
      e = (unsigned)strtoul(tail + 1, &tail, 0);
      if (*tail) return -1;
      v <<= e;
      break;
    case '\0': break;
    default: return -1;
  }
  *out = v;
  return 0;
}

int main(int argc, char **argv)
{
  uint64_t pmin = 0, pmax = 0, kmin = 0, kmax = 0, v = 0;
  uint32_t nmin = 0, nmax = 0, kstep = 0, koffset = 0, qmax = 0;
  int32_t c = 1;
  int threads = (int)sysconf(_SC_NPROCESSORS_ONLN);
  const char *outfn = NULL;
  int opt;
  while ((opt = getopt(argc, argv, "p:P:k:K:n:N:RM:s:Q:t:f:q")) != -1) {
    if (optarg && opt != 'f' && parse_u64(optarg, &v)) {
      fprintf(stderr, "bad number for -%c: %s\n", opt, optarg);
      return 2;
    }
    switch (opt) {
      case 'p': pmin = v; break;
      case 'P': pmax = v; break;
      case 'k': kmin = v; break;
      case 'K': kmax = v; break;
      case 'n': nmin = (uint32_t)v; break;
      case 'N': nmax = (uint32_t)v; break;
      case 'R': c = -1; break;
      case 'M': kstep = (uint32_t)v; if (koffset >= kstep) koffset = kstep / 2; break;
      case 's': koffset = (uint32_t)v; break;
      case 'Q': qmax = (uint32_t)v; break;
      case 't': threads = (int)v; break;
      case 'f': outfn = optarg; break;
      case 'q': break;
      default: return 2;
    }
  }
  ppo_params pp;
  int rc = ppo_normalize(&pp, pmin, pmax, kmin, kmax, nmin, nmax, c, kstep, koffset, qmax);
  if (rc) {
    fprintf(stderr, "invalid parameters (%d)\n", rc);
    return 1;
  }
  fprintf(stderr, "kmin=%" PRIu64 " kmax=%" PRIu64 " nmin=%u nmax=%u nstep=%u qmax=%u\n",
          pp.kmin, pp.kmax, pp.nmin, pp.nmax, pp.nstep, pp.qmax);
  struct timespec t0, t1;
  clock_gettime(CLOCK_MONOTONIC, &t0);
  size_t cap = 1 << 20;
  ppo_factor *f = malloc(cap * sizeof *f);
  uint64_t count = 0, sum = 0;
  long nf = ppo_run(&pp, threads, f, cap, &count, &sum);
  clock_gettime(CLOCK_MONOTONIC, &t1);
  double secs = (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec);
  FILE *out = outfn ? fopen(outfn, "w") : stdout;
  if (!out) { perror(outfn); return 1; }
  for (long i = 0; i < nf && (size_t)i < cap; i++)
    fprintf(out, "%" PRIu64 " | %" PRIu64 "*2^%u%+d\n", f[i].p, f[i].k, f[i].n, f[i].c);
  if (outfn) fclose(out);
  fprintf(stderr, "count=%" PRIu64 ",sum=0x%016" PRIx64 "\n", count, sum);
  fprintf(stderr, "factors=%ld elapsed=%.3f s threads=%d\n", nf, secs, threads);
  free(f);
  return 0;
}
