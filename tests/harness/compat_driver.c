/* compat_driver.c -- test harness for libppsgpu_appcu.so (pps/appcu.h ABI).

   Plays the part of the reference's main.c + pps/app.c around the ABI: defines
   the globals they define (pps/app.h:88-96, main.h:57-60) and bmsg/bexit/
   bmprefix, then calls cuda_init, cuda_app_init, check_ns, get_factors_found,
   cuda_finalize in the order pps/app.c:649-790, 797-827, 1224-1286 does, with
   the same double buffering (walk batch i while batch i-1's flags are read).

   usage: compat_driver PRIMES_FILE pmin pmax kmin kmax nmin nmax sign nstep [mthreads]
   PRIMES_FILE holds little-endian uint64 primes.  Prints the subsection starts
   and one line "p mask" per prime with a non-zero flag byte.
*/
#include <inttypes.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "appcu_compat.h"

struct n_subsection {
  unsigned int n_subsection_start[9];
  unsigned int *first_n_subsection;
};
struct n_subsection *thread_subsections;
unsigned int nmin, nmax;
int search_proth = 1;
uint64_t kmax, kmin;
int num_threads = 1;
uint64_t pmin, pmax, pstart;
unsigned int quiet_opt = 1;

void bmsg(const char *msg) { fputs(msg, stderr); }
char *bmprefix(void) { return ""; }
void bexit(int status)
{
  fprintf(stderr, "bexit(%d)\n", status);
  exit(status == 0 ? 0 : 3);
}

static void emit(const uint64_t *P, const unsigned char *ff, unsigned n)
{
  for (unsigned i = 0; i < n; i++)
    if (ff[i]) printf("%" PRIu64 " %u\n", P[i], (unsigned)ff[i]);
}

int main(int argc, char **argv)
{
  if (argc < 10) {
    fprintf(stderr, "usage: %s PRIMES pmin pmax kmin kmax nmin nmax sign nstep [m]\n", argv[0]);
    return 2;
  }
  FILE *f = fopen(argv[1], "rb");
  if (!f) { perror(argv[1]); return 2; }
  fseek(f, 0, SEEK_END);
  long bytes = ftell(f);
  fseek(f, 0, SEEK_SET);
  size_t np = (size_t)bytes / 8;
  uint64_t *all = malloc(np * 8 + 8);
  if (fread(all, 8, np, f) != np) { perror("read"); return 2; }
  fclose(f);
  pmin = strtoull(argv[2], 0, 0);
  pmax = strtoull(argv[3], 0, 0);
  kmin = strtoull(argv[4], 0, 0);
  kmax = strtoull(argv[5], 0, 0);
  nmin = (unsigned)strtoul(argv[6], 0, 0);
  nmax = (unsigned)strtoul(argv[7], 0, 0);
  search_proth = atoi(argv[8]);
  ld_nstep = (unsigned)strtoul(argv[9], 0, 0);
  unsigned m = argc > 10 ? (unsigned)strtoul(argv[10], 0, 0) : 0;

  thread_subsections = calloc(1, sizeof *thread_subsections);
  cuda_init();
  unsigned cnt = cuda_app_init(0, 0, m);
  if (cnt == 0) { fprintf(stderr, "no device\n"); return 4; }
  printf("nstep %u\n", ld_nstep);
  printf("starts");
  for (int j = 0; j <= 8; j++) printf(" %u", thread_subsections[0].n_subsection_start[j]);
  printf("\n");

  uint64_t *P = malloc((size_t)cnt * 8), *lastP = malloc((size_t)cnt * 8);
  unsigned char *ff = malloc(cnt);
  unsigned last_len = 0;
  int started = 0;
  for (size_t off = 0; off < np; off += cnt) {
    unsigned len = (unsigned)((np - off) < cnt ? (np - off) : cnt);
    memcpy(P, all + off, (size_t)len * 8);
    /* pad a partial batch with a composite, as pps/app.c:1264-1270 does */
    if (len < cnt) {
      uint64_t c = P[len - 1];
      while (c % 3 != 0) c += 2;
      for (unsigned i = len; i < cnt; i++) P[i] = c;
    }
    if (started) get_factors_found(ff, cnt, 0, NULL);
    check_ns(P, cnt, 0);
    if (started) emit(lastP, ff, last_len);
    memcpy(lastP, P, (size_t)cnt * 8);
    last_len = len;
    started = 1;
  }
  if (started) {
    get_factors_found(ff, cnt, 0, NULL);
    emit(lastP, ff, last_len);
  }
  cuda_finalize();
  free(all); free(P); free(lastP); free(ff);
  return 0;
}
