/* plugin_driver.c -- test harness for libppsgpu_app.so (include/pps_app.h).

   Plays the part of the reference's main.c around the plugin hooks, in the
   order main.c:887-1266 calls them: app_banner, app_parse_option per option,
   app_init, app_thread_init, app_thread_fun per full batch, app_thread_fun1 for
   the rest, app_write_checkpoint / app_read_checkpoint, app_thread_fini,
   app_fini.  Primes come from a file (little-endian uint64, in order) instead of
   sieve.c.  Prints count=...,sum=0x... like main.c:1232.

   usage: plugin_driver PRIMES_FILE -pPMIN -PPMAX [plugin options...]
*/
#include <errno.h>
#include <getopt.h>
#include <inttypes.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "pps_app.h"

int num_threads = 1;
uint64_t pmin, pmax, pstart;
unsigned int quiet_opt = 1;

/* main.c's number parser (putil.c parse_uint64 / parse_uint) is the
   executable's to provide; this stand-in reads the forms the tests pass:
   decimal or 0x numbers with an optional decimal exponent eN, or one suffix
   K M G T P (powers of 1000) or k m g t p (powers of 1024).  0 ok,
   -1 unparsable, -2 out of range. */
static int scale_checked(uint64_t *v, uint64_t f, unsigned long times, uint64_t hi)
{
  while (times--) {
    if (*v > hi / f) return -2;
    *v *= f;
  }
  return 0;
}

int parse_uint64(uint64_t *result, const char *str, uint64_t lo, uint64_t hi)
{
  static const char dec[] = "KMGTP", bin[] = "kmgtp";
  char *end;
  errno = 0;
  uint64_t v = strtoull(str, &end, 0);
  if (end == str) return -1;
  if (errno) return -2;
  int rc = 0;
  const char *d;
  if (*end == 'e' || *end == 'E') {
    char *e2;
    unsigned long x = strtoul(end + 1, &e2, 10);
    if (e2 == end + 1 || *e2) return -1;
    rc = scale_checked(&v, 10, x, hi);
  } else if (*end && end[1] == '\0' && (d = strchr(dec, *end)) != NULL) {
    rc = scale_checked(&v, 1000, (unsigned long)(d - dec) + 1, hi);
  } else if (*end && end[1] == '\0' && (d = strchr(bin, *end)) != NULL) {
    rc = scale_checked(&v, 1024, (unsigned long)(d - bin) + 1, hi);
  } else if (*end) {
    return -1;
  }
  if (rc) return rc;
  if (v < lo || v > hi) return -2;
  *result = v;
  return 0;
}

int parse_uint(unsigned int *result, const char *str, unsigned int lo, unsigned int hi)
{
  uint64_t v;
  int rc = parse_uint64(&v, str, lo, hi);
  if (rc == 0) *result = (unsigned int)v;
  return rc;
}

void bmsg(const char *msg) { fputs(msg, stderr); }
char *bmprefix(void) { return ""; }
void bexit(int status)
{
  fprintf(stderr, "bexit(%d)\n", status);
  exit(status == 0 ? 0 : 3);
}

int main(int argc, char **argv)
{
  if (argc < 2) return 2;
  FILE *f = fopen(argv[1], "rb");
  if (!f) { perror(argv[1]); return 2; }
  fseek(f, 0, SEEK_END);
  size_t np = (size_t)ftell(f) / 8;
  fseek(f, 0, SEEK_SET);
  uint64_t *all = malloc(np * 8 + 8);
  if (np && fread(all, 8, np, f) != np) return 2;
  fclose(f);

  app_banner();
  optind = 2;
  int opt;
  while ((opt = getopt(argc, argv, "p:P:q" PPS_APP_SHORT_OPTS)) != -1) {
    if (opt == 'p') pmin = strtoull(optarg, 0, 0);
    else if (opt == 'P') pmax = strtoull(optarg, 0, 0);
    else if (opt == 'q') quiet_opt = 1;
    else if (app_parse_option(opt, optarg, NULL) != 0) {
      fprintf(stderr, "invalid argument -%c %s\n", opt, optarg ? optarg : "");
      return 2;
    }
  }
  pstart = pmin | 1;
  app_init();
  unsigned cnt = app_thread_init(0);
  if (cnt == 0) { fprintf(stderr, "no device\n"); return 4; }
  uint64_t *P = malloc((size_t)cnt * 8), *K = malloc((size_t)cnt * 8);
  uint64_t count = 0, sum = 0;
  unsigned plen = 0;
  for (size_t i = 0; i < np; i++) {
    P[plen++] = all[i];
    count++;
    sum += all[i];
    if (plen == cnt) {
      app_thread_fun(0, P, K, cnt);
      plen = 0;
    }
  }
  app_thread_fun1(0, P, K, cnt, plen);
  FILE *cp = tmpfile();
  app_write_checkpoint(cp);
  rewind(cp);
  printf("checkpoint_ok=%d\n", app_read_checkpoint(cp));
  fclose(cp);
  app_thread_fini(0);
  app_fini(pmax);
  printf("count=%" PRIu64 ",sum=0x%016" PRIx64 "\n", count, sum);
  free(all); free(P); free(K);
  return 0;
}
