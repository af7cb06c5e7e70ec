// pps_input.cu -- input sieve files (-i): reading and the per-job key table.
//
// Host code only.  Restates the reference's file handling:
//   scan_input_file   pps/app.c:190-347  format detection, extents, side
//   read_newpgen_file pps/app.c:349-401  "k n" lines into the bitmap
//   read_abcd_file    pps/app.c:403-517  per-k blocks of n deltas (the twin
//                     build: per-n blocks of k-index deltas)
//   test_factor       pps/app.c:180-183  the bitmap as the output rule
// The reference's bitmap (one bit per (n - nmin, (k - kmin) / kstep)) becomes a
// sorted table of those bit numbers, which the device filter searches.
#include <inttypes.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <utility>
#include <vector>

#include "pps_engine_impl.h"

struct pps_input {
  int32_t format = 0;  // 1 NewPGen, 2 ABCD
  int32_t sign = 1;    // PPS_SIGN_TWIN for the twin build's formats
  bool k_index = false;  // twin ABCD: records hold the k index a (k = kstep a + koffset)
  std::vector<std::pair<uint64_t, uint32_t>> recs;  // (k, n) in file order
  uint64_t k0 = 0, k1 = 0;
  uint32_t n0 = 0, n1 = 0;
};

namespace {

constexpr int32_t FORMAT_NEWPGEN = 1, FORMAT_ABCD = 2;  // pps/app.c:81-82

bool abcd_header(const char* line, uint64_t* k, char* ch, uint32_t* n) {
  return sscanf(line, " ABCD %" SCNu64 "*2^$a%c1 [%u]", k, ch, n) == 3;
}

// The twin build's ABCD header (pps/app.c:212-213, 429-431): one n, both sides,
// the first k index a.
bool twin_abcd_header(const char* line, uint32_t* n, uint64_t* a) {
  uint32_t m = 0;
  return sscanf(line, " ABCD (6*$a+3)*2^%u+1 & (6*$a+3)*2^%u-1 [%" SCNu64 "]", &m, n, a) == 3 && m == *n;
}

}  // namespace

extern "C" int pps_input_read(const char* path, pps_job_spec* spec, pps_input** out) {
  if (!path || !spec || !out) return set_err(PPS_ERR_INVALID_PARAM, "null argument");
  *out = nullptr;
  FILE* f = fopen(path, "r");
  if (!f) return set_err(PPS_ERR_FOPEN, "%s: cannot open", path);
  std::vector<std::string> lines;
  {
    char buf[4096];
    std::string cur;
    while (fgets(buf, sizeof buf, f)) {
      cur += buf;
      if (!cur.empty() && cur.back() == '\n') {
        cur.pop_back();
        lines.push_back(cur);
        cur.clear();
      }
    }
    if (!cur.empty()) lines.push_back(cur);
    const bool bad = ferror(f) != 0;
    fclose(f);
    if (bad) return set_err(PPS_ERR_SCANF, "%s: read error", path);
  }
  // the scan (and with it format detection) runs only when a k or n bound is missing
  const bool scan = !(spec->kmin && spec->kmax && spec->nmin && spec->nmax);
  auto in = new pps_input();
  auto fail = [&](const char* what) {
    delete in;
    return set_err(PPS_ERR_SCANF, "%s `%s'", what, path);
  };
  uint64_t k = 0;
  uint32_t n = 0;
  char ch = 0;
  if (spec->sign == PPS_SIGN_TWIN) {
    // the twin build's formats (pps/app.c:208-216): ABCD per n with k-index
    // deltas, or NewPGen ":T:" -- the latter only while scanning
    in->sign = PPS_SIGN_TWIN;
    if (!lines.empty() && twin_abcd_header(lines[0].c_str(), &n, &k)) {
      in->format = FORMAT_ABCD;
      in->k_index = true;
      in->recs.emplace_back(k, n);
      for (size_t i = 1; i < lines.size(); ++i) {
        const char* s = lines[i].c_str();
        if (s[0] >= '0' && s[0] <= '9') {  // a k-index delta (pps/app.c:258-262, 474-477)
          k += strtoull(s, nullptr, 10);
          in->recs.emplace_back(k, n);
        } else if (twin_abcd_header(s, &n, &k)) {
          in->recs.emplace_back(k, n);
        } else if (s[strspn(s, " \t\r")] != '\0') {
          break;
        }
      }
    } else if (scan) {
      uint64_t p0 = 0;
      if (lines.empty() || sscanf(lines[0].c_str(), " %" SCNu64 ":T:%*c:2:%c", &p0, &ch) != 2 || ch != '3')
        return fail("Invalid header in input file");
      in->format = FORMAT_NEWPGEN;
      for (size_t i = 1; i < lines.size(); ++i) {
        if (sscanf(lines[i].c_str(), " %" SCNu64 " %u", &k, &n) != 2) {
          if (lines[i].find_first_not_of(" \t\r") == std::string::npos) continue;
          break;
        }
        in->recs.emplace_back(k, n);
      }
      if (in->recs.empty()) return fail("Invalid line 2 in input file");
    } else {
      return fail("Invalid header in input file");  // read as ABCD (pps/app.c:97)
    }
  } else if (!lines.empty() && abcd_header(lines[0].c_str(), &k, &ch, &n)) {
    in->format = FORMAT_ABCD;
    in->sign = ch == '+' ? 1 : -1;
    in->recs.emplace_back(k, n);
    for (size_t i = 1; i < lines.size(); ++i) {
      const char* s = lines[i].c_str();
      if (s[0] >= '0' && s[0] <= '9') {  // an n delta (pps/app.c:455-476)
        n += (uint32_t)strtoul(s, nullptr, 10);
        in->recs.emplace_back(k, n);
      } else if (abcd_header(s, &k, &ch, &n)) {
        in->recs.emplace_back(k, n);
      } else if (s[strspn(s, " \t\r")] != '\0') {
        break;  // neither a delta nor a header ends the file (pps/app.c:488-496)
      }
    }
  } else if (scan) {
    uint64_t p0 = 0;
    int c = 0;
    if (lines.empty() || sscanf(lines[0].c_str(), " %" SCNu64 ":P:%*c:2:%d", &p0, &c) != 2 ||
        (c != 1 && c != -1 && c != 255 && c != 257))
      return fail("Invalid header in input file");
    in->format = FORMAT_NEWPGEN;
    in->sign = (int32_t)(signed char)c;  // 255 and 257 as the reference's (char) cast reads them
    for (size_t i = 1; i < lines.size(); ++i) {
      if (sscanf(lines[i].c_str(), " %" SCNu64 " %u", &k, &n) != 2) {
        if (lines[i].find_first_not_of(" \t\r") == std::string::npos) continue;
        break;
      }
      in->recs.emplace_back(k, n);
    }
    if (in->recs.empty()) return fail("Invalid line 2 in input file");
  } else {
    return fail("Invalid header in input file");  // read as ABCD (pps/app.c:97, 424-434)
  }
  in->k0 = in->k1 = in->recs[0].first;
  in->n0 = in->n1 = in->recs[0].second;
  for (const auto& r : in->recs) {
    in->k0 = std::min(in->k0, r.first);
    in->k1 = std::max(in->k1, r.first);
    in->n0 = std::min(in->n0, r.second);
    in->n1 = std::max(in->n1, r.second);
  }
  in->n1++;  // pps/app.c:319
  if (in->k_index) {  // the indices as k (pps/app.c:325-331)
    const uint64_t kstep = spec->kstep ? spec->kstep : 6, koffset = spec->koffset ? spec->koffset : 3;
    in->k0 = kstep * in->k0 + koffset;
    in->k1 = kstep * in->k1 + koffset;
  }
  if (scan) {  // pps/app.c:335-346, and the side from the header (pps/app.c:216, 225)
    spec->sign = in->sign;
    if (spec->kmin < in->k0) spec->kmin = in->k0;
    if (spec->kmax == 0 || spec->kmax > in->k1) spec->kmax = in->k1;
    if (spec->nmin < in->n0) spec->nmin = in->n0;
    if (spec->nmax == 0 || spec->nmax > in->n1) spec->nmax = in->n1;
  }
  *out = in;
  return PPS_OK;
}

extern "C" int pps_input_get_info(const pps_input* in, pps_input_info* info) {
  if (!in || !info) return set_err(PPS_ERR_INVALID_PARAM, "null argument");
  info->format = in->format;
  info->sign = in->sign;
  info->records = in->recs.size();
  info->k0 = in->k0;
  info->k1 = in->k1;
  info->n0 = in->n0;
  info->n1 = in->n1;
  return PPS_OK;
}

extern "C" void pps_input_free(pps_input* in) { delete in; }

// ---------------------------------------------------------------- checkpoints
// main.c:304-326 write_checkpoint and pps/app.c:1348-1352 app_write_checkpoint.
extern "C" int pps_checkpoint_format(const pps_checkpoint* c, char* buf, size_t cap) {
  if (!c || (!buf && cap)) return set_err(PPS_ERR_INVALID_PARAM, "null argument");
  const uint64_t checksum = c->pmin + c->p + c->count + c->sum;
  const int n = snprintf(buf, cap,
                         "pmin=%" PRIu64 ",p=%" PRIu64 ",count=%" PRIu64 ",sum=0x%016" PRIx64
                         ",checksum=0x%016" PRIx64 "\nnmin=%u,nmax=%u,factor_count=%u\n",
                         c->pmin, c->p, c->count, c->sum, checksum, c->nmin, c->nmax, c->factor_count);
  if (n < 0) return set_err(PPS_ERR_INVALID_PARAM, "format");
  if ((size_t)n >= cap) return set_err(PPS_ERR_OVERFLOW, "checkpoint text needs %d bytes", n + 1);
  return n;
}

// main.c:332-372 read_checkpoint and pps/app.c:1301-1334 app_read_checkpoint
// (the factors-file check of the latter is the caller's).
extern "C" int pps_checkpoint_parse(const char* text, const pps_job_params* jp, pps_checkpoint* c) {
  if (!text || !jp || !c) return set_err(PPS_ERR_INVALID_PARAM, "null argument");
  pps_checkpoint r;
  memset(&r, 0, sizeof r);
  uint64_t checksum = 0;
  int used = 0;
  if (sscanf(text, "pmin=%" SCNu64 ",p=%" SCNu64 ",count=%" SCNu64 ",sum=0x%" SCNx64 ",checksum=0x%" SCNx64 "\n%n",
             &r.pmin, &r.p, &r.count, &r.sum, &checksum, &used) != 5 || used == 0)
    return set_err(PPS_ERR_INVALID_PARAM, "invalid checkpoint: first line");
  if (r.pmin != jp->pmin || r.p <= jp->pmin || r.p >= jp->pmax)
    return set_err(PPS_ERR_INVALID_PARAM, "invalid checkpoint: p outside the job");
  if (sscanf(text + used, "nmin=%u,nmax=%u,factor_count=%u", &r.nmin, &r.nmax, &r.factor_count) != 3)
    return set_err(PPS_ERR_INVALID_PARAM, "invalid checkpoint: second line");
  if (r.nmin != jp->nmin || r.nmax != jp->nmax) return set_err(PPS_ERR_INVALID_PARAM, "invalid checkpoint: n range");
  if (r.pmin + r.p + r.count + r.sum != checksum) return set_err(PPS_ERR_INVALID_PARAM, "invalid checkpoint: checksum");
  *c = r;
  return PPS_OK;
}

// The reference's bitmap for one job as sorted bit numbers
// (n - nmin) * width + kidx, width = (kmax - kmin) / kstep + 1.
int input_keys_for_job(const pps_input* in, const pps_job_params* jp, std::vector<uint64_t>* keys,
                       uint64_t* width) {
  const uint64_t kstep = jp->kstep, koffset = jp->koffset;
  const uint64_t w = (jp->kmax - jp->kmin) / kstep + 1;
  const unsigned __int128 bits = (unsigned __int128)(jp->nmax - jp->nmin + 1) * w;
  if (bits >> 64) return set_err(PPS_ERR_INSUFFICIENT_RESOURCE, "input bitmap too large");
  const uint64_t b0 = (jp->kmin - koffset) / kstep;  // pps/app.c:703
  keys->clear();
  keys->reserve(in->recs.size());
  for (const auto& r : in->recs) {
    const uint64_t k = r.first;
    const uint32_t n = r.second;
    uint64_t bit;
    if (in->format == FORMAT_NEWPGEN) {
      if (k % kstep != koffset) return set_err(PPS_ERR_SCANF, "Invalid line in input file: k=%" PRIu64, k);
      if (k < jp->kmin || k > jp->kmax) continue;
      bit = k / kstep - b0;  // pps/app.c:392
    } else if (in->k_index) {
      if (k < b0) continue;  // k is the twin build's index a (pps/app.c:451, 484)
      bit = k - b0;
      if (bit >= w) continue;
    } else {
      if (k < jp->kmin) continue;  // the reference writes before its bitmap here
      bit = (k - jp->kmin) / kstep;  // pps/app.c:438-441
      if (bit >= w) continue;
    }
    if (n < jp->nmin || n > jp->nmax) continue;
    keys->push_back((uint64_t)(n - jp->nmin) * w + bit);
  }
  std::sort(keys->begin(), keys->end());
  keys->erase(std::unique(keys->begin(), keys->end()), keys->end());
  *width = w;
  return PPS_OK;
}
