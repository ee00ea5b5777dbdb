// qdg_schedule.cpp -- FFT schedules of the line transforms: radix order and
// lines per batch, per line length and precision.
//
// The reference hands its transforms to FFTW, which picks an algorithm per
// size by planning and keeps the result as wisdom (src/fft/FFTGlobal.cpp:
// 26-84, src/fft/fft.cpp:98-122).  Here the schedules come from a table that
// the project's autotuner (qdng_gb300/autotune.py) writes after timing the
// candidates on the GPU: fft_schedules.txt next to libqdg.so, read once per
// process.  A size without an entry uses the greedy order (largest radices
// first).  Overrides set through the C ABI take precedence; the autotuner
// uses them to time candidates.
//
// Table lines: "<context> <n> <precision> <radix,radix,...> <lines>", with
// context "plan" (plans and their propagators) or "ensemble", precision
// "fp64", "df64" or "mixed", lines the step kernel's lines per batch
// (0: automatic).  '#' starts a comment.
#include <dlfcn.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/qdg.h"
#include "qdg_schedule.h"

namespace qdg {

namespace {

struct Entry {
  std::vector<int> radix;
  int lines = 0;
};
typedef std::tuple<int, int, int> Key;  // context, n, precision

std::mutex g_mu;
bool g_loaded = false;
bool g_use_table = true;
std::map<Key, Entry> g_table, g_override;

bool valid_radices(int n, const std::vector<int> &r) {
  if (r.empty() || r.size() > 16) return false;
  long long p = 1;
  for (int x : r) {
    if (x != 2 && x != 3 && x != 4 && x != 5 && x != 8 && x != 16) return false;
    p *= x;
  }
  return p == n;
}

int parse_precision(const std::string &s) {
  if (s == "fp64") return QDG_PREC_FP64;
  if (s == "mixed") return QDG_PREC_MIXED;
  if (s == "df64") return QDG_PREC_DF64;
  return -1;
}

int parse_context(const std::string &s) { return s == "plan" ? SCHED_PLAN : s == "ensemble" ? SCHED_ENSEMBLE : -1; }

// Directory of this library (the table sits next to it).
std::string library_dir() {
  Dl_info info;
  if (dladdr((void *)&library_dir, &info) == 0 || !info.dli_fname) return ".";
  std::string p(info.dli_fname);
  const size_t k = p.rfind('/');
  return k == std::string::npos ? "." : p.substr(0, k);
}

void load_table_locked() {
  if (g_loaded) return;
  g_loaded = true;
  const char *env = getenv("QDG_FFT_SCHEDULES");
  const std::string path = env ? env : library_dir() + "/fft_schedules.txt";
  std::ifstream f(path);
  std::string line;
  while (std::getline(f, line)) {
    const size_t h = line.find('#');
    if (h != std::string::npos) line.resize(h);
    std::istringstream in(line);
    std::string ctx, prec, rad;
    int n = 0, lines = 0;
    if (!(in >> ctx >> n >> prec >> rad >> lines)) continue;
    Entry e;
    e.lines = lines;
    std::stringstream rs(rad);
    std::string tok;
    while (std::getline(rs, tok, ',')) e.radix.push_back(atoi(tok.c_str()));
    const int c = parse_context(ctx), pr = parse_precision(prec);
    if (c < 0 || pr < 0 || !valid_radices(n, e.radix) || lines < 0 || lines > 64) continue;  // a bad line is skipped
    g_table[Key(c, n, pr)] = e;
  }
}

bool lookup(int context, int n, int precision, Entry &out) {
  std::lock_guard<std::mutex> lock(g_mu);
  load_table_locked();
  auto it = g_override.find(Key(context, n, precision));
  if (it != g_override.end()) { out = it->second; return true; }
  if (!g_use_table) return false;
  it = g_table.find(Key(context, n, precision));
  if (it != g_table.end()) { out = it->second; return true; }
  return false;
}

}  // namespace

bool greedy_radix(int n, RadixPlan &rp) {
  rp.n = n;
  rp.nstages = 0;
  int m = n;
  while (m % 16 == 0 && rp.nstages < 16) { rp.radix[rp.nstages++] = 16; m /= 16; }
  if (m % 8 == 0 && rp.nstages < 16) { rp.radix[rp.nstages++] = 8; m /= 8; }
  if (m % 4 == 0 && rp.nstages < 16) { rp.radix[rp.nstages++] = 4; m /= 4; }
  if (m % 2 == 0 && rp.nstages < 16) { rp.radix[rp.nstages++] = 2; m /= 2; }
  while (m % 3 == 0 && rp.nstages < 16) { rp.radix[rp.nstages++] = 3; m /= 3; }
  while (m % 5 == 0 && rp.nstages < 16) { rp.radix[rp.nstages++] = 5; m /= 5; }
  return m == 1;
}

bool any_radix(int n, RadixPlan &rp) {
  if (n < 1) return false;
  greedy_radix(n, rp);
  int m = n;
  for (int i = 0; i < rp.nstages; ++i) m /= rp.radix[i];
  // the other prime factors, ascending, one direct-DFT stage each
  for (int p = 7; m > 1 && rp.nstages < 16; p += 2) {
    if ((long long)p * p > m) p = m;  // what is left is prime
    while (m % p == 0 && rp.nstages < 16) { rp.radix[rp.nstages++] = p; m /= p; }
  }
  return m == 1;
}

bool generic_radix(const RadixPlan &rp) {
  for (int i = 0; i < rp.nstages; ++i) {
    const int r = rp.radix[i];
    if (r != 2 && r != 3 && r != 4 && r != 5 && r != 8 && r != 16) return true;
  }
  return false;
}

bool schedule_radix(int context, int n, int precision, RadixPlan &rp) {
  Entry e;
  if (lookup(context, n, precision, e)) {
    rp.n = n;
    rp.nstages = (int)e.radix.size();
    for (int i = 0; i < rp.nstages; ++i) rp.radix[i] = e.radix[i];
    return true;
  }
  return greedy_radix(n, rp);
}

int schedule_lines(int context, int n, int precision) {
  Entry e;
  return lookup(context, n, precision, e) ? e.lines : 0;
}

}  // namespace qdg

qdg_status qdg_fft_schedule_set(int32_t context, int32_t n, int32_t precision, const int32_t *radices,
                                int32_t nstages, int32_t lines) {
  if ((context != qdg::SCHED_PLAN && context != qdg::SCHED_ENSEMBLE) || n < 2 || nstages < 1 || nstages > 16 ||
      !radices || lines < 0 || lines > 64)
    return QDG_EINVAL;
  if (precision != QDG_PREC_FP64 && precision != QDG_PREC_MIXED && precision != QDG_PREC_DF64) return QDG_EINVAL;
  qdg::Entry e;
  e.radix.assign(radices, radices + nstages);
  e.lines = lines;
  if (!qdg::valid_radices(n, e.radix)) return QDG_EINVAL;
  std::lock_guard<std::mutex> lock(qdg::g_mu);
  qdg::g_override[qdg::Key(context, n, precision)] = e;
  return QDG_OK;
}

qdg_status qdg_fft_schedule_get(int32_t context, int32_t n, int32_t precision, int32_t *radices, int32_t *nstages,
                                int32_t *lines) {
  if (!radices || !nstages || !lines || n < 2) return QDG_EINVAL;
  qdg::RadixPlan rp;
  if (!qdg::schedule_radix(context, n, precision, rp)) return QDG_EUNSUPPORTED;
  for (int i = 0; i < rp.nstages; ++i) radices[i] = rp.radix[i];
  *nstages = rp.nstages;
  *lines = qdg::schedule_lines(context, n, precision);
  return QDG_OK;
}

qdg_status qdg_fft_schedule_reset(int32_t use_table) {
  std::lock_guard<std::mutex> lock(qdg::g_mu);
  qdg::g_override.clear();
  qdg::g_use_table = use_table != 0;
  return QDG_OK;
}
