// K10: autotuner. Shape choices of the hot kernels (threads per block and
// lanes per row of the batched Lanczos kernel, lanes per row of the CSR SpMV)
// are timed on the caller's own data the first time a problem class is seen
// and remembered in a JSON file keyed by the class (kernel, value precision,
// real or complex, dimension and mean row length rounded to powers of two).
//
// File: $BLQH_TUNE_CACHE, else $HOME/.cache/blqh_gb300/tune.json (kept in
// memory only when neither can be written). BLQH_TUNE=0 turns tuning off (the
// fixed defaults are used). Entries: "key": [choice_a, choice_b, best_ms].
#include <sys/stat.h>
#include <unistd.h>

#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <string>

#include "blqh_internal.h"

namespace {

struct Entry {
  int a = 0, b = 0;
  double ms = 0;
};

std::mutex g_tune_mu;
std::map<std::string, Entry> g_tune;
bool g_loaded = false;
std::string g_loaded_path;  // file the in-memory table was read from

std::string cache_path() {
  if (const char* p = getenv("BLQH_TUNE_CACHE")) return p;
  if (const char* h = getenv("HOME")) return std::string(h) + "/.cache/blqh_gb300/tune.json";
  return "";
}

// Minimal reader of the file this unit writes: "key": [a, b, ms] pairs. The
// table follows the cache file: when the path changes the table is re-read.
void load_locked() {
  const std::string path = cache_path();
  if (g_loaded && path == g_loaded_path) return;
  g_loaded = true;
  g_loaded_path = path;
  g_tune.clear();
  if (path.empty()) return;
  FILE* f = fopen(path.c_str(), "r");
  if (!f) return;
  std::string s;
  char buf[4096];
  size_t n;
  while ((n = fread(buf, 1, sizeof buf, f)) > 0) s.append(buf, n);
  fclose(f);
  size_t i = 0;
  while ((i = s.find('"', i)) != std::string::npos) {
    const size_t j = s.find('"', i + 1);
    if (j == std::string::npos) break;
    const std::string key = s.substr(i + 1, j - i - 1);
    const size_t lb = s.find('[', j), rb = s.find(']', j);
    if (lb == std::string::npos || rb == std::string::npos || rb < lb) break;
    Entry e;
    if (sscanf(s.c_str() + lb + 1, "%d , %d , %lf", &e.a, &e.b, &e.ms) == 3) g_tune[key] = e;
    i = rb + 1;
  }
}

void mkdirs(const std::string& path) {
  for (size_t p = 1; p < path.size(); p++)
    if (path[p] == '/') mkdir(path.substr(0, p).c_str(), 0755);
}

void save_locked() {
  const std::string path = cache_path();
  if (path.empty()) return;
  mkdirs(path);
  const std::string tmp = path + ".tmp" + std::to_string((long)getpid());
  FILE* f = fopen(tmp.c_str(), "w");
  if (!f) return;
  fprintf(f, "{\n");
  size_t k = 0;
  for (const auto& kv : g_tune)
    fprintf(f, "  \"%s\": [%d, %d, %.6g]%s\n", kv.first.c_str(), kv.second.a, kv.second.b, kv.second.ms,
            ++k < g_tune.size() ? "," : "");
  fprintf(f, "}\n");
  fclose(f);
  rename(tmp.c_str(), path.c_str());
}

int log2_bucket(double v) { return v > 1 ? (int)std::lround(std::log2(v)) : 0; }

}  // namespace

bool tune_enabled() {
  const char* e = getenv("BLQH_TUNE");
  return !(e && e[0] == '0');
}

std::string tune_key(const char* kernel, int prec, int cplx, int64_t dim, double mean_row, int extra) {
  char b[160];
  snprintf(b, sizeof b, "%s|p%d|c%d|d2^%d|r2^%d|x%d", kernel, prec, cplx, log2_bucket((double)dim),
           log2_bucket(mean_row), extra);
  return b;
}

bool tune_lookup(const std::string& key, int* a, int* b) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  load_locked();
  auto it = g_tune.find(key);
  if (it == g_tune.end()) return false;
  *a = it->second.a;
  *b = it->second.b;
  return true;
}

void tune_store(const std::string& key, int a, int b, double ms) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  load_locked();
  g_tune[key] = Entry{a, b, ms};
  save_locked();
}
