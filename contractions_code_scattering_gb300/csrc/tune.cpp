// Autotuner: choices of tile schedules, kernel variants and batch sizes, cached
// per (knob, problem shape) key.
//
// A knob's candidates all compute the same results (up to rounding); only their
// speed differs with the shape and the device.  Kernel-level knobs are measured
// by re-launching each candidate on the live arguments of the call that first
// meets the key (the kernels involved are idempotent: they overwrite their
// outputs from unchanged inputs); batch-size knobs are measured on successive
// batches of the call's real work (engine_split.cu), so nothing is computed
// twice.  Measurements use CUDA events on the call's stream, after one untimed
// run of every candidate (first launches pay for module loading).
#include <algorithm>
#include <cfloat>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <set>
#include <sstream>

#include "ctr_internal.h"

namespace ctr {

namespace {

struct Entry {
  int choice = 0;
  std::vector<double> ms;  // per candidate (empty when loaded from a file)
};

std::mutex g_mu;
std::map<std::string, Entry> g_table;
std::map<std::string, int> g_forced;
std::set<std::string> g_fresh;  // keys measured since the mode was last set
int g_mode = 0;

}  // namespace

int tune_mode() { return capturing() ? 0 : g_mode; }

std::string tune_key(const char* knob, const std::string& shape) { return std::string(knob) + "|" + shape; }

int tune_forced(const char* knob) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_forced.find(knob);
  return it == g_forced.end() ? -1 : it->second;
}

bool tune_lookup(const std::string& key, int* choice) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_table.find(key);
  if (it == g_table.end()) return false;
  if (g_mode == 2 && !capturing() && !g_fresh.count(key)) return false;  // re-measure
  *choice = it->second.choice;
  return true;
}

void tune_store(const std::string& key, int choice, const std::vector<double>& ms) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_table[key] = Entry{choice, ms};
  g_fresh.insert(key);
}

bool tune_peek(const char* knob, const std::string& shape, int ncand, int dflt, int* choice) {
  const int forced = tune_forced(knob);
  if (forced >= 0) {
    *choice = forced;
    return forced < ncand;
  }
  if (tune_lookup(tune_key(knob, shape), choice) && *choice < ncand) return true;
  if (tune_mode() == 0) {
    *choice = dflt;
    return true;
  }
  return false;
}

int tune_resolve(const char* knob, const std::string& shape, int ncand, int dflt, cudaStream_t s,
                 const std::function<int(int)>& run, int* choice) {
  const int forced = tune_forced(knob);
  if (forced >= 0) {
    if (forced >= ncand) return fail(CTR_ERR_ARG, "tuning knob %s forced to %d, which is not below %d", knob, forced, ncand);
    *choice = forced;
    return CTR_OK;
  }
  const std::string key = tune_key(knob, shape);
  if (tune_lookup(key, choice) && *choice < ncand) return CTR_OK;
  if (tune_mode() == 0) {
    *choice = dflt;
    return CTR_OK;
  }
  cudaEvent_t e0, e1;
  CTR_CUDA(cudaEventCreate(&e0));
  CTR_CUDA(cudaEventCreate(&e1));
  std::vector<double> ms(ncand, DBL_MAX);
  int rc = CTR_OK;
  for (int c = 0; c < ncand && rc == CTR_OK; c++) rc = run(c);  // untimed: module loading, caches
  for (int rep = 0; rep < 3 && rc == CTR_OK; rep++)
    for (int c = 0; c < ncand && rc == CTR_OK; c++) {
      cudaEventRecord(e0, s);
      rc = run(c);
      cudaEventRecord(e1, s);
      if (rc != CTR_OK) break;
      float t = 0.f;
      cudaError_t e = cudaEventSynchronize(e1);
      if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
      if (e != cudaSuccess) rc = cuda_fail(e, "tuning events", __FILE__, __LINE__);
      ms[c] = std::min(ms[c], (double)t);
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  CTR_TRY(rc);
  int best = 0;
  for (int c = 1; c < ncand; c++)
    if (ms[c] < ms[best]) best = c;
  tune_store(key, best, ms);
  *choice = best;
  return CTR_OK;
}

}  // namespace ctr

extern "C" {

int ctr_tune_set_mode(int mode) {
  if (mode < 0 || mode > 2) return ctr::fail(CTR_ERR_ARG, "tuning mode %d not in {0,1,2}", mode);
  std::lock_guard<std::mutex> lk(ctr::g_mu);
  ctr::g_mode = mode;
  ctr::g_fresh.clear();
  return CTR_OK;
}

int ctr_tune_force(const char* knob, int value) {
  if (!knob || !*knob || std::strchr(knob, '|')) return ctr::fail(CTR_ERR_ARG, "ctr_tune_force: bad knob name");
  std::lock_guard<std::mutex> lk(ctr::g_mu);
  if (value < 0)
    ctr::g_forced.erase(knob);
  else
    ctr::g_forced[knob] = value;
  return CTR_OK;
}

int ctr_tune_report(char* buf, int buflen) {
  if (!buf || buflen < 3) return ctr::fail(CTR_ERR_ARG, "ctr_tune_report: buffer too small");
  std::ostringstream o;
  o << "{";
  {
    std::lock_guard<std::mutex> lk(ctr::g_mu);
    bool first = true;
    for (auto& kv : ctr::g_table) {
      o << (first ? "" : ", ") << "\"" << kv.first << "\": {\"choice\": " << kv.second.choice << ", \"ms\": [";
      for (size_t i = 0; i < kv.second.ms.size(); i++) {
        char t[32];
        snprintf(t, sizeof(t), "%s%.4f", i ? ", " : "", kv.second.ms[i]);
        o << t;
      }
      o << "]}";
      first = false;
    }
    for (auto& kv : ctr::g_forced) {
      o << (first ? "" : ", ") << "\"" << kv.first << "|forced\": {\"choice\": " << kv.second << ", \"ms\": []}";
      first = false;
    }
  }
  o << "}";
  const std::string s = o.str();
  if ((int)s.size() + 1 > buflen) return ctr::fail(CTR_ERR_ARG, "ctr_tune_report: buffer too small");
  std::memcpy(buf, s.c_str(), s.size() + 1);
  return CTR_OK;
}

void ctr_tune_clear(void) {
  std::lock_guard<std::mutex> lk(ctr::g_mu);
  ctr::g_table.clear();
  ctr::g_fresh.clear();
}

int ctr_tune_save(const char* path) {
  if (!path) return ctr::fail(CTR_ERR_ARG, "ctr_tune_save: null path");
  std::ofstream f(path);
  if (!f) return ctr::fail(CTR_ERR_IO, "ctr_tune_save: cannot open %s", path);
  std::lock_guard<std::mutex> lk(ctr::g_mu);
  for (auto& kv : ctr::g_table) f << kv.first << " " << kv.second.choice << "\n";
  return f ? CTR_OK : ctr::fail(CTR_ERR_IO, "ctr_tune_save: write to %s failed", path);
}

int ctr_tune_load(const char* path) {
  if (!path) return ctr::fail(CTR_ERR_ARG, "ctr_tune_load: null path");
  std::ifstream f(path);
  if (!f) return ctr::fail(CTR_ERR_IO, "ctr_tune_load: cannot open %s", path);
  std::map<std::string, ctr::Entry> add;
  std::string line;
  int ln = 0;
  while (std::getline(f, line)) {
    ln++;
    if (line.empty()) continue;
    const size_t sp = line.rfind(' ');
    if (sp == std::string::npos || sp == 0 || line.find('|') == std::string::npos || line.find('|') > sp)
      return ctr::fail(CTR_ERR_IO, "ctr_tune_load: %s:%d is not \"knob|shape choice\"", path, ln);
    char* end = nullptr;
    const long v = std::strtol(line.c_str() + sp + 1, &end, 10);
    if (!end || *end != '\0' || v < 0 || v > 1 << 30)
      return ctr::fail(CTR_ERR_IO, "ctr_tune_load: %s:%d has a bad choice", path, ln);
    add[line.substr(0, sp)] = ctr::Entry{(int)v, {}};
  }
  std::lock_guard<std::mutex> lk(ctr::g_mu);
  for (auto& kv : add) ctr::g_table[kv.first] = kv.second;
  return CTR_OK;
}

}  // extern "C"
