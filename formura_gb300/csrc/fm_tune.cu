// fm_tune.cu — storage of the tuning knobs declared in fm_tune.h.
#include <map>
#include <mutex>
#include <string>

#include "fm_common.cuh"
#include "fm_tune.h"

namespace {
std::mutex g_mu;
std::map<std::string, int> &knobs() {
  static std::map<std::string, int> m;
  return m;
}
}  // namespace

namespace fm {
int tune_get(const char *key, int fallback) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = knobs().find(key);
  return it == knobs().end() ? fallback : it->second;
}

long long spin_limit() {
  const int v = tune_get("sync.spin_limit", 0);
  return v >= 1 ? (long long)v : kSpinLimitDefault;
}
}  // namespace fm

extern "C" int fm_tune_set(const char *key, int value) {
  FM_CHECK_ARG(key && *key, "fm_tune_set: empty key");
  std::lock_guard<std::mutex> lk(g_mu);
  knobs()[key] = value;
  return FM_OK;
}

extern "C" int fm_tune_clear(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  knobs().clear();
  return FM_OK;
}

extern "C" int fm_tune_get(const char *key, int fallback) { return fm::tune_get(key, fallback); }
