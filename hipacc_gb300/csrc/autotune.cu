// autotune.cu -- the tile-configuration cache and its JSON persistence.
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>

#include "autotune.h"

namespace hgb {

namespace {
std::mutex g_mu;
std::map<std::string, std::pair<int, float>> g_cache;
bool g_enabled = false;
}  // namespace

bool autotune_enabled() { return g_enabled; }

int autotune_lookup(const char *key) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_cache.find(key);
  return it == g_cache.end() ? -1 : it->second.first;
}

void autotune_store(const char *key, int cfg, float ms) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_cache[key] = {cfg, ms};
}

}  // namespace hgb

using namespace hgb;

extern "C" {

int hgb_autotune_enable(int on) {
  g_enabled = on != 0;
  return HGB_OK;
}

int hgb_autotune_clear(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_cache.clear();
  return HGB_OK;
}

int hgb_autotune_count(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  return (int)g_cache.size();
}

// {"<key>": [cfg, ms], ...}
int hgb_autotune_save(const char *path) {
  HGB_REQUIRE(path, "hgb_autotune_save: null path");
  FILE *f = fopen(path, "w");
  if (!f) return set_error(HGB_ERR_INVALID, std::string("hgb_autotune_save: cannot open ") + path);
  std::lock_guard<std::mutex> lk(g_mu);
  fprintf(f, "{");
  bool first = true;
  for (auto &kv : g_cache) {
    fprintf(f, "%s\n  \"%s\": [%d, %.6f]", first ? "" : ",", kv.first.c_str(), kv.second.first, kv.second.second);
    first = false;
  }
  fprintf(f, "\n}\n");
  fclose(f);
  return HGB_OK;
}

int hgb_autotune_load(const char *path) {
  HGB_REQUIRE(path, "hgb_autotune_load: null path");
  FILE *f = fopen(path, "r");
  if (!f) return set_error(HGB_ERR_INVALID, std::string("hgb_autotune_load: cannot open ") + path);
  std::string s;
  char buf[4096];
  size_t n;
  while ((n = fread(buf, 1, sizeof(buf), f)) > 0) s.append(buf, n);
  fclose(f);
  std::lock_guard<std::mutex> lk(g_mu);
  size_t pos = 0;
  int loaded = 0;
  while ((pos = s.find('"', pos)) != std::string::npos) {
    size_t end = s.find('"', pos + 1);
    if (end == std::string::npos) break;
    std::string key = s.substr(pos + 1, end - pos - 1);
    int cfg = -1;
    float ms = 0.f;
    if (sscanf(s.c_str() + end + 1, " : [ %d , %f ]", &cfg, &ms) == 2 && cfg >= 0) {
      g_cache[key] = {cfg, ms};
      ++loaded;
    }
    pos = end + 1;
  }
  return loaded > 0 || s.find('"') == std::string::npos ? HGB_OK
                                                        : set_error(HGB_ERR_INVALID, "hgb_autotune_load: no entries");
}

}  // extern "C"
