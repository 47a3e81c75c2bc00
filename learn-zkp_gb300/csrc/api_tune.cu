// libbasefold_gpu.so: the launch-shape autotuner.
//
// A pcs proves at one size (num_vars, blowup), so its best launch shapes are
// fixed per pcs: threads per NTT block and butterfly layers per NTT pass
// (the shared-memory tile, i.e. the NTT radix per pass), how many Merkle
// levels run in the single-block top kernel, and from which round on the
// open runs in the single-block tail.  bf_pcs_autotune times whole proofs
// (commit, evaluation, open, with this library's transcript) on random data
// for each candidate, one parameter at a time, and keeps the fastest; the
// result also goes into a process-wide cache keyed by (device name,
// num_vars, blowup) that every later pcs of that size starts from and that
// can be saved to and loaded from a JSON file.  The choice changes only how
// work is launched, never a byte of the proof.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <tuple>
#include <vector>

#include "api_common.h"

using namespace bfapi;

namespace {

constexpr int kVals = bf::kTuneVals;

void to_vals(const bf::Tune& t, int* v) {
  v[0] = t.ntt_threads;
  v[1] = t.ntt_max_T;
  v[2] = t.top_nodes;
  v[3] = t.tail_log;
  v[4] = t.subtree_log;
  v[5] = t.ntt_kind;
  v[6] = t.gf_mix;
  v[7] = t.ntt_ws_warps;
}

// The first n (>= 4) values over `base`: callers of the four-value form keep
// the other shapes as they are.
bf::Tune from_vals(const int* v, int n, const bf::Tune& base) {
  bf::Tune t = base;
  t.ntt_threads = v[0];
  t.ntt_max_T = v[1];
  t.top_nodes = v[2];
  t.tail_log = v[3];
  if (n > 4) t.subtree_log = v[4];
  if (n > 5) t.ntt_kind = v[5];
  if (n > 6) t.gf_mix = v[6];
  if (n > 7) t.ntt_ws_warps = v[7];
  return t;
}

// ---- per-(device, num_vars, blowup) cache of tuned shapes ------------------
// Filled by bf_pcs_autotune and bf_tune_cache_load, read by bf_pcs_setup (so
// every pcs the engine makes for a size picks that size's shapes up), and
// written by bf_tune_cache_save as a small JSON file:
//   {"version": 1, "entries": [
//    {"device": "NVIDIA GB300", "num_vars": 24, "log2_c": 1, "tune": [256, 12, 512, 8, 16, 1], "ms": 41.2},
//    ...]}
struct CacheEntry {
  bf::Tune tune;
  double ms;
};
std::mutex g_cache_mu;
std::map<std::tuple<std::string, int, int>, CacheEntry> g_cache;

std::string device_name(int dev) {
  static std::mutex mu;
  static std::map<int, std::string> names;
  std::lock_guard<std::mutex> lk(mu);
  auto it = names.find(dev);
  if (it != names.end()) return it->second;
  cudaDeviceProp prop;
  std::string name = cudaGetDeviceProperties(&prop, dev) == cudaSuccess ? std::string(prop.name) : "unknown";
  names[dev] = name;
  return name;
}

// Value of `"key": <int>` in `line` (-1 when absent).
bool json_int(const std::string& line, const char* key, long* out) {
  const std::string k = std::string("\"") + key + "\":";
  const size_t at = line.find(k);
  if (at == std::string::npos) return false;
  char* end = nullptr;
  *out = std::strtol(line.c_str() + at + k.size(), &end, 10);
  return end != line.c_str() + at + k.size();
}

// One commit + eval + open on device-resident `data`; host wall time in ms.
int prove_once(bf_pcs* p, const void* data, const std::vector<uint8_t>& point, std::vector<uint8_t>& proof,
               double* ms) {
  const auto t0 = std::chrono::steady_clock::now();
  bf_commitment* cm = nullptr;
  uint8_t root[32], value[16];
  TRY(bf_commit_device(p, data, 1, &cm, root));
  std::unique_ptr<bf_commitment, void (*)(bf_commitment*)> guard(cm, bf_commitment_free);
  TRY(bf_eval(p, cm, point.empty() ? nullptr : point.data(), value));
  bf_challenger ch;  // GenericChallenger::keccak256()
  ch.c.observe(root, 32);
  ch.c.observe(value, 16);
  size_t len = 0;
  TRY(bf_open(p, cm, point.empty() ? nullptr : point.data(), value, 1, &ch, proof.data(), proof.size(), &len));
  const auto t1 = std::chrono::steady_clock::now();
  *ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  return BF_OK;
}

}  // namespace

namespace bfapi {
void tune_cache_apply(bf_pcs* p) {
  if (p->device < 0) return;
  const auto key = std::make_tuple(device_name(p->device), p->d, p->log2_c);
  std::lock_guard<std::mutex> lk(g_cache_mu);
  auto it = g_cache.find(key);
  if (it != g_cache.end() && bf::tune_valid(it->second.tune)) p->tune = it->second.tune;
}
}  // namespace bfapi

extern "C" {

int bf_pcs_get_tune(const bf_pcs* p, int* vals, int n) {
  if (!p || !vals || n < 4) return fail(BF_ERR_ARG, "need at least 4 values");
  int v[kVals];
  to_vals(p->tune, v);
  for (int k = 0; k < n && k < kVals; ++k) vals[k] = v[k];
  return BF_OK;
}

int bf_pcs_set_tune(bf_pcs* p, const int* vals, int n) {
  if (!p || !vals || n < 4) return fail(BF_ERR_ARG, "need at least 4 values");
  const bf::Tune t = from_vals(vals, n, p->tune);
  if (!bf::tune_valid(t))
    return fail(BF_ERR_ARG,
                "bad tune (ntt_threads %d, ntt_max_T %d, top_nodes %d, tail_log %d, subtree_log %d, ntt_kind %d, "
                "gf_mix %d, ntt_ws_warps %d)",
                t.ntt_threads, t.ntt_max_T, t.top_nodes, t.tail_log, t.subtree_log, t.ntt_kind, t.gf_mix,
                t.ntt_ws_warps);
  p->tune = t;
  return BF_OK;
}

int bf_tune_cache_load(const char* path) {
  if (!path) return fail(BF_ERR_ARG, "null path");
  std::ifstream f(path);
  if (!f) return fail(BF_ERR_ARG, "cannot read %s", path);
  std::string line;
  int count = 0;
  std::lock_guard<std::mutex> lk(g_cache_mu);
  while (std::getline(f, line)) {
    const size_t dk = line.find("\"device\": \"");
    if (dk == std::string::npos) continue;
    const size_t d0 = dk + 11, d1 = line.find('"', d0);
    long nv = -1, lc = -1;
    const size_t tk = line.find("\"tune\": [");
    if (d1 == std::string::npos || tk == std::string::npos || !json_int(line, "num_vars", &nv) ||
        !json_int(line, "log2_c", &lc))
      return fail(BF_ERR_ARG, "%s: malformed entry: %s", path, line.c_str());
    int v[kVals];
    int k = 0;
    const char* c = line.c_str() + tk + 9;
    for (; k < kVals; ++k) {
      char* end = nullptr;
      v[k] = (int)std::strtol(c, &end, 10);
      if (end == c) break;
      c = end;
      while (*c == ',' || *c == ' ') ++c;
    }
    if (k < 4) return fail(BF_ERR_ARG, "%s: tune needs at least 4 values: %s", path, line.c_str());
    const bf::Tune t = from_vals(v, k, bf::Tune());
    if (!bf::tune_valid(t)) return fail(BF_ERR_ARG, "%s: invalid tune: %s", path, line.c_str());
    double ms = 0;
    const size_t mk = line.find("\"ms\":");
    if (mk != std::string::npos) ms = std::strtod(line.c_str() + mk + 5, nullptr);
    g_cache[std::make_tuple(line.substr(d0, d1 - d0), (int)nv, (int)lc)] = CacheEntry{t, ms};
    ++count;
  }
  return count;
}

int bf_tune_cache_save(const char* path) {
  if (!path) return fail(BF_ERR_ARG, "null path");
  std::ostringstream o;
  o << "{\"version\": 1, \"entries\": [\n";
  {
    std::lock_guard<std::mutex> lk(g_cache_mu);
    size_t i = 0;
    for (const auto& kv : g_cache) {
      int v[kVals];
      to_vals(kv.second.tune, v);
      char buf[384];
      std::snprintf(buf, sizeof(buf),
                    " {\"device\": \"%s\", \"num_vars\": %d, \"log2_c\": %d, \"tune\": [%d, %d, %d, %d, %d, %d, %d, "
                    "%d], \"ms\": %.4f}%s\n",
                    std::get<0>(kv.first).c_str(), std::get<1>(kv.first), std::get<2>(kv.first), v[0], v[1], v[2], v[3],
                    v[4], v[5], v[6], v[7], kv.second.ms, ++i < g_cache.size() ? "," : "");
      o << buf;
    }
  }
  o << "]}\n";
  std::ofstream f(path);
  if (!f) return fail(BF_ERR_ARG, "cannot write %s", path);
  f << o.str();
  return f.good() ? BF_OK : fail(BF_ERR_ARG, "write to %s failed", path);
}

int bf_tune_cache_clear(void) {
  std::lock_guard<std::mutex> lk(g_cache_mu);
  g_cache.clear();
  return BF_OK;
}

int bf_pcs_autotune(bf_pcs* p, int reps, char* report, size_t cap) {
  if (!p) return fail(BF_ERR_ARG, "null argument");
  if (p->device < 0) return fail(BF_ERR_ARG, "verifier-only pcs (device < 0)");
  if (reps < 1 || reps > 100) return fail(BF_ERR_ARG, "reps must be 1..100");
  DeviceGuard g(p->device);
  const int d = p->d;
  const size_t N = (size_t)1 << d;
  DevBuf data;
  CU(data.alloc(16 * N));
  CU(bf::launch_fill_random(data.as<uint4>(), N, 0x5eed0000ull + (uint64_t)d, p->stream));
  CU(cudaStreamSynchronize(p->stream));
  // a point with no coordinate 0 or 1 (those are rejected by open)
  std::vector<uint8_t> point(16 * (size_t)d);
  uint64_t x = 0x243f6a8885a308d3ull;
  for (auto& b : point) {
    x = x * 6364136223846793005ull + 1442695040888963407ull;
    b = (uint8_t)(x >> 56);
  }
  for (int k = 0; k < d; ++k) point[16 * k + 7] |= 0x10;  // nonzero, and not ONE (whose byte 7 is 0)
  std::vector<uint8_t> proof(bf_pcs_proof_size(p, 1, 1));

  const bf::Tune start = p->tune;
  auto measure = [&](const bf::Tune& t, double* best_ms) -> int {
    p->tune = t;
    double ms = 0;
    TRY(prove_once(p, data.p, point, proof, &ms));  // warm-up: pool allocations, caches
    std::vector<double> v;
    for (int r = 0; r < reps; ++r) {
      TRY(prove_once(p, data.p, point, proof, &ms));
      v.push_back(ms);
    }
    std::sort(v.begin(), v.end());
    *best_ms = v[v.size() / 2];
    return BF_OK;
  };
  struct Axis {
    const char* name;
    int slot;  // index in the get/set value order
    std::vector<int> values;
  };
  std::vector<int> tails;
  for (int t = 3; t <= bf::kTailMaxLeavesLog; ++t) tails.push_back(t);
  const std::vector<Axis> axes = {
      {"ntt_kind", 5, {2, 0, 1, 3}},
      {"ntt_max_T", 1, {10, 11, 12}},
      {"ntt_threads", 0, {128, 256, 512}},
      {"top_nodes", 2, {128, 256, 512, 1024, 2048}},
      {"subtree_log", 4, {12, 14, 16, 18}},
      {"tail_log", 3, tails},
      {"gf_mix", 6, {0, 2, 3, 4}},
      {"ntt_ws_warps", 7, {8, 4, 6, 10}},
  };
  bf::Tune best = start;
  double best_ms = 0;
  int rc = measure(best, &best_ms);
  if (rc < 0) {
    p->tune = start;
    return rc;
  }
  std::string rep = "{\"start_ms\": " + std::to_string(best_ms) + ", \"axes\": {";
  for (size_t a = 0; a < axes.size(); ++a) {
    const Axis& ax = axes[a];
    rep += (a ? ", \"" : "\"") + std::string(ax.name) + "\": {";
    bool first = true;
    for (int v : ax.values) {
      int vals[kVals];
      to_vals(best, vals);
      vals[ax.slot] = v;
      const bf::Tune t = from_vals(vals, kVals, best);
      if (!bf::tune_valid(t)) continue;
      double ms = 0;
      rc = measure(t, &ms);
      if (rc < 0) {
        p->tune = start;
        return rc;
      }
      rep += (first ? "\"" : ", \"") + std::to_string(v) + "\": " + std::to_string(ms);
      first = false;
      if (ms < best_ms) {
        best_ms = ms;
        best = t;
      }
    }
    rep += "}";
  }
  p->tune = best;
  {
    std::lock_guard<std::mutex> lk(g_cache_mu);
    g_cache[std::make_tuple(device_name(p->device), p->d, p->log2_c)] = CacheEntry{best, best_ms};
  }
  int vals[kVals];
  to_vals(best, vals);
  char tail[256];
  std::snprintf(tail, sizeof(tail),
                "}, \"best_ms\": %.4f, \"tune\": {\"ntt_threads\": %d, \"ntt_max_T\": %d, \"top_nodes\": %d, "
                "\"tail_log\": %d, \"subtree_log\": %d, \"ntt_kind\": %d, \"gf_mix\": %d, \"ntt_ws_warps\": %d}}",
                best_ms, vals[0], vals[1], vals[2], vals[3], vals[4], vals[5], vals[6], vals[7]);
  rep += tail;
  if (report && cap) {
    std::strncpy(report, rep.c_str(), cap - 1);
    report[cap - 1] = '\0';
  }
  return BF_OK;
}

}  // extern "C"
