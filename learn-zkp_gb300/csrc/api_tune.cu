// libbasefold_gpu.so: the launch-shape autotuner.
//
// A pcs proves at one size (num_vars, blowup), so its best launch shapes are
// fixed per pcs: threads per NTT block and butterfly layers per NTT pass
// (the shared-memory tile, i.e. the NTT radix per pass), how many Merkle
// levels run in the single-block top kernel, and from which round on the
// open runs in the single-block tail.  bf_pcs_autotune times whole proofs
// (commit, evaluation, open, with this library's transcript) on random data
// for each candidate, one parameter at a time, and keeps the fastest.  The
// choice changes only how work is launched, never a byte of the proof.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "api_common.h"

using namespace bfapi;

namespace {

void to_vals(const bf::Tune& t, int* v) {
  v[0] = t.ntt_threads;
  v[1] = t.ntt_max_T;
  v[2] = t.top_nodes;
  v[3] = t.tail_log;
}

bf::Tune from_vals(const int* v) {
  bf::Tune t;
  t.ntt_threads = v[0];
  t.ntt_max_T = v[1];
  t.top_nodes = v[2];
  t.tail_log = v[3];
  return t;
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

extern "C" {

int bf_pcs_get_tune(const bf_pcs* p, int* vals, int n) {
  if (!p || !vals || n < 4) return fail(BF_ERR_ARG, "need 4 values");
  to_vals(p->tune, vals);
  return BF_OK;
}

int bf_pcs_set_tune(bf_pcs* p, const int* vals, int n) {
  if (!p || !vals || n < 4) return fail(BF_ERR_ARG, "need 4 values");
  const bf::Tune t = from_vals(vals);
  if (!bf::tune_valid(t))
    return fail(BF_ERR_ARG, "bad tune (ntt_threads %d, ntt_max_T %d, top_nodes %d, tail_log %d)", vals[0], vals[1],
                vals[2], vals[3]);
  p->tune = t;
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
      {"ntt_max_T", 1, {10, 11, 12}},
      {"ntt_threads", 0, {128, 256, 512}},
      {"top_nodes", 2, {128, 256, 512, 1024, 2048}},
      {"tail_log", 3, tails},
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
      int vals[4];
      to_vals(best, vals);
      vals[ax.slot] = v;
      const bf::Tune t = from_vals(vals);
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
  int vals[4];
  to_vals(best, vals);
  char tail[160];
  std::snprintf(tail, sizeof(tail),
                "}, \"best_ms\": %.4f, \"tune\": {\"ntt_threads\": %d, \"ntt_max_T\": %d, \"top_nodes\": %d, "
                "\"tail_log\": %d}}",
                best_ms, vals[0], vals[1], vals[2], vals[3]);
  rep += tail;
  if (report && cap) {
    std::strncpy(report, rep.c_str(), cap - 1);
    report[cap - 1] = '\0';
  }
  return BF_OK;
}

}  // extern "C"
