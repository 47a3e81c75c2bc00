// libbasefold_gpu.so: the Basefold verifier on the host.
#include <cstring>
#include <vector>

#include "api_common.h"

using bfh::u128;
using namespace bfapi;

// ===========================================================================
// Verifier (host): basefold.rs:234-324.  Not on the prover's hot path; the
// reference runs it on the CPU as well.
// ===========================================================================
namespace {

struct ParsedProof {
  std::vector<std::vector<u128>> round_polys;
  std::vector<u128> final_poly;
  std::vector<std::array<uint8_t, 32>> pi_comms;
  struct Ext {
    u128 sibling;
    std::vector<std::array<uint8_t, 32>> path;
  };
  struct Opening {
    std::vector<u128> leaves;
    std::vector<std::array<uint8_t, 32>> path;
    std::vector<Ext> ext;
  };
  std::vector<Opening> openings;
};

struct Rd {
  const uint8_t* p;
  size_t n, off = 0;
  bool ok = true;
  uint64_t u64() {
    if (off + 8 > n) { ok = false; return 0; }
    uint64_t v;
    std::memcpy(&v, p + off, 8);
    off += 8;
    return v;
  }
  u128 elem() {
    if (off + 16 > n) { ok = false; return 0; }
    u128 v = bfh::load(p + off);
    off += 16;
    return v;
  }
  std::array<uint8_t, 32> dig() {
    std::array<uint8_t, 32> d{};
    if (off + 32 > n) { ok = false; return d; }
    std::memcpy(d.data(), p + off, 32);
    off += 32;
    return d;
  }
  bool len(uint64_t& v, uint64_t lim) {
    v = u64();
    if (v > lim) ok = false;
    return ok;
  }
};

bool parse_proof(const uint8_t* b, size_t n, ParsedProof& pf) {
  Rd r{b, n};
  uint64_t a, k;
  if (!r.len(a, 64)) return false;
  pf.round_polys.resize(a);
  for (auto& rp : pf.round_polys) {
    if (!r.len(k, 16)) return false;
    for (uint64_t i = 0; i < k; ++i) rp.push_back(r.elem());
  }
  if (!r.len(a, 1 << 20)) return false;
  for (uint64_t i = 0; i < a; ++i) pf.final_poly.push_back(r.elem());
  if (!r.len(a, 64)) return false;
  for (uint64_t i = 0; i < a; ++i) pf.pi_comms.push_back(r.dig());
  if (!r.len(a, 1 << 16)) return false;
  pf.openings.resize(a);
  for (auto& o : pf.openings) {
    if (!r.len(k, 1 << 16)) return false;
    for (uint64_t i = 0; i < k; ++i) o.leaves.push_back(r.elem());
    if (!r.len(k, 64)) return false;
    for (uint64_t i = 0; i < k; ++i) o.path.push_back(r.dig());
    if (!r.len(k, 64)) return false;
    o.ext.resize(k);
    for (auto& e : o.ext) {
      e.sibling = r.elem();
      uint64_t m;
      if (!r.len(m, 64)) return false;
      for (uint64_t i = 0; i < m; ++i) e.path.push_back(r.dig());
    }
  }
  return r.ok && r.off == n;
}

bool merkle_verify_host(const uint8_t root[32], int log_h, uint64_t index, const std::vector<u128>& row,
                        const std::vector<std::array<uint8_t, 32>>& path) {
  if ((int)path.size() != log_h) return false;
  std::vector<uint8_t> bytes(16 * row.size());
  for (size_t i = 0; i < row.size(); ++i) bfh::store(bytes.data() + 16 * i, row[i]);
  uint8_t cur[32], buf[64];
  bfh::keccak256(bytes.data(), bytes.size(), cur);
  for (int k = 0; k < log_h; ++k) {
    if ((index >> k) & 1) {
      std::memcpy(buf, path[k].data(), 32);
      std::memcpy(buf + 32, cur, 32);
    } else {
      std::memcpy(buf, cur, 32);
      std::memcpy(buf + 32, path[k].data(), 32);
    }
    bfh::keccak256(buf, 64, cur);
  }
  return std::memcmp(cur, root, 32) == 0;
}

uint64_t rev_bits(uint64_t x, int bits) {
  uint64_t r = 0;
  for (int i = 0; i < bits; ++i) r |= ((x >> i) & 1) << (bits - 1 - i);
  return r;
}

}  // namespace

extern "C" int bf_verify(const bf_pcs* p, const uint8_t root[32], const uint8_t* point, const uint8_t* values,
                         size_t width, int n_evals, bf_challenger* chp, const uint8_t* proof, size_t proof_len) {
  if (!p || !root || !chp || (!proof && proof_len)) return fail(BF_ERR_ARG, "null argument");
  if (n_evals == 0) return BF_VERIFY_OK;
  if (n_evals != 1 || width == 0 || !values || (p->d > 0 && !point)) return fail(BF_ERR_ARG, "bad evals");
  ParsedProof pf;
  if (!parse_proof(proof, proof_len, pf)) return BF_VERIFY_MALFORMED;
  bfh::Challenger& ch = chp->c;
  const u128 ONE = bfh::one();
  const int d = p->d, L = p->L, log2_c = p->log2_c;
  std::vector<u128> vals(width), scalars;
  for (size_t i = 0; i < width; ++i) vals[i] = bfh::load(values + 16 * i);
  u128 claim = 0;
  if (width == 1) {
    scalars = {ONE};
    claim = vals[0];
  } else {
    scalars = sample_scalars_by_eq(width, ch);
    for (size_t i = 0; i < width; ++i) claim ^= bfh::mul(scalars[i], vals[i]);
  }
  if ((int)pf.round_polys.size() != d || (int)pf.pi_comms.size() != d) return BF_VERIFY_MALFORMED;
  u128 sc = claim;
  std::vector<u128> xs(d);  // challenge of round i at xs[i]
  for (int k = 0; k < d; ++k) {
    ch.observe(pf.pi_comms[k].data(), 32);
    const auto& comp = pf.round_polys[k];
    if (comp.size() != 2) return BF_VERIFY_MALFORMED;
    ch.observe_elem(comp[0]);
    ch.observe_elem(comp[1]);
    const u128 rp[3] = {comp[0], sc ^ comp[1], comp[1]};  // Eval::decompress (eval.rs:68-79)
    const u128 x = ch.sample_elem();
    sc = horner(rp, 3, x);
    xs[d - 1 - k] = x;
  }
  for (u128 v : pf.final_poly) ch.observe_elem(v);
  if (pf.final_poly.size() != 1) return BF_VERIFY_MALFORMED;
  u128 eqv = ONE;
  for (int k = 0; k < d; ++k) eqv = bfh::mul(eqv, ONE ^ bfh::load(point + 16 * k) ^ xs[k]);
  if (bfh::mul(pf.final_poly[0], eqv) != sc) return BF_VERIFY_INVALID_FINAL_POLY;
  const size_t Q = p->Q;
  std::vector<uint64_t> idxs(Q);
  for (size_t q = 0; q < Q; ++q) idxs[q] = ch.sample_bits(L);
  if (pf.openings.size() != Q) return BF_VERIFY_MALFORMED;
  for (size_t q = 0; q < Q; ++q) {
    const uint64_t idx = idxs[q];
    const auto& o = pf.openings[q];
    if (o.leaves.size() != width || (int)o.ext.size() != d) return BF_VERIFY_MALFORMED;
    if (!merkle_verify_host(root, L, idx, o.leaves, o.path)) return BF_VERIFY_MMCS;
    u128 folded = 0;
    for (size_t i = 0; i < width; ++i) folded ^= bfh::mul(scalars[i], o.leaves[i]);
    for (int k = 0; k < d; ++k) {
      const int i = d - 1 - k;
      const uint64_t ni = (uint64_t)1 << (log2_c + i);
      const uint64_t sib = ((idx / ni) & 1) ^ 1;
      const uint64_t ii = idx % ni;
      std::vector<u128> v2(2, folded);
      v2[sib] = o.ext[k].sibling;
      if (!merkle_verify_host(pf.pi_comms[k].data(), log2_c + i, ii, v2, o.ext[k].path)) return BF_VERIFY_MMCS;
      // interpolate (binary_reed_solomon.rs:98-109): twiddle = stage (d-1-i) entry bitrev(ii)
      const int s = d - 1 - i;
      const uint64_t K = rev_bits(ii, log2_c + i);
      u128 t = 0;
      for (int b = 0; b < log2_c + i; ++b)
        if ((K >> b) & 1) t ^= p->bases[s][b];
      u128 lo = v2[0], hi = v2[1];
      hi ^= lo;
      lo ^= bfh::mul(hi, t);
      folded = lo ^ bfh::mul(hi ^ lo, xs[i]);
    }
    if (pf.final_poly[0] != folded) return BF_VERIFY_INVALID_QUERY;  // encode0 = [f; c]
  }
  return BF_VERIFY_OK;
}

