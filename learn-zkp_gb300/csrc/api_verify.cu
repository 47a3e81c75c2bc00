// libbasefold_gpu.so: the Basefold verifier on the host.
#include <algorithm>
#include <cstring>
#include <thread>
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
  bool skip(uint64_t m) {
    if (!ok || m > n - off) {
      ok = false;
      return false;
    }
    off += m;
    return true;
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


// ===========================================================================
// Verifier of many proofs: the transcripts on host threads, every query's
// Merkle paths and fold chain on the GPU (kernels_verify.cu).  Each job's
// result and challenger end as bf_verify's would.
// ===========================================================================
namespace {

// Where each field of a serialized BasefoldProof sits (bincode layout,
// basefold.rs:49-66); accepts exactly what parse_proof accepts.
struct Layout {
  struct Ext {
    uint64_t sib, path, path_n;
  };
  struct Open {
    uint64_t leaves, leaves_n, path, path_n, ext0, ext_n;
  };
  std::vector<uint64_t> rp_off, rp_n;
  uint64_t final_off = 0, final_n = 0, pi_off = 0, pi_n = 0;
  std::vector<Open> open;
  std::vector<Ext> ext;
};

bool parse_layout(const uint8_t* b, size_t n, Layout& lay) {
  Rd r{b, n};
  uint64_t a, k;
  if (!r.len(a, 64)) return false;
  for (uint64_t i = 0; i < a; ++i) {
    if (!r.len(k, 16)) return false;
    lay.rp_off.push_back(r.off);
    lay.rp_n.push_back(k);
    if (!r.skip(16 * k)) return false;
  }
  if (!r.len(a, 1 << 20)) return false;
  lay.final_off = r.off;
  lay.final_n = a;
  if (!r.skip(16 * a)) return false;
  if (!r.len(a, 64)) return false;
  lay.pi_off = r.off;
  lay.pi_n = a;
  if (!r.skip(32 * a)) return false;
  if (!r.len(a, 1 << 16)) return false;
  lay.open.resize(a);
  for (auto& o : lay.open) {
    if (!r.len(k, 1 << 16)) return false;
    o.leaves = r.off;
    o.leaves_n = k;
    if (!r.skip(16 * k)) return false;
    if (!r.len(k, 64)) return false;
    o.path = r.off;
    o.path_n = k;
    if (!r.skip(32 * k)) return false;
    if (!r.len(k, 64)) return false;
    o.ext0 = lay.ext.size();
    o.ext_n = k;
    for (uint64_t e = 0; e < k; ++e) {
      Layout::Ext x;
      x.sib = r.off;
      if (!r.skip(16)) return false;
      uint64_t m;
      if (!r.len(m, 64)) return false;
      x.path = r.off;
      x.path_n = m;
      if (!r.skip(32 * m)) return false;
      lay.ext.push_back(x);
    }
  }
  return r.ok && r.off == n;
}

struct VJob {
  int status = -1;  // decided on the host (BF_VERIFY_*), or -1: queries 0..nq_dev-1 go to the device
  Layout lay;
  std::vector<u128> rounds_x;  // challenge of each round, in round order
  std::vector<u128> scalars;   // width > 1
  std::vector<uint64_t> idx;   // query positions
  size_t nq_dev = 0;
  int after = BF_VERIFY_OK;  // status of query nq_dev, decided by its structure (or OK: none left)
  uint64_t elems = 0, proof = 0;  // device image offsets
};

// The transcript part of bf_verify for one job: the same observations,
// samples and checks, in the same order.
void verify_host_part(const bf_pcs* p, const bf_verify_job& jb, VJob& v) {
  const uint8_t* pf = jb.proof;
  if (!parse_layout(pf, jb.proof_len, v.lay)) {
    v.status = BF_VERIFY_MALFORMED;
    return;
  }
  const Layout& lay = v.lay;
  bfh::Challenger& ch = jb.challenger->c;
  const u128 ONE = bfh::one();
  const int d = p->d, L = p->L, log2_c = p->log2_c;
  const size_t width = jb.width;
  u128 claim = 0;
  if (width == 1) {
    v.scalars = {ONE};
    claim = bfh::load(jb.values);
  } else {
    v.scalars = sample_scalars_by_eq(width, ch);
    for (size_t i = 0; i < width; ++i) claim ^= bfh::mul(v.scalars[i], bfh::load(jb.values + 16 * i));
  }
  if ((int)lay.rp_n.size() != d || (int)lay.pi_n != d) {
    v.status = BF_VERIFY_MALFORMED;
    return;
  }
  u128 sc = claim;
  v.rounds_x.resize(d);
  for (int k = 0; k < d; ++k) {
    ch.observe(pf + lay.pi_off + 32 * (size_t)k, 32);
    if (lay.rp_n[k] != 2) {
      v.status = BF_VERIFY_MALFORMED;
      return;
    }
    const u128 c0 = bfh::load(pf + lay.rp_off[k]), c2 = bfh::load(pf + lay.rp_off[k] + 16);
    ch.observe_elem(c0);
    ch.observe_elem(c2);
    const u128 rp[3] = {c0, sc ^ c2, c2};  // Eval::decompress (eval.rs:68-79)
    const u128 x = ch.sample_elem();
    sc = horner(rp, 3, x);
    v.rounds_x[k] = x;
  }
  for (uint64_t i = 0; i < lay.final_n; ++i) ch.observe_elem(bfh::load(pf + lay.final_off + 16 * i));
  if (lay.final_n != 1) {
    v.status = BF_VERIFY_MALFORMED;
    return;
  }
  u128 eqv = ONE;  // eq_eval(point, r) with r[k] the challenge of round d-1-k
  for (int k = 0; k < d; ++k) eqv = bfh::mul(eqv, ONE ^ bfh::load(jb.point + 16 * k) ^ v.rounds_x[d - 1 - k]);
  if (bfh::mul(bfh::load(pf + lay.final_off), eqv) != sc) {
    v.status = BF_VERIFY_INVALID_FINAL_POLY;
    return;
  }
  const size_t Q = p->Q;
  v.idx.resize(Q);
  for (size_t q = 0; q < Q; ++q) v.idx[q] = ch.sample_bits(L);
  if (lay.open.size() != Q) {
    v.status = BF_VERIFY_MALFORMED;
    return;
  }
  // queries in order until one whose shape decides it: a wrong row width or
  // round count is malformed, a path of the wrong length fails its Merkle check
  for (size_t q = 0; q < Q; ++q) {
    const Layout::Open& o = lay.open[q];
    if (o.leaves_n != width || (int)o.ext_n != d) {
      v.after = BF_VERIFY_MALFORMED;
      break;
    }
    bool bad = (int)o.path_n != L;
    for (int k = 0; k < d && !bad; ++k) bad = (int)lay.ext[o.ext0 + k].path_n != log2_c + (d - 1 - k);
    if (bad) {
      v.after = BF_VERIFY_MMCS;
      break;
    }
    v.nq_dev = q + 1;
  }
  if (v.nq_dev == 0) v.status = v.after;
}

template <class F>
void parallel_jobs(size_t count, F&& f) {
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t nt = std::min<size_t>({(size_t)hw, (size_t)16, (count + 3) / 4});
  if (nt <= 1) {
    for (size_t i = 0; i < count; ++i) f(i);
    return;
  }
  std::vector<std::thread> th;
  for (size_t t = 0; t < nt; ++t)
    th.emplace_back([&, t] {
      for (size_t i = t; i < count; i += nt) f(i);
    });
  for (auto& x : th) x.join();
}

inline uint64_t align16(uint64_t x) { return (x + 15) & ~(uint64_t)15; }

}  // namespace

extern "C" int bf_verify_batch(bf_pcs* p, bf_verify_job* jobs, size_t count) {
  if (!p || (count && !jobs)) return fail(BF_ERR_ARG, "null argument");
  if (p->device < 0) return fail(BF_ERR_ARG, "verifier-only pcs (device < 0): use bf_verify");
  for (size_t j = 0; j < count; ++j) {
    const bf_verify_job& jb = jobs[j];
    if (!jb.root || !jb.challenger || (!jb.proof && jb.proof_len) || jb.width == 0 || jb.width > 4096 ||
        !jb.values || (p->d > 0 && !jb.point))
      return fail(BF_ERR_ARG, "bad verify job %zu", j);
    jobs[j].result = BF_VERIFY_OK;
  }
  if (count == 0) return BF_OK;
  std::lock_guard<std::mutex> lk(p->verify_mu);
  DeviceGuard g(p->device);
  const int d = p->d;
  const uint64_t Q = p->Q;
  // Device image: [jobs | queries | rounds | elements | proofs], then scratch
  // and flags.  Every job owns Q query slots and fixed element and proof
  // ranges, so one pass over the jobs fills it; slots a job does not use
  // (queries decided on the host) are marked inactive.
  const uint64_t nq = count * Q;
  if (nq > 0xffffffffull / (uint64_t)(d + 2)) return fail(BF_ERR_ARG, "too many queries in one batch");
  std::vector<VJob> v(count);
  const uint64_t off_jobs = 0;
  const uint64_t off_queries = align16(off_jobs + sizeof(bf::VerifyJob) * count);
  const uint64_t off_rounds = align16(off_queries + sizeof(bf::VerifyQuery) * nq);
  uint64_t cur = align16(off_rounds + sizeof(bf::VerifyRound) * nq * d);
  for (size_t j = 0; j < count; ++j) {
    v[j].elems = cur;
    cur += 32 + 16 * (uint64_t)d + (jobs[j].width > 1 ? 16 * (uint64_t)jobs[j].width : 0);
  }
  const uint64_t header = align16(cur);  // what the kernels read besides the proofs
  cur = header;
  for (size_t j = 0; j < count; ++j) {
    v[j].proof = cur;
    cur = align16(cur + jobs[j].proof_len);
  }
  const uint64_t image = cur;
  const uint64_t off_pairs = image, off_flags = off_pairs + 32 * nq * d;
  const uint64_t flag_bytes = nq * (uint64_t)(d + 2);
  const uint64_t dev_bytes = align16(off_flags + flag_bytes);
  if (nq > 0) {
    CU(p->verify_pin.ensure(image + align16(flag_bytes)));
    if (p->verify_dev.bytes < dev_bytes) CU(p->verify_dev.alloc(dev_bytes));
  }
  uint8_t* h = p->verify_pin.b();
  uint8_t* dv = reinterpret_cast<uint8_t*>(p->verify_dev.p);
  cudaStream_t st = p->stream;
  std::vector<cudaError_t> copy_err(count, cudaSuccess);
  parallel_jobs(count, [&](size_t j) {
    VJob& x = v[j];
    const bf_verify_job& jb = jobs[j];
    verify_host_part(p, jb, x);
    if (Q == 0) return;
    const Layout& lay = x.lay;
    const size_t active = x.status < 0 ? x.nq_dev : 0;
    bf::VerifyJob rec{};
    rec.root = x.elems;
    rec.challenges = x.elems + 32;
    rec.scalars = x.elems + 32 + 16 * (uint64_t)d;
    rec.pi_comms = x.proof + (active ? lay.pi_off : 0);
    rec.final_poly = x.proof + (active ? lay.final_off : 0);
    rec.width = (uint32_t)jb.width;
    std::memcpy(h + off_jobs + sizeof(rec) * j, &rec, sizeof(rec));
    if (active) {
      std::memcpy(h + x.elems, jb.root, 32);
      for (int k = 0; k < d; ++k) bfh::store(h + x.elems + 32 + 16 * k, x.rounds_x[k]);
      if (jb.width > 1)
        for (size_t w = 0; w < jb.width; ++w) bfh::store(h + rec.scalars + 16 * w, x.scalars[w]);
    }
    for (uint64_t q = 0; q < Q; ++q) {
      bf::VerifyQuery vq{};
      vq.job = q < active ? (uint32_t)j : bf::kVerifyInactive;
      const uint64_t gq = j * Q + q;
      if (q < active) {
        const Layout::Open& o = lay.open[q];
        vq.idx = x.idx[q];
        vq.leaves = x.proof + o.leaves;
        vq.path = x.proof + o.path;
        for (int k = 0; k < d; ++k) {
          const Layout::Ext& e = lay.ext[o.ext0 + k];
          bf::VerifyRound vr{x.proof + e.sib, x.proof + e.path};
          std::memcpy(h + off_rounds + sizeof(vr) * (gq * d + k), &vr, sizeof(vr));
        }
      }
      std::memcpy(h + off_queries + sizeof(vq) * gq, &vq, sizeof(vq));
    }
    if (active && jb.proof_len) {  // stage the proof and start its copy while other jobs are prepared
      std::memcpy(h + x.proof, jb.proof, jb.proof_len);
      copy_err[j] = cudaSetDevice(p->device);  // worker threads start on device 0
      if (copy_err[j] == cudaSuccess)
        copy_err[j] = cudaMemcpyAsync(dv + x.proof, h + x.proof, jb.proof_len, cudaMemcpyHostToDevice, st);
    }
  });
  for (cudaError_t e : copy_err) CU(e);
  if (nq > 0) {
    CU(cudaMemcpyAsync(dv, h, header, cudaMemcpyHostToDevice, st));
    bf::VerifyParams vp{};
    vp.blob = dv;
    vp.jobs = reinterpret_cast<const bf::VerifyJob*>(dv + off_jobs);
    vp.queries = reinterpret_cast<const bf::VerifyQuery*>(dv + off_queries);
    vp.rounds = reinterpret_cast<const bf::VerifyRound*>(dv + off_rounds);
    vp.tw = p->tw_view.as<bf::TwiddleView>();
    vp.pairs = reinterpret_cast<uint4*>(dv + off_pairs);
    vp.final_bad = dv + off_flags;
    vp.path_bad = dv + off_flags + nq;
    vp.nq = (uint32_t)nq;
    vp.d = d;
    vp.log2_c = p->log2_c;
    CU(bf::launch_verify(vp, st));
    uint8_t* flags = h + image;
    CU(cudaMemcpyAsync(flags, dv + off_flags, flag_bytes, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    // per job, the first query that fails decides (basefold.rs:284-322 checks
    // them in order): a bad path is an Mmcs error, a bad chain InvalidQuery
    for (size_t j = 0; j < count; ++j) {
      VJob& x = v[j];
      if (x.status >= 0) continue;
      x.status = x.after;
      for (size_t q = 0; q < x.nq_dev; ++q) {
        const uint64_t gq = j * Q + q;
        bool path_bad = false;
        for (int l = 0; l <= d && !path_bad; ++l) path_bad = flags[nq + (uint64_t)l * nq + gq] != 0;
        if (path_bad) {
          x.status = BF_VERIFY_MMCS;
          break;
        }
        if (flags[gq]) {
          x.status = BF_VERIFY_INVALID_QUERY;
          break;
        }
      }
    }
  }
  for (size_t j = 0; j < count; ++j) jobs[j].result = v[j].status < 0 ? v[j].after : v[j].status;
  return BF_OK;
}
