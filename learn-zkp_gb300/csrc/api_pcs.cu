// libbasefold_gpu.so: setup, commit, eval, transcript objects, timing and
// test hooks.
//
// The prover keeps every array of the path in device memory: evaluations,
// codeword, Merkle trees, folded codewords and their trees, the sumcheck
// polynomial and its eq table.  What crosses to the host is what the caller
// receives (roots, evaluations, the proof) and, at the end of an open, the
// transcript state from which the query positions are sampled.
#include <nvtx3/nvToolsExt.h>
#include <cuda_runtime.h>

#include <algorithm>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <memory>

#include "api_common.h"

using bfh::u128;

namespace bfapi {

void pcs_acquire(bf_pcs* p) { p->refs.fetch_add(1, std::memory_order_relaxed); }

void pcs_release(bf_pcs* p) {
  if (p->refs.fetch_sub(1, std::memory_order_acq_rel) != 1) return;
  if (p->device < 0) {  // a verifier-only pcs touches no device
    delete p;
    return;
  }
  DeviceGuard g(p->device);
  delete p;
}

namespace {
thread_local std::string g_err;
}

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

const std::string& last_error() { return g_err; }

cudaEvent_t Profiler::get() {
  if (!pool.empty()) {
    cudaEvent_t e = pool.back();
    pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}

Profiler::~Profiler() {
  for (auto& p : pending) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  for (auto e : pool) cudaEventDestroy(e);
}

void Profiler::drain() {
  for (auto& p : pending) {
    float t = 0.f;
    if (cudaEventElapsedTime(&t, p.a, p.b) == cudaSuccess) {
      ms[p.cls] += t;
      count[p.cls] += 1;
    }
    pool.push_back(p.a);
    pool.push_back(p.b);
  }
  pending.clear();
}

// NVTX range names of the kernel classes (in P_* order); the ranges cost
// nothing unless a profiler is attached.
static const char* const kProfNames[kProfClasses] = {"encode", "leaves", "tree", "pi_leaves", "fold",   "fix",
                                                     "eq",     "gather", "open_tail", "transcript", "encode_last"};

ProfScope::ProfScope(Profiler& p, cudaStream_t s, int c) : pr(p), st(s), cls(c) {
  nvtxRangePushA(kProfNames[cls]);
  if (pr.on) {
    a = pr.get();
    cudaEventRecord(a, st);
  }
}

ProfScope::~ProfScope() {
  if (pr.on) {
    cudaEvent_t b = pr.get();
    cudaEventRecord(b, st);
    pr.pending.push_back({cls, a, b});
  }
  nvtxRangePop();
}

DeviceGuard::DeviceGuard(int dev) {
  cudaGetDevice(&prev);
  if (dev >= 0 && prev != dev) cudaSetDevice(dev);
}

DeviceGuard::~DeviceGuard() {
  int cur = -1;
  cudaGetDevice(&cur);
  if (prev >= 0 && cur != prev) cudaSetDevice(prev);
}

// Formula 8 of 2024/504 (binary_reed_solomon.rs:56-59); a non-finite or
// non-positive quotient saturates to 0 like Rust's float-to-usize cast.
size_t num_queries(int lambda, int log2_c) {
  double c = (double)((size_t)1 << log2_c);
  double delta = (1.0 + 1.0 / c) / 2.0;
  double q = std::ceil((double)lambda / -std::log2(delta));
  if (!(q > 0) || !std::isfinite(q)) return 0;
  return (size_t)q;
}

// univariate horner (p3/src/poly/univariate.rs:5-12)
u128 horner(const u128* c, int n, u128 x) {
  u128 acc = 0;
  for (int k = n - 1; k >= 0; --k) acc = bfh::mul(acc, x) ^ c[k];
  return acc;
}

void put_u64(std::vector<uint8_t>& b, uint64_t v) {
  for (int i = 0; i < 8; ++i) b.push_back((uint8_t)(v >> (8 * i)));
}

void put_elem(std::vector<uint8_t>& b, u128 v) {
  uint8_t t[16];
  bfh::store(t, v);
  b.insert(b.end(), t, t + 16);
}

std::vector<u128> eq_table_host(const std::vector<u128>& x) {
  std::vector<u128> e((size_t)1 << x.size(), 0);
  e[0] = bfh::one();
  for (size_t i = 0; i < x.size(); ++i) {  // eq_expand (multilinear.rs:216-222)
    const size_t h = (size_t)1 << i;
    for (size_t k = 0; k < h; ++k) {
      const u128 hv = bfh::mul(e[k], x[i]);
      e[h + k] = hv;
      e[k] ^= hv;
    }
  }
  return e;
}

std::vector<u128> sample_scalars_by_eq(size_t n, bfh::Challenger& ch) {
  int log_n = 0;
  while (((size_t)1 << log_n) < n) ++log_n;
  std::vector<u128> r;
  for (int i = 0; i < log_n; ++i) r.push_back(ch.sample_elem());
  std::vector<u128> eq = eq_table_host(r);
  eq.resize(n);
  return eq;
}

}  // namespace bfapi

using namespace bfapi;

bf_pcs::~bf_pcs() {
  if (aux) cudaStreamSynchronize(aux);
  if (aux2) cudaStreamSynchronize(aux2);
  if (stream) cudaStreamSynchronize(stream);
  sc_ws.release();
  eval_ws.release();
  evalc_ws.release();
  if (stream) cudaStreamSynchronize(stream);
  if (pool) cudaMemPoolDestroy(pool);
  if (stream && own_stream) cudaStreamDestroy(stream);
  if (aux) cudaStreamDestroy(aux);
  if (aux2) cudaStreamDestroy(aux2);
  if (ev_fork) cudaEventDestroy(ev_fork);
  if (ev_join) cudaEventDestroy(ev_join);
  for (cudaEvent_t e : slice_ev)
    if (e) cudaEventDestroy(e);
}

// ---------------------------------------------------------------------------
// Setup: additive-NTT twiddle bases (p3/src/field/binary.rs:23-53).
// W_0(x) = x, W_{i+1}(x) = W_i(x)^2 + W_i(x) W_i(beta_i); stage s has basis
// W_s(beta_{s+1+b}) / W_s(beta_s), beta_i = basis(i) = from_canonical(1<<i)
// (p3/src/polyval.rs:167-172).
// ---------------------------------------------------------------------------
namespace {

u128 mul_x(u128 v) {
  bool carry = (v >> 127) & 1;
  v <<= 1;
  if (carry) v ^= (u128)1 ^ ((u128)1 << 121) ^ ((u128)1 << 126) ^ ((u128)1 << 127);
  return v;
}

// x^256 mod P: from_canonical(v) = v * x^256 * x^-128.
u128 r2_const() {
  static u128 r2 = 0;
  if (!r2) {
    u128 v = 1;
    for (int i = 0; i < 256; ++i) v = mul_x(v);
    r2 = v;
  }
  return r2;
}

std::vector<std::vector<u128>> stage_bases(int L) {
  std::vector<std::vector<u128>> out(L);
  if (L == 0) return out;
  auto beta = [](int i) { return bfh::mul((u128)1 << i, r2_const()); };
  u128 wbi = beta(0);
  std::vector<u128> wb;
  for (int i = 1; i < L; ++i) wb.push_back(beta(i));
  for (int s = 0; s < L; ++s) {
    u128 inv_i = bfh::inv(wbi);
    for (u128 w : wb) out[s].push_back(bfh::mul(w, inv_i));
    if (wb.empty()) break;
    auto q = [wbi](u128 w) { return bfh::sq(w) ^ bfh::mul(w, wbi); };
    u128 first = q(wb[0]);
    std::vector<u128> rest;
    for (size_t b = 1; b < wb.size(); ++b) rest.push_back(q(wb[b]));
    wbi = first;
    wb = rest;
  }
  return out;
}

int build_twiddles(bf_pcs* p) {
  const int L = p->L;
  p->bases = stage_bases(L);
  const auto& bases = p->bases;
  // stage s table has 2^(L-1-s) entries: lo covers the low 12 bits of K, hi the rest.
  std::vector<u128> host;
  std::vector<size_t> lo_off(L), hi_off(L);
  for (int s = 0; s < L; ++s) {
    const int bits = L - 1 - s;
    const int lo_bits = bits < bf::kTwLoBits ? bits : bf::kTwLoBits;
    const int hi_bits = bits - lo_bits;
    lo_off[s] = host.size();
    size_t base = host.size();
    host.resize(base + ((size_t)1 << lo_bits), 0);
    for (int b = 0; b < lo_bits; ++b) {
      size_t h = (size_t)1 << b;
      for (size_t k = 0; k < h; ++k) host[base + h + k] = host[base + k] ^ bases[s][b];
    }
    hi_off[s] = host.size();
    base = host.size();
    host.resize(base + ((size_t)1 << hi_bits), 0);
    for (int b = 0; b < hi_bits; ++b) {
      size_t h = (size_t)1 << b;
      for (size_t k = 0; k < h; ++k) host[base + h + k] = host[base + k] ^ bases[s][lo_bits + b];
    }
  }
  CU(p->tw_tables.alloc(host.size() * 16 + 16));
  CU(cudaMemcpy(p->tw_tables.p, host.data(), host.size() * 16, cudaMemcpyHostToDevice));
  const uint4* t = p->tw_tables.as<uint4>();
  for (int s = 0; s < L; ++s) {
    p->tw_host.lo[s] = t + lo_off[s];
    p->tw_host.hi[s] = t + hi_off[s];
  }
  CU(p->tw_view.alloc(sizeof(bf::TwiddleView)));
  CU(cudaMemcpy(p->tw_view.p, &p->tw_host, sizeof(bf::TwiddleView), cudaMemcpyHostToDevice));
  return BF_OK;
}

}  // namespace

namespace bfapi {

// The codeword and tree buffers of `cm` from the pcs's pool (kept when they
// are already there, e.g. for a captured graph's fixed buffers).
int commit_alloc(bf_pcs* p, bf_commitment* cm, cudaStream_t st) {
  const size_t nd = p->n_d(), w = cm->width;
  const bool pairs = p->d > 0 && w == 1;
  if (!cm->cw.p) CU(cm->cw.alloc_async(16 * nd * w, p->pool, st));
  if (!cm->tree.p) CU(cm->tree.alloc_async(32 * (2 * nd - 1), p->pool, st));
  if (pairs && !cm->pi_tree.p) CU(cm->pi_tree.alloc_async(32 * (nd - 1), p->pool, st));
  return BF_OK;
}

// Encode + Merkle commit of `data` on stream `st`; the codeword root and
// (width 1) the first folded-codeword root are copied to roots_pin[0..64)
// (pinned) when the stream reaches that point.
int commit_enqueue(bf_pcs* p, bf_commitment* cm, const uint4* data, cudaStream_t st, uint8_t* roots_pin,
                   bool fork_trees, const cudaEvent_t* slice_ready, int slices) {
  const size_t nd = p->n_d(), w = cm->width;
  // For width 1 the first open round commits the codeword itself (as pairs),
  // so that tree is built here; wider data is first combined in open.
  const bool pairs = p->d > 0 && w == 1;
  TRY(commit_alloc(p, cm, st));
  uint4* cw = cm->cw.as<uint4>();
  uint4* tree = cm->tree.as<uint4>();
  uint4* pit = cm->pi_tree.as<uint4>();
  {
    // encode; for width 1 and d >= 1 the last NTT pass also hashes the leaves
    ProfScope ps(p->prof, st, P_ENCODE);
    cudaEvent_t la = nullptr, lb = nullptr;
    if (p->prof.on) {
      la = p->prof.get();
      lb = p->prof.get();
    }
    // the pcs's second streams and events only serve work on its own stream
    // (engine jobs of one size share the pcs on streams of their own)
    const bool own = st == p->stream;
    const cudaError_t e = bf::launch_encode(data, cw, p->d, p->log2_c, w, p->tw_view.as<bf::TwiddleView>(), st,
                                            pairs ? tree : nullptr, pairs ? pit : nullptr, p->tune, slice_ready,
                                            slices, own ? p->aux2 : nullptr, own ? p->ev_fork : nullptr,
                                            own ? p->ev_join : nullptr, la, lb);
    if (p->prof.on) p->prof.pending.push_back({P_ENCODE_LAST, la, lb});
    CU(e);
  }
  if (!pairs) {
    ProfScope ps(p->prof, st, P_LEAVES);
    CU(bf::launch_leaves_elem(cw, tree, nd, w, st));
  }
  if (pairs && fork_trees && st == p->stream && p->aux) {
    // the two trees are independent: the folded-codeword tree on the second
    // stream, joined before the roots are read
    ProfScope ps(p->prof, st, P_TREE);  // one scope from the fork to the join
    CU(cudaEventRecord(p->ev_fork, st));
    CU(cudaStreamWaitEvent(p->aux, p->ev_fork, 0));
    CU(bf::launch_tree(pit, nd / 2, p->aux, nullptr, p->tune));
    CU(bf::launch_tree(tree, nd, st, nullptr, p->tune));
    CU(cudaEventRecord(p->ev_join, p->aux));
    CU(cudaStreamWaitEvent(st, p->ev_join, 0));
  } else {
    ProfScope ps(p->prof, st, P_TREE);
    CU(bf::launch_tree(tree, nd, st, nullptr, p->tune));
    if (pairs) CU(bf::launch_tree(pit, nd / 2, st, nullptr, p->tune));
  }
  CU(cudaMemcpyAsync(roots_pin, tree + 2 * (2 * nd - 2), 32, cudaMemcpyDeviceToHost, st));
  if (pairs) CU(cudaMemcpyAsync(roots_pin + 32, pit + 2 * (nd - 2), 32, cudaMemcpyDeviceToHost, st));
  return BF_OK;
}

// MultiPoly::evaluate (multilinear.rs:124-141) of the commitment's data at
// `point` (host, d elements) on stream `st`: fix the top variable with the
// last coordinate, repeatedly, in `scratch` (2^(d-1) elements).  The value
// lands in value_pin[0..16).
int eval_enqueue(bf_pcs* p, const bf_commitment* cm, const uint8_t* point, uint4* scratch, cudaStream_t st,
                 uint8_t* value_pin, const uint4** value_dev, const uint4* point_dev) {
  const int d = p->d;
  const size_t w = cm->width;
  const uint4* data = cm->data.as<uint4>();
  if (value_dev) *value_dev = d == 0 ? data : scratch;
  if (d == 0) {
    CU(cudaMemcpyAsync(value_pin, data, 16 * w, cudaMemcpyDeviceToHost, st));
    return BF_OK;
  }
  auto coord = [&](int k) {
    uint4 r{};
    if (!point_dev) std::memcpy(&r, point + 16 * k, 16);
    return r;
  };
  auto coord_dev = [&](int k) { return point_dev ? point_dev + k : nullptr; };
  for (size_t col = 0; col < w; ++col) {  // one value per column (basefold.rs:126-131)
    {
      ProfScope ps(p->prof, st, P_FIX);
      if (w == 1)
        CU(bf::launch_fix(data, scratch, (size_t)1 << (d - 1), coord(d - 1), nullptr, 0, nullptr, st,
                          coord_dev(d - 1)));
      else
        CU(bf::launch_fix_column(data, w, col, scratch, (size_t)1 << (d - 1), coord(d - 1), st, coord_dev(d - 1)));
    }
    // large levels one launch each; the last (<= kEvalTailMaxVars) in one block
    const int tail = std::min(d - 1, bf::kEvalTailMaxVars);
    for (int k = d - 2; k >= tail; --k) {
      ProfScope ps(p->prof, st, P_FIX);
      CU(bf::launch_fix(scratch, scratch, (size_t)1 << k, coord(k), nullptr, 0, nullptr, st, coord_dev(k)));
    }
    if (tail > 0) {
      bf::EvalTail et{};
      et.nvars = tail;
      et.rp = point_dev;
      for (int k = 0; k < tail; ++k) et.r[k] = coord(k);
      ProfScope ps(p->prof, st, P_FIX);
      CU(bf::launch_eval_tail(scratch, et, st));
    }
    CU(cudaMemcpyAsync(value_pin + 16 * col, scratch, 16, cudaMemcpyDeviceToHost, st));
  }
  return BF_OK;
}

}  // namespace bfapi

namespace {

int commit_device(bf_pcs* p, bf_commitment* cm, const uint4* data, const cudaEvent_t* slice_ready = nullptr,
                  int slices = 0) {
  TRY(commit_enqueue(p, cm, data, p->stream, p->pinned.b(), true, slice_ready, slices));
  CU(cudaStreamSynchronize(p->stream));
  p->prof.drain();
  bfh::digest_from_interleaved(p->pinned.b(), cm->root);  // tree roots are stored interleaved
  bfh::digest_from_interleaved(p->pinned.b() + 32, cm->pi_root);
  return BF_OK;
}

}  // namespace

extern "C" {

int bf_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return BF_ERR_ARG;
  const std::string& e = last_error();
  size_t n = e.size() < len - 1 ? e.size() : len - 1;
  std::memcpy(buf, e.data(), n);
  buf[n] = 0;
  return BF_OK;
}

int bf_kernel_launches(uint64_t* count) {
  if (!count) return fail(BF_ERR_ARG, "null argument");
  *count = bf::launches_total();
  return BF_OK;
}

int bf_device_info(int device, int* num_sms, int* cc_major, int* cc_minor) {
  int n = 0;
  CU(cudaGetDeviceCount(&n));
  if (device < 0 || device >= n) return fail(BF_ERR_ARG, "device %d out of range (%d devices)", device, n);
  if (num_sms) CU(cudaDeviceGetAttribute(num_sms, cudaDevAttrMultiProcessorCount, device));
  if (cc_major) CU(cudaDeviceGetAttribute(cc_major, cudaDevAttrComputeCapabilityMajor, device));
  if (cc_minor) CU(cudaDeviceGetAttribute(cc_minor, cudaDevAttrComputeCapabilityMinor, device));
  return BF_OK;
}

int bf_pcs_setup(int device, int lambda, int log2_c, int num_vars, void* stream, bf_pcs** out) {
  if (!out) return fail(BF_ERR_ARG, "out is null");
  *out = nullptr;
  if (lambda < 0 || log2_c < 0 || log2_c > 4 || num_vars < 0 || num_vars + log2_c > 30)
    return fail(BF_ERR_ARG, "unsupported code parameters lambda=%d log2_c=%d num_vars=%d", lambda, log2_c, num_vars);
  std::unique_ptr<bf_pcs> p(new bf_pcs());
  p->device = device;
  p->lambda = lambda;
  p->log2_c = log2_c;
  p->d = num_vars;
  p->L = num_vars + log2_c;
  p->Q = num_queries(lambda, log2_c);
  if (device < 0) {  // verifier-only object: no GPU is touched
    p->bases = stage_bases(p->L);
    *out = p.release();
    return BF_OK;
  }
  CU(cudaSetDevice(device));
  if (stream) {
    p->stream = reinterpret_cast<cudaStream_t>(stream);
  } else {
    CU(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
    p->own_stream = true;
  }
  CU(cudaStreamCreateWithFlags(&p->aux, cudaStreamNonBlocking));
  {
    // aux2 runs work that should be dispatched ahead of the main stream's
    // waiting blocks (the next cosets' first NTT pass beside a last pass)
    int lo_prio = 0, hi_prio = 0;
    CU(cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio));
    CU(cudaStreamCreateWithPriority(&p->aux2, cudaStreamNonBlocking, hi_prio));
  }
  CU(cudaEventCreateWithFlags(&p->ev_fork, cudaEventDisableTiming));
  CU(cudaEventCreateWithFlags(&p->ev_join, cudaEventDisableTiming));
  for (cudaEvent_t& e : p->slice_ev) CU(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  TRY(build_twiddles(p.get()));
  bf::init_kernel_attributes();
  CU(p->pinned.ensure(4096));
  {
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    CU(cudaMemPoolCreate(&p->pool, &props));
    uint64_t keep = ~(uint64_t)0;
    CU(cudaMemPoolSetAttribute(p->pool, cudaMemPoolAttrReleaseThreshold, &keep));
  }
  tune_cache_apply(p.get());  // shapes tuned earlier for this device and size, if any
  *out = p.release();
  return BF_OK;
}

void bf_pcs_free(bf_pcs* pcs) {
  if (pcs) pcs_release(pcs);
}

size_t bf_pcs_num_queries(const bf_pcs* pcs) { return pcs ? pcs->Q : 0; }

size_t bf_pcs_proof_size(const bf_pcs* p, size_t width, int n_evals) {
  if (!p) return 0;
  if (n_evals == 0) return 32;
  return 8 + (size_t)p->d * 40 + 24 + 8 + 32 * (size_t)p->d + 8 + p->Q * p->block_bytes(width);
}

int bf_commit(bf_pcs* p, const uint8_t* evals, size_t width, bf_commitment** out, uint8_t root[32]) {
  if (!p || !evals || !out) return fail(BF_ERR_ARG, "null argument");
  if (p->device < 0) return fail(BF_ERR_ARG, "verifier-only pcs (device < 0)");
  *out = nullptr;
  if (width == 0 || width > 4096) return fail(BF_ERR_ARG, "width %zu out of range (1..4096)", width);
  DeviceGuard g(p->device);
  std::unique_ptr<bf_commitment> cm(new bf_commitment());
  cm->pcs = p;
  cm->width = width;
  const size_t n = (size_t)1 << p->d;
  CU(cm->data.alloc_async(16 * n * width, p->pool, p->stream));
  if (p->d >= 16) {
    // copy in slices on the second stream; the first NTT pass takes each
    // slice as it lands (pinned `evals` overlap the copy with the pass)
    const int S = bf_pcs::kH2DSlices;
    const size_t slice = 16 * (n / S) * width;
    CU(cudaEventRecord(p->ev_fork, p->stream));  // the allocation
    CU(cudaStreamWaitEvent(p->aux, p->ev_fork, 0));
    for (int k = 0; k < S; ++k) {
      CU(cudaMemcpyAsync(cm->data.as<uint8_t>() + k * slice, evals + k * slice, slice, cudaMemcpyHostToDevice,
                         p->aux));
      CU(cudaEventRecord(p->slice_ev[k], p->aux));
    }
    TRY(commit_device(p, cm.get(), cm->data.as<uint4>(), p->slice_ev, S));
  } else {
    CU(cudaMemcpyAsync(cm->data.p, evals, 16 * n * width, cudaMemcpyHostToDevice, p->stream));
    TRY(commit_device(p, cm.get(), cm->data.as<uint4>()));
  }
  if (root) std::memcpy(root, cm->root, 32);
  pcs_acquire(p);
  *out = cm.release();
  return BF_OK;
}

int bf_commit_device(bf_pcs* p, const void* d_evals, size_t width, bf_commitment** out, uint8_t root[32]) {
  if (!p || !d_evals || !out) return fail(BF_ERR_ARG, "null argument");
  if (p->device < 0) return fail(BF_ERR_ARG, "verifier-only pcs (device < 0)");
  *out = nullptr;
  if (width == 0 || width > 4096) return fail(BF_ERR_ARG, "width %zu out of range (1..4096)", width);
  if (reinterpret_cast<uintptr_t>(d_evals) & 15) return fail(BF_ERR_ARG, "device evaluations must be 16-byte aligned");
  DeviceGuard g(p->device);
  std::unique_ptr<bf_commitment> cm(new bf_commitment());
  cm->pcs = p;
  cm->width = width;
  cm->data.p = const_cast<void*>(d_evals);
  cm->data.owned = false;
  cm->data.bytes = 16 * ((size_t)1 << p->d) * width;
  TRY(commit_device(p, cm.get(), reinterpret_cast<const uint4*>(d_evals)));
  if (root) std::memcpy(root, cm->root, 32);
  pcs_acquire(p);
  *out = cm.release();
  return BF_OK;
}

void bf_commitment_free(bf_commitment* cm) {
  if (!cm) return;
  bf_pcs* p = cm->pcs;
  {
    DeviceGuard g(p->device);
    delete cm;  // buffers return to the pcs's pool in stream order
  }
  pcs_release(p);
}

int bf_commitment_root(const bf_commitment* cm, uint8_t root[32]) {
  if (!cm || !root) return fail(BF_ERR_ARG, "null argument");
  std::memcpy(root, cm->root, 32);
  return BF_OK;
}

int bf_commitment_data(const bf_commitment* cm, uint8_t* evals, size_t cap) {
  if (!cm || !evals) return fail(BF_ERR_ARG, "null argument");
  if (cap < cm->data.bytes) return fail(BF_ERR_BUFFER, "need %zu bytes", cm->data.bytes);
  DeviceGuard g(cm->pcs->device);
  CU(cudaMemcpyAsync(evals, cm->data.p, cm->data.bytes, cudaMemcpyDeviceToHost, cm->pcs->stream));
  CU(cudaStreamSynchronize(cm->pcs->stream));
  return BF_OK;
}

namespace {
// Values of every column of a w > 1 matrix at a host point in one pass over
// the matrix: the point's eq table against all columns (the columns'
// MultiPoly::evaluate values, basefold.rs:126-131), into value_pin.
int eval_cols_enqueue(bf_pcs* p, const uint4* data, size_t w, const uint8_t* point, uint8_t* value_pin) {
  const int d = p->d;
  const size_t n = (size_t)1 << d;
  auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t o_lo = up(16 * (size_t)(d > 0 ? d : 1)), o_hi = o_lo + up(16 * 4096), o_eq = o_hi + up(16 * 65536);
  const size_t o_acc = o_eq + up(16 * n), total = o_acc + up(16 * w);
  if (p->evalc_ws.bytes < total) CU(p->evalc_ws.alloc(total));
  uint8_t* ws = p->evalc_ws.as<uint8_t>();
  if (d > 0) {
    std::memcpy(value_pin + 16 * w, point, 16 * (size_t)d);
    CU(cudaMemcpyAsync(ws, value_pin + 16 * w, 16 * (size_t)d, cudaMemcpyHostToDevice, p->stream));
  }
  uint4* eq = reinterpret_cast<uint4*>(ws + o_eq);
  uint32_t* acc = reinterpret_cast<uint32_t*>(ws + o_acc);
  {
    ProfScope ps(p->prof, p->stream, P_EQ);
    CU(bf::launch_eq_table(reinterpret_cast<const uint4*>(ws), d, eq, reinterpret_cast<uint4*>(ws + o_lo),
                           reinterpret_cast<uint4*>(ws + o_hi), p->stream));
  }
  CU(cudaMemsetAsync(acc, 0, 16 * w, p->stream));
  {
    ProfScope ps(p->prof, p->stream, P_FIX);
    CU(bf::launch_eval_cols(eq, data, n, w, acc, p->stream));
  }
  CU(cudaMemcpyAsync(value_pin, acc, 16 * w, cudaMemcpyDeviceToHost, p->stream));
  return BF_OK;
}
}  // namespace

int bf_eval(bf_pcs* p, const bf_commitment* cm, const uint8_t* point, uint8_t* values) {
  if (!p || !cm || !values || (p->d > 0 && !point)) return fail(BF_ERR_ARG, "null argument");
  DeviceGuard g(p->device);
  const size_t half = p->d > 0 ? ((size_t)1 << (p->d - 1)) : 1;
  CU(p->pinned.ensure(16 * cm->width + 16 * (size_t)p->d + 64));
  if (cm->width > 1 && p->d <= bf::kEqTableMaxVars) {
    TRY(eval_cols_enqueue(p, cm->data.as<uint4>(), cm->width, point, p->pinned.b()));
    CU(cudaStreamSynchronize(p->stream));
    p->prof.drain();
    std::memcpy(values, p->pinned.b(), 16 * cm->width);
    return BF_OK;
  }
  if (p->eval_ws.bytes < 16 * half) CU(p->eval_ws.alloc(16 * half));
  TRY(eval_enqueue(p, cm, point, p->eval_ws.as<uint4>(), p->stream, p->pinned.b()));
  CU(cudaStreamSynchronize(p->stream));
  p->prof.drain();
  std::memcpy(values, p->pinned.b(), 16 * cm->width);
  return BF_OK;
}

int bf_eval_data(bf_pcs* p, const void* evals, int on_device, size_t width, const uint8_t* point, uint8_t* values) {
  if (!p || !evals || !values || (p->d > 0 && !point)) return fail(BF_ERR_ARG, "null argument");
  if (p->device < 0) return fail(BF_ERR_ARG, "verifier-only pcs (device < 0)");
  if (width == 0 || width > 4096) return fail(BF_ERR_ARG, "width %zu out of range (1..4096)", width);
  if (on_device && (reinterpret_cast<uintptr_t>(evals) & 15))
    return fail(BF_ERR_ARG, "device evaluations must be 16-byte aligned");
  DeviceGuard g(p->device);
  // the data of a commitment that is never made: the caller's device buffer,
  // or a pool copy of the host rows (released in stream order)
  bf_commitment cm;
  cm.pcs = p;
  cm.width = width;
  const size_t bytes = 16 * width * ((size_t)1 << p->d);
  if (on_device) {
    cm.data.p = const_cast<void*>(evals);
    cm.data.owned = false;
  } else {
    CU(cm.data.alloc_async(bytes, p->pool, p->stream));
    CU(cudaMemcpyAsync(cm.data.p, evals, bytes, cudaMemcpyHostToDevice, p->stream));
  }
  const size_t half = p->d > 0 ? ((size_t)1 << (p->d - 1)) : 1;
  CU(p->pinned.ensure(16 * width + 16 * (size_t)p->d + 64));
  if (width > 1 && p->d <= bf::kEqTableMaxVars) {
    TRY(eval_cols_enqueue(p, cm.data.as<uint4>(), width, point, p->pinned.b()));
  } else {
    if (p->eval_ws.bytes < 16 * half) CU(p->eval_ws.alloc(16 * half));
    TRY(eval_enqueue(p, &cm, point, p->eval_ws.as<uint4>(), p->stream, p->pinned.b()));
  }
  CU(cudaStreamSynchronize(p->stream));
  p->prof.drain();
  std::memcpy(values, p->pinned.b(), 16 * width);
  return BF_OK;
}

// ---- challenger -----------------------------------------------------------
int bf_challenger_new(const uint8_t* initial_state, size_t len, bf_challenger** out) {
  if (!out || (len && !initial_state)) return fail(BF_ERR_ARG, "null argument");
  bf_challenger* c = new bf_challenger();
  if (len) c->c.in.assign(initial_state, initial_state + len);
  *out = c;
  return BF_OK;
}
int bf_challenger_clone(const bf_challenger* ch, bf_challenger** out) {
  if (!ch || !out) return fail(BF_ERR_ARG, "null argument");
  *out = new bf_challenger(*ch);
  return BF_OK;
}
void bf_challenger_free(bf_challenger* ch) { delete ch; }
int bf_challenger_observe(bf_challenger* ch, const uint8_t* bytes, size_t len) {
  if (!ch || (len && !bytes)) return fail(BF_ERR_ARG, "null argument");
  ch->c.observe(bytes, len);
  return BF_OK;
}
int bf_challenger_sample_ext(bf_challenger* ch, uint8_t out[16]) {
  if (!ch || !out) return fail(BF_ERR_ARG, "null argument");
  bfh::store(out, ch->c.sample_elem());
  return BF_OK;
}
int bf_challenger_sample_bits(bf_challenger* ch, int bits, uint64_t* out) {
  if (!ch || !out || bits < 0 || bits > 64) return fail(BF_ERR_ARG, "bad argument");
  *out = ch->c.sample_bits(bits);
  return BF_OK;
}
int bf_challenger_state(const bf_challenger* ch, uint8_t* buf, size_t cap, size_t* len) {
  if (!ch || !len) return fail(BF_ERR_ARG, "null argument");
  std::vector<uint8_t> b = ch->c.blob();
  *len = b.size();
  if (!buf || cap < b.size()) return fail(BF_ERR_BUFFER, "need %zu bytes", b.size());
  std::memcpy(buf, b.data(), b.size());
  return BF_OK;
}
int bf_challenger_from_state(const uint8_t* buf, size_t len, bf_challenger** out) {
  if (!buf || !out) return fail(BF_ERR_ARG, "null argument");
  bf_challenger* c = new bf_challenger();
  if (!c->c.from_blob(buf, len)) {
    delete c;
    return fail(BF_ERR_ARG, "malformed challenger state");
  }
  *out = c;
  return BF_OK;
}

// ---- profiling ---------------------------------------------------------------
int bf_profile_enable(bf_pcs* p, int on) {
  if (!p) return fail(BF_ERR_ARG, "null argument");
  p->prof.on = on != 0;
  for (int k = 0; k < kProfClasses; ++k) {
    p->prof.ms[k] = 0;
    p->prof.count[k] = 0;
  }
  return BF_OK;
}
int bf_profile_read(bf_pcs* p, double* ms, uint64_t* launches, int nclasses) {
  if (!p || p->device < 0) return fail(BF_ERR_ARG, "null argument or verifier-only pcs");
  DeviceGuard g(p->device);
  CU(cudaStreamSynchronize(p->stream));
  p->prof.drain();
  for (int k = 0; k < nclasses && k < kProfClasses; ++k) {
    if (ms) ms[k] = p->prof.ms[k];
    if (launches) launches[k] = p->prof.count[k];
  }
  return BF_OK;
}

// ---- test hooks --------------------------------------------------------------
int bf_test_gf_mul(int device, const uint8_t* a, const uint8_t* b, uint8_t* out, size_t n) {
  if (!a || !b || !out) return fail(BF_ERR_ARG, "null argument");
  CU(cudaSetDevice(device));
  DevBuf da, db, dc;
  CU(da.alloc(16 * n));
  CU(db.alloc(16 * n));
  CU(dc.alloc(16 * n));
  CU(cudaMemcpy(da.p, a, 16 * n, cudaMemcpyHostToDevice));
  CU(cudaMemcpy(db.p, b, 16 * n, cudaMemcpyHostToDevice));
  CU(bf::launch_test_mul(da.as<uint4>(), db.as<uint4>(), dc.as<uint4>(), n, 0));
  CU(cudaMemcpy(out, dc.p, 16 * n, cudaMemcpyDeviceToHost));
  return BF_OK;
}

int bf_test_keccak_f(int device, uint64_t* states, size_t n) {
  if (!states) return fail(BF_ERR_ARG, "null argument");
  CU(cudaSetDevice(device));
  DevBuf ds;
  CU(ds.alloc(200 * n));
  CU(cudaMemcpy(ds.p, states, 200 * n, cudaMemcpyHostToDevice));
  CU(bf::launch_test_keccak(ds.as<uint2>(), n, 0));
  CU(cudaMemcpy(states, ds.p, 200 * n, cudaMemcpyDeviceToHost));
  return BF_OK;
}

}  // extern "C"
