// Host orchestration and the C ABI of libbasefold_gpu.so.
//
// The prover keeps every array of the path in device memory: evaluations,
// codeword, Merkle trees, folded codewords and their trees, the sumcheck
// polynomial and its eq table.  Per round only the Fiat–Shamir transcript
// crosses to the host: a 32-byte Merkle root and one 16-byte reduction go
// down, the 16-byte challenge goes back up as a kernel argument.
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <cmath>
#include <array>
#include <memory>
#include <string>
#include <vector>

#include "../../include/basefold_gpu.h"
#include "bf_internal.h"
#include "host_math.h"

using bfh::u128;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define CU(expr)                                                                          \
  do {                                                                                    \
    cudaError_t e__ = (expr);                                                             \
    if (e__ != cudaSuccess)                                                               \
      return fail(e__ == cudaErrorMemoryAllocation ? BF_ERR_OOM : BF_ERR_CUDA, "%s: %s (%s:%d)", #expr, \
                  cudaGetErrorString(e__), __FILE__, __LINE__);                           \
  } while (0)

#define TRY(expr)              \
  do {                         \
    int rc__ = (expr);         \
    if (rc__ < 0) return rc__; \
  } while (0)

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  bool owned = true;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p && owned) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  cudaError_t alloc(size_t n) {
    release();
    owned = true;
    if (n == 0) n = 16;
    cudaError_t e = cudaMalloc(&p, n);
    if (e == cudaSuccess) bytes = n;
    return e;
  }
  template <class T>
  T* as() const {
    return reinterpret_cast<T*>(p);
  }
};

struct PinnedBuf {
  void* p = nullptr;
  size_t bytes = 0;
  ~PinnedBuf() {
    if (p) cudaFreeHost(p);
  }
  cudaError_t ensure(size_t n) {
    if (n <= bytes) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMallocHost(&p, n);
    if (e == cudaSuccess) bytes = n;
    return e;
  }
  uint8_t* b() const { return reinterpret_cast<uint8_t*>(p); }
};

inline uint4 to_uint4(u128 v) {
  uint4 r;
  std::memcpy(&r, &v, 16);
  return r;
}

constexpr int kProfClasses = 8;
enum ProfClass { P_ENCODE = 0, P_LEAVES = 1, P_TREE = 2, P_PI_LEAVES = 3, P_FOLD = 4, P_FIX = 5, P_EQ = 6, P_GATHER = 7 };

struct Profiler {
  bool on = false;
  struct Pending {
    int cls;
    cudaEvent_t a, b;
  };
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> pool;
  double ms[kProfClasses] = {0};
  uint64_t count[kProfClasses] = {0};
  cudaEvent_t get() {
    if (!pool.empty()) {
      cudaEvent_t e = pool.back();
      pool.pop_back();
      return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
  }
  ~Profiler() {
    for (auto& p : pending) {
      cudaEventDestroy(p.a);
      cudaEventDestroy(p.b);
    }
    for (auto e : pool) cudaEventDestroy(e);
  }
  // Resolve recorded pairs (the stream must have been synchronised).
  void drain() {
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
};

struct ProfScope {
  Profiler& pr;
  cudaStream_t st;
  int cls;
  cudaEvent_t a = nullptr;
  ProfScope(Profiler& p, cudaStream_t s, int c) : pr(p), st(s), cls(c) {
    if (pr.on) {
      a = pr.get();
      cudaEventRecord(a, st);
    }
  }
  ~ProfScope() {
    if (pr.on) {
      cudaEvent_t b = pr.get();
      cudaEventRecord(b, st);
      pr.pending.push_back({cls, a, b});
    }
  }
};

}  // namespace

// ---------------------------------------------------------------------------
// Objects
// ---------------------------------------------------------------------------
struct bf_challenger {
  bfh::Challenger c;
};

struct bf_pcs {
  int device = 0;
  int lambda = 128, log2_c = 1, d = 0, L = 0;
  size_t Q = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  DevBuf tw_tables, tw_view;
  bf::TwiddleView tw_host{};
  std::vector<std::vector<u128>> bases;  // stage bases (host copy, for the verifier)
  // standalone-sumcheck scratch
  DevBuf sc_ws;
  // open workspace (sized for width 1 at this num_vars)
  DevBuf ws;
  bool ws_ready = false;
  uint4* w_point = nullptr;
  uint4* w_pi_fold = nullptr;
  uint4* w_pi_trees = nullptr;
  uint4* w_poly = nullptr;
  uint4* w_heq = nullptr;
  uint4* w_eq_lo = nullptr;
  uint4* w_eq_hi = nullptr;
  uint32_t* w_acc = nullptr;
  uint64_t* w_idx = nullptr;
  uint8_t* w_open = nullptr;
  PinnedBuf pinned;
  Profiler prof;

  size_t n_d() const { return (size_t)1 << L; }
  size_t c() const { return (size_t)1 << log2_c; }
  size_t n_i(int i) const { return c() << i; }
  size_t block_bytes(size_t width) const {
    size_t b = 8 + 16 * width + 8 + 32 * (size_t)L + 8;
    for (int i = 0; i < d; ++i) b += 24 + 32 * (size_t)(log2_c + i);
    return b;
  }
  ~bf_pcs() {
    if (stream && own_stream) cudaStreamDestroy(stream);
  }
};

struct bf_commitment {
  bf_pcs* pcs = nullptr;
  size_t width = 1;
  DevBuf data, cw, tree;
  uint8_t root[32];
};

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

size_t num_queries(int lambda, int log2_c) {
  double c = (double)((size_t)1 << log2_c);
  double delta = (1.0 + 1.0 / c) / 2.0;
  double q = std::ceil((double)lambda / -std::log2(delta));
  if (!(q > 0) || !std::isfinite(q)) return 0;
  return (size_t)q;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

int ensure_workspace(bf_pcs* p) {
  if (p->ws_ready) return BF_OK;
  const int d = p->d;
  const size_t c = p->c();
  const size_t half = d >= 1 ? ((size_t)1 << (d - 1)) : 1;
  const size_t n_point = d > 0 ? d : 1;
  const size_t n_fold = c * (((size_t)1 << d) - 1) + 1;
  const size_t n_pi_tree_digests = (c << 1) * (((size_t)1 << d) - 1) + 1;
  const int hi_vars = d - 1 > 12 ? d - 1 - 12 : 0;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off += align256(bytes);
    return o;
  };
  size_t o_point = take(16 * n_point);
  size_t o_fold = take(16 * n_fold);
  size_t o_trees = take(32 * n_pi_tree_digests);
  size_t o_poly = take(16 * half);
  size_t o_heq = take(16 * half);
  size_t o_lo = take(16 * 4096);
  size_t o_hi = take(16 * ((size_t)1 << hi_vars));
  size_t o_acc = take(64);
  size_t o_idx = take(8 * (p->Q + 1));
  size_t o_open = take(p->block_bytes(1) * (p->Q + 1));
  CU(p->ws.alloc(off));
  uint8_t* b = p->ws.as<uint8_t>();
  p->w_point = reinterpret_cast<uint4*>(b + o_point);
  p->w_pi_fold = reinterpret_cast<uint4*>(b + o_fold);
  p->w_pi_trees = reinterpret_cast<uint4*>(b + o_trees);
  p->w_poly = reinterpret_cast<uint4*>(b + o_poly);
  p->w_heq = reinterpret_cast<uint4*>(b + o_heq);
  p->w_eq_lo = reinterpret_cast<uint4*>(b + o_lo);
  p->w_eq_hi = reinterpret_cast<uint4*>(b + o_hi);
  p->w_acc = reinterpret_cast<uint32_t*>(b + o_acc);
  p->w_idx = reinterpret_cast<uint64_t*>(b + o_idx);
  p->w_open = b + o_open;
  CU(p->pinned.ensure(256 + 16 * n_point + 8 * (p->Q + 1) + p->block_bytes(1) * (p->Q + 1)));
  p->ws_ready = true;
  return BF_OK;
}

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

// Encode + Merkle commit of comm->data (width 1).
int commit_device(bf_pcs* p, bf_commitment* cm, const uint4* data) {
  const size_t nd = p->n_d();
  CU(cm->cw.alloc(16 * nd));
  CU(cm->tree.alloc(32 * (2 * nd - 1)));
  uint4* cw = cm->cw.as<uint4>();
  uint4* tree = cm->tree.as<uint4>();
  {
    ProfScope ps(p->prof, p->stream, P_ENCODE);
    CU(bf::launch_encode(data, cw, p->d, p->log2_c, 1, p->tw_view.as<bf::TwiddleView>(), p->stream));
  }
  {
    ProfScope ps(p->prof, p->stream, P_LEAVES);
    CU(bf::launch_leaves_elem(cw, tree, nd, 1, p->stream));
  }
  {
    ProfScope ps(p->prof, p->stream, P_TREE);
    CU(bf::launch_tree(tree, nd, p->stream));
  }
  CU(cudaMemcpyAsync(p->pinned.b(), tree + 2 * (2 * nd - 2), 32, cudaMemcpyDeviceToHost, p->stream));
  CU(cudaStreamSynchronize(p->stream));
  p->prof.drain();
  std::memcpy(cm->root, p->pinned.b(), 32);
  return BF_OK;
}

void put_u64(std::vector<uint8_t>& b, uint64_t v) {
  for (int i = 0; i < 8; ++i) b.push_back((uint8_t)(v >> (8 * i)));
}
void put_elem(std::vector<uint8_t>& b, u128 v) {
  uint8_t t[16];
  bfh::store(t, v);
  b.insert(b.end(), t, t + 16);
}

u128 horner(const u128* c, int n, u128 x) {
  u128 acc = 0;
  for (int k = n - 1; k >= 0; --k) acc = bfh::mul(acc, x) ^ c[k];
  return acc;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

int bf_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return BF_ERR_ARG;
  size_t n = g_err.size() < len - 1 ? g_err.size() : len - 1;
  std::memcpy(buf, g_err.data(), n);
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
  TRY(build_twiddles(p.get()));
  CU(p->pinned.ensure(4096));
  *out = p.release();
  return BF_OK;
}

void bf_pcs_free(bf_pcs* pcs) {
  if (!pcs) return;
  if (pcs->device < 0) {
    delete pcs;
    return;
  }
  DeviceGuard g(pcs->device);
  if (pcs->stream) cudaStreamSynchronize(pcs->stream);
  delete pcs;
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
  if (width != 1) return fail(BF_ERR_UNSUPPORTED, "width %zu: only width 1 runs on the GPU in this build", width);
  DeviceGuard g(p->device);
  std::unique_ptr<bf_commitment> cm(new bf_commitment());
  cm->pcs = p;
  cm->width = width;
  const size_t n = (size_t)1 << p->d;
  CU(cm->data.alloc(16 * n * width));
  CU(cudaMemcpyAsync(cm->data.p, evals, 16 * n * width, cudaMemcpyHostToDevice, p->stream));
  TRY(commit_device(p, cm.get(), cm->data.as<uint4>()));
  if (root) std::memcpy(root, cm->root, 32);
  *out = cm.release();
  return BF_OK;
}

int bf_commit_device(bf_pcs* p, const void* d_evals, size_t width, bf_commitment** out, uint8_t root[32]) {
  if (!p || !d_evals || !out) return fail(BF_ERR_ARG, "null argument");
  if (p->device < 0) return fail(BF_ERR_ARG, "verifier-only pcs (device < 0)");
  *out = nullptr;
  if (width != 1) return fail(BF_ERR_UNSUPPORTED, "width %zu: only width 1 runs on the GPU in this build", width);
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
  *out = cm.release();
  return BF_OK;
}

void bf_commitment_free(bf_commitment* cm) {
  if (!cm) return;
  DeviceGuard g(cm->pcs->device);
  cudaStreamSynchronize(cm->pcs->stream);
  delete cm;
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

int bf_eval(bf_pcs* p, const bf_commitment* cm, const uint8_t* point, uint8_t* values) {
  if (!p || !cm || !values || (p->d > 0 && !point)) return fail(BF_ERR_ARG, "null argument");
  if (cm->width != 1) return fail(BF_ERR_UNSUPPORTED, "width != 1");
  DeviceGuard g(p->device);
  TRY(ensure_workspace(p));
  const int d = p->d;
  const uint4* data = cm->data.as<uint4>();
  if (d == 0) {
    CU(cudaMemcpyAsync(p->pinned.b(), data, 16, cudaMemcpyDeviceToHost, p->stream));
  } else {
    // MultiPoly::evaluate (multilinear.rs:124-141): fix the top variable with
    // the last coordinate, repeatedly.
    const uint4* in = data;
    for (int k = d - 1; k >= 0; --k) {
      uint4 r;
      std::memcpy(&r, point + 16 * k, 16);
      ProfScope ps(p->prof, p->stream, P_FIX);
      CU(bf::launch_fix(in, p->w_poly, (size_t)1 << k, r, nullptr, 0, nullptr, p->stream));
      in = p->w_poly;
    }
    CU(cudaMemcpyAsync(p->pinned.b(), p->w_poly, 16, cudaMemcpyDeviceToHost, p->stream));
  }
  CU(cudaStreamSynchronize(p->stream));
  p->prof.drain();
  std::memcpy(values, p->pinned.b(), 16);
  return BF_OK;
}

int bf_open(bf_pcs* p, const bf_commitment* cm, const uint8_t* point, const uint8_t* values, int n_evals,
            bf_challenger* chp, uint8_t* proof, size_t cap, size_t* proof_len) {
  if (!p || !cm || !chp || !proof_len) return fail(BF_ERR_ARG, "null argument");
  if (n_evals < 0 || n_evals > 1) return fail(BF_ERR_ARG, "n_evals must be 0 or 1");
  const size_t need = bf_pcs_proof_size(p, cm->width, n_evals);
  *proof_len = need;
  if (!proof || cap < need) return fail(BF_ERR_BUFFER, "proof buffer needs %zu bytes", need);
  if (n_evals == 0) {  // basefold.rs:139-141: Default proof
    std::memset(proof, 0, 32);
    return BF_OK;
  }
  if ((p->d > 0 && !point) || !values) return fail(BF_ERR_ARG, "null point/values");
  if (cm->width != 1) return fail(BF_ERR_UNSUPPORTED, "width != 1");
  DeviceGuard g(p->device);
  TRY(ensure_workspace(p));
  bfh::Challenger& ch = chp->c;
  const int d = p->d, L = p->L, log2_c = p->log2_c;
  const size_t c = p->c();
  cudaStream_t st = p->stream;
  const u128 ONE = bfh::one();

  std::vector<u128> r(d), r_inv, omr_inv;
  for (int k = 0; k < d; ++k) r[k] = bfh::load(point + 16 * k);
  const u128 claim = bfh::load(values);
  // EvalImpr::new / HalfEq::new (eval_impr.rs:20-27, 69-79)
  if (!bfh::batch_inverse(r, r_inv)) return fail(BF_ERR_NOT_INVERTIBLE, "point has a zero coordinate");
  std::vector<u128> omr;
  for (int k = 0; k + 1 < d; ++k) omr.push_back(ONE ^ r[k]);
  if (!bfh::batch_inverse(omr, omr_inv)) return fail(BF_ERR_NOT_INVERTIBLE, "point has a coordinate equal to one");
  // correcting_factor(i) = prod_{k >= i} (1 - r_k)^-1 over k < d-1 (eval_impr.rs:83-90)
  std::vector<u128> corr(d > 0 ? d : 1, ONE);
  for (int i = d - 2; i >= 0; --i) corr[i] = bfh::mul(corr[i + 1], omr_inv[i]);

  const uint4* data = cm->data.as<uint4>();
  const uint4* cw = cm->cw.as<uint4>();
  uint8_t* pin = p->pinned.b();
  std::vector<uint8_t> rounds;  // compressed round polys section
  std::vector<uint8_t> roots;   // pi_comms section
  put_u64(rounds, (uint64_t)d);
  put_u64(roots, (uint64_t)d);

  auto pi_fold_out = [&](int i) { return p->w_pi_fold + c * (((size_t)1 << d) - ((size_t)1 << (i + 1))); };
  auto pi_tree = [&](int i) {
    return p->w_pi_trees + 2 * ((c << 1) * (((size_t)1 << d) - ((size_t)1 << (i + 1))) - (size_t)(d - 1 - i));
  };

  u128 final_val = 0;
  if (d == 0) {
    CU(cudaMemcpyAsync(pin, data, 16, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    final_val = bfh::load(pin);
  } else {
    std::memcpy(pin, point, 16 * (size_t)d);
    CU(cudaMemcpyAsync(p->w_point, pin, 16 * (size_t)d, cudaMemcpyHostToDevice, st));
    {
      ProfScope ps(p->prof, st, P_EQ);
      CU(bf::launch_eq_table(p->w_point, d - 1, p->w_heq, p->w_eq_lo, p->w_eq_hi, st));
    }
    // round d-1: tree over (cw[2s], cw[2s+1]) and sum half_eq * poly_lo
    {
      const size_t ni = p->n_i(d - 1);
      {
        ProfScope ps(p->prof, st, P_PI_LEAVES);
        CU(bf::launch_leaves_pair(cw, pi_tree(d - 1), ni, st));
      }
      {
        ProfScope ps(p->prof, st, P_TREE);
        CU(bf::launch_tree(pi_tree(d - 1), ni, st));
      }
      CU(cudaMemsetAsync(p->w_acc, 0, 16, st));
      {
        ProfScope ps(p->prof, st, P_FIX);
        CU(bf::launch_dot_xor(p->w_heq, data, (size_t)1 << (d - 1), p->w_acc, st));
      }
      CU(cudaMemcpyAsync(pin, pi_tree(d - 1) + 2 * (2 * ni - 2), 32, cudaMemcpyDeviceToHost, st));
      CU(cudaMemcpyAsync(pin + 32, p->w_acc, 16, cudaMemcpyDeviceToHost, st));
      CU(cudaStreamSynchronize(st));
    }
    u128 outer_val = claim, inner_val = 0, delta_prod = ONE;
    for (int i = d - 1; i >= 0; --i) {
      uint8_t root_i[32];
      std::memcpy(root_i, pin, 32);
      const u128 S = bfh::load(pin + 32);
      roots.insert(roots.end(), root_i, root_i + 32);
      ch.observe(root_i, 32);  // basefold.rs:356
      // EvalImprProver::compute_round_poly + decompress (eval_impr.rs:116-127,187-197)
      const u128 sc_val = (i == d - 1) ? outer_val : inner_val;
      const u128 c0 = bfh::mul(corr[i], S);
      const u128 c1 = bfh::mul(sc_val ^ bfh::mul(ONE ^ r[i], c0), r_inv[i]) ^ c0;
      // EvalProver::compute_round_poly (eval.rs:89-106) with delta (eval_impr.rs:45-58)
      const u128 scalar = (i == d - 1) ? ONE : delta_prod;
      const u128 d0 = bfh::mul(scalar, ONE ^ r[i]);
      const u128 d1 = bfh::mul(scalar, r[i] ^ (ONE ^ r[i]));
      const u128 rp[3] = {bfh::mul(c0, d0), bfh::mul(c0, d1) ^ bfh::mul(c1, d0), bfh::mul(c1, d1)};
      put_u64(rounds, 2);
      put_elem(rounds, rp[0]);
      put_elem(rounds, rp[2]);
      ch.observe_elem(rp[0]);  // compress [c0, c2] (eval.rs:64-66)
      ch.observe_elem(rp[2]);
      const u128 x = ch.sample_elem();
      const u128 ic[2] = {c0, c1};
      inner_val = horner(ic, 2, x);  // EvalProver::fix_last_var (eval.rs:108-111)
      outer_val = horner(rp, 3, x);  // SumcheckSubclaim::reduce (lib.rs:41-47)
      delta_prod = bfh::mul(delta_prod, ONE ^ r[i] ^ x);
      const uint4 xr = to_uint4(x);
      // fold pi (binary_reed_solomon.rs:88-96): stage d-1-i
      const size_t ni = p->n_i(i);
      const uint4* pi_in = (i == d - 1) ? cw : pi_fold_out(i + 1);
      {
        ProfScope ps(p->prof, st, P_FOLD);
        CU(bf::launch_fold(pi_in, pi_fold_out(i), ni, p->tw_host.lo[d - 1 - i], p->tw_host.hi[d - 1 - i], xr, st));
      }
      // fix_last_var + next round's reduction
      const uint4* poly_in = (i == d - 1) ? data : p->w_poly;
      if (i > 0) CU(cudaMemsetAsync(p->w_acc, 0, 16, st));
      {
        ProfScope ps(p->prof, st, P_FIX);
        CU(bf::launch_fix(poly_in, p->w_poly, (size_t)1 << i, xr, p->w_heq, i > 0 ? ((size_t)1 << (i - 1)) : 0,
                          i > 0 ? p->w_acc : nullptr, st));
      }
      if (i > 0) {
        const size_t nn = p->n_i(i - 1);
        {
          ProfScope ps(p->prof, st, P_PI_LEAVES);
          CU(bf::launch_leaves_pair(pi_fold_out(i), pi_tree(i - 1), nn, st));
        }
        {
          ProfScope ps(p->prof, st, P_TREE);
          CU(bf::launch_tree(pi_tree(i - 1), nn, st));
        }
        CU(cudaMemcpyAsync(pin, pi_tree(i - 1) + 2 * (2 * nn - 2), 32, cudaMemcpyDeviceToHost, st));
        CU(cudaMemcpyAsync(pin + 32, p->w_acc, 16, cudaMemcpyDeviceToHost, st));
      } else {
        CU(cudaMemcpyAsync(pin, p->w_poly, 16, cudaMemcpyDeviceToHost, st));
      }
      CU(cudaStreamSynchronize(st));
    }
    final_val = bfh::load(pin);
  }
  // final poly + queries (basefold.rs:194-222)
  ch.observe_elem(final_val);
  const size_t Q = p->Q;
  uint64_t* idx_pin = reinterpret_cast<uint64_t*>(pin + 256);
  for (size_t q = 0; q < Q; ++q) idx_pin[q] = ch.sample_bits(L);
  const size_t bb = p->block_bytes(1);
  uint8_t* open_pin = pin + 256 + 8 * (Q + 1);
  if (Q) {
    CU(cudaMemcpyAsync(p->w_idx, idx_pin, 8 * Q, cudaMemcpyHostToDevice, st));
    bf::GatherParams gp{};
    gp.cw = cw;
    gp.cw_tree = cm->tree.as<uint4>();
    gp.pi_first = cw;
    gp.pi_fold = p->w_pi_fold;
    gp.pi_trees = p->w_pi_trees;
    gp.idx = p->w_idx;
    gp.out = p->w_open;
    gp.width = 1;
    gp.block_bytes = bb;
    gp.L = L;
    gp.d = d;
    gp.log2_c = log2_c;
    gp.nq = (int)Q;
    {
      ProfScope ps(p->prof, st, P_GATHER);
      CU(bf::launch_gather(gp, st));
    }
    CU(cudaMemcpyAsync(open_pin, p->w_open, bb * Q, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
  }
  p->prof.drain();
  // assemble BasefoldProof bincode (basefold.rs:49-66)
  uint8_t* o = proof;
  std::memcpy(o, rounds.data(), rounds.size());
  o += rounds.size();
  std::vector<uint8_t> fin;
  put_u64(fin, 1);
  put_elem(fin, final_val);
  std::memcpy(o, fin.data(), fin.size());
  o += fin.size();
  std::memcpy(o, roots.data(), roots.size());
  o += roots.size();
  std::vector<uint8_t> qn;
  put_u64(qn, Q);
  std::memcpy(o, qn.data(), 8);
  o += 8;
  if (Q) std::memcpy(o, open_pin, bb * Q);
  o += bb * Q;
  if ((size_t)(o - proof) != need) return fail(BF_ERR_CUDA, "internal: proof size mismatch");
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

std::vector<u128> eq_host(const std::vector<u128>& x) {
  std::vector<u128> e((size_t)1 << x.size(), 0);
  e[0] = bfh::one();
  for (size_t i = 0; i < x.size(); ++i) {
    size_t h = (size_t)1 << i;
    for (size_t k = 0; k < h; ++k) {
      u128 hv = bfh::mul(e[k], x[i]);
      e[h + k] = hv;
      e[k] ^= hv;
    }
  }
  return e;
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
  } else {  // sample_random_scalars_by_eq (basefold.rs:398-408)
    int lw = 0;
    while (((size_t)1 << lw) < width) ++lw;
    std::vector<u128> rr;
    for (int i = 0; i < lw; ++i) rr.push_back(ch.sample_elem());
    scalars = eq_host(rr);
    scalars.resize(width);
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
// Standalone product sumcheck (sumcheck/src/lib.rs:56-103).
// ===========================================================================
namespace {

int sumcheck_run(cudaStream_t st, DevBuf& scratch, PinnedBuf& pinned, int k, int n, const uint4* polys,
                 const uint8_t* claim_b, bfh::Challenger& ch, uint8_t* out) {
  const size_t N = (size_t)1 << n;
  const u128 ONE = bfh::one();
  u128 sc = bfh::load(claim_b);
  size_t off_r = 16 * (size_t)k * n, off_f = off_r + 16 * (size_t)n, off_c = off_f + 16 * (size_t)k;
  if (n == 0) {  // lib.rs:63-65: no rounds, nothing observed
    CU(cudaMemcpyAsync(pinned.b(), polys, 16, cudaMemcpyDeviceToHost, st));
    for (int j = 1; j < k; ++j)
      CU(cudaMemcpyAsync(pinned.b() + 16 * j, polys + j * N, 16, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    std::memcpy(out + off_f, pinned.b(), 16 * (size_t)k);
    bfh::store(out + off_c, sc);
    return BF_OK;
  }
  const size_t half0 = N / 2;
  if (scratch.bytes < 16 * (size_t)k * half0 + 256) CU(scratch.alloc(16 * (size_t)k * half0 + 256));
  uint32_t* acc = reinterpret_cast<uint32_t*>(scratch.as<uint8_t>() + 16 * (size_t)k * half0);
  uint4* work[3];
  const uint4* in[3];
  for (int j = 0; j < k; ++j) {
    work[j] = scratch.as<uint4>() + j * half0;
    in[j] = polys + j * N;
  }
  ch.observe_elem(sc);  // lib.rs:67
  CU(cudaMemsetAsync(acc, 0, 48, st));
  CU(bf::launch_prod_round_sums(in, k, half0, acc, st));
  CU(cudaMemcpyAsync(pinned.b(), acc, 48, cudaMemcpyDeviceToHost, st));
  CU(cudaStreamSynchronize(st));
  int ri = 0;
  for (int round = n - 1; round >= 0; --round, ++ri) {
    u128 c0 = bfh::load(pinned.b()), c2 = bfh::load(pinned.b() + 16), c3 = bfh::load(pinned.b() + 32);
    std::vector<u128> comp, rp;
    if (k == 2) {
      c0 = bfh::mul(c0, ONE);  // pair scalar ONE (quadratic.rs:118)
      c2 = bfh::mul(c2, ONE);
      comp = {c0, c2};
      rp = {c0, sc ^ c2, c2};  // Quadratic::decompress (quadratic.rs:68-79)
    } else {
      comp = {c0, c2, c3};
      rp = {c0, sc ^ c2 ^ c3, c2, c3};
    }
    for (size_t t = 0; t < comp.size(); ++t) {
      ch.observe_elem(comp[t]);
      bfh::store(out + 16 * ((size_t)ri * k + t), comp[t]);
    }
    const u128 x = ch.sample_elem();
    bfh::store(out + off_r + 16 * (size_t)ri, x);
    sc = horner(rp.data(), (int)rp.size(), x);
    const size_t half = (size_t)1 << round;
    if (round > 0) CU(cudaMemsetAsync(acc, 0, 48, st));
    const uint4* const* src = (round == n - 1) ? in : const_cast<const uint4* const*>(work);
    CU(bf::launch_prod_fix(work, src, k, half, to_uint4(x), half / 2, acc, st));
    if (round > 0) {
      CU(cudaMemcpyAsync(pinned.b(), acc, 48, cudaMemcpyDeviceToHost, st));
    } else {
      for (int j = 0; j < k; ++j) CU(cudaMemcpyAsync(pinned.b() + 16 * j, work[j], 16, cudaMemcpyDeviceToHost, st));
    }
    CU(cudaStreamSynchronize(st));
  }
  std::memcpy(out + off_f, pinned.b(), 16 * (size_t)k);
  bfh::store(out + off_c, sc);
  return BF_OK;
}

}  // namespace

extern "C" int bf_sumcheck_prove_device(bf_pcs* p, int k, int n, const void* d_polys, const uint8_t* claim,
                                        bf_challenger* ch, uint8_t* out) {
  if (!p || !d_polys || !claim || !ch || !out) return fail(BF_ERR_ARG, "null argument");
  if (p->device < 0) return fail(BF_ERR_ARG, "verifier-only pcs (device < 0)");
  if ((k != 2 && k != 3) || n < 0 || n > 30) return fail(BF_ERR_ARG, "k must be 2 or 3, 0 <= num_vars <= 30");
  DeviceGuard g(p->device);
  return sumcheck_run(p->stream, p->sc_ws, p->pinned, k, n, reinterpret_cast<const uint4*>(d_polys), claim, ch->c, out);
}

extern "C" int bf_sumcheck_prove(int device, int k, int n, const uint8_t* polys, const uint8_t* claim,
                                 bf_challenger* ch, uint8_t* out) {
  if (!polys || !claim || !ch || !out) return fail(BF_ERR_ARG, "null argument");
  if ((k != 2 && k != 3) || n < 0 || n > 30) return fail(BF_ERR_ARG, "k must be 2 or 3, 0 <= num_vars <= 30");
  CU(cudaSetDevice(device));
  DevBuf dp, scratch;
  PinnedBuf pinned;
  CU(pinned.ensure(4096));
  const size_t bytes = 16 * (size_t)k * ((size_t)1 << n);
  CU(dp.alloc(bytes));
  cudaStream_t st;
  CU(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() { cudaStreamDestroy(s); }
  } sg{st};
  CU(cudaMemcpyAsync(dp.p, polys, bytes, cudaMemcpyHostToDevice, st));
  return sumcheck_run(st, scratch, pinned, k, n, dp.as<uint4>(), claim, ch->c, out);
}
