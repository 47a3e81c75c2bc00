// C ABI of the prime-field Basefold: Basefold<BabyBear, BinomialExtension
// Field<BabyBear, 5>, ReedSolomonCode<BabyBear>, Keccak256MerkleTreeMmcs>
// (poly-commit/src/basefold.rs, poly-commit/src/basefold/code/reed_solomon.rs).
//
// The GPU holds every array (evaluations, codeword, folded codewords, trees,
// eq tables); the host runs the transcript and the O(num_vars) sumcheck
// scalars, reading 96 bytes back per open round (the folded-codeword root and
// the round's sum).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <memory>
#include <vector>

#include "api_common.h"
#include "bb_host.h"
#include "bb_internal.h"

using namespace bfapi;
using bbh::E;

struct bf_bb_pcs {
  std::atomic<int> refs{1};
  int device = -1;
  // num_vars = log2_k0 + d; the codeword has 2^L rows, L = log2_c + num_vars
  int lambda = 128, log2_c = 1, log2_k0 = 0, d = 0, num_vars = 0, L = 0;
  bool generic = false;              // GenericRandomFoldableCode, else ReedSolomonCode
  std::vector<uint32_t> ts;          // generic: ts[0], .., ts[d-1] back to back (canonical)
  size_t Q = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  // bf_bb_commit copies host evaluations in slices on `aux`; the encode's
  // first stage starts on each slice when its event completes
  static constexpr int kH2DSlices = 8;
  cudaStream_t aux = nullptr;
  cudaEvent_t ev_fork = nullptr;
  cudaEvent_t slice_ev[kH2DSlices] = {};
  // bf_bb_open runs each round's sums and fix on `aux` beside the tree and the
  // fold: ev_dot orders a round's sums before its transcript step, ev_x the
  // challenge before the fix, ev_join `aux` back into the main stream
  cudaEvent_t ev_dot = nullptr, ev_x = nullptr, ev_join = nullptr;
  DevBuf tw;    // butterfly factors: layer s at 2^s - 1, 2^s of them (Shoup pairs, uint2)
  DevBuf tinv;  // fold constants: round i at n_0 (2^i - 1), (2 t_i[j])^-1 for j < n_i (Montgomery)
  DevBuf small;  // 4 KB: the canonical flag, sums, roots
  DevBuf ws;       // grow-only scratch of bf_bb_eval
  DevBuf open_ws;  // grow-only workspace of bf_bb_open
  DevBuf data_ws;  // grow-only copy of host rows for bf_bb_eval_data
  PinnedBuf pin;
  // Commitment buffers (evaluation copy, codeword, tree) come from this
  // stream-ordered pool, which keeps freed memory for the next commit: no
  // cudaMalloc per commit, and no cudaFree (which waits for the whole device).
  cudaMemPool_t pool = nullptr;

  size_t c() const { return (size_t)1 << log2_c; }
  size_t k0() const { return (size_t)1 << log2_k0; }
  int log2_n0() const { return log2_c + log2_k0; }
  size_t n0() const { return (size_t)1 << log2_n0(); }
  size_t n_d() const { return (size_t)1 << L; }
  size_t n_i(int i) const { return n0() << i; }
  size_t tinv_off(int i) const { return n0() * (((size_t)1 << i) - 1); }
  // One query record (basefold.rs:56-65 in bincode): the codeword row and its
  // path, then per round the sibling and its path.
  size_t rec_bytes(size_t w) const {
    size_t words = 2 + w + 2 + 8 * (size_t)L + 2;
    for (int i = 0; i < d; ++i) words += 7 + 8 * (size_t)(log2_n0() + i);
    return 4 * words;
  }
  // round polys (u64 + two E each), final poly (u64 + k_0 E), roots, query count
  size_t header_bytes() const { return 8 + 48 * (size_t)d + 8 + 20 * k0() + 8 + 32 * (size_t)d + 8; }
  // (2 t_i[j])^-1 on the host (the verifier's interpolate)
  uint32_t t_inv_half(int i, size_t j) const {
    const uint32_t t = generic ? ts[tinv_off(i) + j] : bbh::fpow(bbh::two_adic_generator(log2_c + i + 1), j);
    return bbh::finv(bbh::fadd(t, t));
  }
  // encode0 (reed_solomon.rs:66-70, generic.rs:105-110): entry i of m G_0
  E encode0_at(const std::vector<E>& m, size_t i) const {
    if (!generic) return m[0];
    E acc;
    uint32_t pw = 1;
    for (const E& e : m) {
      acc = bbh::eadd(acc, bbh::escale(e, pw));
      pw = bbh::fmul(pw, (uint32_t)i);
    }
    return acc;
  }
  ~bf_bb_pcs() {
    if (device >= 0) {
      cudaSetDevice(device);
      if (stream) cudaStreamSynchronize(stream);
      if (aux) cudaStreamSynchronize(aux);
      tw.release();
      tinv.release();
      small.release();
      ws.release();
      open_ws.release();
      data_ws.release();
      if (stream) cudaStreamSynchronize(stream);
      if (pool) cudaMemPoolDestroy(pool);
      if (own_stream && stream) cudaStreamDestroy(stream);
      if (aux) cudaStreamDestroy(aux);
      if (ev_fork) cudaEventDestroy(ev_fork);
      for (cudaEvent_t e : {ev_dot, ev_x, ev_join})
        if (e) cudaEventDestroy(e);
      for (cudaEvent_t e : slice_ev)
        if (e) cudaEventDestroy(e);
    }
  }
};

struct bf_bb_commitment {
  bf_bb_pcs* pcs = nullptr;
  size_t w = 1;
  DevBuf data;  // canonical evaluations (owned copy, or the caller's device buffer)
  DevBuf cw;    // codeword, Montgomery, n_d rows of w
  DevBuf tree;  // 2 n_d digests, reversed level storage, interleaved lanes
  uint8_t root[32];
};

namespace {

void bb_acquire(bf_bb_pcs* p) { p->refs.fetch_add(1); }
void bb_release(bf_bb_pcs* p) {
  if (p->refs.fetch_sub(1) == 1) delete p;
}

// Relative distance bound of the generic code: appendix C of ePrint
// 2023/1705 as generic.rs:24-39 evaluates it, F::bits() = 31 for BabyBear.
double generic_z_c(double lambda, double log2_f, size_t c, int i, int log2_n_i) {
  if (i == 0) return 1.0 / (double)c;
  return generic_z_c(lambda, log2_f, c, i - 1, log2_n_i - 1) * (log2_f / (log2_f - 1.001)) +
         1.0 / (log2_f - 1.001) *
             ((2.0 * (double)(log2_n_i - 1) + lambda) / (double)((uint64_t)1 << log2_n_i) + 0.6);
}

// RandomFoldableCode::num_queries (reed_solomon.rs:57-64, generic.rs:99-103):
// delta = 1 - distance / 3 in the unique-decoding regime, the Rust cast
// saturating (-inf, NaN and negatives give 0).
size_t bb_num_queries(const bf_bb_pcs& p) {
  const double rel = p.generic ? 1.0 - generic_z_c((double)p.lambda, 31.0, p.c(), p.d, p.L)
                               : 1.0 - 1.0 / (double)p.c();
  const double delta = 1.0 - rel / 3.0;
  const double q = std::ceil((double)p.lambda / -std::log2(delta));
  if (!(q > 0)) return 0;
  if (!std::isfinite(q) || q > 1e15) return (size_t)-1;  // unreachable for lambda <= 2^20
  return (size_t)q;
}

int load_points(const uint8_t* bytes, size_t n, std::vector<E>& out, const char* what) {
  out.resize(n);
  for (size_t k = 0; k < n; ++k) {
    out[k] = bbh::load(bytes + 20 * k);
    if (!bbh::canonical(out[k])) return fail(BF_ERR_ARG, "%s %zu has a coefficient >= p", what, k);
  }
  return BF_OK;
}

// Device eq table of x (2^|x| extension entries) in `ev`.
int eq_table_device(bf_bb_pcs* p, const std::vector<E>& x, uint32_t* ev) {
  std::vector<bb::E5> xd(x.size());
  for (size_t i = 0; i < x.size(); ++i) xd[i] = bbh::to_dev(x[i]);
  CU(bf::bb_launch_eq_table(ev, xd.data(), (int)xd.size(), p->stream));
  return BF_OK;
}

int commit_device(bf_bb_pcs* p, bf_bb_commitment* cm, const uint32_t* data, const cudaEvent_t* slice_ready = nullptr,
                  int slices = 0) {
  const size_t w = cm->w, n = p->n_d();
  CU(cm->cw.alloc_async(4 * n * w, p->pool, p->stream));
  CU(cm->tree.alloc_async(64 * n, p->pool, p->stream));
  uint32_t* flag = p->small.as<uint32_t>();
  CU(cudaMemsetAsync(flag, 0, 4, p->stream));
  CU(bf::bb_launch_encode(data, cm->cw.as<uint32_t>(), p->d, p->log2_c, p->log2_k0, p->generic, w,
                          p->tw.as<uint2>(), flag, p->stream, slice_ready, slices));
  uint4* leaves = cm->tree.as<uint4>();
  CU(bf::bb_launch_leaves_rows(cm->cw.as<uint32_t>(), leaves, n, w, p->L, p->stream));
  uint4* root_dev = p->small.as<uint4>() + 2;
  CU(bf::launch_tree(leaves, n, p->stream, root_dev, bf::Tune()));
  CU(cudaMemcpyAsync(p->pin.b(), p->small.p, 64, cudaMemcpyDeviceToHost, p->stream));
  CU(cudaStreamSynchronize(p->stream));
  uint32_t bad;
  std::memcpy(&bad, p->pin.b(), 4);
  if (bad) return fail(BF_ERR_ARG, "an evaluation is not a canonical BabyBear (>= p)");
  bfh::digest_from_interleaved(p->pin.b() + 32, cm->root);
  return BF_OK;
}

}  // namespace

extern "C" {

static int bb_setup(int device, int lambda, int log2_c, int log2_k0, int num_vars, const uint32_t* ts,
                    size_t ts_len, void* stream, bf_bb_pcs** out) {
  if (!out) return fail(BF_ERR_ARG, "out is null");
  *out = nullptr;
  if (lambda < 0 || log2_c < 0 || num_vars < 0 || log2_k0 < 0 || log2_k0 > num_vars || num_vars + log2_c > 27)
    return fail(BF_ERR_ARG,
                "unsupported code parameters lambda=%d log2_c=%d log2_k_0=%d num_vars=%d (log2_k_0 <= num_vars, "
                "num_vars + log2_c <= 27)",
                lambda, log2_c, log2_k0, num_vars);
  std::unique_ptr<bf_bb_pcs> p(new bf_bb_pcs());
  p->lambda = lambda;
  p->log2_c = log2_c;
  p->log2_k0 = log2_k0;
  p->num_vars = num_vars;
  p->d = num_vars - log2_k0;
  p->L = num_vars + log2_c;
  p->generic = ts != nullptr;
  if (p->generic) {
    const size_t need = p->n0() * (((size_t)1 << p->d) - 1);
    if (ts_len != need)
      return fail(BF_ERR_ARG, "ts holds %zu values; the code needs n_0 (2^d - 1) = %zu", ts_len, need);
    for (size_t k = 0; k < need; ++k)
      if (ts[k] == 0 || ts[k] >= bbh::P) return fail(BF_ERR_ARG, "ts[%zu] = %u is zero or not canonical", k, ts[k]);
    p->ts.assign(ts, ts + need);
  }
  p->Q = bb_num_queries(*p);
  if (device < 0) {  // verifier-only: no GPU is touched
    *out = p.release();
    return BF_OK;
  }
  p->device = device;
  CU(cudaSetDevice(device));
  if (stream) {
    p->stream = reinterpret_cast<cudaStream_t>(stream);
  } else {
    CU(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
    p->own_stream = true;
  }
  CU(p->pin.ensure(4096));
  CU(p->small.alloc(4096));
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
  CU(cudaStreamCreateWithFlags(&p->aux, cudaStreamNonBlocking));
  CU(cudaEventCreateWithFlags(&p->ev_fork, cudaEventDisableTiming));
  for (cudaEvent_t* e : {&p->ev_dot, &p->ev_x, &p->ev_join}) CU(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  for (cudaEvent_t& e : p->slice_ev) CU(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  CU(p->tw.alloc(8 * p->n_d()));
  CU(p->tinv.alloc(4 * p->n0() * (((size_t)1 << p->d) - 1) + 4));
  uint32_t* flag = p->small.as<uint32_t>();
  CU(cudaMemsetAsync(flag, 0, 4, p->stream));
  if (!p->generic) {
    // DIT twiddles: layer s (half-size 2^s) uses g_s = two_adic_generator(s + 1)
    for (int s = 0; s < p->L; ++s)
      CU(bf::bb_launch_pow_shoup(p->tw.as<uint2>() + ((size_t)1 << s) - 1, (size_t)1 << s,
                                 bb::to_mont(bbh::two_adic_generator(s + 1)), p->stream));
    // ReedSolomonCode::new (reed_solomon.rs:20-38): t_i = two_adic_generator(
    // log2_c + i + 1), entry j = (2 t_i^j)^-1 = 2^-1 (t_i^-1)^j
    for (int i = 0; i < p->d; ++i) {
      const uint32_t t_inv = bbh::finv(bbh::two_adic_generator(p->log2_c + i + 1));
      CU(bf::bb_launch_pow_table(p->tinv.as<uint32_t>() + p->tinv_off(i), p->n_i(i), bb::to_mont(t_inv),
                                 bb::MONT_INV2, p->stream));
    }
  } else if (p->d > 0) {
    // generic.rs:43-71: round i's butterflies are layer log2_n0 + i of the
    // encode and its fold constants are (2 ts[i][j])^-1
    DevBuf tdev;
    const size_t total = p->ts.size();
    CU(tdev.alloc(4 * total));
    CU(cudaMemcpyAsync(tdev.p, p->ts.data(), 4 * total, cudaMemcpyHostToDevice, p->stream));
    for (int i = 0; i < p->d; ++i) {
      const int s = p->log2_n0() + i;
      CU(bf::bb_launch_shoup_from(tdev.as<uint32_t>() + p->tinv_off(i), p->tw.as<uint2>() + ((size_t)1 << s) - 1,
                                  p->n_i(i), flag, p->stream));
    }
    CU(bf::bb_launch_tinv(tdev.as<uint32_t>(), p->tinv.as<uint32_t>(), total, flag, p->stream));
    CU(cudaStreamSynchronize(p->stream));  // tdev is released below
  }
  CU(cudaStreamSynchronize(p->stream));
  *out = p.release();
  return BF_OK;
}

int bf_bb_pcs_setup(int device, int lambda, int log2_c, int num_vars, void* stream, bf_bb_pcs** out) {
  return bb_setup(device, lambda, log2_c, 0, num_vars, nullptr, 0, stream, out);
}

int bf_bb_pcs_setup_generic(int device, int lambda, int log2_c, int log2_k_0, int num_vars, const uint32_t* ts,
                            size_t ts_len, void* stream, bf_bb_pcs** out) {
  if (!ts && num_vars > log2_k_0) return fail(BF_ERR_ARG, "ts is null");
  static const uint32_t none = 1;
  return bb_setup(device, lambda, log2_c, log2_k_0, num_vars, ts ? ts : &none, ts_len, stream, out);
}

void bf_bb_pcs_free(bf_bb_pcs* pcs) {
  if (pcs) bb_release(pcs);
}

size_t bf_bb_pcs_num_queries(const bf_bb_pcs* pcs) { return pcs ? pcs->Q : 0; }

size_t bf_bb_pcs_proof_size(const bf_bb_pcs* p, size_t width, int n_evals) {
  if (!p || width == 0) return 0;
  if (n_evals == 0) return 32;  // BasefoldProof::default(): four empty vectors
  return p->header_bytes() + p->Q * p->rec_bytes(width);
}

static int check_commit_args(bf_bb_pcs* p, const void* evals, size_t width, bf_bb_commitment** out) {
  if (!p || !evals || !out) return fail(BF_ERR_ARG, "null argument");
  *out = nullptr;
  if (p->device < 0) return fail(BF_ERR_ARG, "verifier-only pcs (device < 0)");
  if (width == 0 || width > 65536) return fail(BF_ERR_ARG, "width %zu out of range (1..65536)", width);
  return BF_OK;
}

int bf_bb_commit(bf_bb_pcs* p, const uint32_t* evals, size_t width, bf_bb_commitment** out, uint8_t root[32]) {
  TRY(check_commit_args(p, evals, width, out));
  DeviceGuard g(p->device);
  std::unique_ptr<bf_bb_commitment> cm(new bf_bb_commitment());
  cm->pcs = p;
  cm->w = width;
  const size_t bytes = 4 * width << p->num_vars;
  CU(cm->data.alloc_async(bytes, p->pool, p->stream));  // before the fork: `aux` writes it after this point
  if (p->num_vars >= 16) {
    // copy in slices on the second stream; the encode's first stage takes
    // each slice as it lands (pinned `evals` overlap the copy with the encode)
    const int S = bf_bb_pcs::kH2DSlices;
    const size_t slice = bytes / S;
    CU(cudaEventRecord(p->ev_fork, p->stream));
    CU(cudaStreamWaitEvent(p->aux, p->ev_fork, 0));
    for (int k = 0; k < S; ++k) {
      CU(cudaMemcpyAsync(cm->data.as<uint8_t>() + k * slice, reinterpret_cast<const uint8_t*>(evals) + k * slice,
                         slice, cudaMemcpyHostToDevice, p->aux));
      CU(cudaEventRecord(p->slice_ev[k], p->aux));
    }
    TRY(commit_device(p, cm.get(), cm->data.as<uint32_t>(), p->slice_ev, S));
  } else {
    CU(cudaMemcpyAsync(cm->data.p, evals, bytes, cudaMemcpyHostToDevice, p->stream));
    TRY(commit_device(p, cm.get(), cm->data.as<uint32_t>()));
  }
  if (root) std::memcpy(root, cm->root, 32);
  bb_acquire(p);
  *out = cm.release();
  return BF_OK;
}

int bf_bb_commit_device(bf_bb_pcs* p, const void* d_evals, size_t width, bf_bb_commitment** out, uint8_t root[32]) {
  TRY(check_commit_args(p, d_evals, width, out));
  if (reinterpret_cast<uintptr_t>(d_evals) & 3) return fail(BF_ERR_ARG, "device evaluations must be 4-byte aligned");
  DeviceGuard g(p->device);
  std::unique_ptr<bf_bb_commitment> cm(new bf_bb_commitment());
  cm->pcs = p;
  cm->w = width;
  cm->data.p = const_cast<void*>(d_evals);
  cm->data.owned = false;
  cm->data.bytes = 4 * width << p->num_vars;
  TRY(commit_device(p, cm.get(), cm->data.as<uint32_t>()));
  if (root) std::memcpy(root, cm->root, 32);
  bb_acquire(p);
  *out = cm.release();
  return BF_OK;
}

int bf_bb_commitment_root(const bf_bb_commitment* cm, uint8_t root[32]) {
  if (!cm || !root) return fail(BF_ERR_ARG, "null argument");
  std::memcpy(root, cm->root, 32);
  return BF_OK;
}

void bf_bb_commitment_free(bf_bb_commitment* cm) {
  if (!cm) return;
  bf_bb_pcs* p = cm->pcs;
  {
    DeviceGuard g(p->device);
    delete cm;  // owned buffers return to the pcs's pool in stream order
  }
  bb_release(p);
}

namespace {
// The column values of 2^num_vars rows of w canonical words (device memory)
// at a host point: the point's eq table against every column.
int eval_device_rows(bf_bb_pcs* p, const uint32_t* data, size_t w, const uint8_t* point, uint8_t* values) {
  std::vector<E> x;
  TRY(load_points(point, (size_t)p->num_vars, x, "point coordinate"));
  const size_t rows = (size_t)1 << p->num_vars;
  // the sums are 64-bit atomics: their slot starts on a 256-byte boundary
  const size_t eq_bytes = (20 * rows + 255) & ~(size_t)255, acc_bytes = 40 * w;
  if (p->ws.bytes < eq_bytes + acc_bytes) CU(p->ws.alloc(eq_bytes + acc_bytes));
  CU(p->pin.ensure(acc_bytes + 64));
  uint32_t* eq = p->ws.as<uint32_t>();
  unsigned long long* acc = reinterpret_cast<unsigned long long*>(p->ws.as<uint8_t>() + eq_bytes);
  TRY(eq_table_device(p, x, eq));
  CU(cudaMemsetAsync(acc, 0, acc_bytes, p->stream));
  // evaluate = sum over the hypercube of eq(b, point) f(b): the same field
  // value as MultiPoly::evaluate's fix_last_var chain
  if (w == 1)
    CU(bf::bb_launch_dot(eq, data, 1, rows, acc, p->stream));
  else
    CU(bf::bb_launch_eval_cols(eq, data, rows, w, acc, p->stream));
  CU(cudaMemcpyAsync(p->pin.p, acc, acc_bytes, cudaMemcpyDeviceToHost, p->stream));
  CU(cudaStreamSynchronize(p->stream));
  const unsigned long long* s = reinterpret_cast<const unsigned long long*>(p->pin.p);
  for (size_t c = 0; c < w; ++c) bbh::store(values + 20 * c, bbh::from_canonical_sums(s + 5 * c));
  return BF_OK;
}
}  // namespace

int bf_bb_eval(bf_bb_pcs* p, const bf_bb_commitment* cm, const uint8_t* point, uint8_t* values) {
  if (!p || !cm || !values || (p->num_vars > 0 && !point)) return fail(BF_ERR_ARG, "null argument");
  if (cm->pcs != p) return fail(BF_ERR_ARG, "commitment made by another pcs");
  DeviceGuard g(p->device);
  return eval_device_rows(p, cm->data.as<uint32_t>(), cm->w, point, values);
}

int bf_bb_eval_data(bf_bb_pcs* p, const void* evals, int on_device, size_t width, const uint8_t* point,
                    uint8_t* values) {
  if (!p || !evals || !values || (p->num_vars > 0 && !point)) return fail(BF_ERR_ARG, "null argument");
  if (p->device < 0) return fail(BF_ERR_ARG, "verifier-only pcs (device < 0)");
  if (width == 0 || width > 65536) return fail(BF_ERR_ARG, "width %zu out of range (1..65536)", width);
  if (on_device && (reinterpret_cast<uintptr_t>(evals) & 3))
    return fail(BF_ERR_ARG, "device evaluations must be 4-byte aligned");
  DeviceGuard g(p->device);
  if (on_device) return eval_device_rows(p, static_cast<const uint32_t*>(evals), width, point, values);
  // host rows: copied in on the pcs's stream into a grow-only buffer
  const size_t bytes = 4 * width << p->num_vars;
  if (p->data_ws.bytes < bytes) CU(p->data_ws.alloc(bytes));
  CU(cudaMemcpyAsync(p->data_ws.p, evals, bytes, cudaMemcpyHostToDevice, p->stream));
  return eval_device_rows(p, p->data_ws.as<uint32_t>(), width, point, values);
}

int bf_bb_open(bf_bb_pcs* p, const bf_bb_commitment* cm, const uint8_t* point, const uint8_t* values,
               int n_evals, bf_challenger* ch, uint8_t* proof, size_t cap, size_t* proof_len) {
  if (!p || !cm || !ch || !proof_len) return fail(BF_ERR_ARG, "null argument");
  if (cm->pcs != p) return fail(BF_ERR_ARG, "commitment made by another pcs");
  if (n_evals < 0 || n_evals > 1) return fail(BF_ERR_ARG, "n_evals %d: one point or none (basefold.rs:143-144)", n_evals);
  if (n_evals == 0) {  // basefold.rs:139-141
    *proof_len = 32;
    if (!proof || cap < 32) return fail(BF_ERR_BUFFER, "proof buffer of %zu bytes, 32 needed", cap);
    std::memset(proof, 0, 32);
    return BF_OK;
  }
  if (!values || (p->num_vars > 0 && !point)) return fail(BF_ERR_ARG, "null argument");
  const int d = p->d, L = p->L, nv = p->num_vars, lk = p->log2_k0;
  const size_t w = cm->w, Q = p->Q, rec = p->rec_bytes(w), k0 = p->k0();
  const size_t total = p->header_bytes() + Q * rec;
  *proof_len = total;
  if (!proof || cap < total) return fail(BF_ERR_BUFFER, "proof buffer of %zu bytes, %zu needed", cap, total);
  std::vector<E> r, vals;
  TRY(load_points(point, (size_t)nv, r, "point coordinate"));
  TRY(load_points(values, w, vals, "value"));
  bbh::EvalScalars es;
  if (!es.init(r)) return fail(BF_ERR_NOT_INVERTIBLE, "a point coordinate is 0, or 1 below the last");
  DeviceGuard g(p->device);
  bfh::Challenger& tr = ch->c;
  cudaStream_t st = p->stream;

  // Workspace: batched poly and pi (width > 1), half_eq, two fix buffers,
  // the fold outputs of every round, the trees of every round, query indices
  // and records.
  const size_t rows = (size_t)1 << nv, half = rows >> 1;
  const size_t n_fold = p->n0() * (((size_t)1 << d) - 1);  // sum over rounds of n_i
  const size_t wsz[] = {w > 1 ? 20 * rows : 0,
                        w > 1 ? 20 * p->n_d() : 0,
                        20 * (half ? half : 1),
                        20 * half,
                        20 * half,
                        20 * n_fold,
                        64 * n_fold,
                        8 * Q,
                        Q * rec,
                        128,
                        w > 1 ? 20 * rows : 0,
                        sizeof(bf::BbTranscript) + sizeof(bf::BbRoundConsts),
                        (20 + 72) * (size_t)(d > 0 ? d : 1),
                        w > 1 ? 20 * w : 0};
  constexpr int kSlots = sizeof(wsz) / sizeof(wsz[0]);
  size_t off[kSlots + 1] = {0};
  for (int k = 0; k < kSlots; ++k) off[k + 1] = off[k] + ((wsz[k] + 255) & ~(size_t)255);
  if (p->open_ws.bytes < off[kSlots]) CU(p->open_ws.alloc(off[kSlots]));
  uint8_t* base = p->open_ws.as<uint8_t>();
  uint32_t* polyE = reinterpret_cast<uint32_t*>(base + off[0]);
  uint32_t* piE = reinterpret_cast<uint32_t*>(base + off[1]);
  uint32_t* heq = reinterpret_cast<uint32_t*>(base + off[2]);
  uint32_t* fixbuf[2] = {reinterpret_cast<uint32_t*>(base + off[3]), reinterpret_cast<uint32_t*>(base + off[4])};
  uint32_t* folds = reinterpret_cast<uint32_t*>(base + off[5]);
  uint4* trees = reinterpret_cast<uint4*>(base + off[6]);
  uint64_t* idx_dev = reinterpret_cast<uint64_t*>(base + off[7]);
  uint8_t* recs = base + off[8];
  unsigned long long* acc = reinterpret_cast<unsigned long long*>(base + off[9]);
  uint4* root_dev = reinterpret_cast<uint4*>(base + off[9] + 64);  // after the five sums
  uint32_t* poly_canon = reinterpret_cast<uint32_t*>(base + off[10]);  // width > 1: the combined poly, canonical
  // the device transcript, the round constants, each round's challenge (20 bytes) and record (72)
  bf::BbTranscript* tdev = reinterpret_cast<bf::BbTranscript*>(base + off[11]);
  bf::BbRoundConsts* cdev = reinterpret_cast<bf::BbRoundConsts*>(base + off[11] + sizeof(bf::BbTranscript));
  uint32_t* xs_dev = reinterpret_cast<uint32_t*>(base + off[12]);
  uint8_t* rec_dev = base + off[12] + 20 * (size_t)(d > 0 ? d : 1);
  uint32_t* scal_dev = reinterpret_cast<uint32_t*>(base + off[13]);  // width > 1: the batching scalars
  CU(p->pin.ensure(std::max<size_t>(8 * Q + 20 * k0 + 20 * 64 + 256 + sizeof(bf::BbTranscript) +
                                         sizeof(bf::BbRoundConsts) + 72 * (size_t)d,
                                     20 * w)));

  // The polynomial and codeword the folding sumcheck runs on (basefold.rs:154-177).
  E claim;
  const uint32_t* poly = cm->data.as<uint32_t>();
  const uint32_t* pi = cm->cw.as<uint32_t>();
  int base_round = 1;  // the first round's poly and pi are base-field arrays
  if (w == 1) {
    claim = vals[0];
  } else {
    const std::vector<E> s = bbh::scalars_by_eq(w, tr);
    for (size_t c = 0; c < w; ++c) claim = bbh::eadd(claim, bbh::emul(s[c], vals[c]));
    // s R^2 against the canonical evaluations
    bb::E5* sd = reinterpret_cast<bb::E5*>(p->pin.p);
    for (size_t c = 0; c < w; ++c) sd[c] = bbh::to_dev2(s[c]);
    CU(cudaMemcpyAsync(scal_dev, sd, 20 * w, cudaMemcpyHostToDevice, st));
    CU(bf::bb_launch_combine(cm->data.as<uint32_t>(), rows, w, scal_dev, polyE, st));
    // The reference combines the codeword's rows the same way; both codes are
    // linear over the base field, so that combination is the encoding of the
    // combined polynomial, coefficient by coefficient: a 5-column encode of
    // 2^num_vars rows instead of w products per codeword row, the same values.
    CU(bf::bb_launch_from_mont(polyE, poly_canon, 5 * rows, st));
    uint32_t* flag = p->small.as<uint32_t>();
    CU(cudaMemsetAsync(flag, 0, 4, st));
    CU(bf::bb_launch_encode(poly_canon, piE, p->d, p->log2_c, p->log2_k0, p->generic, 5, p->tw.as<uint2>(), flag,
                            st));
    CU(cudaStreamSynchronize(st));  // the staging of the scalars is reused below
    poly = polyE;
    pi = piE;
    base_round = 0;
  }
  // HalfEq over the point's first num_vars - 1 coordinates (eval_impr.rs)
  if (nv > 0) TRY(eq_table_device(p, std::vector<E>(r.begin(), r.end() - 1), heq));

  // prove_interleaved_folding_sumcheck (basefold.rs:335-369) with the
  // transcript on the device: every round is enqueued without waiting, the
  // host reads the transcript back once at the end.
  std::vector<std::array<E, 2>> comp;
  std::vector<std::array<uint8_t, 32>> roots;
  bf::BbGather gp{};
  gp.pi0_base = w == 1;
  const size_t tsz = sizeof(bf::BbTranscript) + sizeof(bf::BbRoundConsts);
  if (d > 0) {
    // the caller's transcript as a sponge: whole 136-byte blocks of its input
    // absorbed here, the rest pending
    bf::BbTranscript t{};
    uint64_t A[25] = {0};
    size_t pos = 0;
    for (; pos + 136 <= tr.in.size(); pos += 136) {
      for (int l = 0; l < 17; ++l) {
        uint64_t v = 0;
        std::memcpy(&v, tr.in.data() + pos + 8 * l, 8);
        A[l] ^= v;
      }
      bfh::keccak_f(A);
    }
    for (int l = 0; l < 25; ++l) t.A[l] = make_uint2((uint32_t)A[l], (uint32_t)(A[l] >> 32));
    t.pend_len = (uint32_t)(tr.in.size() - pos);
    std::memcpy(t.pend, tr.in.data() + pos, t.pend_len);
    t.out_len = (uint32_t)tr.out.size();
    std::memcpy(t.out, tr.out.data(), t.out_len);
    t.outer = bbh::to_dev(claim);
    bf::BbRoundConsts c{};
    const std::vector<E> cf = es.correcting_factors();
    for (int k = 0; k < nv; ++k) {
      c.r[k] = bbh::to_dev(r[k]);
      c.r_inv[k] = bbh::to_dev(es.r_inv[k]);
      c.cf[k] = bbh::to_dev(cf[k]);
    }
    std::memcpy(p->pin.p, &t, sizeof(t));
    std::memcpy(p->pin.b() + sizeof(t), &c, sizeof(c));
    CU(cudaMemcpyAsync(tdev, p->pin.p, tsz, cudaMemcpyHostToDevice, st));
  }
  // A round's sums need only the previous fix and its fix only the round's
  // challenge, so both run on `aux` beside the round's tree and fold: the
  // main stream's chain per round is tree, transcript step, fold.
  struct AuxJoin {  // joins `aux` back into the main stream on every exit
    bf_bb_pcs* p;
    cudaStream_t st;
    bool active = false;
    ~AuxJoin() {
      if (active && cudaEventRecord(p->ev_join, p->aux) == cudaSuccess) cudaStreamWaitEvent(st, p->ev_join, 0);
    }
  } join{p, st};
  cudaStream_t sa = p->aux;
  CU(cudaEventRecord(p->ev_fork, st));  // the eq table, the round-0 poly and the transcript state
  CU(cudaStreamWaitEvent(sa, p->ev_fork, 0));
  join.active = true;
  size_t fold_off = 0, tree_off = 0;
  for (int k = 0; k < d; ++k) {
    const int i = d - 1 - k, li = p->log2_n0() + i;
    const int ri = i + lk;  // the sumcheck round (basefold.rs:356-361)
    const size_t ni = p->n_i(i);
    uint4* tree = trees + 2 * tree_off;
    gp.pi[k] = pi;
    gp.trees[k] = tree;
    const int base_k = k == 0 && base_round;
    if (k == 0) CU(bf::bb_launch_leaves_pairs(pi, base_k, tree, ni, li, st));  // later rounds: made by the fold
    CU(bf::launch_tree(tree, ni, st, root_dev, bf::Tune()));
    CU(cudaMemsetAsync(acc, 0, 40, sa));
    CU(bf::bb_launch_dot(heq, poly, base_k, (size_t)1 << ri, acc, sa));
    CU(cudaEventRecord(p->ev_dot, sa));
    CU(cudaStreamWaitEvent(st, p->ev_dot, 0));
    uint32_t* x_k = xs_dev + 5 * (size_t)k;
    CU(bf::bb_launch_transcript_round(tdev, cdev, k, ri, nv, root_dev, acc, base_k, x_k, rec_dev + 72 * (size_t)k,
                                      st));
    CU(cudaEventRecord(p->ev_x, st));
    CU(cudaStreamWaitEvent(sa, p->ev_x, 0));
    const bb::E5 unused{};
    uint32_t* fixed = fixbuf[k & 1];  // the fix two rounds back and the sums since have read it (stream order)
    CU(bf::bb_launch_fix(poly, base_k, fixed, (size_t)1 << ri, unused, sa, x_k));
    poly = fixed;
    bf::BbFold fp;
    fp.w = pi;
    fp.base = base_k;
    fp.out = folds + 5 * fold_off;
    fp.tinv = p->tinv.as<uint32_t>() + p->tinv_off(i);
    fp.n = ni;
    fp.leaves = i > 0 ? tree + 2 * (2 * ni) : nullptr;  // the next round's tree follows this one
    fp.leaf_bits = li - 1;
    fp.xp = x_k;
    CU(bf::bb_launch_fold(fp, unused, st));
    pi = fp.out;
    fold_off += ni;
    tree_off += 2 * ni;
  }
  CU(cudaEventRecord(p->ev_join, sa));  // the last fix, before the final poly is read
  CU(cudaStreamWaitEvent(st, p->ev_join, 0));
  join.active = false;
  // final_poly (into_ext_poly): the k_0 evaluations left after d fixes, observed
  std::vector<E> fin(k0);
  {
    const int fin_base = d == 0 && base_round;  // still the caller's base-field data
    CU(cudaMemcpyAsync(p->pin.p, poly, (fin_base ? 4 : 20) * k0, cudaMemcpyDeviceToHost, st));
    const size_t chk_off = 20 * k0 + 64;
    const size_t t_off = chk_off + 20 * 64;  // then the transcript, then the round records
    size_t nchk = 0;
    if (d > 0) {  // debug_assert_eq!(encode0(final_poly), pi) (basefold.rs:189), up to 64 entries
      nchk = p->n0() < 64 ? p->n0() : 64;
      CU(cudaMemcpyAsync(p->pin.b() + chk_off, pi, 20 * nchk, cudaMemcpyDeviceToHost, st));
      CU(cudaMemcpyAsync(p->pin.b() + t_off, tdev, sizeof(bf::BbTranscript), cudaMemcpyDeviceToHost, st));
      CU(cudaMemcpyAsync(p->pin.b() + t_off + sizeof(bf::BbTranscript), rec_dev, 72 * (size_t)d,
                         cudaMemcpyDeviceToHost, st));
    }
    CU(cudaStreamSynchronize(st));
    for (size_t t = 0; t < k0; ++t) {
      if (fin_base) {
        uint32_t v;
        std::memcpy(&v, p->pin.b() + 4 * t, 4);
        fin[t] = E::from(v);
      } else {
        uint32_t m[5];
        std::memcpy(m, p->pin.b() + 20 * t, 20);
        for (int q = 0; q < 5; ++q) fin[t].c[q] = bb::from_mont(m[q]);
      }
    }
    for (size_t q = 0; q < nchk; ++q) {
      uint32_t m[5];
      std::memcpy(m, p->pin.b() + chk_off + 20 * q, 20);
      E e;
      for (int t = 0; t < 5; ++t) e.c[t] = bb::from_mont(m[t]);
      if (e != p->encode0_at(fin, q))
        return fail(BF_ERR_CHECK, "the last folded codeword is not the encoding of the final polynomial");
    }
    if (d > 0) {
      // the caller's transcript continues from the device's: after a sample the
      // sponge holds no absorbed block, only pending input bytes
      bf::BbTranscript t;
      std::memcpy(&t, p->pin.b() + t_off, sizeof(t));
      for (int l = 0; l < 25; ++l)
        if (t.A[l].x | t.A[l].y) return fail(BF_ERR_CHECK, "device transcript left an absorbed block");
      tr.in.assign(t.pend, t.pend + t.pend_len);
      tr.out.assign(t.out, t.out + t.out_len);
      const uint8_t* rb = p->pin.b() + t_off + sizeof(bf::BbTranscript);
      for (int k = 0; k < d; ++k) {
        std::array<uint8_t, 32> root;
        std::memcpy(root.data(), rb + 72 * k, 32);
        roots.push_back(root);
        comp.push_back({bbh::load(rb + 72 * k + 32), bbh::load(rb + 72 * k + 52)});
      }
    }
  }
  for (const E& e : fin) bbh::observe_e(tr, e);
  std::vector<uint64_t> idx(Q);
  for (uint64_t& v : idx) v = tr.sample_bits(L);
  if (Q) {
    std::memcpy(p->pin.p, idx.data(), 8 * Q);
    CU(cudaMemcpyAsync(idx_dev, p->pin.p, 8 * Q, cudaMemcpyHostToDevice, st));
    gp.cw = cm->cw.as<uint32_t>();
    gp.cw_tree = cm->tree.as<uint4>();
    gp.idx = idx_dev;
    gp.out = recs;
    gp.w = w;
    gp.rec_bytes = rec;
    gp.L = L;
    gp.d = d;
    gp.log2_n0 = p->log2_n0();
    gp.nq = (int)Q;
    CU(bf::bb_launch_gather(gp, st));
    CU(cudaMemcpyAsync(proof + p->header_bytes(), recs, Q * rec, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
  }
  // BasefoldProof header: round polys, final poly, pi roots, query count
  std::vector<uint8_t> h;
  put_u64(h, (uint64_t)d);
  for (const auto& c : comp) {
    put_u64(h, 2);
    uint8_t b[20];
    for (const E& e : c) {
      bbh::store(b, e);
      h.insert(h.end(), b, b + 20);
    }
  }
  put_u64(h, (uint64_t)k0);
  for (const E& e : fin) {
    uint8_t b[20];
    bbh::store(b, e);
    h.insert(h.end(), b, b + 20);
  }
  put_u64(h, (uint64_t)d);
  for (const auto& rt : roots) h.insert(h.end(), rt.begin(), rt.end());
  put_u64(h, (uint64_t)Q);
  if (h.size() != p->header_bytes()) return fail(BF_ERR_CHECK, "proof header size mismatch");
  std::memcpy(proof, h.data(), h.size());
  return BF_OK;
}

// ---- verify (basefold.rs:234-324) on the host -------------------------------------
namespace {
struct Reader {
  const uint8_t* p;
  size_t n, off = 0;
  bool ok = true;
  const uint8_t* take(size_t k) {
    if (!ok || k > n - off) {
      ok = false;
      return nullptr;
    }
    const uint8_t* r = p + off;
    off += k;
    return r;
  }
  uint64_t u64() {
    const uint8_t* q = take(8);
    uint64_t v = 0;
    if (q) std::memcpy(&v, q, 8);
    return v;
  }
  bool e(E& out) {
    const uint8_t* q = take(20);
    if (!q) return false;
    out = bbh::load(q);
    return bbh::canonical(out);
  }
};
struct Dg {
  uint8_t b[32];
};
Dg hash_bytes(const uint8_t* m, size_t n) {
  Dg d;
  bfh::keccak256(m, n, d.b);
  return d;
}
Dg leaf_row(const uint32_t* row, size_t w) {
  std::vector<uint8_t> b(4 * w);
  std::memcpy(b.data(), row, 4 * w);
  return hash_bytes(b.data(), b.size());
}
Dg leaf_pair(const E& a, const E& b) {
  uint8_t m[40];
  bbh::store(m, a);
  bbh::store(m + 20, b);
  return hash_bytes(m, 40);
}
// MerkleTreeMmcs::verify_batch for one matrix: the path from leaf `idx` of a
// `height`-leaf tree to `root`.
bool verify_path(const uint8_t root[32], Dg leaf, uint64_t idx, const std::vector<Dg>& path, size_t height) {
  size_t h = 0;
  while (((size_t)1 << h) < height) ++h;
  if (path.size() != h) return false;
  uint8_t buf[64];
  for (const Dg& s : path) {
    if (idx & 1) {
      std::memcpy(buf, s.b, 32);
      std::memcpy(buf + 32, leaf.b, 32);
    } else {
      std::memcpy(buf, leaf.b, 32);
      std::memcpy(buf + 32, s.b, 32);
    }
    leaf = hash_bytes(buf, 64);
    idx >>= 1;
  }
  return std::memcmp(leaf.b, root, 32) == 0;
}
bool read_path(Reader& rd, std::vector<Dg>& path) {
  const uint64_t n = rd.u64();
  if (!rd.ok || n > 64) return false;
  path.resize(n);
  for (Dg& g : path) {
    const uint8_t* q = rd.take(32);
    if (!q) return false;
    std::memcpy(g.b, q, 32);
  }
  return true;
}
}  // namespace

int bf_bb_verify(const bf_bb_pcs* p, const uint8_t root[32], const uint8_t* point, const uint8_t* values,
                 size_t width, int n_evals, bf_challenger* ch, const uint8_t* proof, size_t proof_len) {
  if (!p || !root || !ch || (!proof && proof_len)) return fail(BF_ERR_ARG, "null argument");
  if (n_evals < 0 || n_evals > 1) return fail(BF_ERR_ARG, "n_evals %d: one point or none", n_evals);
  if (n_evals == 0) return BF_VERIFY_OK;  // basefold.rs:241-243
  if (!values || (p->num_vars > 0 && !point)) return fail(BF_ERR_ARG, "null argument");
  if (width == 0) return fail(BF_ERR_ARG, "width 0");
  const int d = p->d, lk = p->log2_k0;
  std::vector<E> r, vals;
  TRY(load_points(point, (size_t)p->num_vars, r, "point coordinate"));
  TRY(load_points(values, width, vals, "value"));
  bfh::Challenger& tr = ch->c;
  std::vector<E> scalars = {E::one()};
  E claim = vals[0];
  if (width > 1) {  // basefold.rs:253-259
    scalars = bbh::scalars_by_eq(width, tr);
    claim = E();
    for (size_t c = 0; c < width; ++c) claim = bbh::eadd(claim, bbh::emul(scalars[c], vals[c]));
  }
  Reader rd{proof, proof_len};
  if (rd.u64() != (uint64_t)d || !rd.ok) return BF_VERIFY_MALFORMED;
  std::vector<std::array<E, 2>> comp((size_t)d);
  for (auto& c : comp) {
    if (rd.u64() != 2 || !rd.e(c[0]) || !rd.e(c[1])) return BF_VERIFY_MALFORMED;
  }
  std::vector<E> fin(p->k0());
  if (rd.u64() != (uint64_t)p->k0()) return BF_VERIFY_MALFORMED;
  for (E& e : fin)
    if (!rd.e(e)) return BF_VERIFY_MALFORMED;
  if (rd.u64() != (uint64_t)d || !rd.ok) return BF_VERIFY_MALFORMED;
  std::vector<Dg> pi_comms((size_t)d);
  for (Dg& g : pi_comms) {
    const uint8_t* q = rd.take(32);
    if (!q) return BF_VERIFY_MALFORMED;
    std::memcpy(g.b, q, 32);
  }
  // verify_interleaved_folding_sumcheck (basefold.rs:371-396)
  bbh::Subclaim sc;
  sc.value = claim;
  for (int k = 0; k < d; ++k) {
    tr.observe(pi_comms[k].b, 32);
    bbh::observe_e(tr, comp[k][0]);
    bbh::observe_e(tr, comp[k][1]);
    // Eval::decompress_round_poly: c1 = claim - 2 c0 - c2
    const E c1 = bbh::esub(bbh::esub(sc.value, bbh::eadd(comp[k][0], comp[k][0])), comp[k][1]);
    const E x = bbh::sample_e(tr);
    const E rp[3] = {comp[k][0], c1, comp[k][1]};
    sc.reduce(rp, 3, x);
  }
  for (const E& e : fin) bbh::observe_e(tr, e);
  const std::vector<E> rr = sc.r();
  // evaluate(final_poly, point_lo) * eq_eval(point_hi, r) (basefold.rs:271-275):
  // fix_last_var with point_lo from its last coordinate down
  std::vector<E> ev = fin;
  for (int k = lk - 1; k >= 0; --k) {
    const size_t mid = ev.size() / 2;
    for (size_t b = 0; b < mid; ++b) ev[b] = bbh::eadd(ev[b], bbh::emul(r[k], bbh::esub(ev[b + mid], ev[b])));
    ev.resize(mid);
  }
  const size_t nhi = r.size() - (size_t)lk;
  if (bbh::emul(ev[0], bbh::eq_eval(r.data() + lk, rr.data(), nhi < rr.size() ? nhi : rr.size())) != sc.value)
    return BF_VERIFY_INVALID_FINAL_POLY;
  // pi_0 = encode0(final_poly) (basefold.rs:277)
  std::vector<E> pi0(p->n0());
  for (size_t i = 0; i < pi0.size(); ++i) pi0[i] = p->encode0_at(fin, i);
  const size_t Q = p->Q;
  std::vector<uint64_t> idx(Q);
  for (uint64_t& v : idx) v = tr.sample_bits(p->L);
  if (rd.u64() != (uint64_t)Q || !rd.ok) return BF_VERIFY_MALFORMED;
  std::vector<uint32_t> row(width);
  std::vector<Dg> path;
  for (size_t qi = 0; qi < Q; ++qi) {
    const uint64_t q = idx[qi];
    if (rd.u64() != (uint64_t)width) return BF_VERIFY_MALFORMED;
    const uint8_t* vp = rd.take(4 * width);
    if (!vp) return BF_VERIFY_MALFORMED;
    std::memcpy(row.data(), vp, 4 * width);
    for (uint32_t v : row)
      if (v >= bbh::P) return BF_VERIFY_MALFORMED;
    if (!read_path(rd, path)) return BF_VERIFY_MALFORMED;
    if (!verify_path(root, leaf_row(row.data(), width), q, path, p->n_d())) return BF_VERIFY_MMCS;
    E folded;
    for (size_t c = 0; c < width; ++c) folded = bbh::eadd(folded, bbh::escale(scalars[c], row[c]));
    if (rd.u64() != (uint64_t)d) return BF_VERIFY_MALFORMED;
    for (int k = 0; k < d; ++k) {
      const int i = d - 1 - k;
      const size_t ni = p->n_i(i);
      const size_t sib = ((q / ni) & 1) ^ 1, j = q % ni;
      E other;
      if (!rd.e(other)) return BF_VERIFY_MALFORMED;
      if (!read_path(rd, path)) return BF_VERIFY_MALFORMED;
      E v[2] = {folded, folded};
      v[sib] = other;
      if (!verify_path(pi_comms[k].b, leaf_pair(v[0], v[1]), j, path, ni)) return BF_VERIFY_MMCS;
      // interpolate (code.rs:86-91) with (2 t_i[j])^-1 and round i's challenge rr[i]
      const uint32_t t = p->t_inv_half(i, j);
      const E l = bbh::escale(bbh::eadd(v[0], v[1]), (bbh::P + 1) / 2);
      const E hh = bbh::escale(bbh::esub(v[0], v[1]), t);
      folded = bbh::eadd(l, bbh::emul(bbh::esub(hh, l), rr[i]));
    }
    if (folded != pi0[q % p->n0()]) return BF_VERIFY_INVALID_QUERY;  // pi_0[idx % n_0] (basefold.rs:316-318)
  }
  return rd.off == proof_len ? BF_VERIFY_OK : BF_VERIFY_MALFORMED;
}

int bf_challenger_sample_bb_ext(bf_challenger* ch, uint8_t out[20]) {
  if (!ch || !out) return fail(BF_ERR_ARG, "null argument");
  bbh::store(out, bbh::sample_e(ch->c));
  return BF_OK;
}

}  // extern "C"
