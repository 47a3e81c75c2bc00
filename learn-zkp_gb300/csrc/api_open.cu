// libbasefold_gpu.so: Basefold::open (poly-commit/src/basefold.rs:133-232).
//
// Two drivers over one session (device workspace, pinned staging):
//  * round-level, for a caller-held transcript: each round the device returns
//    the folded-codeword Merkle root and the compressed sumcheck round
//    polynomial; the caller's transcript observes them and samples the
//    challenge; the device then folds, fixes the variable and builds the
//    next round's tree;
//  * device-resident (bf_open, the engine): the library's transcript lives in
//    device memory and every round is queued at once (kernels_tail.cu); the
//    host samples only the query positions from the returned state.
// Both then gather the query openings and write the bincode proof.  Sessions
// own their device workspace, so several can be in flight on different
// streams.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <vector>

#include "api_common.h"

using bfh::u128;
using namespace bfapi;

struct bf_open_session {
  bf_pcs* p = nullptr;
  const bf_commitment* cm = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t ev = nullptr;
  int d = 0;
  size_t w = 1;            // columns of the commitment
  int i = 0;               // current round (d-1 .. 0); -1 once every round is done
  bool msg_ready = false;  // host message of the current round computed
  bool pending = false;    // device work enqueued, its result not read yet
  bool final_ready = false;
  std::vector<u128> r, r_inv, corr;
  u128 outer_val = 0, inner_val = 0, delta_prod = 0;
  uint8_t root[32] = {0};
  u128 rp[3] = {0, 0, 0};
  u128 c01[2] = {0, 0};
  u128 final_val = 0;
  std::vector<uint8_t> rounds, roots;
  DevBuf ws;
  uint4* w_point = nullptr;
  uint4* w_pi_fold = nullptr;
  uint4* w_pi_trees = nullptr;
  uint4* w_poly = nullptr;
  uint4* w_heq = nullptr;
  uint4* w_eq_lo = nullptr;
  uint4* w_eq_hi = nullptr;
  uint8_t* w_stage = nullptr;  // per round: root (32 B) + sumcheck reduction (16 B)
  uint64_t* w_idx = nullptr;
  uint8_t* w_open = nullptr;
  // width > 1: the eq-scalar combinations of the codeword rows (the first
  // round's folded codeword) and of the data rows (the sumcheck polynomial),
  // basefold.rs:166-183, and the first round's tree
  uint4* w_scalars = nullptr;
  uint4* w_pi_first = nullptr;
  uint4* w_pi_first_tree = nullptr;
  uint4* w_poly_first = nullptr;
  // device transcript: per-round scalars, the OpenState, the round records
  uint8_t* w_tail = nullptr;
  bf::OpenState* w_state = nullptr;
  uint8_t* w_rec = nullptr;
  bool resident_pending = false;   // a device-transcript open is in flight
  bool gather_pending = false;     // query openings in flight
  std::unique_ptr<PinnedBuf> pin;  // [0,64) staging, [64,64+16(w+d)) scalars and point, indices,
                                   // openings, device-transcript results; inputs at tail_in_off()
  uint64_t* idx_pin = nullptr;
  uint8_t* open_pin = nullptr;
  uint8_t* res_pin = nullptr;

  size_t c() const { return p->c(); }
  uint4* pi_fold_out(int k) const { return w_pi_fold + c() * (((size_t)1 << d) - ((size_t)1 << (k + 1))); }
  // tree of round k <= d-2 (round d-1's tree is the commitment's)
  uint4* pi_tree(int k) const {
    return w_pi_trees + 2 * ((c() << 1) * (((size_t)1 << (d - 1)) - ((size_t)1 << (k + 1))) - (size_t)(d - 2 - k));
  }
  uint8_t* stage(int k) const { return w_stage + 48 * (size_t)k; }
  const uint4* first_pi() const { return w == 1 ? cm->cw.as<uint4>() : w_pi_first; }
  const uint4* first_poly() const { return w == 1 ? cm->data.as<uint4>() : w_poly_first; }
  const uint4* first_tree() const { return w == 1 ? cm->pi_tree.as<uint4>() : w_pi_first_tree; }
  // Pinned offset of the device-transcript inputs: past the staging, the eq
  // scalars and the point, whose host-to-device copies may still be queued
  // when the resident open is enqueued.
  size_t tail_in_off() const { return 64 + 16 * ((size_t)(d > 0 ? d : 1) + w); }
  // Root of round d-1's tree on the device: the commitment's pair tree for
  // width 1, the combined rows' tree otherwise.
  const uint4* first_root_dev() const {
    return w == 1 ? cm->pi_tree.as<uint4>() + 2 * (p->n_d() - 2) : reinterpret_cast<const uint4*>(stage(d - 1));
  }
  ~bf_open_session() {
    if (st) cudaStreamSynchronize(st);
    if (ev) cudaEventDestroy(ev);
    ws.release();
    if (pin) {
      // keep the pinned staging for the next session of this pcs
      std::lock_guard<std::mutex> lk(p->pinned_mu);
      p->pinned_cache.push_back(std::move(pin));
    }
  }
};

namespace {

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

// Device-transcript workspace: per round 3 scalars (r_i, r_i^-1, correcting
// factor), the OpenState, then 64 bytes per round (root, c0, c2) and the
// final polynomial.
size_t state_off(int d) { return align256(48 * (size_t)(d > 0 ? d : 1)); }
size_t rec_off(int d) { return state_off(d) + align256(sizeof(bf::OpenState)); }
size_t rec_bytes(int d) { return 64 * (size_t)d + 16; }
size_t tail_bytes(int d) { return rec_off(d) + rec_bytes(d); }

int session_alloc(bf_open_session* s) {
  bf_pcs* p = s->p;
  const int d = s->d;
  const size_t c = p->c();
  const size_t half = d >= 1 ? ((size_t)1 << (d - 1)) : 1;
  const size_t n_point = d > 0 ? d : 1;
  const size_t n_fold = c * (((size_t)1 << d) - 1) + 1;
  const size_t n_tree = d >= 2 ? (c << 1) * (((size_t)1 << (d - 1)) - 1) - (size_t)(d - 1) + 1 : 1;
  const int hi_vars = d - 1 > 12 ? d - 1 - 12 : 0;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off += align256(bytes);
    return o;
  };
  const size_t o_point = take(16 * n_point), o_fold = take(16 * n_fold), o_tree = take(32 * n_tree);
  const size_t o_poly = take(16 * half), o_heq = take(16 * half), o_lo = take(16 * 4096);
  const size_t o_hi = take(16 * ((size_t)1 << hi_vars)), o_stage = take(48 * n_point);
  const size_t bb = p->block_bytes(s->w);
  const size_t o_idx = take(8 * (p->Q + 1)), o_open = take(bb * (p->Q + 1));
  const size_t o_tail = take(tail_bytes(d));
  size_t o_sc = 0, o_pif = 0, o_pift = 0, o_polyf = 0;
  if (s->w > 1) {
    o_sc = take(16 * s->w);
    o_pif = take(16 * p->n_d());
    o_pift = take(32 * p->n_d());
    o_polyf = take(16 * ((size_t)1 << d));
  }
  CU(s->ws.alloc_async(off, p->pool, s->st));
  uint8_t* b = s->ws.as<uint8_t>();
  if (s->w > 1) {
    s->w_scalars = reinterpret_cast<uint4*>(b + o_sc);
    s->w_pi_first = reinterpret_cast<uint4*>(b + o_pif);
    s->w_pi_first_tree = reinterpret_cast<uint4*>(b + o_pift);
    s->w_poly_first = reinterpret_cast<uint4*>(b + o_polyf);
  }
  s->w_tail = b + o_tail;
  s->w_state = reinterpret_cast<bf::OpenState*>(b + o_tail + state_off(d));
  s->w_rec = b + o_tail + rec_off(d);
  s->w_point = reinterpret_cast<uint4*>(b + o_point);
  s->w_pi_fold = reinterpret_cast<uint4*>(b + o_fold);
  s->w_pi_trees = reinterpret_cast<uint4*>(b + o_tree);
  s->w_poly = reinterpret_cast<uint4*>(b + o_poly);
  s->w_heq = reinterpret_cast<uint4*>(b + o_heq);
  s->w_eq_lo = reinterpret_cast<uint4*>(b + o_lo);
  s->w_eq_hi = reinterpret_cast<uint4*>(b + o_hi);
  s->w_stage = b + o_stage;
  s->w_idx = reinterpret_cast<uint64_t*>(b + o_idx);
  s->w_open = b + o_open;
  const size_t res_off = align16(64 + 16 * (n_point + s->w) + 8 * (p->Q + 1) + bb * (p->Q + 1));
  const size_t pin_bytes =
      std::max(res_off + align16(rec_bytes(d)) + sizeof(bf::OpenState),
               s->tail_in_off() + 48 * n_point + sizeof(bf::OpenState));
  {
    std::lock_guard<std::mutex> lk(p->pinned_mu);
    if (!p->pinned_cache.empty()) {
      s->pin = std::move(p->pinned_cache.back());
      p->pinned_cache.pop_back();
    }
  }
  if (!s->pin) s->pin.reset(new PinnedBuf());
  CU(s->pin->ensure(pin_bytes));
  s->idx_pin = reinterpret_cast<uint64_t*>(s->pin->b() + 64 + 16 * (n_point + s->w));
  s->open_pin = reinterpret_cast<uint8_t*>(s->idx_pin + (p->Q + 1));
  s->res_pin = s->pin->b() + res_off;
  return BF_OK;
}

// Reads the result of the enqueued work and computes the host-side message of
// the current round: EvalImprProver::compute_round_poly + decompress
// (eval_impr.rs:116-127,187-197) lifted by EvalProver (eval.rs:89-106).
int ensure_message(bf_open_session* s) {
  if (s->pending) {
    CU(cudaStreamSynchronize(s->st));
    s->p->prof.drain();
    s->pending = false;
  }
  if (s->i < 0) {
    if (!s->final_ready) {
      s->final_val = bfh::load(s->pin->b());
      s->final_ready = true;
    }
    return BF_OK;
  }
  if (s->msg_ready) return BF_OK;
  const int i = s->i, d = s->d;
  const u128 ONE = bfh::one();
  if (i == d - 1 && s->w == 1)
    std::memcpy(s->root, s->cm->pi_root, 32);
  else
    bfh::digest_from_interleaved(s->pin->b(), s->root);  // a tree root, stored interleaved
  const u128 S = bfh::load(s->pin->b() + 32);
  const u128 sc_val = (i == d - 1) ? s->outer_val : s->inner_val;
  const u128 c0 = bfh::mul(s->corr[i], S);
  const u128 c1 = bfh::mul(sc_val ^ bfh::mul(ONE ^ s->r[i], c0), s->r_inv[i]) ^ c0;
  const u128 scalar = (i == d - 1) ? ONE : s->delta_prod;  // delta_scalar (eval_impr.rs:45-51)
  const u128 d0 = bfh::mul(scalar, ONE ^ s->r[i]);
  const u128 d1 = bfh::mul(scalar, s->r[i] ^ (ONE ^ s->r[i]));
  s->c01[0] = c0;
  s->c01[1] = c1;
  s->rp[0] = bfh::mul(c0, d0);
  s->rp[1] = bfh::mul(c0, d1) ^ bfh::mul(c1, d0);
  s->rp[2] = bfh::mul(c1, d1);
  s->msg_ready = true;
  return BF_OK;
}

}  // namespace

namespace bfapi {

// First round run by the single-block kernel: the largest i <= d-1 whose
// folded codeword has at most 2^(tail_log+1) entries.
int tail_first_round(const bf_pcs* p, int d) {
  const int lim = p->tune.tail_log + 1 - p->log2_c;
  return std::min(d - 1, lim);
}

// Host side of a device-transcript open: the per-round scalars and the
// starting OpenState (transcript `ch`, claim, delta = 1) in the pinned
// staging.
int open_resident_prepare(bf_open_session* s, const bfh::Challenger& ch) {
  const int d = s->d;
  if (s->i != d - 1 || s->msg_ready || s->resident_pending)
    return fail(BF_ERR_ARG, "a device-transcript open starts before the first round");
  if (ch.in.size() > (size_t)bf::kTrMax || ch.out.size() > 32)
    return fail(BF_ERR_ARG, "transcript state too large for the device (%zu input bytes)", ch.in.size());
  const size_t n_point = d > 0 ? d : 1;
  // Inputs go where no copy still in flight reads (the start's scalar and
  // point copies): scalars per round, then the OpenState image.
  uint8_t* in = s->pin->b() + s->tail_in_off();
  for (int i = 0; i < d; ++i) {
    bfh::store(in + 48 * i, s->r[i]);
    bfh::store(in + 48 * i + 16, s->r_inv[i]);
    bfh::store(in + 48 * i + 32, s->corr[i]);
  }
  bf::OpenState img;
  std::memset(&img, 0, sizeof(img));
  if (!ch.in.empty()) std::memcpy(img.tr.in, ch.in.data(), ch.in.size());
  if (!ch.out.empty()) std::memcpy(img.tr.out, ch.out.data(), ch.out.size());
  img.tr.in_len = (int)ch.in.size();
  img.tr.out_len = (int)ch.out.size();
  img.outer = to_uint4(s->outer_val);
  img.delta = to_uint4(bfh::one());
  std::memcpy(in + 48 * n_point, &img, sizeof(img));
  return BF_OK;
}

// Device side: every round of `s` and the final polynomial with the
// transcript on the device, from the staging; root_dev / value_dev, when
// given, are observed first (the commitment root and the evaluation on the
// device, the value becoming the claim).  Results are copied to the pinned
// staging; no event is recorded.
int open_resident_enqueue_device(bf_open_session* s, const uint4* root_dev, const uint4* value_dev) {
  bf_pcs* p = s->p;
  const int d = s->d;
  const size_t n_point = d > 0 ? d : 1;
  const uint8_t* in = s->pin->b() + s->tail_in_off();
  cudaStream_t st = s->st;
  if (d > 0) CU(cudaMemcpyAsync(s->w_tail, in, 48 * (size_t)d, cudaMemcpyHostToDevice, st));
  CU(cudaMemcpyAsync(s->w_state, in + 48 * n_point, sizeof(bf::OpenState), cudaMemcpyHostToDevice, st));
  if (root_dev || value_dev) CU(bf::launch_open_observe(s->w_state, root_dev, value_dev, st));
  const uint4* scal = reinterpret_cast<const uint4*>(s->w_tail);
  const uint4* xp = &s->w_state->x;
  const int i_tail = d > 0 ? tail_first_round(p, d) : -1;
  for (int i = d - 1; i > i_tail; --i) {  // large rounds: one kernel per step
    const uint4* root_i = (i == d - 1) ? s->first_root_dev() : reinterpret_cast<const uint4*>(s->stage(i));
    {
      ProfScope ps(p->prof, st, P_TRANSCRIPT);
      CU(bf::launch_open_round(s->w_state, i, d, scal, root_i, reinterpret_cast<const uint4*>(s->stage(i) + 32),
                               s->w_rec + 64 * (size_t)(d - 1 - i), st));
    }
    {
      // fold (binary_reed_solomon.rs:88-96) + next leaves, and fix_last_var
      // (multilinear.rs:183-198) + next reduction, in one launch
      ProfScope ps(p->prof, st, P_FOLD);
      bf::FoldFixParams fp{};
      fp.pi = (i == d - 1) ? s->first_pi() : s->pi_fold_out(i + 1);
      fp.pi_out = s->pi_fold_out(i);
      fp.leaves = s->pi_tree(i - 1);
      fp.n_leaves = p->n_i(i) / 2;
      fp.tlo = p->tw_host.lo[d - 1 - i];
      fp.thi = p->tw_host.hi[d - 1 - i];
      fp.poly_in = (i == d - 1) ? s->first_poly() : s->w_poly;
      fp.poly_out = s->w_poly;
      fp.half = (size_t)1 << i;
      fp.heq = s->w_heq;
      fp.next_half = (size_t)1 << (i - 1);
      fp.acc = reinterpret_cast<uint32_t*>(s->stage(i - 1) + 32);
      fp.xp = xp;
      CU(bf::launch_fold_fix(fp, uint4{}, st));
    }
    {
      ProfScope ps(p->prof, st, P_TREE);
      CU(bf::launch_tree(s->pi_tree(i - 1), p->n_i(i - 1), st, reinterpret_cast<uint4*>(s->stage(i - 1)),
                         p->tune));
    }
  }
  bf::TailParams tp{};
  tp.i0 = i_tail;
  tp.d = d;
  tp.log2_c = p->log2_c;
  tp.pi_first = s->first_pi();
  tp.pi_fold = s->w_pi_fold;
  tp.pi_trees = s->w_pi_trees;
  tp.poly_first = s->first_poly();
  tp.poly = s->w_poly;
  tp.heq = s->w_heq;
  if (i_tail >= 0) {
    tp.root_i0 = (i_tail == d - 1) ? s->first_root_dev() : reinterpret_cast<const uint4*>(s->stage(i_tail));
    tp.S_i0 = reinterpret_cast<const uint4*>(s->stage(i_tail) + 32);
  }
  tp.scal = scal;
  tp.tw = p->tw_view.as<bf::TwiddleView>();
  tp.state = s->w_state;
  tp.result = s->w_rec + 64 * (size_t)(d - 1 - i_tail);
  {
    ProfScope ps(p->prof, st, P_TAIL);
    CU(bf::launch_open_tail(tp, st));
  }
  CU(cudaMemcpyAsync(s->res_pin, s->w_rec, rec_bytes(d), cudaMemcpyDeviceToHost, st));
  CU(cudaMemcpyAsync(s->res_pin + align16(rec_bytes(d)), s->w_state, sizeof(bf::OpenState), cudaMemcpyDeviceToHost,
                     st));
  return BF_OK;
}

// Enqueues every round of `s`, and the final polynomial, with the transcript
// on the device, starting from `ch` (see open_resident_prepare /
// open_resident_enqueue_device); nothing is read back until
// open_resident_complete.
int open_resident_enqueue(bf_open_session* s, const bfh::Challenger& ch, const uint4* root_dev,
                          const uint4* value_dev) {
  TRY(open_resident_prepare(s, ch));
  TRY(open_resident_enqueue_device(s, root_dev, value_dev));
  CU(cudaEventRecord(s->ev, s->st));
  s->pending = true;
  s->resident_pending = true;
  s->msg_ready = false;
  return BF_OK;
}

// Reads the device-transcript open: the rounds' roots and compressed round
// polynomials, the final polynomial, and the transcript state (into `ch`).
int open_resident_complete(bf_open_session* s, bfh::Challenger& ch) {
  if (!s->resident_pending) return fail(BF_ERR_ARG, "no device-transcript open in flight");
  CU(cudaStreamSynchronize(s->st));
  s->p->prof.drain();
  s->pending = false;
  s->resident_pending = false;
  const int d = s->d;
  const uint8_t* res = s->res_pin;
  bf::OpenState img;
  std::memcpy(&img, res + align16(rec_bytes(d)), sizeof(img));
  if (img.status & 1) return fail(BF_ERR_ARG, "transcript input outgrew the device buffer");
  if (img.status & 2)
    return fail(BF_ERR_CHECK, "self-check failed: the last folded codeword is not encode0(final polynomial)");
  for (int k = 0; k < d; ++k) {
    const uint8_t* rec = res + 64 * (size_t)k;
    s->roots.insert(s->roots.end(), rec, rec + 32);
    put_u64(s->rounds, 2);
    s->rounds.insert(s->rounds.end(), rec + 32, rec + 64);
  }
  s->final_val = bfh::load(res + 64 * (size_t)d);
  ch.in.assign(img.tr.in, img.tr.in + img.tr.in_len);
  ch.out.assign(img.tr.out, img.tr.out + img.tr.out_len);
  s->i = -1;
  s->final_ready = true;
  return BF_OK;
}

// Gather of the openings at `indices` (basefold.rs:204-221) and their copy
// to the host; open_finish_complete waits and writes the proof.
int open_finish_enqueue(bf_open_session* s, const uint64_t* indices, size_t nq) {
  bf_pcs* p = s->p;
  if (s->i >= 0) return fail(BF_ERR_ARG, "rounds remain");
  if (nq != p->Q) return fail(BF_ERR_ARG, "expected %zu query indices, got %zu", p->Q, nq);
  if (nq && !indices) return fail(BF_ERR_ARG, "null argument");
  TRY(ensure_message(s));
  const size_t bb = p->block_bytes(s->w);
  for (size_t q = 0; q < nq; ++q) {
    if (indices[q] >= p->n_d()) return fail(BF_ERR_ARG, "query index %llu out of range", (unsigned long long)indices[q]);
    s->idx_pin[q] = indices[q];
  }
  cudaStream_t st = s->st;
  if (nq) {
    CU(cudaMemcpyAsync(s->w_idx, s->idx_pin, 8 * nq, cudaMemcpyHostToDevice, st));
    bf::GatherParams gp{};
    gp.cw = s->cm->cw.as<uint4>();
    gp.cw_tree = s->cm->tree.as<uint4>();
    gp.pi_first = s->first_pi();
    gp.pi_first_tree = s->first_tree();
    gp.pi_fold = s->w_pi_fold;
    gp.pi_trees = s->w_pi_trees;
    gp.idx = s->w_idx;
    gp.out = s->w_open;
    gp.width = s->w;
    gp.block_bytes = bb;
    gp.L = p->L;
    gp.d = s->d;
    gp.log2_c = p->log2_c;
    gp.nq = (int)nq;
    {
      ProfScope ps(p->prof, st, P_GATHER);
      CU(bf::launch_gather(gp, st));
    }
    CU(cudaMemcpyAsync(s->open_pin, s->w_open, bb * nq, cudaMemcpyDeviceToHost, st));
  }
  CU(cudaEventRecord(s->ev, st));
  s->pending = true;
  s->gather_pending = true;
  return BF_OK;
}

// BasefoldProof bincode (basefold.rs:49-66): round polys, final poly,
// pi_comms, openings.
int open_finish_complete(bf_open_session* s, uint8_t* proof, size_t cap, size_t* proof_len) {
  bf_pcs* p = s->p;
  if (!s->gather_pending) return fail(BF_ERR_ARG, "no openings in flight");
  const size_t need = bf_pcs_proof_size(p, s->w, 1);
  *proof_len = need;
  if (!proof || cap < need) return fail(BF_ERR_BUFFER, "proof buffer needs %zu bytes", need);
  CU(cudaStreamSynchronize(s->st));
  p->prof.drain();
  s->pending = false;
  s->gather_pending = false;
  const size_t nq = p->Q, bb = p->block_bytes(s->w);
  uint8_t* o = proof;
  std::memcpy(o, s->rounds.data(), s->rounds.size());
  o += s->rounds.size();
  std::vector<uint8_t> fin;
  put_u64(fin, 1);
  put_elem(fin, s->final_val);
  std::memcpy(o, fin.data(), fin.size());
  o += fin.size();
  std::memcpy(o, s->roots.data(), s->roots.size());
  o += s->roots.size();
  std::vector<uint8_t> qn;
  put_u64(qn, nq);
  std::memcpy(o, qn.data(), 8);
  o += 8;
  if (nq) std::memcpy(o, s->open_pin, bb * nq);
  o += bb * nq;
  if ((size_t)(o - proof) != need) return fail(BF_ERR_CUDA, "internal: proof size mismatch");
  return BF_OK;
}

}  // namespace bfapi

extern "C" {

int bf_open_start(bf_pcs* p, const bf_commitment* cm, const uint8_t* point, const uint8_t* values,
                  const uint8_t* scalars, void* stream, bf_open_session** out) {
  if (!values) return fail(BF_ERR_ARG, "null argument");
  return open_start_impl(p, cm, point, values, scalars, stream, out);
}

}  // extern "C"

namespace bfapi {

// A session for `cm` on `stream` with its device workspace and pinned
// staging; no device work.
int open_session_create(bf_pcs* p, const bf_commitment* cm, void* stream, bf_open_session** out) {
  if (!p || !cm || !out) return fail(BF_ERR_ARG, "null argument");
  *out = nullptr;
  if (p->device < 0) return fail(BF_ERR_ARG, "verifier-only pcs (device < 0)");
  if (cm->pcs != p) return fail(BF_ERR_ARG, "commitment belongs to another pcs");
  DeviceGuard g(p->device);
  std::unique_ptr<bf_open_session> s(new bf_open_session());
  s->p = p;
  s->cm = cm;
  s->w = cm->width;
  s->st = stream ? reinterpret_cast<cudaStream_t>(stream) : p->stream;
  CU(cudaEventCreateWithFlags(&s->ev, cudaEventDisableTiming));
  s->d = p->d;
  s->i = s->d - 1;
  TRY(session_alloc(s.get()));
  pcs_acquire(p);
  *out = s.release();
  return BF_OK;
}

// Host side of starting an open at `point`: the round scalars and the claim,
// the point (and the eq scalars) written to the session's pinned staging,
// the rounds reset.  `values` may be null when the evaluation will be
// observed on the device (width 1).
int open_session_prepare(bf_open_session* s, const uint8_t* point, const uint8_t* values, const uint8_t* scalars) {
  const int d = s->d;
  const size_t w = s->w;
  if (d > 0 && !point) return fail(BF_ERR_ARG, "null argument");
  if (!values && w != 1) return fail(BF_ERR_ARG, "null argument");
  if (w > 1 && !scalars) return fail(BF_ERR_ARG, "width > 1 needs the eq scalars");
  if (s->pending) return fail(BF_ERR_ARG, "session busy");
  const u128 ONE = bfh::one();
  s->i = d - 1;
  s->msg_ready = s->final_ready = s->resident_pending = s->gather_pending = false;
  s->r.assign(d, 0);
  for (int k = 0; k < d; ++k) s->r[k] = bfh::load(point + 16 * k);
  if (w == 1) {
    s->outer_val = values ? bfh::load(values) : 0;
  } else {  // claim = <scalars, values> (basefold.rs:176)
    u128 claim = 0;
    for (size_t c = 0; c < w; ++c) claim ^= bfh::mul(bfh::load(scalars + 16 * c), bfh::load(values + 16 * c));
    s->outer_val = claim;
  }
  s->inner_val = 0;
  s->delta_prod = ONE;
  // EvalImpr::new / HalfEq::new (eval_impr.rs:20-27, 69-79)
  if (!bfh::batch_inverse(s->r, s->r_inv)) return fail(BF_ERR_NOT_INVERTIBLE, "point has a zero coordinate");
  std::vector<u128> omr, omr_inv;
  for (int k = 0; k + 1 < d; ++k) omr.push_back(ONE ^ s->r[k]);
  if (!bfh::batch_inverse(omr, omr_inv)) return fail(BF_ERR_NOT_INVERTIBLE, "point has a coordinate equal to one");
  // correcting_factor(i) = prod_{i <= k < d-1} (1 - r_k)^-1 (eval_impr.rs:83-90)
  s->corr.assign(d > 0 ? d : 1, ONE);
  for (int i = d - 2; i >= 0; --i) s->corr[i] = bfh::mul(s->corr[i + 1], omr_inv[i]);
  s->rounds.clear();
  s->roots.clear();
  put_u64(s->rounds, (uint64_t)d);
  put_u64(s->roots, (uint64_t)d);
  uint8_t* pin = s->pin->b();
  if (w > 1) std::memcpy(pin + 64, scalars, 16 * w);
  if (d > 0) std::memcpy(pin + 64 + 16 * w, point, 16 * (size_t)d);
  return BF_OK;
}

// Device side of the start, from the staging: row combination and the first
// round's tree (width > 1), the point, the half-eq table and the first
// round's reduction.  No event is recorded.
int open_session_enqueue_start(bf_open_session* s) {
  bf_pcs* p = s->p;
  const bf_commitment* cm = s->cm;
  const int d = s->d;
  const size_t w = s->w;
  uint8_t* pin = s->pin->b();
  cudaStream_t st = s->st;
  if (w > 1) {  // combine rows with the eq scalars (basefold.rs:166-183)
    CU(cudaMemcpyAsync(s->w_scalars, pin + 64, 16 * w, cudaMemcpyHostToDevice, st));
    {
      ProfScope ps(p->prof, st, P_FIX);
      CU(bf::launch_combine_rows(cm->data.as<uint4>(), (size_t)1 << d, w, s->w_scalars, s->w_poly_first, st));
    }
    // The reference combines the codeword's rows the same way; the code is
    // linear over the field, so that combination is the encoding of the
    // combined polynomial: one width-1 encode of 2^d elements instead of
    // w products per codeword row, the same values.
    ProfScope ps(p->prof, st, P_ENCODE);
    const cudaError_t e = bf::launch_encode(s->w_poly_first, s->w_pi_first, d, p->log2_c, 1,
                                            p->tw_view.as<bf::TwiddleView>(), st, nullptr, nullptr, p->tune);
    if (e != cudaSuccess) return fail(BF_ERR_CUDA, "encode of the combined polynomial: %s", cudaGetErrorString(e));
  }
  if (d == 0) {
    CU(cudaMemcpyAsync(pin, s->first_poly(), 16, cudaMemcpyDeviceToHost, st));
    return BF_OK;
  }
  if (w > 1) {  // the first round's tree over the combined codeword pairs
    ProfScope ps(p->prof, st, P_TREE);
    const size_t n1 = p->n_i(d - 1);
    CU(bf::launch_leaves_pair(s->w_pi_first, s->w_pi_first_tree, n1, st));
    CU(bf::launch_tree(s->w_pi_first_tree, n1, st, reinterpret_cast<uint4*>(s->stage(d - 1)), p->tune));
  }
  CU(cudaMemcpyAsync(s->w_point, pin + 64 + 16 * w, 16 * (size_t)d, cudaMemcpyHostToDevice, st));
  CU(cudaMemsetAsync(s->stage(d - 1) + 32, 0, 16, st));
  if (d >= 2) CU(cudaMemsetAsync(s->w_stage, 0, 48 * (size_t)(d - 1), st));
  {
    ProfScope ps(p->prof, st, P_EQ);
    CU(bf::launch_eq_table(s->w_point, d - 1, s->w_heq, s->w_eq_lo, s->w_eq_hi, st));
  }
  {
    ProfScope ps(p->prof, st, P_FIX);
    CU(bf::launch_dot_xor(s->w_heq, s->first_poly(), (size_t)1 << (d - 1),
                          reinterpret_cast<uint32_t*>(s->stage(d - 1) + 32), st));
  }
  CU(cudaMemcpyAsync(pin, s->stage(d - 1), 48, cudaMemcpyDeviceToHost, st));
  return BF_OK;
}

const uint4* open_session_point_dev(const bf_open_session* s) { return s->w_point; }

void open_session_mark_launched(bf_open_session* s) {
  s->pending = true;
  s->resident_pending = true;
}

cudaStream_t open_session_stream(const bf_open_session* s) { return s->st; }
void open_session_set_stream(bf_open_session* s, cudaStream_t st) { s->st = st; }
cudaEvent_t open_session_event(const bf_open_session* s) { return s->ev; }

// bf_open_start; `values` may be null when a device-transcript open will
// observe the evaluation on the device (width 1).
int open_start_impl(bf_pcs* p, const bf_commitment* cm, const uint8_t* point, const uint8_t* values,
                    const uint8_t* scalars, void* stream, bf_open_session** out) {
  if (!p || !cm || !out || (p->d > 0 && !point)) return fail(BF_ERR_ARG, "null argument");
  if (!values && cm->width != 1) return fail(BF_ERR_ARG, "null argument");
  if (cm->width > 1 && !scalars) return fail(BF_ERR_ARG, "width > 1 needs the eq scalars");
  *out = nullptr;
  bf_open_session* raw = nullptr;
  TRY(open_session_create(p, cm, stream, &raw));
  std::unique_ptr<bf_open_session> s(raw);
  DeviceGuard g(p->device);
  TRY(open_session_prepare(s.get(), point, values, scalars));
  TRY(open_session_enqueue_start(s.get()));
  CU(cudaEventRecord(s->ev, s->st));
  s->pending = true;
  *out = s.release();
  return BF_OK;
}

}  // namespace bfapi

extern "C" {

int bf_open_poll(bf_open_session* s) {
  if (!s) return fail(BF_ERR_ARG, "null argument");
  if (!s->pending) return 1;
  cudaError_t e = cudaEventQuery(s->ev);
  if (e == cudaSuccess) return 1;
  if (e == cudaErrorNotReady) return 0;
  CU(e);
  return 0;
}

int bf_open_round(bf_open_session* s, int* round, uint8_t pi_root[32], uint8_t round_poly[32]) {
  if (!s || !round) return fail(BF_ERR_ARG, "null argument");
  DeviceGuard g(s->p->device);
  TRY(ensure_message(s));
  *round = s->i;
  if (s->i < 0) return BF_OK;
  if (pi_root) std::memcpy(pi_root, s->root, 32);
  if (round_poly) {  // compressed [c0, c2] (eval.rs:64-66)
    bfh::store(round_poly, s->rp[0]);
    bfh::store(round_poly + 16, s->rp[2]);
  }
  return BF_OK;
}

int bf_open_challenge(bf_open_session* s, const uint8_t r_i[16]) {
  if (!s || !r_i) return fail(BF_ERR_ARG, "null argument");
  DeviceGuard g(s->p->device);
  TRY(ensure_message(s));
  if (s->i < 0) return fail(BF_ERR_ARG, "every round is done");
  bf_pcs* p = s->p;
  const int i = s->i, d = s->d;
  const u128 ONE = bfh::one();
  s->roots.insert(s->roots.end(), s->root, s->root + 32);
  put_u64(s->rounds, 2);
  put_elem(s->rounds, s->rp[0]);
  put_elem(s->rounds, s->rp[2]);
  const u128 x = bfh::load(r_i);
  s->inner_val = horner(s->c01, 2, x);  // EvalProver::fix_last_var (eval.rs:108-111)
  s->outer_val = horner(s->rp, 3, x);   // SumcheckSubclaim::reduce (sumcheck/src/lib.rs:41-47)
  s->delta_prod = bfh::mul(s->delta_prod, ONE ^ s->r[i] ^ x);
  const uint4 xr = to_uint4(x);
  cudaStream_t st = s->st;
  // fold (binary_reed_solomon.rs:88-96) with the stage d-1-i twiddles,
  // fused with the leaves of the next round's tree
  const size_t ni = p->n_i(i);
  const uint4* pi_in = (i == d - 1) ? s->first_pi() : s->pi_fold_out(i + 1);
  const uint4* tlo = p->tw_host.lo[d - 1 - i];
  const uint4* thi = p->tw_host.hi[d - 1 - i];
  {
    ProfScope ps(p->prof, st, P_FOLD);
    if (i > 0)
      CU(bf::launch_fold_leaves(pi_in, s->pi_fold_out(i), s->pi_tree(i - 1), ni / 2, tlo, thi, xr, st));
    else
      CU(bf::launch_fold(pi_in, s->pi_fold_out(i), ni, tlo, thi, xr, st));
  }
  // fix_last_var (multilinear.rs:183-198) + next round's reduction
  const uint4* poly_in = (i == d - 1) ? s->first_poly() : s->w_poly;
  {
    ProfScope ps(p->prof, st, P_FIX);
    CU(bf::launch_fix(poly_in, s->w_poly, (size_t)1 << i, xr, s->w_heq, i > 0 ? ((size_t)1 << (i - 1)) : 0,
                      i > 0 ? reinterpret_cast<uint32_t*>(s->stage(i - 1) + 32) : nullptr, st));
  }
  uint8_t* pin = s->pin->b();
  if (i > 0) {
    {
      ProfScope ps(p->prof, st, P_TREE);
      CU(bf::launch_tree(s->pi_tree(i - 1), p->n_i(i - 1), st, reinterpret_cast<uint4*>(s->stage(i - 1)),
                         p->tune));
    }
    CU(cudaMemcpyAsync(pin, s->stage(i - 1), 48, cudaMemcpyDeviceToHost, st));
  } else {
    CU(cudaMemcpyAsync(pin, s->w_poly, 16, cudaMemcpyDeviceToHost, st));
  }
  CU(cudaEventRecord(s->ev, st));
  s->pending = true;
  s->msg_ready = false;
  s->i -= 1;
  return BF_OK;
}

int bf_open_final(bf_open_session* s, uint8_t final_poly[16]) {
  if (!s || !final_poly) return fail(BF_ERR_ARG, "null argument");
  if (s->i >= 0) return fail(BF_ERR_ARG, "rounds remain");
  DeviceGuard g(s->p->device);
  TRY(ensure_message(s));
  bfh::store(final_poly, s->final_val);
  return BF_OK;
}

int bf_open_finish(bf_open_session* s, const uint64_t* indices, size_t nq, uint8_t* proof, size_t cap,
                   size_t* proof_len) {
  if (!s || !proof_len || (nq && !indices)) return fail(BF_ERR_ARG, "null argument");
  bf_pcs* p = s->p;
  if (s->i >= 0) return fail(BF_ERR_ARG, "rounds remain");
  if (nq != p->Q) return fail(BF_ERR_ARG, "expected %zu query indices, got %zu", p->Q, nq);
  const size_t need = bf_pcs_proof_size(p, s->w, 1);
  *proof_len = need;
  if (!proof || cap < need) return fail(BF_ERR_BUFFER, "proof buffer needs %zu bytes", need);
  DeviceGuard g(p->device);
  TRY(open_finish_enqueue(s, indices, nq));
  return open_finish_complete(s, proof, cap, proof_len);
}

void bf_open_session_free(bf_open_session* s) {
  if (!s) return;
  bf_pcs* p = s->p;
  {
    DeviceGuard g(p->device);
    delete s;
  }
  pcs_release(p);
}

// Whole open with this library's transcript (basefold.rs:133-232).
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
  bfh::Challenger& ch = chp->c;
  std::vector<uint8_t> scal;
  if (cm->width > 1) {  // sample_random_scalars_by_eq (basefold.rs:166-167,398-408)
    std::vector<u128> sc = sample_scalars_by_eq(cm->width, ch);
    scal.resize(16 * sc.size());
    for (size_t c = 0; c < sc.size(); ++c) bfh::store(scal.data() + 16 * c, sc[c]);
  }
  bf_open_session* s = nullptr;
  TRY(bf_open_start(p, cm, point, values, scal.empty() ? nullptr : scal.data(), nullptr, &s));
  std::unique_ptr<bf_open_session, void (*)(bf_open_session*)> guard(s, bf_open_session_free);
  // every round and the final polynomial with the transcript on the device
  // (basefold.rs:185-196, 335-369), then the queries on the host; a pending
  // transcript input too long for the device buffer drives the rounds from
  // the host instead (same kernels)
  const bool fits = ch.in.size() + 64 <= (size_t)bf::kTrMax && ch.out.size() <= 32;
  if (fits) {
    TRY(open_resident_enqueue(s, ch, nullptr, nullptr));
    TRY(open_resident_complete(s, ch));
  } else {
    while (true) {
      int round;
      uint8_t root[32], poly[32];
      TRY(bf_open_round(s, &round, root, poly));
      if (round < 0) break;
      ch.observe(root, 32);  // basefold.rs:356
      ch.observe(poly, 32);  // sumcheck/src/lib.rs:97
      uint8_t r[16];
      bfh::store(r, ch.sample_elem());
      TRY(bf_open_challenge(s, r));
    }
    uint8_t fin[16];
    TRY(bf_open_final(s, fin));
    ch.observe(fin, 16);  // basefold.rs:196
  }
  std::vector<uint64_t> idx(p->Q);
  for (size_t q = 0; q < p->Q; ++q) idx[q] = ch.sample_bits(p->L);  // basefold.rs:200-203
  size_t len = 0;
  TRY(bf_open_finish(s, idx.data(), idx.size(), proof, cap, &len));
  *proof_len = len;
  return BF_OK;
}

}  // extern "C"
