// Internal interface between the host orchestration (api.cu) and the
// kernels (kernels.cu).  Not part of the public C ABI.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>

namespace bf {

constexpr int kMaxStages = 32;
constexpr int kTwLoBits = 12;  // twiddle(s, K) = lo_s[K & 4095] ^ hi_s[K >> 12]

// Per-stage views of the additive-NTT twiddle tables.  Stage s of
// AddtiveNtt::new(L) (p3/src/field/binary.rs:23-53) has 2^(L-1-s) entries,
// entry K being the XOR of the stage's basis values selected by the bits of K.
// That map is GF(2)-linear in K, so a twiddle is the XOR of one entry of a
// table over the low 12 bits and one of a table over the remaining bits.
struct TwiddleView {
  const uint4* lo[kMaxStages];
  const uint4* hi[kMaxStages];
};

// Launch shapes and thresholds, chosen per (num_vars, blowup) by the
// autotuner (bf_pcs_autotune) or left at these defaults.
constexpr int kNttMaxT = 12;  // largest shared-memory tile of an NTT pass: 2^12 elements
struct Tune {
  int ntt_threads = 256;  // threads per block of the shared-memory NTT pass: 128, 256 or 512
  int ntt_max_T = 12;     // butterfly layers per NTT pass (tile 2^T), 6 .. kNttMaxT
  int top_nodes = 512;    // Merkle levels at or below this many nodes run in one block (64 .. 4096)
  int tail_log = 8;       // open rounds whose next tree has <= 2^tail_log leaves run in one block (1 .. 11)
  int subtree_log = 16;   // Merkle levels of 2^10 .. 2^subtree_log nodes run as one launch (10 .. 20)
  // NTT pass kind: 0 every pass layer by layer in shared memory; 1 tiles of
  // 2^9 .. 2^13 register-blocked; 2 as 0, with the last pass (and its leaf
  // hashing) warp-specialized; 3 as 0, two-pass encodes with the cosets
  // pipelined (the next cosets' first pass beside a coset's last pass)
  int ntt_kind = 2;
  int gf_mix = 0;        // NTT passes without hashing: 32 x 32 products per field product from 16-bit pieces (0 .. 4)
  int ntt_ws_warps = 8;  // warp-specialized last pass: butterfly warps of its 16 (2 .. 14; the rest hash)
};
constexpr int kTuneVals = 8;  // the Tune fields above, in order, as the C ABI's value vector
bool tune_valid(const Tune& t);

// Launchers (all asynchronous on `st`).
// `tw` points to a TwiddleView in device memory.  When `leaves` and
// `pair_leaves` are given (n >= 1), the last pass also writes the codeword
// leaves and the first folded-codeword leaves.
// With `slices` > 0, slice k of the input (rows [k N/slices, (k+1) N/slices))
// is ready once slice_ready[k] has completed: the first pass waits for each
// slice before the blocks that read it, its launches alternating between st
// and st2 (joined back to st through the events ev_a, ev_b) when those are
// given.  last_a / last_b (when given) are recorded on st around the last
// pass (the kernel-class timing of the last pass with its leaf hashing).
cudaError_t launch_encode(const uint4* m, uint4* cw, int n, int log2_c, size_t width, const TwiddleView* tw,
                          cudaStream_t st, uint4* leaves = nullptr, uint4* pair_leaves = nullptr,
                          const Tune& tune = Tune(), const cudaEvent_t* slice_ready = nullptr,
                          int slices = 0, cudaStream_t st2 = nullptr, cudaEvent_t ev_a = nullptr,
                          cudaEvent_t ev_b = nullptr, cudaEvent_t last_a = nullptr, cudaEvent_t last_b = nullptr);
cudaError_t launch_leaves_elem(const uint4* cw, uint4* leaves, size_t n, size_t width, cudaStream_t st);
cudaError_t launch_leaves_pair(const uint4* pi, uint4* leaves, size_t n, cudaStream_t st);
// Build every level above `leaves` (n leaves, power of two); levels are stored
// one after another right after the leaves.  Root = last digest, also copied
// to `root_out` (32 bytes) when it is not null.
cudaError_t launch_tree(uint4* leaves, size_t n, cudaStream_t st, uint4* root_out = nullptr,
                        const Tune& tune = Tune());
// SplitMix64 words as field elements (autotuner inputs).
cudaError_t launch_fill_random(uint4* out, size_t n, uint64_t seed, cudaStream_t st);

cudaError_t launch_eq_table(const uint4* r, int nvars, uint4* out, uint4* tmp_lo, uint4* tmp_hi, cudaStream_t st);
cudaError_t launch_dot_xor(const uint4* x, const uint4* y, size_t n, uint32_t* acc, cudaStream_t st);
// The fold and fix challenge is `r`, or *xp when xp is not null (a challenge
// sampled on the device).
cudaError_t launch_fold(const uint4* pi, uint4* out, size_t n_out, const uint4* tw_lo, const uint4* tw_hi, uint4 r,
                        cudaStream_t st, const uint4* xp = nullptr);
cudaError_t launch_fold_leaves(const uint4* pi, uint4* out, uint4* leaves, size_t n_leaves, const uint4* tw_lo,
                               const uint4* tw_hi, uint4 r, cudaStream_t st, const uint4* xp = nullptr);
cudaError_t launch_fix(const uint4* in, uint4* out, size_t half, uint4 r, const uint4* heq, size_t next_half,
                       uint32_t* acc, cudaStream_t st, const uint4* xp = nullptr);
cudaError_t launch_fix_column(const uint4* in, size_t width, size_t col, uint4* out, size_t half, uint4 r,
                              cudaStream_t st, const uint4* xp = nullptr);
// A round of open (i >= 1) in one launch: the fold of `pi` into `pi_out`
// with the next round's leaves (launch_fold_leaves) and the fix of
// `poly_in` into `poly_out` with the next round's reduction into `acc`
// (launch_fix).  The challenge is *xp when xp is set, else r.
struct FoldFixParams {
  const uint4* pi;
  uint4* pi_out;
  uint4* leaves;
  size_t n_leaves;
  const uint4* tlo;
  const uint4* thi;
  const uint4* poly_in;
  uint4* poly_out;
  size_t half;
  const uint4* heq;
  size_t next_half;
  uint32_t* acc;
  const uint4* xp;
  unsigned fold_blocks, fix_blocks, fix_stride;  // set by the launcher
};
cudaError_t launch_fold_fix(const FoldFixParams& p, uint4 r, cudaStream_t st);
cudaError_t launch_combine_rows(const uint4* rows, size_t nrows, size_t width, const uint4* scalars, uint4* out,
                                cudaStream_t st);
// acc[4 c .. 4 c + 3] ^= sum_r eq[r] * data[r w + c] for every column c < w.
cudaError_t launch_eval_cols(const uint4* eq, const uint4* data, size_t rows, size_t w, uint32_t* acc,
                             cudaStream_t st);
constexpr int kEqTableMaxVars = 28;  // launch_eq_table: up to 12 + 16 variables
// The last `nvars` (<= kEvalTailMaxVars) fixes of MultiPoly::evaluate in one
// block, in place on buf[0 .. 2^nvars): variable k is fixed with r[k] (or
// rp[k] in device memory when rp is not null), top first; the value lands in
// buf[0].
constexpr int kEvalTailMaxVars = 12;
struct EvalTail {
  uint4 r[kEvalTailMaxVars];
  const uint4* rp;
  int nvars;
};
cudaError_t launch_eval_tail(uint4* buf, const EvalTail& p, cudaStream_t st);

// Gather of the query openings, written in the proof's bincode layout.
struct GatherParams {
  const uint4* cw;         // codeword, NTT order, rows of `width`
  const uint4* cw_tree;    // codeword tree, reversed storage per level
  const uint4* pi_first;       // folded codeword of the first round (= cw when width is 1)
  const uint4* pi_first_tree;  // its tree
  const uint4* pi_fold;        // outputs of the folds of rounds d-1 .. 0, one after another
  const uint4* pi_trees;       // trees of rounds d-2 .. 0, one after another
  const uint64_t* idx;     // query positions
  uint8_t* out;            // Q blocks of `block_bytes`
  size_t width;
  size_t block_bytes;
  int L;        // log2 n_d
  int d;        // rounds
  int log2_c;
  int nq;
};
cudaError_t launch_gather(const GatherParams& p, cudaStream_t st);

// Standalone product sumcheck.
cudaError_t launch_prod_round_sums(const uint4* const* polys, int k, size_t half, uint32_t* acc, cudaStream_t st);
cudaError_t launch_prod_fix(uint4* const* out, const uint4* const* in, int k, size_t half, uint4 r,
                            size_t next_half, uint32_t* acc, cudaStream_t st, const uint4* xp = nullptr);

unsigned long long launches_total();
unsigned long long launches_this_thread();  // launched by the calling thread
void count_launch();
void add_launches(long long n);  // kernels run by a replayed CUDA graph (negative: captured, not run)
// Function attributes (dynamic shared memory) set once per device, outside
// any stream capture.
void init_kernel_attributes();

// ---- Fiat-Shamir on the device
// HashChallenger<u8, Keccak256Hash, 32> (p3/src/challenger.rs) as bytes: the
// pending input and the unread output of the last digest.
constexpr int kTrMax = 512;
struct alignas(16) DevTranscript {
  uint8_t in[kTrMax];
  uint8_t out[32];
  int in_len, out_len, pad_[2];
};
// Device-resident state of one open (basefold.rs:133-232): the transcript,
// the claim of the first sumcheck round (`outer`, the evaluation), the
// EvalProver claim of the later rounds (`inner`), the product of delta
// scalars (eval_impr.rs:45-51) and the last challenge.  status bit 0: the
// transcript input outgrew kTrMax; bit 1: the last folded codeword is not
// encode0 of the final polynomial (basefold.rs:198).
struct alignas(16) OpenState {
  DevTranscript tr;
  uint4 outer, inner, delta, x;
  int status, pad_[3];
};
// Observes the commitment root (32 bytes at `root`) and the evaluation
// (16 bytes at `value`, which also becomes the claim), as the caller of open
// does (poly-commit/src/lib.rs:80-100).
cudaError_t launch_open_observe(OpenState* s, const uint4* root, const uint4* value, cudaStream_t st);
// The transcript step of round i: round polynomial from the reduction
// S = sum half_eq * poly_lo (eval_impr.rs:116-127, eval.rs:89-106), observe
// root and [c0, c2], sample the challenge into s->x.  `rec` receives root,
// c0, c2 (64 bytes).  `scal` holds r_i, r_i^-1, correcting factor per round.
cudaError_t launch_open_round(OpenState* s, int i, int d, const uint4* scal, const uint4* root, const uint4* S,
                              uint8_t* rec, cudaStream_t st);
// One round of the product sumcheck's transcript on the device (warp):
// from the sums acc = [c0, c2, c3] (sumcheck/src/function/quadratic.rs
// 116-127 for k = 2; its k = 3 extension), observe the compressed round
// polynomial, sample the challenge into s->x, and advance the claim
// s->outer to the round polynomial at x (lib.rs:95-103).  `rec` receives
// the compressed polynomial (16 k bytes) and the challenge (16 bytes).
cudaError_t launch_sumcheck_round(OpenState* s, int k, const uint32_t* acc, uint8_t* rec, cudaStream_t st);

// ---- the last rounds of open in one block, then the final polynomial
constexpr int kTailThreads = 256;
constexpr int kTailMaxLeavesLog = 11;    // largest Tune::tail_log
struct TailParams {
  int i0, d, log2_c;        // rounds i0 .. 0 (i0 = -1: none)
  const uint4* pi_first;    // folded codeword input of round d-1
  uint4* pi_fold;           // fold outputs of rounds d-1 .. 0
  uint4* pi_trees;          // trees of rounds d-2 .. 0
  const uint4* poly_first;  // sumcheck polynomial of round d-1
  uint4* poly;              // sumcheck polynomial after each fix (in place)
  const uint4* heq;         // half eq table
  const uint4* root_i0;     // root of round i0's tree (32 B)
  const uint4* S_i0;        // reduction of round i0 (16 B)
  const uint4* scal;        // per round i: r_i, r_i^-1, correcting factor
  const TwiddleView* tw;
  OpenState* state;
  uint8_t* result;          // per round: root, c0, c2 (64 B); then the final polynomial (16 B)
};
cudaError_t launch_open_tail(const TailParams& p, cudaStream_t st);

// ---- Basefold::verify of many proofs (basefold.rs:284-320) on the device.
// Offsets are byte offsets into `blob`, multiples of 8.  All proofs share one
// pcs (num_vars d, blowup 2^log2_c) and are checked query by query.
struct VerifyJob {
  uint64_t root;        // 32-byte commitment
  uint64_t pi_comms;    // the proof's d folded-codeword roots, 32 bytes apart
  uint64_t final_poly;  // the proof's final polynomial (one element)
  uint64_t challenges;  // round challenges in round order (16 bytes each)
  uint64_t scalars;     // width > 1: the eq scalars of the columns
  uint32_t width;
  uint32_t pad;
};
constexpr uint32_t kVerifyInactive = 0xffffffffu;  // a query slot with nothing to check
struct VerifyQuery {
  uint32_t job;     // kVerifyInactive: an unused slot
  uint32_t pad;
  uint64_t idx;     // sampled position in the codeword
  uint64_t leaves;  // the opened row (16*width bytes)
  uint64_t path;    // its L sibling digests
};
struct VerifyRound {
  uint64_t sibling;  // the opened sibling element of round k
  uint64_t path;     // its log2 n_i sibling digests
};
struct VerifyParams {
  const uint8_t* blob;
  const VerifyJob* jobs;
  const VerifyQuery* queries;  // nq
  const VerifyRound* rounds;   // nq * d, query-major
  const TwiddleView* tw;
  uint4* pairs;                // nq * d * 2 elements (scratch)
  uint8_t* final_bad;          // nq: fold chain != final polynomial
  uint8_t* path_bad;           // (d + 1) * nq, level-major: level 0 = codeword path, 1 + k = round k
  uint32_t nq;
  int d, log2_c;
};
cudaError_t launch_verify(const VerifyParams& p, cudaStream_t st);

// Test hooks.
cudaError_t launch_test_mul(const uint4* a, const uint4* b, uint4* out, size_t n, cudaStream_t st);
cudaError_t launch_test_keccak(uint2* states, size_t n, cudaStream_t st);

}  // namespace bf
