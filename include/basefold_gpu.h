/*
 * basefold_gpu.h — C ABI of the GB300 Basefold prover (libbasefold_gpu.so).
 *
 * Drop-in boundary for the Basefold polynomial commitment of han0110/learn-zkp
 * instantiated as
 *   Basefold<Polyval, Polyval, BinaryReedSolomonCode<Polyval>,
 *            Keccak256MerkleTreeMmcs<Polyval>>
 * behind its `PolyCommitScheme` trait (poly-commit/src/lib.rs:20-51) and the
 * standalone sumcheck prover (sumcheck/src/lib.rs:56-103).  The reference
 * exposes Rust traits, not an FFI; each entry point below names the trait
 * method or function it replaces, so a Rust crate can bind these symbols
 * with `extern "C"` declarations and implement the trait over them.
 *
 * Conventions
 *  - Field element: 16 bytes, the raw little-endian u128 that `Polyval`
 *    stores (Montgomery form, p3/src/polyval.rs:30-34), exactly the bytes
 *    bincode writes for it.
 *  - Digest / commitment: 32 bytes (Plonky3 `Hash<Polyval, u8, 32>`).
 *  - Evaluations: row-major, `width` columns (one multilinear polynomial per
 *    column, 2^num_vars rows) — the reference's `RowMajorMatrix<F>` Data
 *    (poly-commit/src/basefold.rs:96-97).  The engine (bf_engine_*) runs
 *    width 1 only.
 *  - Proofs: the bincode 1.3 bytes of `BasefoldProof` (basefold.rs:49-66).
 *  - Every call returns 0 on success or a negative BF_ERR_* code; the text of
 *    the last error on the calling thread is available from bf_last_error.
 *    bf_verify additionally returns the BF_VERIFY_* results.
 *  - A bf_pcs and everything made from it belong to one host thread at a
 *    time; all GPU work runs on the pcs's stream.
 *  - Free in any order: a freed bf_pcs lives on until its last commitment
 *    and open session are freed.
 */
#ifndef BASEFOLD_GPU_H
#define BASEFOLD_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BF_OK 0
#define BF_ERR_ARG (-1)          /* bad argument or size */
#define BF_ERR_CUDA (-2)         /* CUDA runtime failure */
#define BF_ERR_OOM (-3)          /* device or pinned allocation failed */
#define BF_ERR_BUFFER (-4)       /* caller buffer too small; required size returned */
#define BF_ERR_UNSUPPORTED (-5)  /* configuration this build does not run on the GPU */
#define BF_ERR_NOT_INVERTIBLE (-6) /* a point coordinate r with r = 0 or r = 1 */
#define BF_ERR_CHECK (-7)        /* a self-check of the prover failed (the reference's debug asserts) */
#define BF_ERR_CANCELLED (-8)    /* an engine job cancelled before it started */

#define BF_VERIFY_OK 0
#define BF_VERIFY_INVALID_FINAL_POLY 1 /* BasefoldError::InvalidFinalPoly (basefold.rs:79-84) */
#define BF_VERIFY_INVALID_QUERY 2      /* BasefoldError::InvalidQuery */
#define BF_VERIFY_MMCS 3               /* BasefoldError::Mmcs */
#define BF_VERIFY_MALFORMED 4          /* proof bytes do not parse */

typedef struct bf_pcs bf_pcs;
typedef struct bf_commitment bf_commitment;
typedef struct bf_challenger bf_challenger;
typedef struct bf_open_session bf_open_session;
typedef struct bf_engine bf_engine;

/* One commit + eval + open job of the engine (the reference harness,
 * poly-commit/src/lib.rs:80-100, with GenericChallenger::keccak256()). */
typedef struct {
  int32_t num_vars;      /* in: log2 of the number of evaluations */
  int32_t status;        /* out: 0 done, 1 pending, < 0 BF_ERR_* */
  const void* evals;     /* in: 2^num_vars elements (host or device memory) */
  const uint8_t* point;  /* in: num_vars elements, host memory */
  uint8_t* proof;        /* in: caller buffer for the bincode proof */
  size_t proof_cap;      /* in: its size (bf_engine_proof_size) */
  size_t proof_len;      /* out */
  double latency_ms;     /* out: submission to completion */
  uint8_t root[32];      /* out: commitment */
  uint8_t value[16];     /* out: evaluation at the point */
} bf_job;

/* Text of the last error on this thread (NUL-terminated, truncated to len). */
int bf_last_error(char* buf, size_t len);

/* Device facts: number of SMs and compute capability. */
int bf_device_info(int device, int* num_sms, int* cc_major, int* cc_minor);
/* Number of CUDA kernels this library has launched since it was loaded. */
int bf_kernel_launches(uint64_t* count);

/* ---- PolyCommitScheme::setup (poly-commit/src/lib.rs:29; basefold.rs:104-110)
 * with BinaryReedSolomonCode::new(lambda, log2_c, num_vars)
 * (binary_reed_solomon.rs:20-27).  Builds the additive-NTT twiddle tables of
 * AddtiveNtt::new(log2_c + num_vars) (p3/src/field/binary.rs:23-53) on the
 * device.  `stream` is a cudaStream_t to run on, or NULL for a private one.
 * device < 0 makes a verifier-only object that never touches a GPU (only
 * bf_verify, bf_pcs_num_queries and bf_pcs_proof_size accept it). */
int bf_pcs_setup(int device, int lambda, int log2_c, int num_vars, void* stream, bf_pcs** out);
void bf_pcs_free(bf_pcs* pcs);
/* RandomFoldableCode::num_queries (binary_reed_solomon.rs:56-59). */
size_t bf_pcs_num_queries(const bf_pcs* pcs);
/* Size in bytes of a proof for `width` columns and n_evals (0 or 1) points. */
size_t bf_pcs_proof_size(const bf_pcs* pcs, size_t width, int n_evals);

/* ---- PolyCommitScheme::commit (lib.rs:31; basefold.rs:112-120): encode
 * (binary_reed_solomon.rs:67-82) + Merkle commit of the codeword.
 * `evals` is host memory (2^num_vars * width elements, copied in). */
int bf_commit(bf_pcs* pcs, const uint8_t* evals, size_t width, bf_commitment** out, uint8_t root[32]);
/* Same, with `d_evals` already in device memory.  The commitment keeps a
 * reference to it (no copy): the buffer must outlive the commitment. */
int bf_commit_device(bf_pcs* pcs, const void* d_evals, size_t width, bf_commitment** out, uint8_t root[32]);
/* The commitment's device buffers return, in stream order, to a memory pool
 * owned by its pcs, which keeps them for the next commitments until the pcs
 * itself is freed (no cudaMalloc or cudaFree per commit). */
void bf_commitment_free(bf_commitment* comm);
/* AsRef<Commitment> of BasefoldCommitmentData (basefold.rs:37-47). */
int bf_commitment_root(const bf_commitment* comm, uint8_t root[32]);
/* PolyCommitScheme::data (lib.rs:33): copies the evaluations back to host. */
int bf_commitment_data(const bf_commitment* comm, uint8_t* evals, size_t cap);

/* ---- PolyCommitScheme::eval (lib.rs:35; basefold.rs:126-131): the value of
 * every column's multilinear extension at `point` (num_vars elements), on
 * the device-resident evaluations.  Writes `width` elements. */
int bf_eval(bf_pcs* pcs, const bf_commitment* comm, const uint8_t* point, uint8_t* values);
/* ---- PolyCommitScheme::eval(&self, data: &Data, point) (lib.rs:35;
 * basefold.rs:126-131 over MultiPoly::evaluate, p3/src/poly/multilinear.rs:
 * 124-141) for data that has no commitment: `evals` holds 2^num_vars rows of
 * `width` columns, in host memory (on_device 0: copied in on the pcs's
 * stream) or device memory (on_device 1: 16-byte aligned, not modified).
 * The evaluation runs on the GPU; writes `width` elements to `values`. */
int bf_eval_data(bf_pcs* pcs, const void* evals, int on_device, size_t width, const uint8_t* point,
                 uint8_t* values);

/* ---- PolyCommitScheme::open (lib.rs:37-42; basefold.rs:133-232).
 * n_evals is 0 (empty proof) or 1 (one PolyEvals: `point` of num_vars
 * elements, `values` of `width` elements).  `ch` is the caller's challenger
 * state, advanced in place (the reference takes it by value; pass a clone
 * to keep the original).  Writes the bincode proof; *proof_len receives its
 * size (also when BF_ERR_BUFFER is returned). */
int bf_open(bf_pcs* pcs, const bf_commitment* comm, const uint8_t* point, const uint8_t* values, int n_evals,
            bf_challenger* ch, uint8_t* proof, size_t cap, size_t* proof_len);

/* ---- PolyCommitScheme::open driven round by round by the caller's own
 * transcript (any FieldChallenger): the device computes each round's
 * folded-codeword Merkle root and compressed round polynomial [c0, c2]; the
 * caller observes both (basefold.rs:356, sumcheck/src/lib.rs:97), samples the
 * challenge and passes it back.  After the last round the caller observes the
 * final polynomial (basefold.rs:196), samples the query indices
 * (basefold.rs:200-203) and finishes.  `stream` (cudaStream_t or NULL for the
 * pcs's stream) lets several sessions overlap on the GPU.
 * bf_open_start: begins open (basefold.rs:133-193) for one point; for a
 *   commitment of width > 1, `scalars` holds the caller's eq scalars
 *   (sample_random_scalars_by_eq, basefold.rs:398-408; width elements), which
 *   combine the rows (basefold.rs:166-183); NULL for width 1.
 * bf_open_round: waits for the device and writes the current round index
 *   (d-1 .. 0, or -1 once every round is done), its root and round poly.
 * bf_open_challenge: applies the round's challenge; returns without waiting.
 * bf_open_poll: 1 when the session's enqueued work has finished, else 0.
 * bf_open_final: the final polynomial (one element) after the last round.
 * bf_open_finish: gathers the openings at the caller's indices (exactly
 *   num_queries of them) and writes the bincode proof. */
int bf_open_start(bf_pcs* pcs, const bf_commitment* comm, const uint8_t* point, const uint8_t* values,
                  const uint8_t* scalars, void* stream, bf_open_session** out);
int bf_open_round(bf_open_session* s, int* round, uint8_t pi_root[32], uint8_t round_poly[32]);
int bf_open_challenge(bf_open_session* s, const uint8_t r[16]);
int bf_open_poll(bf_open_session* s);
int bf_open_final(bf_open_session* s, uint8_t final_poly[16]);
int bf_open_finish(bf_open_session* s, const uint64_t* indices, size_t nq, uint8_t* proof, size_t cap,
                   size_t* proof_len);
void bf_open_session_free(bf_open_session* s);

/* ---- Launch-shape autotuner.  No counterpart in the reference.
 * A pcs's launch shapes are six integers: threads per block of the
 * shared-memory NTT pass (128, 256, 512), butterfly layers per NTT pass
 * (6..12, a tile of 2^T elements: the NTT radix per pass), the largest
 * Merkle level run by the single-block top kernel (64..4096, a power of
 * two), the single-block open tail (rounds whose next tree has
 * <= 2^tail_log leaves, 1..11), the Merkle levels per launch (levels of
 * 2^10 .. 2^subtree_log nodes run as one launch, 10..20), and the NTT pass
 * kind (0: layer by layer in shared memory; 1: tiles of 2^9..2^13 elements
 * register-blocked; 2: as 0 with the last pass and its leaf hashing
 * warp-specialized, butterfly warps and hashing warps on two tile buffers;
 * 3: as 0 with the cosets of a two-pass encode pipelined, the next cosets'
 * first pass on a high-priority stream beside a coset's last pass).
 * They change how work is launched, never the proof bytes.  bf_pcs_autotune times `reps` whole proofs (commit + eval + open)
 * on random device data per candidate, one parameter at a time, keeps the
 * fastest in the pcs and in the tune cache, and writes a JSON report
 * (timings per candidate, ms) into `report` when given.
 * get/set: vals = {ntt_threads, ntt_max_T, top_nodes, tail_log, subtree_log,
 * ntt_kind}; n >= 4 (set leaves the values past n unchanged). */
int bf_pcs_autotune(bf_pcs* pcs, int reps, char* report, size_t cap);
int bf_pcs_get_tune(const bf_pcs* pcs, int* vals, int n);
int bf_pcs_set_tune(bf_pcs* pcs, const int* vals, int n);
/* The tune cache: launch shapes per (device name, num_vars, log2_c), filled
 * by bf_pcs_autotune and bf_tune_cache_load; bf_pcs_setup (and so every pcs
 * the engine makes for a size) starts from the entry for its device and size.
 * The file is JSON: {"version": 1, "entries": [{"device": ..., "num_vars":
 * ..., "log2_c": ..., "tune": [six values], "ms": ...}, ...]}, one entry per
 * line.  load merges the file's entries (returns how many) and save writes
 * every entry. */
int bf_tune_cache_load(const char* path);
int bf_tune_cache_save(const char* path);
int bf_tune_cache_clear(void);

/* ---- Prover engine: many jobs of different sizes in flight at once.
 * Each job runs on one stream of a pool: at admission its commit,
 * evaluation and whole open (transcript on the device) are queued at once;
 * the host only samples the query positions and reads the proof back.  The
 * engine admits jobs while streams (max_inflight) and the HBM budget
 * (mem_budget bytes, 0 = 80% of free memory) allow, so requests join while
 * others run.  Proofs are identical to bf_commit/bf_eval/bf_open one at a
 * time.  (No counterpart in the reference, which proves one polynomial at a
 * time on the CPU.)
 * bf_engine_autotune: reps > 0 autotunes (bf_pcs_autotune) each size the
 *   first time a job of that size is admitted; 0 (default) keeps defaults.
 * bf_engine_set_tune: the launch shapes of bf_pcs_set_tune (4 to 6 values)
 *   for every size, current and future (an autotune, if on, still runs
 *   after).  Without it each size starts from the tune cache's entry.
 *   Call only while no job is in flight.
 * bf_engine_graphs (default off): on, each slot keeps, per job size, fixed
 *   buffers and one captured CUDA graph of the commit, evaluation and
 *   device-transcript open; a job then costs a staging write, one copy of
 *   its evaluations and one graph launch (lower latency for a job alone).
 *   Idle slots' buffers count toward mem_budget and are dropped when a job
 *   of another size needs the room.  Off: every job enqueues its kernels one
 *   by one on pool memory (as fast or faster with many jobs in flight).
 *   Call only while no job is in flight.
 * Completed jobs (query sampling, openings, proof) are finished on a few
 *   host threads of the engine, apart from the scheduling thread.
 * bf_engine_prove: runs `count` jobs to completion on the calling thread.
 * bf_engine_start/stop + submit/poll: serving from a background thread;
 *   submitted bf_job structs must stay valid until returned by poll. */
int bf_engine_create(int device, int lambda, int log2_c, int max_inflight, size_t mem_budget, bf_engine** out);
void bf_engine_free(bf_engine* e);
size_t bf_engine_proof_size(bf_engine* e, int num_vars);
int bf_engine_prove(bf_engine* e, bf_job* jobs, size_t count, int device_input);
int bf_engine_start(bf_engine* e);
int bf_engine_stop(bf_engine* e);
int bf_engine_submit(bf_engine* e, bf_job* job, int device_input);
int bf_engine_poll(bf_engine* e, bf_job** done, size_t cap, size_t* n);
/* Cancels a submitted job that is still waiting for admission: it leaves the
 * queue with status BF_ERR_CANCELLED and is returned by bf_engine_poll.  A job
 * whose GPU work has been queued cannot be cancelled (BF_ERR_ARG). */
int bf_engine_cancel(bf_engine* e, bf_job* job);
int bf_engine_autotune(bf_engine* e, int reps);
int bf_engine_set_tune(bf_engine* e, const int* vals, int n);
int bf_engine_graphs(bf_engine* e, int on);
/* Serving policy.  smallest_first != 0: a free slot takes the queued job with
 * the fewest variables (default: arrival order).  prio_max_vars >= 0: jobs of
 * at most that many variables run on high-priority CUDA streams (direct
 * launches; graph replay keeps normal priority), whose blocks are dispatched
 * ahead of the waiting blocks of larger jobs (default -1: off).  Call only
 * while no job is in flight. */
int bf_engine_schedule(bf_engine* e, int smallest_first, int prio_max_vars);
/* Host-side accounting since creation: out = {ms spent admitting jobs
 * (allocation, capture, staging, enqueue), of which ms in graph launches,
 * ms completing jobs (query sampling, proof readout), plans built, plans
 * dropped, jobs done}. */
int bf_engine_stats(bf_engine* e, double* out, int n);

/* ---- Evaluation that allocates nothing.  No counterpart in the reference.
 * The multilinear extension of the 2^num_vars evaluations at `point`, the
 * same value bf_eval returns, for callers that cannot allocate device memory
 * at this point — e.g. a service whose device memory is all carved into
 * fixed per-request slots, or a latency-critical loop where
 * cudaMalloc/cudaFree would synchronise the device.  Inputs and output are
 * the caller's: `d_evals` and `d_value` (16 bytes) in device memory, both
 * 16-byte aligned (otherwise BF_ERR_ARG), `point` in host memory; the work
 * is queued on `stream` (cudaStream_t, NULL = default stream) and the call
 * does not wait for it.  Scratch is a fixed 1 MiB array in the library's
 * device image, so num_vars <= 17 (larger sizes return BF_ERR_ARG; use
 * bf_eval).  Every call on a device shares that array and it keeps the last
 * call's contents: calls whose GPU work overlaps (other streams or threads)
 * race.  The first call on each device looks up the array's device address;
 * make that first call before any stream capture, and do not reset the
 * device (cudaDeviceReset) after it. */
int bf_eval_noalloc(const void* d_evals, int num_vars, const uint8_t* point, void* d_value, void* stream);

/* ---- PolyCommitScheme::verify (lib.rs:44-50; basefold.rs:234-324) on the
 * host.  Returns BF_VERIFY_* (>= 0) or a negative BF_ERR_*. */
int bf_verify(const bf_pcs* pcs, const uint8_t root[32], const uint8_t* point, const uint8_t* values, size_t width,
              int n_evals, bf_challenger* ch, const uint8_t* proof, size_t proof_len);

/* ---- PolyCommitScheme::verify of many proofs of one pcs at once: each job
 * is one bf_verify call with n_evals = 1 (basefold.rs:234-324).  The
 * transcripts are replayed on host threads; the Merkle paths and fold chains
 * of every query run on the GPU (the pcs must be on a device).  Each job's
 * `result` and challenger end exactly as bf_verify's would.  Returns BF_OK or
 * a negative BF_ERR_* (nothing is verified then).  Calls on one pcs are
 * serialized. */
typedef struct bf_verify_job {
  const uint8_t* root;        /* 32-byte commitment */
  const uint8_t* point;       /* num_vars field elements */
  const uint8_t* values;      /* width field elements */
  size_t width;
  bf_challenger* challenger;  /* the caller's transcript (observed root and values) */
  const uint8_t* proof;
  size_t proof_len;
  int result;                 /* out: BF_VERIFY_* */
} bf_verify_job;
int bf_verify_batch(bf_pcs* pcs, bf_verify_job* jobs, size_t count);

/* ---- Fiat–Shamir transcript: GenericChallenger<Polyval, Keccak256Hash>
 * (p3/src/challenger.rs:24-83) over Plonky3's HashChallenger. */
/* GenericChallenger::new(initial_state) (challenger.rs:36-42); keccak256()
 * is an empty initial state (challenger.rs:45-49). */
int bf_challenger_new(const uint8_t* initial_state, size_t len, bf_challenger** out);
int bf_challenger_clone(const bf_challenger* ch, bf_challenger** out);
void bf_challenger_free(bf_challenger* ch);
/* CanObserve<T>::observe of bincode bytes (challenger.rs:51-60). */
int bf_challenger_observe(bf_challenger* ch, const uint8_t* bytes, size_t len);
/* CanSample<E>::sample of one field element (challenger.rs:62-74). */
int bf_challenger_sample_ext(bf_challenger* ch, uint8_t out[16]);
/* CanSampleBits<usize>::sample_bits (challenger.rs:76-83). */
int bf_challenger_sample_bits(bf_challenger* ch, int bits, uint64_t* out);
/* Serialized state: [u64 in_len][input buffer][u64 out_len][output buffer]. */
int bf_challenger_state(const bf_challenger* ch, uint8_t* buf, size_t cap, size_t* len);
int bf_challenger_from_state(const uint8_t* buf, size_t len, bf_challenger** out);

/* ---- Standalone sumcheck prover: prove_sumcheck (sumcheck/src/lib.rs:56-79)
 * of sum_b prod_{j<k} f_j(b).  k = 2 is Quadratic with the single pair
 * (ONE, 0, 1) (function/quadratic.rs:84-134); k = 3 is this project's
 * product-of-three extension (compressed round polynomial [c0, c2, c3]).
 * `polys` holds k arrays of 2^num_vars elements back to back (host memory
 * for bf_sumcheck_prove, device memory for bf_sumcheck_prove_device, which
 * does not modify them).  Output: num_vars compressed round polynomials
 * (k elements each, round num_vars-1 first), then the num_vars challenges,
 * then the k final evaluations, then the final subclaim. */
int bf_sumcheck_prove(int device, int k, int num_vars, const uint8_t* polys, const uint8_t* claim,
                      bf_challenger* ch, uint8_t* out);
int bf_sumcheck_prove_device(bf_pcs* pcs, int k, int num_vars, const void* d_polys, const uint8_t* claim,
                             bf_challenger* ch, uint8_t* out);

/* ---- Timing of the kernel classes (CUDA events on the pcs's stream).
 * When enabled, every launch group is bracketed by events; bf_profile_read
 * returns accumulated milliseconds and launch counts per class:
 * 0 encode (NTT passes), 1 codeword leaves, 2 tree levels, 3 folded-codeword
 * leaves, 4 fold, 5 fix + sumcheck reduction, 6 eq table, 7 query gather,
 * 8 single-block last rounds of open, 9 on-device transcript steps, 10 the
 * last NTT pass with the leaf hashing it carries (also inside class 0). */
int bf_profile_enable(bf_pcs* pcs, int on);
int bf_profile_read(bf_pcs* pcs, double* ms, uint64_t* launches, int nclasses);

/* ---- Test hooks: device field products and Keccak-f[1600] permutations on
 * host buffers (n elements / n states of 25 little-endian lanes). */
int bf_test_gf_mul(int device, const uint8_t* a, const uint8_t* b, uint8_t* out, size_t n);
int bf_test_keccak_f(int device, uint64_t* states, size_t n);

/* ---- Prime-field Basefold: the same PolyCommitScheme instantiated as
 *   Basefold<BabyBear, BinomialExtensionField<BabyBear, 5>,
 *            ReedSolomonCode<BabyBear>, Keccak256MerkleTreeMmcs<BabyBear>>
 * (poly-commit/benches/poly-commit.rs:28-43,114-123; code/reed_solomon.rs).
 * Conventions of this section:
 *  - A BabyBear (p = 15 * 2^27 + 1) is its canonical value as a u32
 *    (< p), little-endian: the bytes bincode writes for it.  Evaluations are
 *    row-major u32, 2^num_vars rows of `width` (RowMajorMatrix<BabyBear>);
 *    a value >= p is rejected with BF_ERR_ARG.
 *  - An extension element is its five coefficients (of 1, X, .., X^4 with
 *    X^5 = 2), canonical u32 each: 20 bytes.  Points are num_vars of them;
 *    values `width` of them.
 *  - The transcript is a bf_challenger: the byte-level HashChallenger is the
 *    same for both fields; the prime path samples field elements from it as
 *    GenericChallenger<BabyBear, _> does (bf_challenger_sample_bb_ext).
 *  - Same ownership and threading rules as bf_pcs. */
typedef struct bf_bb_pcs bf_bb_pcs;
typedef struct bf_bb_commitment bf_bb_commitment;

/* PolyCommitScheme::setup with ReedSolomonCode::new(lambda, log2_c,
 * num_vars) (reed_solomon.rs:19-39); num_vars + log2_c <= 27.  device < 0
 * makes a verifier-only pcs (bf_bb_verify, sizes). */
int bf_bb_pcs_setup(int device, int lambda, int log2_c, int num_vars, void* stream, bf_bb_pcs** out);
/* PolyCommitScheme::setup with GenericRandomFoldableCode::
 * reed_solomon_g_0_with_random_ts(lambda, log2_c, log2_k_0, d, rng)
 * (code/generic.rs:43-71), d = num_vars - log2_k_0.  The random vectors the
 * reference draws from its RNG are given: `ts` holds ts[0], .., ts[d-1]
 * back to back (n_0 << i canonical nonzero BabyBears each, n_0 =
 * 2^(log2_c + log2_k_0); ts_len = n_0 (2^d - 1)).  G_0 is the reference's
 * (row i = powers of i).  Proofs carry k_0 = 2^log2_k_0 final values. */
int bf_bb_pcs_setup_generic(int device, int lambda, int log2_c, int log2_k_0, int num_vars, const uint32_t* ts,
                            size_t ts_len, void* stream, bf_bb_pcs** out);
void bf_bb_pcs_free(bf_bb_pcs* pcs);
/* RandomFoldableCode::num_queries (reed_solomon.rs:57-64, generic.rs:
 * 99-103 with F::bits() = 31). */
size_t bf_bb_pcs_num_queries(const bf_bb_pcs* pcs);
/* Exact bincode size of the proof of a width-`width` open of n_evals (0 or
 * 1) points. */
size_t bf_bb_pcs_proof_size(const bf_bb_pcs* pcs, size_t width, int n_evals);
/* PolyCommitScheme::commit (basefold.rs:112-120): host evaluations
 * (bf_bb_commit, pinned memory overlaps the copy best) or device memory
 * (bf_bb_commit_device, 4-byte aligned, read and kept by reference until
 * the commitment is freed). */
int bf_bb_commit(bf_bb_pcs* pcs, const uint32_t* evals, size_t width, bf_bb_commitment** out, uint8_t root[32]);
int bf_bb_commit_device(bf_bb_pcs* pcs, const void* d_evals, size_t width, bf_bb_commitment** out,
                        uint8_t root[32]);
int bf_bb_commitment_root(const bf_bb_commitment* comm, uint8_t root[32]);
void bf_bb_commitment_free(bf_bb_commitment* comm);
/* PolyCommitScheme::eval (basefold.rs:126-131): `values` receives the
 * width column evaluations at the point (width x 20 bytes). */
int bf_bb_eval(bf_bb_pcs* pcs, const bf_bb_commitment* comm, const uint8_t* point, uint8_t* values);
/* PolyCommitScheme::eval(&self, data: &Data, point) for data that has no
 * commitment: 2^num_vars rows of `width` canonical words in host memory
 * (on_device 0: copied in) or device memory (on_device 1: 4-byte aligned,
 * not modified); evaluated on the GPU into `values` (width x 20 bytes). */
int bf_bb_eval_data(bf_bb_pcs* pcs, const void* evals, int on_device, size_t width, const uint8_t* point,
                    uint8_t* values);
/* PolyCommitScheme::open (basefold.rs:133-232) of n_evals points (0: the
 * default proof, as the reference returns for no evaluations; 1: `point`
 * and the commitment's width `values`); the transcript advances exactly as
 * the reference's.  Returns BF_ERR_BUFFER with *proof_len set when cap is
 * too small, and BF_ERR_NOT_INVERTIBLE for a coordinate r = 0 (or r = 1
 * below the last). */
int bf_bb_open(bf_bb_pcs* pcs, const bf_bb_commitment* comm, const uint8_t* point, const uint8_t* values,
               int n_evals, bf_challenger* ch, uint8_t* proof, size_t cap, size_t* proof_len);
/* PolyCommitScheme::verify (basefold.rs:234-324), on the host; n_evals 0
 * accepts anything, as the reference does.  Returns BF_VERIFY_* (>= 0) or
 * a negative BF_ERR_*. */
int bf_bb_verify(const bf_bb_pcs* pcs, const uint8_t root[32], const uint8_t* point, const uint8_t* values,
                 size_t width, int n_evals, bf_challenger* ch, const uint8_t* proof, size_t proof_len);
/* CanSample<BinomialExtensionField<BabyBear, 5>>::sample (challenger.rs:
 * 62-74): five BabyBears, each from 4 bytes shifted right by one and
 * rejected while >= p. */
int bf_challenger_sample_bb_ext(bf_challenger* ch, uint8_t out[20]);

#ifdef __cplusplus
}
#endif
#endif
