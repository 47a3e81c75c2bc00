// Shared host-side definitions of libbasefold_gpu.so: error reporting,
// device/pinned buffers, kernel-class timing and the ABI objects.
#pragma once
#include <cuda_runtime.h>

#include <array>
#include <atomic>
#include <cstdint>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/basefold_gpu.h"
#include "bf_internal.h"
#include "host_math.h"

namespace bfapi {

using bfh::u128;

// Records the message as the calling thread's last error and returns `code`.
int fail(int code, const char* fmt, ...);
const std::string& last_error();

#define CU(expr)                                                                                      \
  do {                                                                                                \
    cudaError_t e__ = (expr);                                                                         \
    if (e__ != cudaSuccess)                                                                           \
      return ::bfapi::fail(e__ == cudaErrorMemoryAllocation ? BF_ERR_OOM : BF_ERR_CUDA, "%s: %s (%s:%d)", \
                           #expr, cudaGetErrorString(e__), __FILE__, __LINE__);                       \
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
  cudaStream_t pool_stream = nullptr;  // set when allocated from a stream-ordered pool
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p && owned) {
      if (pool_stream)
        cudaFreeAsync(p, pool_stream);
      else
        cudaFree(p);
    }
    p = nullptr;
    bytes = 0;
    pool_stream = nullptr;
  }
  cudaError_t alloc(size_t n) {
    release();
    owned = true;
    if (n == 0) n = 16;
    cudaError_t e = cudaMalloc(&p, n);
    if (e == cudaSuccess) bytes = n;
    return e;
  }
  // Stream-ordered allocation from `pool`, released in stream order on `st`.
  cudaError_t alloc_async(size_t n, cudaMemPool_t pool, cudaStream_t st) {
    release();
    owned = true;
    if (n == 0) n = 16;
    cudaError_t e = cudaMallocFromPoolAsync(&p, n, pool, st);
    if (e == cudaSuccess) {
      bytes = n;
      pool_stream = st;
    }
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
  PinnedBuf() = default;
  PinnedBuf(const PinnedBuf&) = delete;
  PinnedBuf& operator=(const PinnedBuf&) = delete;
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

// Kernel classes timed with CUDA events when profiling is on.
// P_ENCODE_LAST is the last NTT pass alone (with the leaf hashing it
// carries); it is also inside P_ENCODE.
constexpr int kProfClasses = 11;
enum ProfClass {
  P_ENCODE = 0, P_LEAVES = 1, P_TREE = 2, P_PI_LEAVES = 3, P_FOLD = 4, P_FIX = 5, P_EQ = 6, P_GATHER = 7,
  P_TAIL = 8, P_TRANSCRIPT = 9, P_ENCODE_LAST = 10
};

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
  cudaEvent_t get();
  ~Profiler();
  void drain();  // resolve recorded pairs; the stream must have been synchronised
};

struct ProfScope {
  Profiler& pr;
  cudaStream_t st;
  int cls;
  cudaEvent_t a = nullptr;
  ProfScope(Profiler& p, cudaStream_t s, int c);
  ~ProfScope();
};

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev);
  ~DeviceGuard();
};

size_t num_queries(int lambda, int log2_c);
u128 horner(const u128* c, int n, u128 x);
void put_u64(std::vector<uint8_t>& b, uint64_t v);
void put_elem(std::vector<uint8_t>& b, u128 v);
// MultiPoly::eq(x, ONE) on the host (p3/src/poly/multilinear.rs:41-64).
std::vector<u128> eq_table_host(const std::vector<u128>& x);
// sample_random_scalars_by_eq (poly-commit/src/basefold.rs:398-408).
std::vector<u128> sample_scalars_by_eq(size_t n, bfh::Challenger& ch);

}  // namespace bfapi

struct bf_pcs;
struct bf_commitment;
namespace bfapi {
int commit_alloc(bf_pcs* p, bf_commitment* cm, cudaStream_t st);
// With fork_trees (and st the pcs's own stream) the codeword tree and the
// first folded-codeword tree are built concurrently on the pcs's second stream.
int commit_enqueue(bf_pcs* p, bf_commitment* cm, const uint4* data, cudaStream_t st, uint8_t* roots_pin,
                   bool fork_trees = false, const cudaEvent_t* slice_ready = nullptr, int slices = 0);
// The value lands in value_pin; *value_dev (when given) receives where it
// lives on the device.  With point_dev the coordinates are read from device
// memory at run time (for graph capture), else taken from the host `point`.
int eval_enqueue(bf_pcs* p, const bf_commitment* cm, const uint8_t* point, uint4* scratch, cudaStream_t st,
                 uint8_t* value_pin, const uint4** value_dev = nullptr, const uint4* point_dev = nullptr);
}  // namespace bfapi

struct bf_open_session;
namespace bfapi {
int open_start_impl(bf_pcs* p, const bf_commitment* cm, const uint8_t* point, const uint8_t* values,
                    const uint8_t* scalars, void* stream, bf_open_session** out);
// The pieces of open_start_impl / open_resident_enqueue, for graph capture:
// host-side preparation (pinned staging) apart from the device work.
int open_session_create(bf_pcs* p, const bf_commitment* cm, void* stream, bf_open_session** out);
int open_session_prepare(bf_open_session* s, const uint8_t* point, const uint8_t* values, const uint8_t* scalars);
int open_session_enqueue_start(bf_open_session* s);
const uint4* open_session_point_dev(const bf_open_session* s);
void open_session_mark_launched(bf_open_session* s);  // the resident open was launched by a graph
cudaStream_t open_session_stream(const bf_open_session* s);
// Moves the session's later work (the query gather and proof readout) to `st`;
// its earlier work must have completed.
void open_session_set_stream(bf_open_session* s, cudaStream_t st);
cudaEvent_t open_session_event(const bf_open_session* s);
int open_resident_prepare(bf_open_session* s, const bfh::Challenger& ch);
int open_resident_enqueue_device(bf_open_session* s, const uint4* root_dev, const uint4* value_dev);
int open_resident_enqueue(bf_open_session* s, const bfh::Challenger& ch, const uint4* root_dev,
                          const uint4* value_dev);
int open_resident_complete(bf_open_session* s, bfh::Challenger& ch);
int open_finish_enqueue(bf_open_session* s, const uint64_t* indices, size_t nq);
int open_finish_complete(bf_open_session* s, uint8_t* proof, size_t cap, size_t* proof_len);
}  // namespace bfapi

namespace bfapi {
void pcs_acquire(bf_pcs* p);
void pcs_release(bf_pcs* p);
// Launch shapes from the tune cache for the pcs's device and size, if any.
void tune_cache_apply(bf_pcs* p);
}  // namespace bfapi

struct bf_challenger {
  bfh::Challenger c;
};

struct bf_pcs {
  // Holders: the caller (until bf_pcs_free) and every commitment and open
  // session made from it; the last to let go destroys it, so frees in any
  // order are safe.
  std::atomic<int> refs{1};
  int device = 0;
  int lambda = 128, log2_c = 1, d = 0, L = 0;
  size_t Q = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  cudaStream_t aux = nullptr;   // second stream for independent work of one commit
  cudaStream_t aux2 = nullptr;  // third: the first NTT pass of a sliced host commit
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // bf_commit copies host evaluations in slices on `aux`; the first NTT pass
  // starts on each slice when its event completes
  static constexpr int kH2DSlices = 8;
  cudaEvent_t slice_ev[kH2DSlices] = {};
  // Commitments and open sessions draw their buffers from this pool; it keeps
  // freed memory for reuse instead of returning it to the driver.
  cudaMemPool_t pool = nullptr;
  bfapi::DevBuf tw_tables, tw_view;
  bf::TwiddleView tw_host{};
  std::vector<std::vector<bfh::u128>> bases;  // stage bases (host copy, for the verifier)
  bfapi::DevBuf sc_ws;                        // standalone-sumcheck scratch
  bfapi::DevBuf eval_ws;                      // bf_eval scratch
  bfapi::DevBuf evalc_ws;                     // bf_eval of w > 1 columns: point, eq table, sums
  bfapi::PinnedBuf pinned;
  std::vector<std::unique_ptr<bfapi::PinnedBuf>> pinned_cache;  // staging kept between open sessions
  std::mutex pinned_mu;                                          // guards pinned_cache (sessions on several threads)
  bfapi::Profiler prof;
  bf::Tune tune;  // launch shapes and thresholds (bf_pcs_autotune / bf_pcs_set_tune)
  // bf_verify_batch staging (grow-only): proofs and query records in, flags out
  bfapi::PinnedBuf verify_pin;
  bfapi::DevBuf verify_dev;
  std::mutex verify_mu;

  size_t n_d() const { return (size_t)1 << L; }
  size_t c() const { return (size_t)1 << log2_c; }
  size_t n_i(int i) const { return c() << i; }
  // Bytes of one query opening in the proof (basefold.rs:56-65).
  size_t block_bytes(size_t width) const {
    size_t b = 8 + 16 * width + 8 + 32 * (size_t)L + 8;
    for (int i = 0; i < d; ++i) b += 24 + 32 * (size_t)(log2_c + i);
    return b;
  }
  ~bf_pcs();
};

struct bf_commitment {
  bf_pcs* pcs = nullptr;
  size_t width = 1;
  bfapi::DevBuf data, cw, tree;
  // Tree of the first open round's folded codeword (for width 1 it is the
  // codeword itself, paired (2s, 2s+1) in NTT order), built at commit time.
  bfapi::DevBuf pi_tree;
  uint8_t root[32];
  uint8_t pi_root[32];
};
