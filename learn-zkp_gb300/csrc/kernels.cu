// CUDA kernels of the Basefold prover path (sm_103a).
//
// Layout conventions shared by every kernel:
//  * a field element is a uint4 (raw little-endian Montgomery-form u128);
//  * a digest is two uint4 (32 bytes); inside the Merkle trees its four
//    64-bit lanes are stored bit-interleaved (keccak.cuh), converted to
//    bytes wherever a digest leaves a tree (openings, roots);
//  * the codeword of a commitment and every folded codeword of `open` are
//    kept in additive-NTT output order ("NTT order"): position q holds the
//    codeword entry at bitrev(q).  The reference materialises the bit
//    reversal (binary_reed_solomon.rs:80-81); here it is absorbed into
//    indexing.  In NTT order the folding pair (j, j + n_i) of
//    binary_reed_solomon.rs:88-96 is the adjacent pair (2t, 2t+1) and its
//    twiddle is entry t of the stage table with no bit reversal;
//  * every Merkle level is stored "reversed": node m of a level with 2^h
//    nodes sits at bitrev_h(m).  Then node s of the next level is
//    H(prev[s] || prev[s + half]) — both children in the two contiguous
//    halves of the level below — so every level is one coalesced pass.
#include <cuda_runtime.h>
#include <atomic>
#include <algorithm>
#include <cstdint>

#include "bf_internal.h"
#include "gf128.cuh"
#include "keccak.cuh"

namespace bf {

__device__ __forceinline__ uint32_t brev_bits(uint32_t x, int bits) { return bits ? (__brev(x) >> (32 - bits)) : 0u; }
__device__ __forceinline__ uint64_t brev_bits64(uint64_t x, int bits) {
  return bits ? (__brevll(x) >> (64 - bits)) : 0ull;
}

__device__ __forceinline__ uint4 gf_one() { return make_uint4(1u, 0u, 0u, 0xc2000000u); }

// Number of kernels this library has launched (all devices, all streams).
// The per-thread count lets a graph capture learn how many kernels it holds
// while other threads launch.
static std::atomic<unsigned long long> g_launches{0};
static thread_local unsigned long long t_launches = 0;
unsigned long long launches_total() { return g_launches.load(); }
unsigned long long launches_this_thread() { return t_launches; }
void count_launch() {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  ++t_launches;
}
void add_launches(long long n) { g_launches.fetch_add((unsigned long long)n, std::memory_order_relaxed); }
#define COUNT_LAUNCH() count_launch()

static int g_num_sms = 0;
static int num_sms() {
  if (g_num_sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_num_sms <= 0) g_num_sms = 1;
  }
  return g_num_sms;
}

static unsigned grid_for(size_t n, int threads, int per_sm = 8) {
  size_t want = (n + threads - 1) / threads;
  size_t cap = (size_t)num_sms() * per_sm;
  if (want > cap) want = cap;
  if (want == 0) want = 1;
  return (unsigned)want;
}

// One element per thread for the long grid-stride kernels (Merkle levels and
// leaves, fold): blocks then live microseconds instead of the whole
// launch, so work of other streams (other jobs of the engine) gets SM room as
// blocks retire rather than only when the launch ends.
static unsigned grid_short(size_t n, int threads) {
  size_t want = (n + threads - 1) / threads;
  if (want > 0x7fffffffull) want = 0x7fffffffull;
  if (want == 0) want = 1;
  return (unsigned)want;
}

// ---------------------------------------------------------------------------
// Reed–Solomon encoding (binary_reed_solomon.rs:67-82 with the coset NTTs of
// binary.rs:55-105).  Codeword = additive NTT of pad(bitrev(m)) over
// L = n + log2_c bits; its top log2_c layers only replicate m (the padding is
// zero and every stage table starts with 0), so coset j is a size-2^n NTT of
// bitrev(m) with stage-s twiddles K = (j << (n-1-s)) | k.
//
// One launch runs T consecutive layers [s_lo, s_lo+T) on tiles of 2^T
// elements held in shared memory: element x = (hi << (s_lo+T)) | (a << s_lo) | u.
// The first launch reads m directly (bit reversal and replication folded
// into the load: for fixed u the tile's m-indices are one contiguous run).
// ---------------------------------------------------------------------------
struct PassParams {
  int n, s_lo, T, first;
  int width;  // row width of m and cw; blockIdx.y is the column
  // First pass split into 2^piece_log launches (input slices): launch
  // `piece` runs the butterfly columns u = (m << piece_log) | bitrev(piece),
  // whose input tiles bitrev(u) (rows [c 2^T, (c+1) 2^T)) are slice `piece`.
  // Unsplit (piece_log 0) block m runs column m, so neighbouring blocks write
  // neighbouring elements.
  int piece_log, piece;
  // Last pass only: also hash the codeword leaves H(cw[q]) and the first
  // folded-codeword leaves H(cw[2s] || cw[2s+1]) from the tile in shared
  // memory (null: no hashing).  The hashing is integer-ALU work and the
  // butterflies are multiplier work, so co-resident blocks in the two phases
  // keep both pipes busy.
  uint4* leaves;
  uint4* pair_leaves;
  int log2_c;      // cosets: the persistent last pass walks c 2^(n-T) tiles
  int ntt_warps;   // warp-specialized last pass: warps on butterflies (the rest hash)
  int coset0;      // the launch covers cosets coset0, coset0 + 1, ... (grid / tiles per coset of them)
};

// H: field products take H of their nine 32 x 32 products from the 16-bit
// form (gf_mul_mix), moving multiplier work of the passes without hashing,
// which are bound by the wide multiplies, onto the ALU pipe.
template <bool HASH, int H = 0>
__global__ void __launch_bounds__(512) ntt_pass_kernel(const uint4* __restrict__ m, uint4* __restrict__ cw,
                                                      PassParams p, const TwiddleView* __restrict__ tw) {
  extern __shared__ uint4 sm[];
  const int n = p.n, T = p.T, s_lo = p.s_lo;
  const uint32_t tiles_per_coset = 1u << (n - T);
  uint32_t j, rem;
  if (p.first) {
    const int shift = n - T - p.piece_log;  // log2 of this launch's blocks per coset
    j = blockIdx.x >> shift;
    rem = ((blockIdx.x & ((1u << shift) - 1u)) << p.piece_log) | brev_bits((uint32_t)p.piece, p.piece_log);
  } else {
    j = blockIdx.x >> (n - T);
    rem = blockIdx.x & (tiles_per_coset - 1);
  }
  j += (uint32_t)p.coset0;
  const uint32_t u = rem & ((1u << s_lo) - 1u);
  const uint32_t hi = rem >> s_lo;
  const uint32_t tsize = 1u << T;
  const size_t coset_base = (size_t)j << n;
  const size_t w = (size_t)p.width, col = blockIdx.y;

  if (p.first) {
    const size_t base = (size_t)brev_bits(u, s_lo) << T;
    for (uint32_t i = threadIdx.x; i < tsize; i += blockDim.x) sm[brev_bits(i, T)] = m[(base + i) * w + col];
  } else {
    for (uint32_t i = threadIdx.x; i < tsize; i += blockDim.x) {
      const size_t x = ((size_t)hi << (s_lo + T)) | ((size_t)i << s_lo) | u;
      sm[i] = cw[(coset_base + x) * w + col];
    }
  }
  __syncthreads();

  for (int l = T - 1; l >= 0; --l) {
    const int s = s_lo + l;
    const uint4* __restrict__ lo_tab = tw->lo[s];
    const uint4* __restrict__ hi_tab = tw->hi[s];
    const uint32_t kbase = (j << (n - 1 - s)) | (hi << (T - 1 - l));
    const uint32_t lmask = (1u << l) - 1u;
    for (uint32_t bi = threadIdx.x; bi < (tsize >> 1); bi += blockDim.x) {
      const uint32_t a = ((bi >> l) << (l + 1)) | (bi & lmask);
      const uint32_t K = kbase | (bi >> l);
      uint4 x0 = sm[a], x1 = sm[a + (1u << l)];
      // twiddle K is the XOR of independent stage bases over K's bits: zero
      // only for K = 0 (the whole top layer of coset 0, half the next, ...)
      if (K != 0) x0 = gf_add(x0, gf_mul_mix<H>(x1, gf_add(lo_tab[K & 4095u], hi_tab[K >> 12])));  // lo += hi * t
      x1 = gf_add(x1, x0);  // hi += lo
      sm[a] = x0;
      sm[a + (1u << l)] = x1;
    }
    __syncthreads();
  }

  for (uint32_t i = threadIdx.x; i < tsize; i += blockDim.x) {
    const size_t x = ((size_t)hi << (s_lo + T)) | ((size_t)i << s_lo) | u;
    cw[(coset_base + x) * w + col] = sm[i];
  }
  if (HASH) {
    // last pass: s_lo = 0, the tile is the contiguous run [coset_base + hi 2^T, +2^T)
    const size_t q0 = coset_base + ((size_t)hi << T);
    for (uint32_t k = threadIdx.x; k < (tsize >> 1); k += blockDim.x) {
      const uint4 e0 = sm[2 * k], e1 = sm[2 * k + 1];
      const size_t q = q0 + 2 * k;
      store_digest(p.leaves, q, hash_elem(e0));
      store_digest(p.leaves, q + 1, hash_elem(e1));
      store_digest(p.pair_leaves, q >> 1, hash_pair(e0, e1));
    }
  }
}

// ---------------------------------------------------------------------------
// Register-blocked NTT pass for tiles of 2^9 .. 2^13 elements.  The tile's T
// layers run in phases of (up to) four: in a phase with base bit b, thread t
// holds the 16 elements a(t, e) = tpart(t, b) | (e << b), e < 16, whose tile
// indices differ only in bits [b, b+4), so the phase's layers are butterflies
// between registers with no exchange.  Between phases the tile goes once
// through shared memory (a transpose); a 2^12 tile takes three phases and two
// transposes instead of twelve shared-memory layers with a barrier each.
// Within a layer the 8 butterflies of a thread share at most 8 twiddles, and
// by GF(2)-linearity twiddle(K | v) = twiddle(K) + lo[v] for the v < 8 low
// bits that vary between them: one table pair lookup and block-uniform lo[v]
// loads per layer instead of a lookup per butterfly.
// ---------------------------------------------------------------------------
constexpr int kNttRegMinT = 9;   // smallest tile of the register-blocked pass (32 threads)
constexpr int kNttRegMaxT = 13;  // largest (512 threads)

// Shared-memory slot of tile index a: the low three bits are XORed with bits
// 4..6, so every phase's reads and writes (16-byte elements, 8 lanes per
// shared-memory wavefront) fall in 8 distinct bank groups.
__device__ __forceinline__ uint32_t ntt_slot(uint32_t a) { return a ^ ((a >> 4) & 7u); }

// Tile index held by thread t as element e in the phase with base bit b.
__device__ __forceinline__ uint32_t ntt_elem(uint32_t t, uint32_t e, int b) {
  return (t & ((1u << b) - 1u)) | (e << b) | ((t >> b) << (b + 4));
}

// Layers b+ll_hi .. b of one phase on the thread's 16 registers.  A is the
// thread's tile index with bits [b, b+4) clear, extended by the tile's index
// within its coset above bit T (so that A >> (l+1) is the twiddle index's
// position part at layer l); the stage-s twiddle index of the butterfly at
// element e0 is K = (j << (n-1-s)) | (A >> (l+1)) | (e0 >> (ll+1)).
__device__ __forceinline__ void ntt_phase(uint4 (&x)[16], int b, int ll_hi, uint32_t A, uint32_t j, int n, int s_lo,
                                          const TwiddleView* __restrict__ tw) {
#pragma unroll
  for (int ll = 3; ll >= 0; --ll) {
    if (ll > ll_hi) continue;
    const int l = b + ll, s = s_lo + l;
    const uint4* __restrict__ lo_tab = tw->lo[s];
    const uint4* __restrict__ hi_tab = tw->hi[s];
    const uint32_t Kb = (j << (n - 1 - s)) | (A >> (l + 1));
    const uint4 tb = gf_add(lo_tab[Kb & 4095u], hi_tab[Kb >> 12]);
#pragma unroll
    for (int v = 0; v < (8 >> ll); ++v) {
      const uint4 tv = v ? gf_add(tb, lo_tab[v]) : tb;
      // twiddle index 0 (the top layer of coset 0, half the next, ...) has
      // twiddle 0: the product is skipped
      const bool mul = (Kb | (uint32_t)v) != 0u;
#pragma unroll
      for (int w = 0; w < (1 << ll); ++w) {
        const int e0 = (v << (ll + 1)) | w, e1 = e0 | (1 << ll);
        if (mul) x[e0] = gf_add(x[e0], gf_mul(x[e1], tv));  // lo += hi * t
        x[e1] = gf_add(x[e1], x[e0]);                        // hi += lo
      }
    }
  }
}

template <bool HASH>
__global__ void __launch_bounds__(512) ntt_reg_kernel(const uint4* __restrict__ m, uint4* __restrict__ cw, PassParams p,
                                                     const TwiddleView* __restrict__ tw) {
  extern __shared__ uint4 sm[];
  const int n = p.n, T = p.T, s_lo = p.s_lo;
  const uint32_t nthr = 1u << (T - 4), t = threadIdx.x;
  uint32_t j, rem;
  if (p.first) {
    const int shift = n - T - p.piece_log;
    j = blockIdx.x >> shift;
    rem = ((blockIdx.x & ((1u << shift) - 1u)) << p.piece_log) | brev_bits((uint32_t)p.piece, p.piece_log);
  } else {
    j = blockIdx.x >> (n - T);
    rem = blockIdx.x & ((1u << (n - T)) - 1u);
  }
  j += (uint32_t)p.coset0;
  const uint32_t u = rem & ((1u << s_lo) - 1u);
  const uint32_t hi = rem >> s_lo;
  const size_t coset_base = (size_t)j << n;
  const size_t w = (size_t)p.width, col = blockIdx.y;
  const bool last = s_lo == 0;
  uint4 x[16];

  int b = T - 4;
  if (p.first) {
    // coalesced rows of m, bit-reversed into the tile through shared memory
    const size_t base = (size_t)brev_bits(u, s_lo) << T;
#pragma unroll
    for (int e = 0; e < 16; ++e) x[e] = m[(base + t + nthr * e) * w + col];
#pragma unroll
    for (int e = 0; e < 16; ++e) sm[ntt_slot(brev_bits(t + nthr * e, T))] = x[e];
    __syncthreads();
#pragma unroll
    for (int e = 0; e < 16; ++e) x[e] = sm[ntt_slot(ntt_elem(t, e, b))];
  } else {
#pragma unroll
    for (int e = 0; e < 16; ++e) {
      const size_t xx = ((size_t)hi << (s_lo + T)) | ((size_t)ntt_elem(t, e, b) << s_lo) | u;
      x[e] = cw[(coset_base + xx) * w + col];
    }
  }
  int top = T - 1;
  while (true) {
    const uint32_t A = (hi << T) | ntt_elem(t, 0, b);
    ntt_phase(x, b, top - b, A, j, n, s_lo, tw);
    top = b - 1;
    if (top < 0) break;
    const int nb = top > 3 ? top - 3 : 0;
    __syncthreads();  // every thread has read the previous arrangement
#pragma unroll
    for (int e = 0; e < 16; ++e) sm[ntt_slot(ntt_elem(t, e, b))] = x[e];
    __syncthreads();
#pragma unroll
    for (int e = 0; e < 16; ++e) x[e] = sm[ntt_slot(ntt_elem(t, e, nb))];
    b = nb;
  }
  if (!last) {
#pragma unroll
    for (int e = 0; e < 16; ++e) {
      const size_t xx = ((size_t)hi << (s_lo + T)) | ((size_t)ntt_elem(t, e, 0) << s_lo) | u;
      cw[(coset_base + xx) * w + col] = x[e];
    }
    return;
  }
  // last pass: the tile is the contiguous run [coset_base + hi 2^T, +2^T);
  // stored and hashed from shared memory in coalesced order
  __syncthreads();
#pragma unroll
  for (int e = 0; e < 16; ++e) sm[ntt_slot(ntt_elem(t, e, 0))] = x[e];
  __syncthreads();
  const size_t q0 = coset_base + ((size_t)hi << T);
#pragma unroll 4
  for (int e = 0; e < 16; ++e) {
    const uint32_t i = t + nthr * e;
    cw[(q0 + i) * w + col] = sm[ntt_slot(i)];
  }
  if (HASH) {
    for (uint32_t k = t; k < (8u * nthr); k += nthr) {
      const uint4 e0 = sm[ntt_slot(2 * k)], e1 = sm[ntt_slot(2 * k + 1)];
      const size_t q = q0 + 2 * k;
      store_digest(p.leaves, q, hash_elem(e0));
      store_digest(p.leaves, q + 1, hash_elem(e1));
      store_digest(p.pair_leaves, q >> 1, hash_pair(e0, e1));
    }
  }
}

// ---------------------------------------------------------------------------
// Warp-specialized last NTT pass with the leaf hashing.  Its butterflies are
// multiplier work (IMAD.WIDE on the FMA pipe) and its leaf hashes ALU work;
// in a block whose warps all run one phase and then the other, one pipe idles
// while the other works.  Here the first ntt_warps warps of a 16-warp block
// run the butterflies of tile k into one of two shared-memory buffers while
// the other warps hash tile k-1 out of the other buffer, so both pipes stay
// busy through the whole pass.  The block is persistent (tiles b, b + grid,
// ...).  Named barriers: 1 between the butterfly warps' layers, 2 + buffer
// "tile ready" (butterfly warps arrive, hashing warps wait), 4 + buffer
// "buffer free" (the reverse).
// ---------------------------------------------------------------------------
constexpr int kNttWsThreads = 512;
constexpr int kNttWsMaxT = 12;  // two 2^12-element buffers: 128 KB of shared memory

__device__ __forceinline__ void named_sync(int id, int count) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}
__device__ __forceinline__ void named_arrive(int id, int count) {
  asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(count) : "memory");
}

__global__ void __launch_bounds__(kNttWsThreads, 1) ntt_last_ws_kernel(const uint4* __restrict__ m,
                                                                      uint4* __restrict__ cw, PassParams p,
                                                                      const TwiddleView* __restrict__ tw) {
  extern __shared__ uint4 sm[];
  const int n = p.n, T = p.T;
  const uint32_t tsize = 1u << T;
  const uint32_t tiles_per_coset = 1u << (n - T);
  const uint32_t tiles = tiles_per_coset << p.log2_c;
  const uint32_t nthr = 32u * (uint32_t)p.ntt_warps;
  const uint32_t K = blockIdx.x < tiles ? (tiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;  // this block's tiles
  if (threadIdx.x < nthr) {
    // butterfly warps
    const uint32_t t = threadIdx.x;
    for (uint32_t k = 0; k < K; ++k) {
      const uint32_t tile = blockIdx.x + k * gridDim.x;
      const uint32_t j = tile >> (n - T), hi = tile & (tiles_per_coset - 1);
      const size_t q0 = ((size_t)j << n) + ((size_t)hi << T);
      uint4* buf = sm + ((k & 1u) << T);
      if (k >= 2) named_sync(4 + (int)(k & 1u), kNttWsThreads);  // the hashing warps are done with it
      if (p.first) {  // a single pass (T = n): m bit-reversed into the tile
        for (uint32_t i = t; i < tsize; i += nthr) buf[brev_bits(i, T)] = m[i];
      } else {
        for (uint32_t i = t; i < tsize; i += nthr) buf[i] = cw[q0 + i];
      }
      named_sync(1, (int)nthr);
      for (int l = T - 1; l >= 0; --l) {
        const uint4* __restrict__ lo_tab = tw->lo[l];
        const uint4* __restrict__ hi_tab = tw->hi[l];
        const uint32_t kbase = (j << (n - 1 - l)) | (hi << (T - 1 - l));
        const uint32_t lmask = (1u << l) - 1u;
        for (uint32_t bi = t; bi < (tsize >> 1); bi += nthr) {
          const uint32_t a = ((bi >> l) << (l + 1)) | (bi & lmask);
          const uint32_t Kt = kbase | (bi >> l);
          uint4 x0 = buf[a], x1 = buf[a + (1u << l)];
          if (Kt != 0) x0 = gf_add(x0, gf_mul(x1, gf_add(lo_tab[Kt & 4095u], hi_tab[Kt >> 12])));
          x1 = gf_add(x1, x0);
          buf[a] = x0;
          buf[a + (1u << l)] = x1;
        }
        named_sync(1, (int)nthr);
      }
      for (uint32_t i = t; i < tsize; i += nthr) cw[q0 + i] = buf[i];
      named_arrive(2 + (int)(k & 1u), kNttWsThreads);  // tile k is ready to hash
    }
  } else {
    // hashing warps
    const uint32_t t = threadIdx.x - nthr, hthr = blockDim.x - nthr;
    for (uint32_t k = 0; k < K; ++k) {
      const uint32_t tile = blockIdx.x + k * gridDim.x;
      const uint32_t j = tile >> (n - T), hi = tile & (tiles_per_coset - 1);
      const size_t q0 = ((size_t)j << n) + ((size_t)hi << T);
      const uint4* buf = sm + ((k & 1u) << T);
      named_sync(2 + (int)(k & 1u), kNttWsThreads);
      for (uint32_t kk = t; kk < (tsize >> 1); kk += hthr) {
        const uint4 e0 = buf[2 * kk], e1 = buf[2 * kk + 1];
        const size_t q = q0 + 2 * kk;
        store_digest(p.leaves, q, hash_elem(e0));
        store_digest(p.leaves, q + 1, hash_elem(e1));
        store_digest(p.pair_leaves, q >> 1, hash_pair(e0, e1));
      }
      if (k + 2 < K) named_arrive(4 + (int)(k & 1u), kNttWsThreads);  // the butterfly warps may refill it
    }
  }
}

// n = 0: every coset is the single row of m.
__global__ void replicate_kernel(const uint4* __restrict__ m, uint4* __restrict__ cw, size_t c, size_t w) {
  for (size_t i = threadIdx.x; i < c * w; i += blockDim.x) cw[i] = m[i % w];
}

void init_kernel_attributes() {
  static std::atomic<uint64_t> done{0};
  int dev = 0;
  cudaGetDevice(&dev);
  const uint64_t bit = 1ull << (dev & 63);
  if (done.load() & bit) return;
  cudaFuncSetAttribute(ntt_pass_kernel<false, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)(sizeof(uint4) << kNttMaxT));
  cudaFuncSetAttribute(ntt_pass_kernel<false, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)(sizeof(uint4) << kNttMaxT));
  cudaFuncSetAttribute(ntt_pass_kernel<false, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)(sizeof(uint4) << kNttMaxT));
  cudaFuncSetAttribute(ntt_pass_kernel<false, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)(sizeof(uint4) << kNttMaxT));
  cudaFuncSetAttribute(ntt_pass_kernel<false, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)(sizeof(uint4) << kNttMaxT));
  cudaFuncSetAttribute(ntt_pass_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)(sizeof(uint4) << kNttMaxT));
  cudaFuncSetAttribute(ntt_reg_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)(sizeof(uint4) << kNttRegMaxT));
  cudaFuncSetAttribute(ntt_reg_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)(sizeof(uint4) << kNttRegMaxT));
  cudaFuncSetAttribute(ntt_last_ws_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)(2 * sizeof(uint4) << kNttWsMaxT));
  done.fetch_or(bit);
}

bool tune_valid(const Tune& t) {
  const bool threads_ok = t.ntt_threads == 128 || t.ntt_threads == 256 || t.ntt_threads == 512;
  const bool top_ok = t.top_nodes >= 64 && t.top_nodes <= 4096 && (t.top_nodes & (t.top_nodes - 1)) == 0;
  return threads_ok && t.ntt_max_T >= 6 && t.ntt_max_T <= kNttMaxT && top_ok && t.tail_log >= 1 &&
         t.tail_log <= kTailMaxLeavesLog && t.subtree_log >= 10 && t.subtree_log <= 20 && t.ntt_kind >= 0 &&
         t.ntt_kind <= 3 && t.gf_mix >= 0 && t.gf_mix <= 4 && t.ntt_ws_warps >= 2 && t.ntt_ws_warps <= 14;
}

static void launch_ntt_nohash(dim3 grid, int threads, size_t smem, cudaStream_t s, const uint4* m, uint4* cw,
                              const PassParams& p, const TwiddleView* tw, int gf_mix) {
  switch (gf_mix) {
    case 1: ntt_pass_kernel<false, 1><<<grid, threads, smem, s>>>(m, cw, p, tw); break;
    case 2: ntt_pass_kernel<false, 2><<<grid, threads, smem, s>>>(m, cw, p, tw); break;
    case 3: ntt_pass_kernel<false, 3><<<grid, threads, smem, s>>>(m, cw, p, tw); break;
    case 4: ntt_pass_kernel<false, 4><<<grid, threads, smem, s>>>(m, cw, p, tw); break;
    default: ntt_pass_kernel<false, 0><<<grid, threads, smem, s>>>(m, cw, p, tw); break;
  }
}

// Two-pass encode with the cosets pipelined (NTT kind 3): the first pass of
// coset 0 on st; then the first passes of the other cosets on st2 (a
// high-priority stream, so their blocks are dispatched as the running blocks
// retire) while the last pass of coset 0 — its leaf hashing ALU-bound where
// the first pass is multiplier-bound — runs on st; then the last passes of
// the other cosets.  Co-resident blocks of the two passes keep both pipes of
// an SM busy.
static cudaError_t encode_pipelined(const uint4* m, uint4* cw, int n, int log2_c, const TwiddleView* tw,
                                    cudaStream_t st, cudaStream_t st2, cudaEvent_t ev_a, cudaEvent_t ev_b,
                                    uint4* leaves, uint4* pair_leaves, const Tune& tune, int T0,
                                    cudaEvent_t last_a, cudaEvent_t last_b) {
  const size_t c = (size_t)1 << log2_c;
  const int T1 = n - T0;
  auto params = [&](int first, int T, int coset0) {
    PassParams p{};
    p.n = n;
    p.T = T;
    p.s_lo = first ? n - T : 0;
    p.first = first;
    p.width = 1;
    p.leaves = first ? nullptr : leaves;
    p.pair_leaves = first ? nullptr : pair_leaves;
    p.log2_c = log2_c;
    p.coset0 = coset0;
    return p;
  };
  auto launch = [&](const PassParams& p, unsigned blocks, cudaStream_t s) {
    const int threads = std::max(32, std::min(tune.ntt_threads, 1 << (p.T - 1)));
    if (p.leaves)
      ntt_pass_kernel<true><<<blocks, threads, sizeof(uint4) << p.T, s>>>(m, cw, p, tw);
    else
      launch_ntt_nohash(dim3(blocks), threads, sizeof(uint4) << p.T, s, m, cw, p, tw, tune.gf_mix);
    COUNT_LAUNCH();
    return cudaGetLastError();
  };
  const unsigned tiles0 = 1u << (n - T0), tiles1 = 1u << (n - T1);
  cudaError_t e = launch(params(1, T0, 0), tiles0, st);
  if (e == cudaSuccess) e = cudaEventRecord(ev_a, st);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(st2, ev_a, 0);
  if (e == cudaSuccess && c > 1) e = launch(params(1, T0, 1), (unsigned)((c - 1) * tiles0), st2);
  if (e == cudaSuccess) e = cudaEventRecord(ev_b, st2);
  if (e == cudaSuccess && last_a) e = cudaEventRecord(last_a, st);
  if (e == cudaSuccess) e = launch(params(0, T1, 0), tiles1, st);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(st, ev_b, 0);
  if (e == cudaSuccess && c > 1) e = launch(params(0, T1, 1), (unsigned)((c - 1) * tiles1), st);
  if (e == cudaSuccess && last_b) e = cudaEventRecord(last_b, st);
  return e;
}

cudaError_t launch_encode(const uint4* m, uint4* cw, int n, int log2_c, size_t width, const TwiddleView* tw,
                          cudaStream_t st, uint4* leaves, uint4* pair_leaves, const Tune& tune,
                          const cudaEvent_t* slice_ready, int slices, cudaStream_t st2, cudaEvent_t ev_a,
                          cudaEvent_t ev_b, cudaEvent_t last_a, cudaEvent_t last_b) {
  if (width == 0 || width > 65535 || (width != 1 && (leaves || pair_leaves))) return cudaErrorInvalidValue;
  if (!tune_valid(tune)) return cudaErrorInvalidValue;
  const size_t c = (size_t)1 << log2_c;
  if (n == 0) {
    if (last_a) cudaEventRecord(last_a, st);
    replicate_kernel<<<1, 128, 0, st>>>(m, cw, c, width);
    COUNT_LAUNCH();
    if (last_b) cudaEventRecord(last_b, st);
    return cudaGetLastError();
  }
  init_kernel_attributes();
  // Fewest passes whose tiles fit 2^ntt_max_T, then more (smaller tiles) while
  // a pass would have fewer blocks than SMs and tiles stay >= 2^5.
  int passes = (n + tune.ntt_max_T - 1) / tune.ntt_max_T;
  while (passes < n) {
    const int T = (n + passes - 1) / passes;
    const int T_next = (n + passes) / (passes + 1);
    if ((c << (n - T)) >= (size_t)num_sms() || T_next < 5) break;
    ++passes;
  }
  if (tune.ntt_kind == 3 && passes == 2 && leaves && pair_leaves && slices == 0 && st2 && ev_a && ev_b)
    return encode_pipelined(m, cw, n, log2_c, tw, st, st2, ev_a, ev_b, leaves, pair_leaves, tune, (n + 1) / 2,
                            last_a, last_b);
  int top = n;
  for (int pidx = 0; pidx < passes; ++pidx) {
    const int remaining = passes - pidx;
    const int T = (top + remaining - 1) / remaining;  // balanced split, largest first
    PassParams p;
    p.n = n;
    p.T = T;
    p.s_lo = top - T;
    p.first = (pidx == 0);
    p.width = (int)width;
    const bool last = (pidx == passes - 1);
    p.leaves = last ? leaves : nullptr;
    p.pair_leaves = last ? pair_leaves : nullptr;
    p.log2_c = log2_c;
    p.ntt_warps = tune.ntt_ws_warps;
    p.coset0 = 0;
    // one butterfly per thread and layer at most: 2^(T-1) threads, >= one warp
    const int threads = std::max(32, std::min(tune.ntt_threads, 1 << (T - 1)));
    const uint32_t tiles = 1u << (n - T);
    // the first pass may start on each slice of the input as it arrives
    // (slices a power of two, at most the tiles per coset)
    const bool split = p.first && slices > 0 && (slices & (slices - 1)) == 0 && tiles >= (uint32_t)slices;
    const int pieces = split ? slices : 1;
    int piece_log = 0;
    while ((1 << piece_log) < pieces) ++piece_log;
    if (p.first && slices > 0 && !split) {
      cudaError_t e = cudaStreamWaitEvent(st, slice_ready[slices - 1], 0);  // copies are in order
      if (e != cudaSuccess) return e;
    }
    // Pieces alternate between st and st2 (when given): launches on one
    // stream run one after another, and a piece of a few hundred blocks ends
    // in a mostly idle wave; on two streams the next piece fills it.
    const bool two = pieces > 1 && st2 && ev_a && ev_b;
    if (last && last_a) {  // the last pass is one launch on st (it never takes slices)
      cudaError_t e = cudaEventRecord(last_a, st);
      if (e != cudaSuccess) return e;
    }
    if (two) {
      cudaError_t e = cudaEventRecord(ev_a, st);  // st2 after everything before the pass on st
      if (e == cudaSuccess) e = cudaStreamWaitEvent(st2, ev_a, 0);
      if (e != cudaSuccess) return e;
    }
    for (int piece = 0; piece < pieces; ++piece) {
      cudaStream_t sp = (two && (piece & 1)) ? st2 : st;
      if (pieces > 1) {
        cudaError_t e = cudaStreamWaitEvent(sp, slice_ready[piece], 0);
        if (e != cudaSuccess) return e;
      }
      p.piece_log = piece_log;
      p.piece = piece;
      const dim3 grid((unsigned)(c * (tiles >> piece_log)), (unsigned)width);
      const bool reg = tune.ntt_kind == 1 && T >= kNttRegMinT && T <= kNttRegMaxT;
      const bool ws = tune.ntt_kind == 2 && p.leaves && pieces == 1 && T <= kNttWsMaxT && T >= 6;
      if (ws)
        ntt_last_ws_kernel<<<(unsigned)std::min<size_t>(c * tiles, (size_t)num_sms()), kNttWsThreads,
                             2 * sizeof(uint4) << T, sp>>>(m, cw, p, tw);
      else if (reg && p.leaves)
        ntt_reg_kernel<true><<<grid, 1 << (T - 4), sizeof(uint4) << T, sp>>>(m, cw, p, tw);
      else if (reg)
        ntt_reg_kernel<false><<<grid, 1 << (T - 4), sizeof(uint4) << T, sp>>>(m, cw, p, tw);
      else if (p.leaves)
        ntt_pass_kernel<true><<<grid, threads, sizeof(uint4) << T, sp>>>(m, cw, p, tw);
      else
        launch_ntt_nohash(grid, threads, sizeof(uint4) << T, sp, m, cw, p, tw, tune.gf_mix);
      COUNT_LAUNCH();
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return e;
    }
    if (two) {  // the rest of the encode waits for the pieces on st2
      cudaError_t e = cudaEventRecord(ev_b, st2);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(st, ev_b, 0);
      if (e != cudaSuccess) return e;
    }
    if (last && last_b) {
      cudaError_t e = cudaEventRecord(last_b, st);
      if (e != cudaSuccess) return e;
    }
    top -= T;
  }
  return cudaSuccess;
}

// ---------------------------------------------------------------------------
// Merkle trees (Keccak256MerkleTreeMmcs, p3/src/merkle_tree.rs:8-21).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) leaves_elem_kernel(const uint4* __restrict__ cw, uint4* __restrict__ leaves,
                                                          size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    store_digest(leaves, i, hash_elem(cw[i]));
}

// Folded-codeword leaf s = H(pi[2s] || pi[2s+1]): the row (pi[j], pi[j+n_i])
// of the width-2 matrix committed at basefold.rs:350-355, in NTT order.
__global__ void __launch_bounds__(128) leaves_pair_kernel(const uint4* __restrict__ pi, uint4* __restrict__ leaves,
                                                          size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    store_digest(leaves, i, hash_pair(pi[2 * i], pi[2 * i + 1]));
}

__global__ void __launch_bounds__(128) level_kernel(const uint4* __restrict__ prev, uint4* __restrict__ next,
                                                    size_t n_next) {
  for (size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x; s < n_next; s += (size_t)gridDim.x * blockDim.x)
    store_digest(next, s, hash_node(load_digest(prev, s), load_digest(prev, s + n_next)));
}

// The remaining levels of a small tree, in one block; the root is also
// copied to `root_out` when given.
__global__ void __launch_bounds__(256) tree_top_kernel(uint4* level, size_t n, uint4* root_out) {
  const WarpKeccak wk;
  const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  uint4* cur = level;
  while (n > 1) {
    const size_t h = n >> 1;
    uint4* nxt = cur + 2 * n;
    if (h <= (size_t)nwarps) {  // latency-bound: one warp per node
      for (size_t s = warp; s < h; s += nwarps) warp_hash_node(wk, cur, s, h, nxt);
    } else {
      for (size_t s = threadIdx.x; s < h; s += blockDim.x)
        store_digest(nxt, s, hash_node(load_digest(cur, s), load_digest(cur, s + h)));
    }
    __syncthreads();
    cur = nxt;
    n = h;
  }
  if (root_out && threadIdx.x == 0) store_digest(root_out, 0, load_digest(cur, 0));
}

// Leaf of a row of `width` elements: keccak256 of its 16*width bytes
// (GenericHasher over the row's bincode, p3/src/symmetric.rs:16-25), any
// number of 136-byte blocks; a warp stages the blocks of 32 rows through
// shared memory (keccak_rows_warp) so that its loads read whole row runs.
__global__ void __launch_bounds__(128) leaves_rows_kernel(const uint4* __restrict__ cw, uint4* __restrict__ leaves,
                                                          size_t n, size_t width) {
  __shared__ uint32_t stage[4][32 * kStagePitch];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t* words = reinterpret_cast<const uint32_t*>(cw);
  const size_t row_words = 4 * width;
  auto word_at = [&](size_t row, uint32_t i) { return words[row * row_words + i]; };
  for (size_t r0 = ((size_t)blockIdx.x * 4 + warp) * 32; r0 < n; r0 += (size_t)gridDim.x * 128) {
    const Digest dg = keccak_rows_warp(stage[warp], r0, n, (uint32_t)row_words, word_at);
    if (r0 + lane < n) store_digest(leaves, r0 + lane, dg);
  }
}

cudaError_t launch_leaves_elem(const uint4* cw, uint4* leaves, size_t n, size_t width, cudaStream_t st) {
  if (width == 1)
    leaves_elem_kernel<<<grid_short(n, 128), 128, 0, st>>>(cw, leaves, n);
  else
    leaves_rows_kernel<<<grid_short(n, 128), 128, 0, st>>>(cw, leaves, n, width);
  COUNT_LAUNCH();
  return cudaGetLastError();
}

cudaError_t launch_leaves_pair(const uint4* pi, uint4* leaves, size_t n, cudaStream_t st) {
  leaves_pair_kernel<<<grid_short(n, 128), 128, 0, st>>>(pi, leaves, n);
  COUNT_LAUNCH();
  return cudaGetLastError();
}

// Levels 1..k above `level` (n nodes), stored one after another after it, in
// one launch.  Block b owns the top nodes [b M, (b+1) M) of level k
// (n >> k nodes), M = 2^(9-k), and at level k - j the runs s + m (n >> k),
// m < 2^j, of their subtrees: node i of a level has children i and
// i + (its level's size) below, so a block only reads what it wrote and
// __syncthreads separates the levels.  Level 1 has one node per thread.
constexpr int kSubtreeThreads = 256;
__global__ void __launch_bounds__(kSubtreeThreads) subtree_kernel(uint4* level, size_t n, int k) {
  const size_t nk = n >> k;
  const int log_m = 9 - k;  // M = 2^log_m top nodes per block
  const size_t a = (size_t)blockIdx.x << log_m;
  uint4* cur = level;
  size_t ncur = n;
  for (int j = 1; j <= k; ++j) {
    const size_t h = ncur >> 1;
    uint4* nxt = cur + 2 * ncur;
    const int per = 1 << (log_m + k - j);  // this block's nodes at level j
    for (int t = threadIdx.x; t < per; t += blockDim.x) {
      const size_t s = a + (size_t)(t & ((1 << log_m) - 1)) + (size_t)(t >> log_m) * nk;
      store_digest(nxt, s, hash_node(load_digest(cur, s), load_digest(cur, s + h)));
    }
    __syncthreads();
    cur = nxt;
    ncur = h;
  }
}

cudaError_t launch_tree(uint4* leaves, size_t n, cudaStream_t st, uint4* root_out, const Tune& tune) {
  uint4* cur = leaves;
  const size_t top_nodes = (size_t)tune.top_nodes;
  const size_t subtree_max = (size_t)1 << tune.subtree_log;  // larger levels: one launch each
  while (n > top_nodes) {
    if (n <= subtree_max && n >= 1024) {  // the latency-bound middle levels in one launch
      int k = 0;
      size_t m = n;
      while (m > top_nodes && k < 9) {
        m >>= 1;
        ++k;
      }
      subtree_kernel<<<(unsigned)(n >> 9), kSubtreeThreads, 0, st>>>(cur, n, k);
      COUNT_LAUNCH();
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return e;
      for (int j = 0; j < k; ++j) {
        cur += 2 * n;
        n >>= 1;
      }
      continue;
    }
    const size_t h = n >> 1;
    uint4* nxt = cur + 2 * n;
    level_kernel<<<grid_short(h, 128), 128, 0, st>>>(cur, nxt, h);
    COUNT_LAUNCH();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    cur = nxt;
    n = h;
  }
  if (n > 1 || root_out) {
    tree_top_kernel<<<1, 256, 0, st>>>(cur, n, root_out);
    COUNT_LAUNCH();
  }
  return cudaGetLastError();
}

__device__ __forceinline__ uint64_t splitmix64(uint64_t& x) {
  uint64_t z = (x += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

__global__ void fill_random_kernel(uint4* out, size_t n, uint64_t seed) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    uint64_t x = seed ^ (i * 0xd1342543de82ef95ull);
    const uint64_t a = splitmix64(x), b = splitmix64(x);
    out[i] = make_uint4((uint32_t)a, (uint32_t)(a >> 32), (uint32_t)b, (uint32_t)(b >> 32));
  }
}

cudaError_t launch_fill_random(uint4* out, size_t n, uint64_t seed, cudaStream_t st) {
  fill_random_kernel<<<grid_for(n, 256), 256, 0, st>>>(out, n, seed);
  COUNT_LAUNCH();
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Sumcheck side of `open` (sumcheck/src/function/eval_impr.rs,
// p3/src/poly/multilinear.rs).
// ---------------------------------------------------------------------------

// eq table over nv <= 16 variables in one block (MultiPoly::eq via
// eq_expand, multilinear.rs:41-64,216-222): bit i of the index <-> r[i].
__global__ void __launch_bounds__(256) eq_small_kernel(const uint4* __restrict__ r, int nv, uint4* out) {
  if (threadIdx.x == 0) out[0] = gf_one();
  __syncthreads();
  for (int i = 0; i < nv; ++i) {
    const uint32_t h = 1u << i;
    const uint4 ri = r[i];
    for (uint32_t k = threadIdx.x; k < h; k += blockDim.x) {
      const uint4 lo = out[k];
      const uint4 hv = gf_mul(lo, ri);
      out[h + k] = hv;
      out[k] = gf_add(lo, hv);
    }
    __syncthreads();
  }
}

// eq(r)[b] = eq(r_lo)[b & mask] * eq(r_hi)[b >> a]
__global__ void eq_combine_kernel(const uint4* __restrict__ lo, int a, const uint4* __restrict__ hi,
                                  uint4* __restrict__ out, size_t n) {
  const size_t mask = ((size_t)1 << a) - 1;
  for (size_t b = (size_t)blockIdx.x * blockDim.x + threadIdx.x; b < n; b += (size_t)gridDim.x * blockDim.x)
    out[b] = gf_mul(lo[b & mask], hi[b >> a]);
}

constexpr int kEqSmall = 12;

cudaError_t launch_eq_table(const uint4* r, int nvars, uint4* out, uint4* tmp_lo, uint4* tmp_hi, cudaStream_t st) {
  if (nvars <= kEqSmall) {
    eq_small_kernel<<<1, 256, 0, st>>>(r, nvars, out);
    COUNT_LAUNCH();
    return cudaGetLastError();
  }
  if (nvars - kEqSmall > 16) return cudaErrorInvalidValue;
  eq_small_kernel<<<1, 256, 0, st>>>(r, kEqSmall, tmp_lo);
  COUNT_LAUNCH();
  eq_small_kernel<<<1, 256, 0, st>>>(r + kEqSmall, nvars - kEqSmall, tmp_hi);
  COUNT_LAUNCH();
  const size_t n = (size_t)1 << nvars;
  eq_combine_kernel<<<grid_for(n, 256), 256, 0, st>>>(tmp_lo, kEqSmall, tmp_hi, out, n);
  COUNT_LAUNCH();
  return cudaGetLastError();
}

// acc ^= sum_i x[i] * y[i]
__global__ void __launch_bounds__(256) dot_xor_kernel(const uint4* __restrict__ x, const uint4* __restrict__ y,
                                                      size_t n, uint32_t* acc) {
  __shared__ uint4 scratch[32];
  uint64_t sum[4] = {0, 0, 0, 0};  // unreduced: one reduction per thread (GF(2)-linear)
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    gf_clmul_acc(x[i], y[i], sum);
  uint4 s = gf_reduce256(sum[0], sum[1], sum[2], sum[3]);
  s = block_xor(s, scratch);
  if (threadIdx.x == 0) atomic_xor4(acc, s);
}

cudaError_t launch_dot_xor(const uint4* x, const uint4* y, size_t n, uint32_t* acc, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  dot_xor_kernel<<<grid_for(n, 256), 256, 0, st>>>(x, y, n, acc);
  COUNT_LAUNCH();
  return cudaGetLastError();
}

// fold + interpolate (binary_reed_solomon.rs:88-109) in NTT order:
// out[t] = lo' + (hi' - lo') r with hi' = hi + lo, lo' = lo + hi' tw[t].
__global__ void __launch_bounds__(256) fold_kernel(const uint4* __restrict__ pi, uint4* __restrict__ out,
                                                   size_t n_out, const uint4* __restrict__ tlo,
                                                   const uint4* __restrict__ thi, uint4 r, const uint4* xp) {
  if (xp) r = *xp;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n_out; t += (size_t)gridDim.x * blockDim.x) {
    const uint4 tw = gf_add(tlo[t & 4095], thi[t >> 12]);
    uint4 lo = pi[2 * t], hi = pi[2 * t + 1];
    hi = gf_add(hi, lo);
    lo = gf_add(lo, gf_mul(hi, tw));
    out[t] = gf_add(lo, gf_mul(gf_add(hi, lo), r));
  }
}

// Fold fused with the next round's leaf hashing: thread s folds the four
// entries pi[4s..4s+3] into out[2s], out[2s+1] and hashes that pair, which is
// leaf s of the next round's folded-codeword tree.
__global__ void __launch_bounds__(128) fold_leaves_kernel(const uint4* __restrict__ pi, uint4* __restrict__ out,
                                                          uint4* __restrict__ leaves, size_t n_leaves,
                                                          const uint4* __restrict__ tlo,
                                                          const uint4* __restrict__ thi, uint4 r,
                                                          const uint4* xp) {
  if (xp) r = *xp;
  for (size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x; s < n_leaves; s += (size_t)gridDim.x * blockDim.x) {
    uint4 f[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const size_t t = 2 * s + k;
      const uint4 tw = gf_add(tlo[t & 4095], thi[t >> 12]);
      uint4 lo = pi[2 * t], hi = pi[2 * t + 1];
      hi = gf_add(hi, lo);
      lo = gf_add(lo, gf_mul(hi, tw));
      f[k] = gf_add(lo, gf_mul(gf_add(hi, lo), r));
      out[t] = f[k];
    }
    store_digest(leaves, s, hash_pair(f[0], f[1]));
  }
}

cudaError_t launch_fold_leaves(const uint4* pi, uint4* out, uint4* leaves, size_t n_leaves, const uint4* tw_lo,
                               const uint4* tw_hi, uint4 r, cudaStream_t st, const uint4* xp) {
  fold_leaves_kernel<<<grid_short(n_leaves, 128), 128, 0, st>>>(pi, out, leaves, n_leaves, tw_lo, tw_hi, r, xp);
  COUNT_LAUNCH();
  return cudaGetLastError();
}

cudaError_t launch_fold(const uint4* pi, uint4* out, size_t n_out, const uint4* tw_lo, const uint4* tw_hi, uint4 r,
                        cudaStream_t st, const uint4* xp) {
  fold_kernel<<<grid_for(n_out, 256), 256, 0, st>>>(pi, out, n_out, tw_lo, tw_hi, r, xp);
  COUNT_LAUNCH();
  return cudaGetLastError();
}

// fix_last_var (multilinear.rs:183-198) fused with the next round's
// sum_b half_eq[b] * poly_lo[b] (eval_impr.rs:187-197).  In-place safe.
__global__ void __launch_bounds__(256, 3) fix_kernel(const uint4* in, uint4* out, size_t half, uint4 r,
                                                  const uint4* __restrict__ heq, size_t next_half, uint32_t* acc,
                                                  const uint4* xp) {
  __shared__ uint4 scratch[32];
  if (xp) r = *xp;
  uint4 s = make_uint4(0, 0, 0, 0);
  for (size_t b = (size_t)blockIdx.x * blockDim.x + threadIdx.x; b < half; b += (size_t)gridDim.x * blockDim.x) {
    const uint4 lo = in[b], hi = in[b + half];
    const uint4 v = gf_add(lo, gf_mul(r, gf_add(hi, lo)));
    out[b] = v;
    if (b < next_half) s = gf_add(s, gf_mul(heq[b], v));
  }
  if (acc) {
    s = block_xor(s, scratch);
    if (threadIdx.x == 0) atomic_xor4(acc, s);
  }
}

// One round of open in one launch: fold_blocks blocks fold the codeword and
// hash the next round's leaves (as fold_leaves_kernel), fix_blocks blocks fix
// the sumcheck polynomial and reduce for the next round (as fix_kernel).
// Both read the round's challenge.  The fix blocks are spread through the
// grid (block S q + S - 1 is fix block q, S = grid / fix_blocks), so their
// multiplier-bound work runs beside the ALU-bound fold blocks instead of
// alone at the end of the launch.
__global__ void __launch_bounds__(128) fold_fix_kernel(FoldFixParams p, uint4 r) {
  __shared__ uint4 scratch[32];
  if (p.xp) r = *p.xp;
  const unsigned S = p.fix_stride, q = blockIdx.x / S;
  const bool fix = blockIdx.x % S == S - 1 && q < p.fix_blocks;
  if (!fix) {
    const unsigned fb = blockIdx.x - (q < p.fix_blocks ? q : p.fix_blocks);  // fix blocks before this one
    const size_t stride = (size_t)p.fold_blocks * blockDim.x;
    for (size_t s = (size_t)fb * blockDim.x + threadIdx.x; s < p.n_leaves; s += stride) {
      uint4 f[2];
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        const size_t t = 2 * s + k;
        const uint4 tw = gf_add(p.tlo[t & 4095], p.thi[t >> 12]);
        uint4 lo = p.pi[2 * t], hi = p.pi[2 * t + 1];
        hi = gf_add(hi, lo);
        lo = gf_add(lo, gf_mul(hi, tw));
        f[k] = gf_add(lo, gf_mul(gf_add(hi, lo), r));
        p.pi_out[t] = f[k];
      }
      store_digest(p.leaves, s, hash_pair(f[0], f[1]));
    }
    return;
  }
  const size_t b0 = (size_t)q * blockDim.x + threadIdx.x;
  const size_t stride = (size_t)p.fix_blocks * blockDim.x;
  uint4 acc = make_uint4(0, 0, 0, 0);
  for (size_t b = b0; b < p.half; b += stride) {
    const uint4 lo = p.poly_in[b], hi = p.poly_in[b + p.half];
    const uint4 v = gf_add(lo, gf_mul(r, gf_add(hi, lo)));
    p.poly_out[b] = v;
    if (b < p.next_half) acc = gf_add(acc, gf_mul(p.heq[b], v));
  }
  acc = block_xor(acc, scratch);
  if (threadIdx.x == 0) atomic_xor4(p.acc, acc);
}

cudaError_t launch_fold_fix(const FoldFixParams& p0, uint4 r, cudaStream_t st) {
  FoldFixParams p = p0;
  p.fold_blocks = grid_short(p.n_leaves, 128);
  p.fix_blocks = grid_for(p.half, 128, 8);  // few blocks: each ends in one atomic
  p.fix_stride = (p.fold_blocks + p.fix_blocks) / p.fix_blocks;  // >= 2 while fold_blocks >= fix_blocks
  fold_fix_kernel<<<p.fold_blocks + p.fix_blocks, 128, 0, st>>>(p, r);
  COUNT_LAUNCH();
  return cudaGetLastError();
}

cudaError_t launch_fix(const uint4* in, uint4* out, size_t half, uint4 r, const uint4* heq, size_t next_half,
                       uint32_t* acc, cudaStream_t st, const uint4* xp) {
  fix_kernel<<<grid_for(half, 256), 256, 0, st>>>(in, out, half, r, heq, next_half, acc, xp);
  COUNT_LAUNCH();
  return cudaGetLastError();
}

// First fix_last_var of column `col` of a row-major matrix with `width`
// columns: out[b] = in[b] + r (in[b + half] - in[b]) on that column.
__global__ void __launch_bounds__(256) fix_column_kernel(const uint4* __restrict__ in, size_t width, size_t col,
                                                         uint4* __restrict__ out, size_t half, uint4 r,
                                                         const uint4* xp) {
  if (xp) r = *xp;
  for (size_t b = (size_t)blockIdx.x * blockDim.x + threadIdx.x; b < half; b += (size_t)gridDim.x * blockDim.x) {
    const uint4 lo = in[b * width + col], hi = in[(b + half) * width + col];
    out[b] = gf_add(lo, gf_mul(r, gf_add(hi, lo)));
  }
}

cudaError_t launch_fix_column(const uint4* in, size_t width, size_t col, uint4* out, size_t half, uint4 r,
                              cudaStream_t st, const uint4* xp) {
  fix_column_kernel<<<grid_for(half, 256), 256, 0, st>>>(in, width, col, out, half, r, xp);
  COUNT_LAUNCH();
  return cudaGetLastError();
}

__global__ void __launch_bounds__(512) eval_tail_kernel(uint4* buf, EvalTail p) {
  for (int k = p.nvars - 1; k >= 0; --k) {
    const uint32_t half = 1u << k;
    const uint4 r = p.rp ? p.rp[k] : p.r[k];
    // in place: thread b writes buf[b] (b < half) and reads buf[b], buf[b + half]
    for (uint32_t b = threadIdx.x; b < half; b += blockDim.x) {
      const uint4 lo = buf[b], hi = buf[b + half];
      buf[b] = gf_add(lo, gf_mul(r, gf_add(hi, lo)));
    }
    __syncthreads();
  }
}

cudaError_t launch_eval_tail(uint4* buf, const EvalTail& p, cudaStream_t st) {
  if (p.nvars < 0 || p.nvars > kEvalTailMaxVars) return cudaErrorInvalidValue;
  if (p.nvars == 0) return cudaSuccess;
  eval_tail_kernel<<<1, 512, 0, st>>>(buf, p);
  COUNT_LAUNCH();
  return cudaGetLastError();
}

// out[row] = sum_c scalars[c] * rows[row * width + c]   (basefold.rs:166-183).
// One thread per row: a block stages 128 rows x 8 columns (one 128-byte run
// per row and column chunk; a warp's loads cover four whole runs) in shared
// memory, pitch 9 elements so a warp's 16-byte reads of one column hit
// distinct banks.  The chunk's scalars are split once (gf_prepare) for all
// 128 rows, and a row sums its unreduced products and reduces once at the
// end (the reduction is GF(2)-linear).
constexpr int kCombRowsB = 128, kCombColsB = 8;
__global__ void __launch_bounds__(kCombRowsB) combine_rows_kernel(const uint4* __restrict__ rows, size_t nrows,
                                                                 size_t width, const uint4* __restrict__ scalars,
                                                                 uint4* __restrict__ out) {
  __shared__ uint4 stage[kCombRowsB * (kCombColsB + 1)];
  __shared__ uint4 prep[kCombColsB * 9];
  for (size_t r0 = (size_t)blockIdx.x * kCombRowsB; r0 < nrows; r0 += (size_t)gridDim.x * kCombRowsB) {
    uint64_t acc[4] = {0, 0, 0, 0};
    for (size_t c0 = 0; c0 < width; c0 += kCombColsB) {
      __syncthreads();  // the previous chunk's reads are done
      if (threadIdx.x < kCombColsB)
        gf_prepare(c0 + threadIdx.x < width ? scalars[c0 + threadIdx.x] : make_uint4(0, 0, 0, 0),
                   reinterpret_cast<uint32_t*>(prep + 9 * threadIdx.x));
      uint4 v[kCombColsB];
#pragma unroll
      for (int k = 0; k < kCombColsB; ++k) {  // element e = k 128 + t: row e / 8, column e % 8
        const uint32_t e = k * kCombRowsB + threadIdx.x;
        const size_t r = r0 + e / kCombColsB, c = c0 + e % kCombColsB;
        v[k] = (r < nrows && c < width) ? rows[r * width + c] : make_uint4(0, 0, 0, 0);
      }
#pragma unroll
      for (int k = 0; k < kCombColsB; ++k) {
        const uint32_t e = k * kCombRowsB + threadIdx.x;
        stage[(e / kCombColsB) * (kCombColsB + 1) + e % kCombColsB] = v[k];
      }
      __syncthreads();
      const uint4* row = stage + threadIdx.x * (kCombColsB + 1);
      const int nc = width - c0 < (size_t)kCombColsB ? (int)(width - c0) : kCombColsB;
      for (int c = 0; c < nc; ++c) gf_clmul_acc(row[c], prep + 9 * c, acc);
    }
    if (r0 + threadIdx.x < nrows) out[r0 + threadIdx.x] = gf_reduce256(acc[0], acc[1], acc[2], acc[3]);
  }
}

cudaError_t launch_combine_rows(const uint4* rows, size_t nrows, size_t width, const uint4* scalars, uint4* out,
                                cudaStream_t st) {
  combine_rows_kernel<<<grid_for(nrows, kCombRowsB), kCombRowsB, 0, st>>>(rows, nrows, width, scalars, out);
  COUNT_LAUNCH();
  return cudaGetLastError();
}

// Column values of a row-major matrix at a point: acc[c] ^= sum_r eq[r] data[r w + c]
// (basefold.rs:126-131: MultiPoly::evaluate of each column, here as the sum against the
// point's eq table, the same field value).  Lane = column (32 per blockIdx.y), warps and
// blocks over the rows, so a warp reads 32 consecutive elements of a row.
__global__ void __launch_bounds__(256) eval_cols_kernel(const uint4* __restrict__ eq, const uint4* __restrict__ data,
                                                       size_t rows, uint32_t w, uint32_t* acc) {
  __shared__ uint4 part[8][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t c = blockIdx.y * 32 + lane;
  uint64_t sum[4] = {0, 0, 0, 0};  // unreduced: one reduction per thread (GF(2)-linear)
  if (c < w)
    for (size_t r = (size_t)blockIdx.x * 8 + warp; r < rows; r += (size_t)gridDim.x * 8)
      gf_clmul_acc(data[r * w + c], eq[r], sum);
  part[warp][lane] = gf_reduce256(sum[0], sum[1], sum[2], sum[3]);
  __syncthreads();
  if (warp == 0 && c < w) {
    uint4 v = part[0][lane];
    for (int q = 1; q < 8; ++q) v = gf_add(v, part[q][lane]);
    atomic_xor4(acc + 4 * (size_t)c, v);
  }
}

cudaError_t launch_eval_cols(const uint4* eq, const uint4* data, size_t rows, size_t w, uint32_t* acc,
                             cudaStream_t st) {
  const size_t by = (w + 31) / 32;
  size_t bx = (rows + 63) / 64;
  const size_t cap = std::max<size_t>(1, (152 * 8 + by - 1) / by);
  if (bx > cap) bx = cap;
  eval_cols_kernel<<<dim3((unsigned)std::max<size_t>(bx, 1), (unsigned)by), 256, 0, st>>>(eq, data, rows,
                                                                                          (uint32_t)w, acc);
  COUNT_LAUNCH();
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Query openings (basefold.rs:200-222 over MerkleTreeMmcs::open_batch),
// written straight into the proof's bincode layout.  One block per query.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void put_u64(uint8_t* out, size_t off, uint64_t v) {
  *reinterpret_cast<uint64_t*>(out + off) = v;
}
__device__ __forceinline__ void put_elem(uint8_t* out, size_t off, uint4 v) {
  uint2* p = reinterpret_cast<uint2*>(out + off);
  p[0] = make_uint2(v.x, v.y);
  p[1] = make_uint2(v.z, v.w);
}
// Digest i of a tree (stored interleaved) as its 32 bytes.
__device__ __forceinline__ void put_digest(uint8_t* out, size_t off, const uint4* tree, size_t i) {
  const Digest d = digest_bytes(load_digest(tree, i));
  put_elem(out, off, d.lo);
  put_elem(out, off + 16, d.hi);
}

__global__ void gather_kernel(GatherParams p) {
  const int q = blockIdx.x;
  const uint64_t idx = p.idx[q];
  uint8_t* out = p.out + (size_t)q * p.block_bytes;
  const int L = p.L, d = p.d;
  const size_t w = p.width;
  // codeword row + path
  const uint64_t qpos = brev_bits64(idx, L);
  if (threadIdx.x == 0) {
    put_u64(out, 0, w);
    put_u64(out, 8 + 16 * w, (uint64_t)L);
  }
  for (size_t c = threadIdx.x; c < w; c += blockDim.x) put_elem(out, 8 + 16 * c, p.cw[qpos * w + c]);
  for (int k = threadIdx.x; k < L; k += blockDim.x) {
    const uint64_t m = (idx >> k) ^ 1ull;
    const size_t off_k = ((size_t)2 << L) - ((size_t)2 << (L - k));
    put_digest(out, 16 + 16 * w + 32 * (size_t)k, p.cw_tree, off_k + brev_bits64(m, L - k));
  }
  size_t off = 16 + 16 * w + 32 * (size_t)L;
  if (threadIdx.x == 0) put_u64(out, off, (uint64_t)d);
  off += 8;
  const size_t c = (size_t)1 << p.log2_c;
  for (int k = 0; k < d; ++k) {
    const int i = d - 1 - k;
    const int Li = p.log2_c + i + 1;  // log2 of the folded codeword size 2 n_i
    const uint64_t ni = (uint64_t)1 << (Li - 1);
    const uint64_t ii = idx & (ni - 1);
    const uint64_t sib = ((idx >> (Li - 1)) & 1) ^ 1;
    const uint4* pi;
    const uint4* tree;
    if (k == 0) {
      pi = p.pi_first;
      tree = p.pi_first_tree;
    } else {
      // input of round i = output of round i+1, after the outputs of rounds d-1 .. i+2
      pi = p.pi_fold + c * (((size_t)1 << d) - ((size_t)1 << (i + 2)));
      // trees of rounds d-2 .. i+1 come first
      tree = p.pi_trees +
             2 * ((c << 1) * (((size_t)1 << (d - 1)) - ((size_t)1 << (i + 1))) - (size_t)(d - 2 - i));
    }
    if (threadIdx.x == 0) {
      put_elem(out, off, pi[2 * brev_bits64(ii, Li - 1) + sib]);
      put_u64(out, off + 16, (uint64_t)(Li - 1));
    }
    for (int kk = threadIdx.x; kk < Li - 1; kk += blockDim.x) {
      const uint64_t m = (ii >> kk) ^ 1ull;
      const size_t loff = ((size_t)1 << Li) - ((size_t)1 << (Li - kk));
      put_digest(out, off + 24 + 32 * (size_t)kk, tree, loff + brev_bits64(m, Li - 1 - kk));
    }
    off += 24 + 32 * (size_t)(Li - 1);
  }
}

cudaError_t launch_gather(const GatherParams& p, cudaStream_t st) {
  if (p.nq == 0) return cudaSuccess;
  gather_kernel<<<p.nq, 64, 0, st>>>(p);
  COUNT_LAUNCH();
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Standalone product sumcheck (sumcheck/src/function/quadratic.rs:100-128 for
// two polynomials; the project's product-of-three extension for k = 3).
// acc[0..3] = c0, acc[4..7] = c2, acc[8..11] = c3.
// ---------------------------------------------------------------------------
struct PolyPtrs {
  const uint4* in[3];
  uint4* out[3];
};

// One GF(2^128) product as a call: the product-sumcheck kernels need several
// per term, and inlined the compiler interleaves them into 255 registers
// (12% occupancy); called one at a time they need about a third of that.
__device__ __noinline__ uint4 gf_mul_call(uint4 a, uint4 b) { return gf_mul(a, b); }

// Coefficients c0, c2 (and c3) of prod_k (lo_k + b_k X), b_k = hi_k - lo_k,
// summed into s0, s2, s3.  For K = 3 the cross term lo1 b2 + b1 lo2 is
// hi1 hi2 + lo1 lo2 + b1 b2 (characteristic 2, lo + b = hi), which reuses two
// products the term needs anyway: 7 products instead of 8.
template <int K>
__device__ __forceinline__ void prod_terms(const uint4 lo[K], const uint4 hi[K], uint4& s0, uint4& s2, uint4& s3) {
  if (K == 2) {
    s0 = gf_add(s0, gf_mul_call(lo[0], lo[1]));
    s2 = gf_add(s2, gf_mul_call(gf_add(hi[0], lo[0]), gf_add(hi[1], lo[1])));
  } else {
    const uint4 b0 = gf_add(hi[0], lo[0]), b1 = gf_add(hi[1], lo[1]), b2 = gf_add(hi[2], lo[2]);
    const uint4 b12 = gf_mul_call(b1, b2);
    const uint4 lo12 = gf_mul_call(lo[1], lo[2]);
    const uint4 cross = gf_add(gf_add(gf_mul_call(hi[1], hi[2]), lo12), b12);  // lo1 b2 + b1 lo2
    s0 = gf_add(s0, gf_mul_call(lo[0], lo12));
    s2 = gf_add(s2, gf_add(gf_mul_call(b0, cross), gf_mul_call(lo[0], b12)));
    s3 = gf_add(s3, gf_mul_call(b0, b12));
  }
}

template <int K>
__global__ void __launch_bounds__(256) prod_sums_kernel(PolyPtrs p, size_t half, uint32_t* acc) {
  __shared__ uint4 scratch[32];
  uint4 s0 = make_uint4(0, 0, 0, 0), s2 = s0, s3 = s0;
  for (size_t b = (size_t)blockIdx.x * blockDim.x + threadIdx.x; b < half; b += (size_t)gridDim.x * blockDim.x) {
    uint4 lo[K], hi[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      lo[k] = p.in[k][b];
      hi[k] = p.in[k][b + half];
    }
    prod_terms<K>(lo, hi, s0, s2, s3);
  }
  s0 = block_xor(s0, scratch);
  __syncthreads();
  s2 = block_xor(s2, scratch);
  __syncthreads();
  if (K == 3) s3 = block_xor(s3, scratch);
  if (threadIdx.x == 0) {
    atomic_xor4(acc, s0);
    atomic_xor4(acc + 4, s2);
    if (K == 3) atomic_xor4(acc + 8, s3);
  }
}

// Fix the top variable of every polynomial at r and accumulate the next
// round's sums.  Each thread produces the pair (b, b + half/2) of the fixed
// polynomials, which is exactly what the next round's sums need.
template <int K>
__global__ void __launch_bounds__(256, 2) prod_fix_kernel(PolyPtrs p, size_t half, uint4 r, uint32_t* acc,
                                                       const uint4* xp) {
  __shared__ uint4 scratch[32];
  if (xp) r = *xp;
  uint4 s0 = make_uint4(0, 0, 0, 0), s2 = s0, s3 = s0;
  const size_t nh = half >> 1;
  if (nh == 0) {  // last round: one output per polynomial
    if (blockIdx.x == 0 && threadIdx.x == 0) {
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const uint4 lo = p.in[k][0], hi = p.in[k][1];
        p.out[k][0] = gf_add(lo, gf_mul(r, gf_add(hi, lo)));
      }
    }
    return;
  }
  for (size_t b = (size_t)blockIdx.x * blockDim.x + threadIdx.x; b < nh; b += (size_t)gridDim.x * blockDim.x) {
    uint4 lo[K], hi[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const uint4 a0 = p.in[k][b], a1 = p.in[k][b + half];
      const uint4 c0 = p.in[k][b + nh], c1 = p.in[k][b + nh + half];
      lo[k] = gf_add(a0, gf_mul_call(r, gf_add(a1, a0)));
      hi[k] = gf_add(c0, gf_mul_call(r, gf_add(c1, c0)));
      p.out[k][b] = lo[k];
      p.out[k][b + nh] = hi[k];
    }
    prod_terms<K>(lo, hi, s0, s2, s3);
  }
  s0 = block_xor(s0, scratch);
  __syncthreads();
  s2 = block_xor(s2, scratch);
  __syncthreads();
  if (K == 3) s3 = block_xor(s3, scratch);
  if (threadIdx.x == 0) {
    atomic_xor4(acc, s0);
    atomic_xor4(acc + 4, s2);
    if (K == 3) atomic_xor4(acc + 8, s3);
  }
}

cudaError_t launch_prod_round_sums(const uint4* const* polys, int k, size_t half, uint32_t* acc, cudaStream_t st) {
  PolyPtrs p{};
  for (int i = 0; i < k; ++i) p.in[i] = polys[i];
  if (k == 2)
    prod_sums_kernel<2><<<grid_for(half, 256), 256, 0, st>>>(p, half, acc);
  else if (k == 3)
    prod_sums_kernel<3><<<grid_for(half, 256), 256, 0, st>>>(p, half, acc);
  else
    return cudaErrorInvalidValue;
  COUNT_LAUNCH();
  return cudaGetLastError();
}

cudaError_t launch_prod_fix(uint4* const* out, const uint4* const* in, int k, size_t half, uint4 r, size_t next_half,
                            uint32_t* acc, cudaStream_t st, const uint4* xp) {
  (void)next_half;
  PolyPtrs p{};
  for (int i = 0; i < k; ++i) {
    p.in[i] = in[i];
    p.out[i] = out[i];
  }
  const size_t work = half > 1 ? half / 2 : 1;
  if (k == 2)
    prod_fix_kernel<2><<<grid_for(work, 256), 256, 0, st>>>(p, half, r, acc, xp);
  else if (k == 3)
    prod_fix_kernel<3><<<grid_for(work, 256), 256, 0, st>>>(p, half, r, acc, xp);
  else
    return cudaErrorInvalidValue;
  COUNT_LAUNCH();
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Test hooks: raw field products and Keccak-f permutations.
// ---------------------------------------------------------------------------
__global__ void test_mul_kernel(const uint4* a, const uint4* b, uint4* out, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = gf_mul(a[i], b[i]);
}

__global__ void test_keccak_kernel(uint2* states, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    uint2 s[25];
#pragma unroll
    for (int k = 0; k < 25; ++k) s[k] = states[25 * i + k];
    keccak_f1600(s);
#pragma unroll
    for (int k = 0; k < 25; ++k) states[25 * i + k] = s[k];
  }
}

cudaError_t launch_test_mul(const uint4* a, const uint4* b, uint4* out, size_t n, cudaStream_t st) {
  test_mul_kernel<<<grid_for(n, 256), 256, 0, st>>>(a, b, out, n);
  COUNT_LAUNCH();
  return cudaGetLastError();
}

cudaError_t launch_test_keccak(uint2* states, size_t n, cudaStream_t st) {
  test_keccak_kernel<<<grid_for(n, 128), 128, 0, st>>>(states, n);
  COUNT_LAUNCH();
  return cudaGetLastError();
}

}  // namespace bf
