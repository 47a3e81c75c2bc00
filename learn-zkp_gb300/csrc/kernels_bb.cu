// CUDA kernels of Basefold over BabyBear with the multiplicative Reed–Solomon
// code (poly-commit/src/basefold/code/reed_solomon.rs) and the extension
// E = BinomialExtensionField<BabyBear, 5> for the open (sm_103a).
//
// The codeword is in natural order (the order Radix2DitParallel::dft_batch
// returns), so the folding pair of round i is (j, j + n_i) (code.rs:66-75)
// and the rows of every folded-codeword matrix are (pi[j], pi[j + half])
// (basefold.rs:350-355).  All of these kernels are memory- or hash-bound
// integer work: Montgomery products on the integer multiplier, Keccak on the
// ALU; nothing here is GEMM-shaped.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "bb.cuh"
#include "bb_internal.h"
#include "bf_internal.h"
#include "keccak.cuh"

namespace bf {

using bb::E5;

namespace {

__device__ __forceinline__ uint32_t brev_bits(uint64_t x, int bits) {
  return bits ? (uint32_t)(__brevll(x) >> (64 - bits)) : 0u;
}

__device__ __forceinline__ uint32_t mont_pow(uint32_t g, uint64_t e) {
  uint32_t r = bb::MONT_ONE;
  while (e) {
    if (e & 1) r = bb::mul(r, g);
    g = bb::mul(g, g);
    e >>= 1;
  }
  return r;
}

__device__ __forceinline__ E5 ld_e5(const uint32_t* p, size_t i) {
  E5 e;
#pragma unroll
  for (int k = 0; k < 5; ++k) e.c[k] = p[5 * i + k];
  return e;
}
__device__ __forceinline__ void st_e5(uint32_t* p, size_t i, const E5& e) {
#pragma unroll
  for (int k = 0; k < 5; ++k) p[5 * i + k] = e.c[k];
}

// keccak256 of one canonical BabyBear (4 bytes): lane 0 holds the value and
// the 0x01 padding byte, lane 16 the final 0x80 (interleaved lanes, as the
// trees store them).
__device__ __forceinline__ Digest hash_base(uint32_t canonical) {
  uint2 s[25];
#pragma unroll
  for (int i = 0; i < 25; ++i) s[i] = make_uint2(0, 0);
  s[0] = bi_from_lane(make_uint2(canonical, 0x01u));
  s[16].y ^= 0x80000000u;
  keccak_f1600_digest<true>(s);
  return digest_from_state(s);
}

// keccak256 of two extension elements, ten canonical BabyBears (40 bytes):
// a row of the folded-codeword matrix as ExtensionMmcs flattens it.
__device__ __forceinline__ Digest hash_pair_e5(const E5& a, const E5& b) {
  uint32_t w[10];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    w[k] = bb::from_mont(a.c[k]);
    w[5 + k] = bb::from_mont(b.c[k]);
  }
  uint2 s[25];
#pragma unroll
  for (int k = 0; k < 5; ++k) s[k] = bi_from_lane(make_uint2(w[2 * k], w[2 * k + 1]));
  keccak256_lanes<true>(s, 5);
  return digest_from_state(s);
}

__device__ __forceinline__ unsigned long long shfl_xor64(unsigned long long v, int o) {
  return __shfl_xor_sync(0xffffffffu, v, o);
}

// Five Montgomery coefficient sums of a warp reduced into every lane.
__device__ __forceinline__ void warp_sum5(unsigned long long s[5]) {
#pragma unroll
  for (int k = 0; k < 5; ++k)
    for (int o = 16; o > 0; o >>= 1) s[k] += shfl_xor64(s[k], o);
}

}  // namespace

// ---- setup -------------------------------------------------------------------
__global__ void bb_pow_table_kernel(uint32_t* out, size_t n, uint32_t g, uint32_t scale) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    out[k] = bb::mul(scale, mont_pow(g, k));
}

// Butterfly factors as Shoup pairs (w canonical, floor(w 2^32 / p)): the
// powers g^k, or the caller's canonical values (*bad set for one >= p).
__global__ void bb_pow_shoup_kernel(uint2* out, size_t n, uint32_t g) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    const uint32_t w = bb::from_mont(mont_pow(g, k));
    out[k] = make_uint2(w, bb::shoup_quot(w));
  }
}
__global__ void bb_shoup_from_kernel(const uint32_t* in, uint2* out, size_t n, uint32_t* bad) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    const uint32_t v = in[k];
    if (v >= bb::P) atomicOr(bad, 1u);
    const uint32_t w = v % bb::P;
    out[k] = make_uint2(w, bb::shoup_quot(w));
  }
}

// Single-row codeword (num_vars = log2_c = 0): the data in Montgomery form.
__global__ void bb_copy_mont_kernel(const uint32_t* in, uint32_t* out, size_t n, uint32_t* bad) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    const uint32_t v = in[k];
    if (v >= bb::P) atomicOr(bad, 1u);
    out[k] = bb::to_mont(v);
  }
}

// Montgomery words back to canonical.
__global__ void bb_from_mont_kernel(const uint32_t* in, uint32_t* out, size_t n) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    out[k] = bb::from_mont(in[k]);
}

// The generic code's fold constants: (2 t)^-1 of every t (Montgomery out),
// and a flag for a t that is zero or not canonical.
__global__ void bb_tinv_kernel(const uint32_t* ts, uint32_t* tinv, size_t n, uint32_t* bad) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    const uint32_t t = ts[k];
    if (t == 0 || t >= bb::P) atomicOr(bad, 1u);
    const uint32_t t2 = bb::to_mont(bb::add(t % bb::P, t % bb::P));
    tinv[k] = mont_pow(t2, bb::P - 2);  // Fermat: the inverse as a power, in Montgomery form
  }
}

// GenericRandomFoldableCode stage 0 (generic.rs:73-86, 120-125): every
// chunk of k_0 message rows times G_0, g_0[i][j] = i^j, into n_0 codeword
// rows: w[b n_0 + i] = sum_j i^j m[b k_0 + j], column by column.
__global__ void bb_stage0_kernel(const uint32_t* __restrict__ m, uint32_t* __restrict__ cw, size_t row0,
                                 size_t rows_out, uint32_t w, int log2_k0, int log2_n0, uint32_t* bad) {
  const size_t total = (row0 + rows_out) * w;
  for (size_t e = row0 * w + (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const size_t x = e / w, c = e - x * w;
    const size_t b = x >> log2_n0;
    const uint32_t i = (uint32_t)(x & (((size_t)1 << log2_n0) - 1));
    const uint32_t im = bb::to_mont(i);
    uint32_t pw = bb::MONT_ONE, acc = 0;
    for (int j = 0; j < (1 << log2_k0); ++j) {
      const uint32_t v = m[((b << log2_k0) + j) * w + c];
      if (v >= bb::P) atomicOr(bad, 1u);
      acc = bb::add(acc, bb::mul(pw, bb::to_mont(v)));
      pw = bb::mul(pw, im);
    }
    cw[e] = acc;
  }
}

// The same stage for k_0 <= 16: a thread takes one column of one chunk, holds
// its k_0 message values and writes the chunk's n_0 codeword rows.  Row i is
// V(i) for V(X) = sum_j m_j X^j, of degree below k_0 (g_0[i][j] = i^j), so only
// rows i < k_0 are dot products; the rest follow from the backward differences
// of V at k_0 - 1 (the (k_0 - 1)-th is constant), k_0 - 1 additions per row.
// The kernel parameter holds g_0[i][j] R^2 mod p for i < k_0, so the Montgomery
// reduction of a product with a canonical message value is the product's
// Montgomery form; two products sum below 2 p^2 < p 2^32 and share one
// reduction.
constexpr int kBbG0Max = 256;
struct BbG0 {
  uint32_t g[kBbG0Max];  // row i < k_0 at g[i k_0]
};

__device__ __forceinline__ uint32_t bb_reduce(uint64_t t) {  // t R^-1 mod p for t < p 2^32
  const uint32_t m = (uint32_t)t * bb::P_INV;
  const uint32_t d = (uint32_t)(t >> 32) - __umulhi(m, bb::P);
  return bb::umin(d, d + bb::P);
}

template <int K0>
__global__ void __launch_bounds__(256) bb_stage0_fast_kernel(const uint32_t* __restrict__ m, uint32_t* __restrict__ cw,
                                                            size_t chunk0, size_t chunks, uint32_t w, int n0,
                                                            const __grid_constant__ BbG0 g0, uint32_t* bad) {
  const size_t total = chunks * w;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    size_t b, c;
    if (total >> 32) {
      b = e / w;
      c = e - b * w;
    } else {  // 32-bit division where the index fits
      const uint32_t q = (uint32_t)e / w;
      b = q;
      c = (uint32_t)e - q * w;
    }
    b += chunk0;
    uint32_t v[K0];
    bool ok = true;
#pragma unroll
    for (int j = 0; j < K0; ++j) {
      v[j] = m[(b * K0 + j) * w + c];
      ok = ok && v[j] < bb::P;
    }
    if (!ok) atomicOr(bad, 1u);
    uint32_t* out = cw + b * (size_t)n0 * w + c;
    uint32_t y[K0];
#pragma unroll
    for (int i = 0; i < K0; ++i) {  // n_0 >= k_0
      const uint32_t* gi = g0.g + i * K0;
      uint32_t acc;
      if (K0 == 1) {
        acc = bb_reduce((uint64_t)v[0] * gi[0]);
      } else {
        acc = bb_reduce((uint64_t)v[0] * gi[0] + (uint64_t)v[1] * gi[1]);
#pragma unroll
        for (int j = 2; j < K0; j += 2)
          acc = bb::add(acc, bb_reduce((uint64_t)v[j] * gi[j] + (uint64_t)v[j + 1] * gi[j + 1]));
      }
      y[i] = acc;
      out[(size_t)i * w] = acc;
    }
    if (n0 > K0) {
      uint32_t D[K0];  // D[k] = k-th backward difference of V at the last row written
      D[0] = y[K0 - 1];
#pragma unroll
      for (int lev = 1; lev < K0; ++lev) {
#pragma unroll
        for (int i = K0 - 1; i >= lev; --i) y[i] = bb::sub(y[i], y[i - 1]);
        D[lev] = y[K0 - 1];
      }
#pragma unroll 1
      for (int i = K0; i < n0; ++i) {
#pragma unroll
        for (int k = K0 - 2; k >= 0; --k) D[k] = bb::add(D[k], D[k + 1]);
        out[(size_t)i * w] = D[0];
      }
    }
  }
}

// ---- encode: radix-2 DIT of the bit-reversed, zero-padded columns -------------
// encode_batch (reed_solomon.rs:71-75) = dft_batch(pad(bit_reverse_rows(m))).
// A DIT with natural-order output takes its input in bit-reversed order,
// where row x holds input row bitrev_L(x): data row x >> log2_c when the low
// log2_c bits of x are zero, else zero.  So the first pass reads the data
// rows spread out and no permutation pass is needed.
//
// One launch runs layers [s_lo, s_lo + T) (half-sizes 2^s) on tiles of 2^T
// rows x = (hi << (s_lo + T)) | (a << s_lo) | u, a < 2^T.  A block holds
// U = 2^lu consecutive u and C = 2^lc consecutive columns of each of those
// rows (column fastest, then u, then a), so that a warp's loads and stores
// cover runs of C U words.  The butterfly at half-size 2^s pairs rows that
// differ in bit s and multiplies by g_s^(x mod 2^s), g_s of order 2^(s+1).
struct BbPass {
  int s_lo, T, first, log2_c, lu, lc;
  uint32_t w, chunks;  // row width; column chunks of 2^lc
  int chunks_log;      // log2(chunks) when chunks is a power of two, else -1
  uint32_t block0;     // the launch runs blocks block0 + blockIdx.x (a first pass split by input slices)
};

// Tile coordinates of a block: the column chunk is the fastest-varying part
// of the (flat) block index, so the chunks of the same rows run together and
// read whole rows of the row-major matrix.
struct BbTile {
  uint32_t u_blk, c0;
  uint64_t hi;
  __device__ __forceinline__ BbTile(const BbPass& p) {
    const uint32_t b = blockIdx.x + p.block0;
    const uint32_t chunk = b % p.chunks, t = b / p.chunks;
    const uint32_t nub_log = (uint32_t)(p.s_lo - p.lu);
    u_blk = t & ((1u << nub_log) - 1u);
    hi = t >> nub_log;
    c0 = chunk << p.lc;
  }
  __device__ __forceinline__ uint64_t row(const BbPass& p, uint32_t e) const {
    const int ic = p.lu + p.lc;
    const uint32_t uu = (e >> p.lc) & ((1u << p.lu) - 1u), a = e >> ic;
    return (hi << (p.s_lo + p.T)) | ((uint64_t)a << p.s_lo) | ((u_blk << p.lu) | uu);
  }
};

// Tile load: eight independent global loads per thread in flight before any
// is used (the loop is latency-bound otherwise).  The first pass reads the
// spread data rows (canonical, checked and converted); later passes the
// codeword (Montgomery).
__device__ __forceinline__ void bb_tile_load(uint32_t* tile, const uint32_t* __restrict__ m, const uint32_t* cw,
                                             const BbPass& p, const BbTile& tl, uint32_t* bad) {
  const uint32_t tsize = 1u << (p.T + p.lu + p.lc);
  const uint64_t cmask = (1ull << p.log2_c) - 1ull;
  for (uint32_t base = 0; base < tsize; base += 8 * blockDim.x) {
    uint32_t v[8];
    bool ok[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const uint32_t e = base + k * blockDim.x + threadIdx.x;
      const uint64_t x = tl.row(p, e);
      const uint32_t c = tl.c0 + (e & ((1u << p.lc) - 1u));
      v[k] = 0;
      ok[k] = e < tsize && c < p.w;
      if (p.first) {
        ok[k] = ok[k] && (x & cmask) == 0;
        if (ok[k]) v[k] = m[(x >> p.log2_c) * p.w + c];
      } else if (ok[k]) {
        v[k] = cw[x * p.w + c];
      }
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const uint32_t e = base + k * blockDim.x + threadIdx.x;
      if (p.first && ok[k]) {
        if (v[k] >= bb::P) atomicOr(bad, 1u);
        v[k] = bb::to_mont(v[k]);
      }
      if (e < tsize) tile[e] = v[k];
    }
  }
}

__device__ __forceinline__ void bb_tile_store(const uint32_t* tile, uint32_t* cw, const BbPass& p, const BbTile& tl) {
  const uint32_t tsize = 1u << (p.T + p.lu + p.lc);
  for (uint32_t e = threadIdx.x; e < tsize; e += blockDim.x) {
    const uint32_t c = tl.c0 + (e & ((1u << p.lc) - 1u));
    if (c < p.w) cw[tl.row(p, e) * p.w + c] = tile[e];
  }
}

__global__ void __launch_bounds__(256) bb_dft_pass_kernel(const uint32_t* __restrict__ m, uint32_t* cw, BbPass p,
                                                         const uint2* __restrict__ tw, uint32_t* bad) {
  extern __shared__ uint32_t tile[];
  const int s_lo = p.s_lo, T = p.T, lu = p.lu, lc = p.lc, ic = lu + lc;
  const BbTile tl(p);
  const uint32_t u_blk = tl.u_blk;
  const uint32_t tsize = 1u << (T + ic);
  bb_tile_load(tile, m, cw, p, tl, bad);
  __syncthreads();
  for (int l = 0; l < T; ++l) {
    const int s = s_lo + l;
    const uint2* __restrict__ tws = tw + ((size_t)1 << s) - 1;
    const uint32_t lmask = (1u << l) - 1u;
    for (uint32_t e = threadIdx.x; e < (tsize >> 1); e += blockDim.x) {
      const uint32_t cu = e & ((1u << ic) - 1u), bi = e >> ic;
      const uint32_t a0 = ((bi >> l) << (l + 1)) | (bi & lmask);
      const uint32_t u = (u_blk << lu) | (cu >> lc);
      const uint32_t k = ((a0 & lmask) << s_lo) | u;
      const uint32_t i0 = (a0 << ic) | cu, i1 = i0 | (1u << (l + ic));
      const uint32_t v = bb::mul_shoup(tile[i1], tws[k]), x0 = tile[i0];
      tile[i0] = bb::add(x0, v);
      tile[i1] = bb::sub(x0, v);
    }
    __syncthreads();
  }
  bb_tile_store(tile, cw, p, tl);
}

// Register-blocked form of the same pass for tiles whose (u, column) slots
// fill a warp (lu + lc = 5): lane = slot, and a warp takes 2^R rows of its
// slots into registers and runs R layers there per round trip through
// shared memory (R = 4: two round trips per 8-layer pass instead of eight).
// Every shared-memory access of a warp is one 128-byte row run.
template <int R>
__device__ __forceinline__ void bb_reg_group(uint32_t* tile, uint32_t q, int l0, int s_lo, uint32_t u, uint32_t lane,
                                             const uint2* __restrict__ tw) {
  const uint32_t a_base = ((q >> l0) << (l0 + R)) | (q & ((1u << l0) - 1u));
  uint32_t v[1 << R];
#pragma unroll
  for (int j = 0; j < (1 << R); ++j) v[j] = tile[((a_base | ((uint32_t)j << l0)) << 5) | lane];
#pragma unroll
  for (int l = 0; l < R; ++l) {
    // The pair (j0, j0 | 2^l) at tile row a0 = a_base | j0 << l0 takes
    // g_s^((a0 mod 2^(l0 + l)) << s_lo | u): its low bits come from a_base and
    // from jj = j0 mod 2^l alone, so the layer needs 2^l distinct factors,
    // table entries base + jj 2^(l0 + s_lo).
    const int s = s_lo + l0 + l;
    const uint32_t lmask = (1u << (l0 + l)) - 1u;
    const uint32_t base = (1u << s) - 1u + (((a_base & lmask) << s_lo) | u);  // 2^L - 1 words in all, L <= 27
    uint2 tf[1 << (R - 1)];
#pragma unroll
    for (int jj = 0; jj < (1 << l); ++jj) tf[jj] = tw[base + ((uint32_t)jj << (l0 + s_lo))];
#pragma unroll
    for (int j0 = 0; j0 < (1 << R); ++j0) {
      if (j0 & (1 << l)) continue;
      const int j1 = j0 | (1 << l);
      const uint32_t x1 = bb::mul_shoup(v[j1], tf[j0 & ((1 << l) - 1)]), x0 = v[j0];
      v[j0] = bb::add(x0, x1);
      v[j1] = bb::sub(x0, x1);
    }
  }
#pragma unroll
  for (int j = 0; j < (1 << R); ++j) tile[((a_base | ((uint32_t)j << l0)) << 5) | lane] = v[j];
}

// Layers of the register group starting at l0 of a T-layer tile: up to 4,
// but no more than T - 3, so the group has 2^(T - r) >= 8 rows of work (one
// per warp) where the tile allows.
__device__ __forceinline__ int bb_group_layers(int T, int l0) {
  int r = T - l0 < 4 ? T - l0 : 4;
  const int cap = T - 3 > 1 ? T - 3 : 1;
  return r < cap ? r : cap;
}

__global__ void __launch_bounds__(256) bb_dft_reg_kernel(const uint32_t* __restrict__ m, uint32_t* cw, BbPass p,
                                                        const uint2* __restrict__ tw, uint32_t* bad) {
  extern __shared__ uint32_t tile[];
  const int s_lo = p.s_lo, T = p.T, lu = p.lu, lc = p.lc;  // lu + lc = 5
  const BbTile tl(p);
  bb_tile_load(tile, m, cw, p, tl, bad);
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const uint32_t u = (tl.u_blk << lu) | (lane >> lc);
  for (int l0 = 0, r; l0 < T; l0 += r) {
    r = bb_group_layers(T, l0);
    for (uint32_t q = warp; q < (1u << (T - r)); q += nwarps) {
      switch (r) {
        case 4: bb_reg_group<4>(tile, q, l0, s_lo, u, lane, tw); break;
        case 3: bb_reg_group<3>(tile, q, l0, s_lo, u, lane, tw); break;
        case 2: bb_reg_group<2>(tile, q, l0, s_lo, u, lane, tw); break;
        default: bb_reg_group<1>(tile, q, l0, s_lo, u, lane, tw); break;
      }
    }
    __syncthreads();
  }
  bb_tile_store(tile, cw, p, tl);
}

// The same pass for matrices wider than 16 columns (lc = 5, lu = 0): a tile is
// 2^T rows x 32 columns, row a of the tile at matrix row x0 + a 2^s_lo, run by
// eight warps.  The tile height is a template parameter, so the layer groups,
// each warp's share of the rows and every shared-memory offset are compile-time
// constants: the pass's instructions are the butterflies (Shoup products by
// the factor pairs), the factor loads and one pointer step per global access.
__host__ __device__ constexpr int bb_wide_group(int T, int l0) {  // layers of the register group starting at l0 (bb_group_layers)
  const int r = T - l0 < 4 ? T - l0 : 4;
  const int cap = T - 3 > 1 ? T - 3 : 1;
  return r < cap ? r : cap;
}

// One register group: layers L0 .. L0 + R - 1 of the tile.  Warp q of the
// 2^(T - R) groups takes rows a_base | j 2^L0 (j < 2^R) into registers.
template <int T, int L0, int R>
__device__ __forceinline__ void bb_wide_layers(uint32_t* tile, int s_lo, uint32_t u, uint32_t lane, uint32_t warp,
                                               const uint2* __restrict__ tw) {
  constexpr uint32_t kWork = 1u << (T - R);
  constexpr uint32_t kIters = kWork >= 8 ? kWork / 8 : 1;
#pragma unroll
  for (uint32_t it = 0; it < kIters; ++it) {
    const uint32_t q = warp + 8u * it;
    if (kWork < 8 && q >= kWork) return;
    const uint32_t qlo = q & ((1u << L0) - 1u);
    uint32_t* rp = tile + ((((q >> L0) << (L0 + R)) | qlo) << 5) + lane;
    uint32_t v[1 << R];
#pragma unroll
    for (int j = 0; j < (1 << R); ++j) v[j] = rp[j << (L0 + 5)];
    // the rows of the pair (j0, j0 | 2^l) agree below bit L0 + l with a_base,
    // whose bits L0 .. L0 + R - 1 are zero: the factor index is qlo 2^s_lo + u
    // plus jj 2^(L0 + s_lo) for jj = j0 mod 2^l
    const uint2* tq = tw + ((qlo << s_lo) | u);
    const uint32_t step = 1u << (L0 + s_lo);
#pragma unroll
    for (int l = 0; l < R; ++l) {
      const uint2* tl = tq + ((1u << (s_lo + L0 + l)) - 1u);
      uint2 tf[1 << (R - 1)];
#pragma unroll
      for (int jj = 0; jj < (1 << l); ++jj) tf[jj] = tl[jj * step];
#pragma unroll
      for (int j0 = 0; j0 < (1 << R); ++j0) {
        if (j0 & (1 << l)) continue;
        const int j1 = j0 | (1 << l);
        const uint32_t x1 = bb::mul_shoup(v[j1], tf[j0 & ((1 << l) - 1)]), x0 = v[j0];
        v[j0] = bb::add(x0, x1);
        v[j1] = bb::sub(x0, x1);
      }
    }
#pragma unroll
    for (int j = 0; j < (1 << R); ++j) rp[j << (L0 + 5)] = v[j];
  }
}

template <int T, int L0>
struct BbWideGroups {
  static __device__ __forceinline__ void run(uint32_t* tile, int s_lo, uint32_t u, uint32_t lane, uint32_t warp,
                                             const uint2* __restrict__ tw) {
    constexpr int R = bb_wide_group(T, L0);
    bb_wide_layers<T, L0, R>(tile, s_lo, u, lane, warp, tw);
    __syncthreads();
    BbWideGroups<T, L0 + R>::run(tile, s_lo, u, lane, warp, tw);
  }
};
template <int T>
struct BbWideGroups<T, T> {
  static __device__ __forceinline__ void run(uint32_t*, int, uint32_t, uint32_t, uint32_t, const uint2*) {}
};

template <int T>
__global__ void __launch_bounds__(256) bb_dft_wide_kernel(const uint32_t* __restrict__ m, uint32_t* cw, BbPass p,
                                                         const uint2* __restrict__ tw, uint32_t* bad) {
  extern __shared__ uint32_t tile[];
  constexpr uint32_t kRows = 1u << T;
  constexpr uint32_t kPer = kRows >= 8 ? kRows / 8 : 1;  // tile rows per warp (rows warp, warp + 8, ..)
  constexpr uint32_t kBatch = kPer < 8 ? kPer : 8;       // global loads in flight per thread
  const int s_lo = p.s_lo;
  const uint32_t b = blockIdx.x + p.block0;
  const uint32_t chunk = p.chunks_log >= 0 ? b & (p.chunks - 1u) : b % p.chunks;
  const uint32_t t = p.chunks_log >= 0 ? b >> p.chunks_log : b / p.chunks;
  const uint32_t u = t & ((1u << s_lo) - 1u);
  const uint64_t x0 = ((uint64_t)(t >> s_lo) << (s_lo + T)) | u;
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t c = (chunk << 5) + lane;
  const bool col_ok = c < p.w;
  const size_t w = p.w;
  const size_t step = ((size_t)8 << s_lo) * w;  // words between a thread's consecutive tile rows
  if (p.first) {  // spread rows: tile row a holds data row (x0 + a) >> log2_c when its low log2_c bits are 0
    const uint32_t cmask = (1u << p.log2_c) - 1u;
#pragma unroll 1
    for (uint32_t k0 = 0; k0 < kPer; k0 += kBatch) {
      uint32_t v[kBatch];
#pragma unroll
      for (uint32_t k = 0; k < kBatch; ++k) {
        const uint32_t a = warp + 8u * (k0 + k);
        const uint64_t x = x0 + a;
        v[k] = 0;
        if ((kRows >= 8 || a < kRows) && col_ok && ((uint32_t)x & cmask) == 0) v[k] = m[(x >> p.log2_c) * w + c];
      }
#pragma unroll
      for (uint32_t k = 0; k < kBatch; ++k) {
        const uint32_t a = warp + 8u * (k0 + k);
        if (v[k] >= bb::P) atomicOr(bad, 1u);
        if (kRows >= 8 || a < kRows) tile[(a << 5) | lane] = bb::to_mont(v[k]);
      }
    }
  } else {
    const uint32_t* src = cw + (x0 + ((size_t)warp << s_lo)) * w + c;
#pragma unroll 1
    for (uint32_t k0 = 0; k0 < kPer; k0 += kBatch) {
      uint32_t v[kBatch];
#pragma unroll
      for (uint32_t k = 0; k < kBatch; ++k) {
        const uint32_t a = warp + 8u * (k0 + k);
        v[k] = ((kRows >= 8 || a < kRows) && col_ok) ? src[0] : 0u;
        src += step;
      }
#pragma unroll
      for (uint32_t k = 0; k < kBatch; ++k) {
        const uint32_t a = warp + 8u * (k0 + k);
        if (kRows >= 8 || a < kRows) tile[(a << 5) | lane] = v[k];
      }
    }
  }
  __syncthreads();
  BbWideGroups<T, 0>::run(tile, s_lo, u, lane, warp, tw);
  if (col_ok) {
    uint32_t* dst = cw + (x0 + ((size_t)warp << s_lo)) * w + c;
#pragma unroll 4
    for (uint32_t k = 0; k < kPer; ++k) {
      const uint32_t a = warp + 8u * k;
      if (kRows >= 8 || a < kRows) *dst = tile[(a << 5) | lane];
      dst += step;
    }
  }
}

// ---- leaves ------------------------------------------------------------------
// Width 1: the row is one BabyBear.
__global__ void __launch_bounds__(128) bb_leaves_one_kernel(const uint32_t* __restrict__ cw, uint4* __restrict__ leaves,
                                                           size_t rows, int bits) {
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < rows; q += (size_t)gridDim.x * blockDim.x)
    store_digest(leaves, brev_bits(q, bits), hash_base(bb::from_mont(cw[q])));
}

// Any width: keccak256 of the row's 4w bytes (GenericHasher over the row's
// bincode, p3/src/symmetric.rs:11-25): canonical words staged by a warp per
// 32 rows (keccak_rows_warp).  Five blocks per SM (96 registers, a few spilled
// words) measured about 1% faster than four at 128 registers.
__global__ void __launch_bounds__(128, 5) bb_leaves_rows_kernel(const uint32_t* __restrict__ cw,
                                                            uint4* __restrict__ leaves, size_t rows, uint32_t w,
                                                            int bits) {
  __shared__ uint32_t stage[4][32 * kStagePitch];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  auto word_at = [&](size_t row, uint32_t i) { return bb::from_mont(cw[row * w + i]); };
  for (size_t r0 = ((size_t)blockIdx.x * 4 + warp) * 32; r0 < rows; r0 += (size_t)gridDim.x * 128) {
    const Digest dg = keccak_rows_warp(stage[warp], r0, rows, w, word_at);
    if (r0 + lane < rows) store_digest(leaves, brev_bits(r0 + lane, bits), dg);
  }
}

// Folded-codeword leaf j = keccak256(pi[j] || pi[j + half]) at bitrev(j);
// the first round's pi of a width-1 commitment is the codeword itself, lifted
// with E::from (basefold.rs:150-155).
__global__ void __launch_bounds__(128) bb_leaves_pairs_kernel(const uint32_t* __restrict__ pi, int base,
                                                             uint4* __restrict__ leaves, size_t half, int bits) {
  for (size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x; j < half; j += (size_t)gridDim.x * blockDim.x) {
    const E5 a = base ? bb::e_from(pi[j]) : ld_e5(pi, j);
    const E5 b = base ? bb::e_from(pi[j + half]) : ld_e5(pi, j + half);
    store_digest(leaves, brev_bits(j, bits), hash_pair_e5(a, b));
  }
}

// ---- rows combined with the batching scalars (basefold.rs:160-176) ------------
// One thread per row.  A block stages 128 rows x 32 columns through shared
// memory with coalesced loads (each warp instruction reads one 128-byte row
// run; 32 of them in flight per warp), then every thread multiplies its
// row's 32 words by the scalars (shared, broadcast reads).  A product
// mul(s', v) is s' v R^-1: the caller passes s' = s R for a Montgomery source
// (the codeword) and s' = s R^2 for canonical evaluations, so every product
// is the Montgomery form of s v without converting the source.  The products
// s' v (source words below p) are summed unreduced in 64 bits, folded to
// hi (2^32 mod p) + lo after every four columns so that four products never
// overflow; the sum is congruent to R times the Montgomery form of the dot
// product, and one Montgomery reduction of it mod p gives that form.
constexpr int kCombRows = 128, kCombCols = 32;
__global__ void __launch_bounds__(kCombRows, 6) bb_combine_kernel(const uint32_t* __restrict__ src, size_t rows,
                                                              uint32_t w, const uint32_t* __restrict__ scalars,
                                                              uint32_t* __restrict__ out) {
  __shared__ uint32_t stage[kCombRows * (kCombCols + 1)];
  __shared__ uint32_t sc[5 * kCombCols];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (size_t r0 = (size_t)blockIdx.x * kCombRows; r0 < rows; r0 += (size_t)gridDim.x * kCombRows) {
    unsigned long long s[5] = {0, 0, 0, 0, 0};
    for (uint32_t c0 = 0; c0 < w; c0 += kCombCols) {
      __syncthreads();  // the previous chunk's reads are done
      for (uint32_t t = threadIdx.x; t < 5 * kCombCols; t += blockDim.x) {
        const uint32_t c = c0 + t / 5;
        sc[t] = c < w ? scalars[5 * c0 + t] : 0u;
      }
#pragma unroll
      for (int h = 0; h < 2; ++h) {  // warp w loads rows w, w + 4, ..: 16 loads in flight per lane
        uint32_t v[kCombRows / 8];
#pragma unroll
        for (int k = 0; k < kCombRows / 8; ++k) {
          const size_t r = r0 + warp + 4 * (k + h * kCombRows / 8);
          const uint32_t c = c0 + lane;
          v[k] = (r < rows && c < w) ? src[r * w + c] : 0u;
        }
#pragma unroll
        for (int k = 0; k < kCombRows / 8; ++k)
          stage[(warp + 4 * (k + h * kCombRows / 8)) * (kCombCols + 1) + lane] = v[k];
      }
      __syncthreads();
      const uint32_t* row = stage + threadIdx.x * (kCombCols + 1);
#pragma unroll 2
      for (int c4 = 0; c4 < kCombCols; c4 += 4) {
#pragma unroll
        for (int c = c4; c < c4 + 4; ++c) {
          const uint32_t x = row[c];
#pragma unroll
          for (int k = 0; k < 5; ++k) s[k] += (unsigned long long)sc[5 * c + k] * x;
        }
#pragma unroll
        for (int k = 0; k < 5; ++k) s[k] = (s[k] >> 32) * (unsigned long long)bb::MONT_ONE + (uint32_t)s[k];
      }
    }
    const size_t r = r0 + threadIdx.x;
    if (r < rows) {
      E5 e;
#pragma unroll
      for (int k = 0; k < 5; ++k) e.c[k] = bb_reduce(s[k] % bb::P);
      st_e5(out, r, e);
    }
  }
}

// ---- column evaluations (basefold.rs:126-131) ---------------------------------
// Lane = column (32 per blockIdx.y), warps and blocks over the rows; the data
// stay canonical and the eq table is Montgomery.
// Products are summed unreduced: a word v is first brought below 2^32 - p by
// one conditional subtraction (v mod p for every 32-bit word), each product
// eq R v (eq in Montgomery form) is then below 4.6e18, and a 64-bit sum is
// folded to hi (2^32 mod p) + lo (below 1.2e18) after every two rows, so three
// products never overflow it.  A thread's sum is congruent to R sum eq v;
// one reduction mod p and one Montgomery reduction give its canonical part.
__global__ void __launch_bounds__(256) bb_eval_cols_kernel(const uint32_t* __restrict__ eq,
                                                          const uint32_t* __restrict__ data, size_t rows, uint32_t w,
                                                          unsigned long long* acc) {
  __shared__ unsigned long long part[8][5][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t c = blockIdx.y * 32 + lane;
  unsigned long long s[5] = {0, 0, 0, 0, 0};
  auto fold = [&]() {
#pragma unroll
    for (int k = 0; k < 5; ++k) s[k] = (s[k] >> 32) * (unsigned long long)bb::MONT_ONE + (uint32_t)s[k];
  };
  if (c < w) {
    const size_t step = (size_t)gridDim.x * 8;
    for (size_t r = (size_t)blockIdx.x * 8 + warp; r < rows; r += 8 * step) {
      uint32_t v[8];  // eight rows' loads in flight before they are used
#pragma unroll
      for (int q = 0; q < 8; ++q) v[q] = r + q * step < rows ? data[(r + q * step) * w + c] : 0u;
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        if (r + q * step >= rows) break;
        const size_t rr = r + q * step;
        const uint32_t x = bb::umin(v[q], v[q] - bb::P);
#pragma unroll
        for (int k = 0; k < 5; ++k) s[k] += (unsigned long long)eq[5 * rr + k] * x;
        if (q & 1) fold();
      }
      fold();
    }
  }
#pragma unroll
  for (int k = 0; k < 5; ++k) part[warp][k][lane] = bb_reduce(s[k] % bb::P);
  __syncthreads();
  if (warp == 0 && c < w) {
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      unsigned long long v = 0;
      for (int q = 0; q < 8; ++q) v += part[q][k][lane];
      if (v) atomicAdd(acc + 5 * (size_t)c + k, v);
    }
  }
}

// ---- multilinear evaluation and the sumcheck side -----------------------------
// MultiPoly::eq (p3/src/poly/multilinear.rs:41-64) expands the table level by
// level with eq_expand (:216-222): hi = lo x_i; lo -= hi.  Here the whole table
// is one launch: entry b is the product over i of x_i (bit i of b set) or
// 1 - x_i, the same field value, since products do not depend on their
// order.  A thread takes 2^kEqLow
// consecutive entries: the product of their common high-bit factors, then the
// expansion of the low bits in registers (one product and one subtraction
// per new entry).
constexpr int kEqLow = 3;
struct BbEqFactors {
  E5 x[kBbMaxRounds], omx[kBbMaxRounds];  // x_i and 1 - x_i (Montgomery)
};
__global__ void __launch_bounds__(256) bb_eq_table_kernel(uint32_t* ev, int n, const __grid_constant__ BbEqFactors f) {
  const int k = n < kEqLow ? n : kEqLow;
  const size_t groups = (size_t)1 << (n - k);
  for (size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x; g < groups; g += (size_t)gridDim.x * blockDim.x) {
    E5 v[1 << kEqLow];
    E5 pre = bb::e_from(bb::MONT_ONE);
    for (int i = k; i < n; ++i) pre = bb::e_mul(pre, ((g >> (i - k)) & 1) ? f.x[i] : f.omx[i]);
    v[0] = pre;
#pragma unroll
    for (int i = 0; i < kEqLow; ++i) {
      if (i >= k) break;
#pragma unroll
      for (int j = 0; j < (1 << i); ++j) {
        const E5 hv = bb::e_mul(v[j], f.x[i]);
        v[(1 << i) + j] = hv;
        v[j] = bb::e_sub(v[j], hv);
      }
    }
#pragma unroll
    for (int j = 0; j < (1 << kEqLow); ++j) {
      if (j >= (1 << k)) break;
      st_e5(ev, (g << k) + j, v[j]);
    }
  }
}

// sum_b heq[b] poly[b] (EvalImprProver::compute_round_poly, eval_impr.rs:
// 187-197) as five coefficient sums: Montgomery for an extension poly,
// canonical for canonical base-field data.
__global__ void __launch_bounds__(256) bb_dot_kernel(const uint32_t* __restrict__ heq, const uint32_t* __restrict__ poly,
                                                    int base, size_t n, unsigned long long* acc) {
  unsigned long long s[5] = {0, 0, 0, 0, 0};
  for (size_t b = (size_t)blockIdx.x * blockDim.x + threadIdx.x; b < n; b += (size_t)gridDim.x * blockDim.x) {
    const E5 h = ld_e5(heq, b);
    // base: canonical data times the Montgomery table gives canonical products
    const E5 t = base ? bb::e_scale(h, poly[b]) : bb::e_mul(h, ld_e5(poly, b));
#pragma unroll
    for (int k = 0; k < 5; ++k) s[k] += t.c[k];
  }
  __shared__ unsigned long long part[5][8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  warp_sum5(s);
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < 5; ++k) part[k][warp] = s[k];
  }
  __syncthreads();
  if (threadIdx.x < 5) {
    unsigned long long v = 0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) v += part[threadIdx.x][q];
    if (v) atomicAdd(acc + threadIdx.x, v);
  }
}

// fix_last_var (multilinear.rs:183-198): out[b] = lo + x (hi - lo).
__global__ void bb_fix_kernel(const uint32_t* in, int base, uint32_t* out, size_t half, E5 x, const uint32_t* xp) {
  if (xp) x = ld_e5(xp, 0);
  for (size_t b = (size_t)blockIdx.x * blockDim.x + threadIdx.x; b < half; b += (size_t)gridDim.x * blockDim.x) {
    if (base) {
      const uint32_t lo = bb::to_mont(in[b]), d = bb::sub(bb::to_mont(in[b + half]), lo);
      E5 r = bb::e_scale(x, d);
      r.c[0] = bb::add(r.c[0], lo);
      st_e5(out, b, r);
    } else {
      const E5 lo = ld_e5(in, b), hi = ld_e5(in, b + half);
      st_e5(out, b, bb::e_add(lo, bb::e_mul(x, bb::e_sub(hi, lo))));
    }
  }
}

// ---- fold (code.rs:66-84) with the next round's leaves ------------------------
// interpolate(t, lo, hi, r) = l + (h - l) r with l = (lo + hi) / 2 and
// h = (lo - hi) t, t = (2 t_i^j)^-1.  Thread s < n/2 makes out[s] and
// out[s + n/2], the row s of the next round's matrix, and hashes it.
__device__ __forceinline__ E5 bb_interp(const E5& lo, const E5& hi, uint32_t t, const E5& x) {
  const E5 l = bb::e_scale(bb::e_add(lo, hi), bb::MONT_INV2);
  const E5 h = bb::e_scale(bb::e_sub(lo, hi), t);
  return bb::e_add(l, bb::e_mul(bb::e_sub(h, l), x));
}
__global__ void __launch_bounds__(128) bb_fold_kernel(BbFold p, E5 x) {
  if (p.xp) x = ld_e5(p.xp, 0);
  const size_t n = p.n, q = n >> 1;
  const size_t work = q ? q : 1;  // n = 1: the single output, no leaves
  for (size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x; s < work; s += (size_t)gridDim.x * blockDim.x) {
    E5 f[2];
    const int outs = q ? 2 : 1;
    for (int k = 0; k < outs; ++k) {
      const size_t j = s + k * q;
      const E5 lo = p.base ? bb::e_from(p.w[j]) : ld_e5(p.w, j);
      const E5 hi = p.base ? bb::e_from(p.w[j + n]) : ld_e5(p.w, j + n);
      f[k] = bb_interp(lo, hi, p.tinv[j], x);
      st_e5(p.out, j, f[k]);
    }
    if (p.leaves && q) store_digest(p.leaves, brev_bits(s, p.leaf_bits), hash_pair_e5(f[0], f[1]));
  }
}

// ---- the open's transcript on the device ---------------------------------------------
// One warp per round: the sponge's lanes live in lanes 0..24 (WarpKeccak), the
// pending input and the output bytes in shared memory, the scalar algebra on
// lane 0 except the delta product, which is a warp product tree.
namespace {
struct TrCtx {
  uint8_t pend[256];
  uint8_t out[32];
  int pend_len, out_len;
};

// XOR the 136-byte block blk (shared memory) into the sponge and permute.
__device__ __forceinline__ uint2 tr_absorb(const WarpKeccak& wk, uint2 a, const uint8_t* blk) {
  if (wk.lane < 17) {
    uint32_t lo = 0, hi = 0;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      lo |= (uint32_t)blk[8 * wk.lane + b] << (8 * b);
      hi |= (uint32_t)blk[8 * wk.lane + 4 + b] << (8 * b);
    }
    a.x ^= lo;
    a.y ^= hi;
  }
  return wk.permute<false>(a);
}

// observe (challenger.rs:51-60): append n bytes (n <= 72) to the input and
// clear the output; a full block is absorbed.  All lanes call.
__device__ uint2 tr_observe(const WarpKeccak& wk, uint2 a, TrCtx& c, const uint8_t* src, int n) {
  const int len = c.pend_len;
  for (int i = wk.lane; i < n; i += 32) c.pend[len + i] = src[i];
  __syncwarp();
  int total = len + n;
  if (total >= 136) {
    a = tr_absorb(wk, a, c.pend);
    __syncwarp();
    uint8_t keep[3];  // the bytes past the block move to the front, 3 per lane at most
    int m = 0;
    for (int i = 136 + wk.lane; i < total; i += 32) keep[m++] = c.pend[i];
    __syncwarp();
    m = 0;
    for (int i = 136 + wk.lane; i < total; i += 32) c.pend[i - 136] = keep[m++];
    total -= 136;
  }
  __syncwarp();
  if (wk.lane == 0) {
    c.pend_len = total;
    c.out_len = 0;
  }
  __syncwarp();
  return a;
}

// One output byte, popped from the end; an empty output is refilled with
// keccak256 of the input, which becomes the new input.  All lanes call and
// get the byte.
__device__ uint8_t tr_sample_byte(const WarpKeccak& wk, uint2& a, TrCtx& c) {
  if (c.out_len == 0) {
    const int len = c.pend_len;
    uint8_t blk8[8];
    if (wk.lane < 17)
      for (int b = 0; b < 8; ++b) {
        const int k = 8 * wk.lane + b;
        uint8_t v = k < len ? c.pend[k] : 0;
        if (k == len) v ^= 0x01u;
        if (k == 135) v ^= 0x80u;
        blk8[b] = v;
      }
    if (wk.lane < 17) {
      uint32_t lo = 0, hi = 0;
      for (int b = 0; b < 4; ++b) {
        lo |= (uint32_t)blk8[b] << (8 * b);
        hi |= (uint32_t)blk8[4 + b] << (8 * b);
      }
      a.x ^= lo;
      a.y ^= hi;
    }
    a = wk.permute<false>(a);
    __syncwarp();
    if (wk.lane < 4)
      for (int b = 0; b < 4; ++b) {
        const uint8_t lo = (uint8_t)(a.x >> (8 * b)), hi = (uint8_t)(a.y >> (8 * b));
        c.out[8 * wk.lane + b] = lo;
        c.out[8 * wk.lane + 4 + b] = hi;
        c.pend[8 * wk.lane + b] = lo;
        c.pend[8 * wk.lane + 4 + b] = hi;
      }
    a = make_uint2(0, 0);  // the digest is the whole new input, still pending
    __syncwarp();
    if (wk.lane == 0) {
      c.pend_len = 32;
      c.out_len = 32;
    }
    __syncwarp();
  }
  const uint8_t b = c.out[c.out_len - 1];
  __syncwarp();
  if (wk.lane == 0) c.out_len -= 1;
  __syncwarp();
  return b;
}

// FromUniformBytes for BabyBear: 4 bytes LE shifted right by one, redrawn
// while >= p; an extension element is five of them (challenger.rs:62-74).
__device__ E5 tr_sample_e(const WarpKeccak& wk, uint2& a, TrCtx& c) {
  E5 e;
  for (int k = 0; k < 5; ++k) {
    uint32_t v;
    do {
      v = 0;
      for (int b = 0; b < 4; ++b) v |= (uint32_t)tr_sample_byte(wk, a, c) << (8 * b);
      v >>= 1;
    } while (v >= bb::P);
    e.c[k] = bb::to_mont(v);
  }
  return e;
}

__device__ __forceinline__ void e5_bytes(const E5& e, uint8_t* b) {
  for (int k = 0; k < 5; ++k) {
    const uint32_t v = bb::from_mont(e.c[k]);
    for (int q = 0; q < 4; ++q) b[4 * k + q] = (uint8_t)(v >> (8 * q));
  }
}
__device__ __forceinline__ E5 shfl_e5(const E5& e, int src) {
  E5 r;
#pragma unroll
  for (int k = 0; k < 5; ++k) r.c[k] = __shfl_sync(0xffffffffu, e.c[k], src);
  return r;
}
}  // namespace

// One folding-sumcheck round (basefold.rs:340-362 with sumcheck/src/lib.rs:81-103
// and EvalImprProver's round polynomial, eval_impr.rs:41-58, 150-162), one warp.
__global__ void __launch_bounds__(32) bb_transcript_round_kernel(BbTranscript* t, const BbRoundConsts* c, int k,
                                                                int ri, int num_vars, const uint4* root_dev,
                                                                const unsigned long long* sums, int canonical,
                                                                uint32_t* x_out, uint8_t* rec) {
  __shared__ TrCtx ctx;
  __shared__ uint8_t msg[72];  // the root, then the compressed round polynomial (canonical bytes)
  const WarpKeccak wk;
  const int lane = wk.lane;
  const bool last = ri + 1 == num_vars;
  const int nf = last ? 0 : min(k, num_vars - ri - 1);  // k: rounds done
  // Every global load first: none depends on another, so they are in flight
  // together instead of one dependent round trip after another.
  const uint32_t* pend_w = reinterpret_cast<const uint32_t*>(t->pend);
  const uint32_t pw0 = pend_w[lane], pw1 = pend_w[lane + 32];
  const uint8_t ob = t->out[lane];
  uint2 a = lane < 25 ? t->A[lane] : make_uint2(0, 0);
  E5 fx{}, fy{};  // the delta factor's x = r[ri+1+j] and y, the challenge sampled j+1 rounds ago
  if (lane < nf) {
    fx = c->r[ri + 1 + lane];
    fy = t->xs[k - 1 - lane];
  }
  unsigned long long sv[5] = {0, 0, 0, 0, 0};
  E5 sc{}, r{}, cf{}, rinv{};
  if (lane == 0) {
    for (int q = 0; q < 5; ++q) sv[q] = sums[q];
    sc = last ? t->outer : t->inner;
    r = c->r[ri];
    cf = c->cf[ri];
    rinv = c->r_inv[ri];
    ctx.pend_len = (int)t->pend_len;
    ctx.out_len = (int)t->out_len;
    const Digest dg = digest_bytes(load_digest(root_dev, 0));
    const uint32_t words[8] = {dg.lo.x, dg.lo.y, dg.lo.z, dg.lo.w, dg.hi.x, dg.hi.y, dg.hi.z, dg.hi.w};
    for (int i = 0; i < 8; ++i)
      for (int b = 0; b < 4; ++b) msg[4 * i + b] = (uint8_t)(words[i] >> (8 * b));
  }
  reinterpret_cast<uint32_t*>(ctx.pend)[lane] = pw0;
  reinterpret_cast<uint32_t*>(ctx.pend)[lane + 32] = pw1;
  ctx.out[lane] = ob;
  __syncwarp();
  a = tr_observe(wk, a, ctx, msg, 32);
  // delta: eq_eval(r[ri+1..], inner.r()) (multilinear.rs:224-229) as a product
  // tree over the warp, factor j = 2 x y + 1 - x - y
  const E5 one = bb::e_from(bb::MONT_ONE);
  E5 f = one;
  if (lane < nf) {
    const E5 xy = bb::e_mul(fx, fy);
    f = bb::e_sub(bb::e_sub(bb::e_add(bb::e_add(xy, xy), one), fx), fy);
  }
  for (int o = 16; o > 0; o >>= 1) f = bb::e_mul(f, shfl_e5(f, lane ^ o));  // every lane: the product
  // the round polynomial from S = sum_b half_eq[b] poly[b] (lane 0)
  E5 c0{}, c1{}, rp0{}, rp1{}, rp2{};
  if (lane == 0) {
    E5 S;
    for (int q = 0; q < 5; ++q) {
      const uint32_t v = (uint32_t)(sv[q] % bb::P);
      S.c[q] = canonical ? bb::to_mont(v) : v;
    }
    const E5 omr = bb::e_sub(one, r);
    c0 = bb::e_mul(cf, S);
    const E5 e1 = bb::e_mul(bb::e_sub(sc, bb::e_mul(omr, c0)), rinv);
    c1 = bb::e_sub(e1, c0);
    const E5 d0 = bb::e_mul(f, omr), d1 = bb::e_mul(f, bb::e_sub(r, omr));
    rp0 = bb::e_mul(c0, d0);
    rp1 = bb::e_add(bb::e_mul(c0, d1), bb::e_mul(c1, d0));
    rp2 = bb::e_mul(c1, d1);
    e5_bytes(rp0, msg + 32);  // Eval::compress_round_poly keeps c0 and c2
    e5_bytes(rp2, msg + 52);
  }
  __syncwarp();
  for (int q = lane; q < 72; q += 32) rec[q] = msg[q];
  a = tr_observe(wk, a, ctx, msg + 32, 40);
  const E5 x = tr_sample_e(wk, a, ctx);
  if (lane == 0) {
    t->inner = bb::e_add(c0, bb::e_mul(c1, x));                            // fix_last_var (eval.rs:108-111)
    t->outer = bb::e_add(rp0, bb::e_mul(x, bb::e_add(rp1, bb::e_mul(x, rp2))));  // horner (univariate.rs:5-12)
    t->xs[k] = x;
    t->rounds = (uint32_t)(k + 1);
    st_e5(x_out, 0, x);
    t->pend_len = (uint32_t)ctx.pend_len;
    t->out_len = (uint32_t)ctx.out_len;
  }
  uint32_t* pend_out = reinterpret_cast<uint32_t*>(t->pend);
  pend_out[lane] = reinterpret_cast<const uint32_t*>(ctx.pend)[lane];
  pend_out[lane + 32] = reinterpret_cast<const uint32_t*>(ctx.pend)[lane + 32];
  t->out[lane] = ctx.out[lane];
  if (lane < 25) t->A[lane] = a;
}

cudaError_t bb_launch_transcript_round(BbTranscript* t, const BbRoundConsts* c, int k, int ri, int num_vars,
                                       const uint4* root_dev, const unsigned long long* sums, int canonical,
                                       uint32_t* x_out, uint8_t* rec, cudaStream_t st) {
  bb_transcript_round_kernel<<<1, 32, 0, st>>>(t, c, k, ri, num_vars, root_dev, sums, canonical, x_out, rec);
  count_launch();
  return cudaGetLastError();
}

// ---- query openings (basefold.rs:200-222) ---------------------------------------
// One block per query; every field of the record sits on a 4-byte boundary.
__device__ __forceinline__ void put64w(uint32_t* o, size_t wo, uint64_t v) {
  o[wo] = (uint32_t)v;
  o[wo + 1] = (uint32_t)(v >> 32);
}
__device__ __forceinline__ void put_digest_words(uint32_t* o, size_t wo, const uint4* tree, size_t i) {
  const Digest dg = digest_bytes(load_digest(tree, i));
  o[wo + 0] = dg.lo.x;
  o[wo + 1] = dg.lo.y;
  o[wo + 2] = dg.lo.z;
  o[wo + 3] = dg.lo.w;
  o[wo + 4] = dg.hi.x;
  o[wo + 5] = dg.hi.y;
  o[wo + 6] = dg.hi.z;
  o[wo + 7] = dg.hi.w;
}
__global__ void bb_gather_kernel(BbGather p) {
  const int t = blockIdx.x;
  const uint64_t idx = p.idx[t];
  uint32_t* o = reinterpret_cast<uint32_t*>(p.out + (size_t)t * p.rec_bytes);
  const int L = p.L, d = p.d;
  const size_t w = p.w;
  if (threadIdx.x == 0) {
    put64w(o, 0, w);
    put64w(o, 2 + w, (uint64_t)L);
  }
  for (size_t c = threadIdx.x; c < w; c += blockDim.x) o[2 + c] = bb::from_mont(p.cw[idx * w + c]);
  size_t wo = 4 + w;
  for (int k = threadIdx.x; k < L; k += blockDim.x) {
    const uint64_t m = (idx >> k) ^ 1ull;
    const size_t off = ((size_t)2 << L) - ((size_t)2 << (L - k));
    put_digest_words(o, wo + 8 * (size_t)k, p.cw_tree, off + brev_bits(m, L - k));
  }
  wo += 8 * (size_t)L;
  if (threadIdx.x == 0) put64w(o, wo, (uint64_t)d);
  wo += 2;
  for (int k = 0; k < d; ++k) {
    const int i = d - 1 - k;
    const int li = p.log2_n0 + i;  // the round's tree has n_i = 2^li leaves
    const uint64_t ni = (uint64_t)1 << li;
    const uint64_t j = idx & (ni - 1), sib = ((idx >> li) & 1) ^ 1;
    if (threadIdx.x == 0) {
      const size_t e = j + sib * ni;
      if (k == 0 && p.pi0_base) {
        o[wo] = bb::from_mont(p.pi[0][e]);
        o[wo + 1] = o[wo + 2] = o[wo + 3] = o[wo + 4] = 0;
      } else {
#pragma unroll
        for (int c = 0; c < 5; ++c) o[wo + c] = bb::from_mont(p.pi[k][5 * e + c]);
      }
      put64w(o, wo + 5, (uint64_t)li);
    }
    wo += 7;
    const uint4* tree = p.trees[k];
    for (int kk = threadIdx.x; kk < li; kk += blockDim.x) {
      const uint64_t m = (j >> kk) ^ 1ull;
      const size_t loff = ((size_t)2 << li) - ((size_t)2 << (li - kk));
      put_digest_words(o, wo + 8 * (size_t)kk, tree, loff + brev_bits(m, li - kk));
    }
    wo += 8 * (size_t)li;
  }
}

// ---- launchers -----------------------------------------------------------------
static unsigned blocks_for(size_t n, int threads) {
  size_t b = (n + threads - 1) / threads;
  if (b > 152u * 64) b = 152u * 64;  // grid-stride beyond 64 blocks per SM
  return b ? (unsigned)b : 1u;
}

cudaError_t bb_launch_pow_shoup(uint2* out, size_t n, uint32_t g_mont, cudaStream_t st) {
  bb_pow_shoup_kernel<<<blocks_for(n, 256), 256, 0, st>>>(out, n, g_mont);
  count_launch();
  return cudaGetLastError();
}

cudaError_t bb_launch_shoup_from(const uint32_t* in, uint2* out, size_t n, uint32_t* bad, cudaStream_t st) {
  bb_shoup_from_kernel<<<blocks_for(n, 256), 256, 0, st>>>(in, out, n, bad);
  count_launch();
  return cudaGetLastError();
}

cudaError_t bb_launch_pow_table(uint32_t* out, size_t n, uint32_t g_mont, uint32_t scale_mont, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  bb_pow_table_kernel<<<blocks_for(n, 256), 256, 0, st>>>(out, n, g_mont, scale_mont);
  count_launch();
  return cudaGetLastError();
}

static int ilog2_ceil(size_t v) {
  int r = 0;
  while (((size_t)1 << r) < v) ++r;
  return r;
}

cudaError_t bb_launch_from_mont(const uint32_t* in, uint32_t* out, size_t n, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  bb_from_mont_kernel<<<blocks_for(n, 256), 256, 0, st>>>(in, out, n);
  count_launch();
  return cudaGetLastError();
}

cudaError_t bb_launch_tinv(const uint32_t* ts, uint32_t* tinv, size_t n, uint32_t* bad, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  bb_tinv_kernel<<<blocks_for(n, 256), 256, 0, st>>>(ts, tinv, n, bad);
  count_launch();
  return cudaGetLastError();
}

cudaError_t bb_launch_encode(const uint32_t* m, uint32_t* cw, int d, int log2_c, int log2_k0, int generic, size_t w,
                             const uint2* tw, uint32_t* bad, cudaStream_t st, const cudaEvent_t* slice_ready,
                             int slices) {
  const int L = d + log2_c + log2_k0;
  if (slices < 1 || !slice_ready) slices = 1;
  // input slice k (data rows [k 2^nv / slices, (k+1) 2^nv / slices)) feeds
  // codeword rows [k 2^L / slices, (k+1) 2^L / slices)
  auto wait_slice = [&](int k) { return slices > 1 ? cudaStreamWaitEvent(st, slice_ready[k], 0) : cudaSuccess; };
  if (!generic && L == 0) {
    for (int k = 0; k < slices; ++k) {
      cudaError_t e = wait_slice(k);
      if (e != cudaSuccess) return e;
    }
    bb_copy_mont_kernel<<<blocks_for(w, 256), 256, 0, st>>>(m, cw, w, bad);
    count_launch();
    return cudaGetLastError();
  }
  const int log2_n0 = log2_c + log2_k0;
  const int first = generic ? log2_n0 : 0;  // the first DIT layer (the butterflies of ts[i-1] are layers log2_n0 + i - 1)

  // The pass plan.
  struct PassPlan {
    BbPass p;
    size_t blocks, words;
    int threads;
  };
  PassPlan plan[kBbMaxRounds + 1];
  int npass = 0;
  const int lc = ilog2_ceil(w < 32 ? w : 32);
  const unsigned chunks = (unsigned)((w + ((size_t)1 << lc) - 1) >> lc);
  // U C <= 32 consecutive words per row run; tiles of 2^(T + lu + lc) <= 8192 words
  auto lu_at = [&](int s_lo) {
    int lu = 0;
    if (s_lo > 0)
      while (lu < s_lo && lc + lu < 5) ++lu;
    return lu;
  };
  auto tmax_at = [&](int s_lo) { return std::min(12, 13 - lc - lu_at(s_lo)); };
  // the greedy split's pass count, then the layers spread evenly over that
  // many passes where the tiles allow (no short last pass of idle warps)
  int passes = 0;
  for (int x = first; x < L; x += tmax_at(x)) ++passes;
  for (int lo = first; lo < L;) {
    const int lu = lu_at(lo);
    int T = (L - lo + passes - 1) / passes;
    if (T > tmax_at(lo)) T = tmax_at(lo);
    --passes;
    if (passes > 0) {  // keep the rest reachable in the passes left
      int reach = 0;
      for (int x = lo + T, k = 0; k < passes && x < L; ++k) {
        reach += tmax_at(x);
        x += tmax_at(x);
      }
      if (lo + T + reach < L) T = tmax_at(lo);
    }
    if (T > L - lo) T = L - lo;
    PassPlan& pp = plan[npass++];
    BbPass& p = pp.p;
    p.s_lo = lo;
    p.T = T;
    p.first = !generic && lo == first;
    p.log2_c = log2_c;
    p.lu = lu;
    p.lc = lc;
    p.w = (uint32_t)w;
    p.chunks = chunks;
    p.chunks_log = (chunks & (chunks - 1)) == 0 ? ilog2_ceil(chunks) : -1;
    p.block0 = 0;
    pp.words = (size_t)1 << (T + lu + lc);
    pp.threads = (int)(pp.words / 2);
    if (pp.threads > 256) pp.threads = 256;
    if (pp.threads < 32) pp.threads = 32;
    pp.blocks = ((size_t)1 << (L - T - lu)) * chunks;  // chunk fastest (BbTile)
    if (pp.blocks > 0x7fffffffu) return cudaErrorInvalidValue;
    lo += T;
  }
  // Blocks [block0, block0 + grid) of a pass.
  auto launch_pass = [&](const PassPlan& pp, size_t block0, size_t grid_blocks) -> cudaError_t {
    BbPass p = pp.p;
    p.block0 = (uint32_t)block0;
    const unsigned grid = (unsigned)grid_blocks;
    const size_t sh = pp.words * sizeof(uint32_t);
    if (p.lc == 5) {  // wider than 16 columns: tiles of whole 32-column runs (T <= 8)
      switch (p.T) {
        case 1: bb_dft_wide_kernel<1><<<grid, 256, sh, st>>>(m, cw, p, tw, bad); break;
        case 2: bb_dft_wide_kernel<2><<<grid, 256, sh, st>>>(m, cw, p, tw, bad); break;
        case 3: bb_dft_wide_kernel<3><<<grid, 256, sh, st>>>(m, cw, p, tw, bad); break;
        case 4: bb_dft_wide_kernel<4><<<grid, 256, sh, st>>>(m, cw, p, tw, bad); break;
        case 5: bb_dft_wide_kernel<5><<<grid, 256, sh, st>>>(m, cw, p, tw, bad); break;
        case 6: bb_dft_wide_kernel<6><<<grid, 256, sh, st>>>(m, cw, p, tw, bad); break;
        case 7: bb_dft_wide_kernel<7><<<grid, 256, sh, st>>>(m, cw, p, tw, bad); break;
        case 8: bb_dft_wide_kernel<8><<<grid, 256, sh, st>>>(m, cw, p, tw, bad); break;
        default: return cudaErrorInvalidValue;
      }
    } else if (p.lu + p.lc == 5) {  // a warp's lanes are one row run: registers take 4 layers per round trip
      bb_dft_reg_kernel<<<grid, 256, sh, st>>>(m, cw, p, tw, bad);
    } else {
      bb_dft_pass_kernel<<<grid, pp.threads, sh, st>>>(m, cw, p, tw, bad);
    }
    count_launch();
    return cudaGetLastError();
  };

  // A pass whose tiles stay inside one input slice (rows 2^(s_lo + T) apart
  // at most, and a whole number of tile rows per slice) runs slice by slice:
  // its k-th part (blocks in order, chunk fastest) covers exactly slice k's
  // codeword rows, so it starts as soon as that slice and the slice's earlier
  // stages are done.  The leading passes that qualify, and the generic code's
  // stage 0, run per slice; the others after the last slice.
  int slog = 0;
  while ((1 << slog) < slices) ++slog;
  const bool pow2 = (1 << slog) == slices;
  int npre = 0;
  if (slices > 1 && pow2)
    while (npre < npass && plan[npre].p.s_lo + plan[npre].p.T + slog <= L) ++npre;

  // generic stage 0: g_0[i][j] = i^j (generic.rs:51-54), times R^2, for the rows i < k_0
  const size_t rows = (size_t)1 << L, part = rows / (size_t)slices;
  const size_t k0 = (size_t)1 << log2_k0, n0 = (size_t)1 << log2_n0;
  const bool fast = generic && log2_k0 <= 4 && part % n0 == 0;
  BbG0 g0;
  if (fast)
    for (size_t i = 0; i < k0; ++i) {
      const uint32_t im = bb::to_mont((uint32_t)i);
      uint32_t pw = bb::MONT_ONE;  // i^j R
      for (size_t j = 0; j < k0; ++j) {
        g0.g[i * k0 + j] = bb::to_mont(pw);
        pw = bb::mul(pw, im);
      }
    }
  for (int k = 0; k < slices; ++k) {
    cudaError_t e = wait_slice(k);
    if (e != cudaSuccess) return e;
    if (generic) {
      if (fast) {
        const size_t nch = part / n0, c0 = (size_t)k * nch;
        const unsigned grid = blocks_for(nch * w, 256);
        switch (log2_k0) {
          case 0: bb_stage0_fast_kernel<1><<<grid, 256, 0, st>>>(m, cw, c0, nch, (uint32_t)w, (int)n0, g0, bad); break;
          case 1: bb_stage0_fast_kernel<2><<<grid, 256, 0, st>>>(m, cw, c0, nch, (uint32_t)w, (int)n0, g0, bad); break;
          case 2: bb_stage0_fast_kernel<4><<<grid, 256, 0, st>>>(m, cw, c0, nch, (uint32_t)w, (int)n0, g0, bad); break;
          case 3: bb_stage0_fast_kernel<8><<<grid, 256, 0, st>>>(m, cw, c0, nch, (uint32_t)w, (int)n0, g0, bad); break;
          default: bb_stage0_fast_kernel<16><<<grid, 256, 0, st>>>(m, cw, c0, nch, (uint32_t)w, (int)n0, g0, bad); break;
        }
      } else {
        bb_stage0_kernel<<<blocks_for(part * w, 256), 256, 0, st>>>(m, cw, (size_t)k * part, part, (uint32_t)w,
                                                                    log2_k0, log2_n0, bad);
      }
      count_launch();
      e = cudaGetLastError();
      if (e != cudaSuccess) return e;
    }
    for (int i = 0; i < npre; ++i) {
      const size_t per = plan[i].blocks / (size_t)slices;
      e = launch_pass(plan[i], per * (size_t)k, per);
      if (e != cudaSuccess) return e;
    }
  }
  for (int i = npre; i < npass; ++i) {
    cudaError_t e = launch_pass(plan[i], 0, plan[i].blocks);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t bb_launch_leaves_rows(const uint32_t* cw, uint4* leaves, size_t rows, size_t w, int bits,
                                  cudaStream_t st) {
  if (w == 1)
    bb_leaves_one_kernel<<<blocks_for(rows, 128), 128, 0, st>>>(cw, leaves, rows, bits);
  else
    bb_leaves_rows_kernel<<<blocks_for(rows, 128), 128, 0, st>>>(cw, leaves, rows, (uint32_t)w, bits);
  count_launch();
  return cudaGetLastError();
}

cudaError_t bb_launch_leaves_pairs(const uint32_t* pi, int base, uint4* leaves, size_t half, int bits,
                                   cudaStream_t st) {
  bb_leaves_pairs_kernel<<<blocks_for(half, 128), 128, 0, st>>>(pi, base, leaves, half, bits);
  count_launch();
  return cudaGetLastError();
}

cudaError_t bb_launch_combine(const uint32_t* src, size_t rows, size_t w, const uint32_t* scalars, uint32_t* out,
                              cudaStream_t st) {
  bb_combine_kernel<<<blocks_for(rows, kCombRows), kCombRows, 0, st>>>(src, rows, (uint32_t)w, scalars, out);
  count_launch();
  return cudaGetLastError();
}

cudaError_t bb_launch_eval_cols(const uint32_t* eq, const uint32_t* data, size_t rows, size_t w,
                                unsigned long long* acc, cudaStream_t st) {
  size_t bx = (rows + 63) / 64;  // at least 8 rows per warp
  const size_t by = (w + 31) / 32;
  // one wave: as many blocks as the SMs hold at once, spread over the column
  // groups (blocks per SM depend on the kernel only; SMs on the current device)
  static const int per_sm = [] {
    int b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, bb_eval_cols_kernel, 256, 0);
    return b > 0 ? b : 4;
  }();
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  size_t cap = (size_t)(sms > 0 ? sms : 152) * (size_t)per_sm / by;
  if (cap < 1) cap = 1;
  if (bx > cap) bx = cap;
  if (bx < 1) bx = 1;
  bb_eval_cols_kernel<<<dim3((unsigned)bx, (unsigned)by), 256, 0, st>>>(eq, data, rows, (uint32_t)w, acc);
  count_launch();
  return cudaGetLastError();
}

cudaError_t bb_launch_eq_table(uint32_t* ev, const bb::E5* x, int n, cudaStream_t st) {
  if (n < 0 || n > kBbMaxRounds) return cudaErrorInvalidValue;
  BbEqFactors f;
  const bb::E5 one = bb::e_from(bb::MONT_ONE);
  for (int i = 0; i < n; ++i) {
    f.x[i] = x[i];
    f.omx[i] = bb::e_sub(one, x[i]);
  }
  const size_t groups = (size_t)1 << (n - (n < kEqLow ? n : kEqLow));
  bb_eq_table_kernel<<<blocks_for(groups, 256), 256, 0, st>>>(ev, n, f);
  count_launch();
  return cudaGetLastError();
}

cudaError_t bb_launch_dot(const uint32_t* heq, const uint32_t* poly, int base, size_t n, unsigned long long* acc,
                          cudaStream_t st) {
  size_t b = (n + 255) / 256;
  if (b > 152 * 8) b = 152 * 8;
  bb_dot_kernel<<<b ? (unsigned)b : 1u, 256, 0, st>>>(heq, poly, base, n, acc);
  count_launch();
  return cudaGetLastError();
}

cudaError_t bb_launch_fix(const uint32_t* in, int base, uint32_t* out, size_t half, const E5& x, cudaStream_t st,
                          const uint32_t* xp) {
  bb_fix_kernel<<<blocks_for(half, 256), 256, 0, st>>>(in, base, out, half, x, xp);
  count_launch();
  return cudaGetLastError();
}

cudaError_t bb_launch_fold(const BbFold& p, const E5& x, cudaStream_t st) {
  const size_t q = p.n / 2;
  bb_fold_kernel<<<blocks_for(q ? q : 1, 128), 128, 0, st>>>(p, x);
  count_launch();
  return cudaGetLastError();
}

cudaError_t bb_launch_gather(const BbGather& p, cudaStream_t st) {
  if (p.nq == 0) return cudaSuccess;
  bb_gather_kernel<<<p.nq, 64, 0, st>>>(p);
  count_launch();
  return cudaGetLastError();
}

}  // namespace bf
