// Device arithmetic in the POLYVAL field GF(2^128).
//
// An element is the raw 128-bit value that the reference's `Polyval` stores
// (p3/src/polyval.rs:30-34): bit i is the coefficient of x^i, words are
// little-endian (x = bits 0-31 ... w = bits 96-127).  Addition is XOR
// (polyval.rs:183-191).  Multiplication is the Montgomery product
// a*b*x^-128 mod P with P = x^128 + x^127 + x^126 + x^121 + 1
// (polyval/portable.rs:20-28), so values stay in the reference's
// representation with no conversion.
//
// The GPU has no carry-less multiply.  The 32x32 carry-less product is taken
// from ordinary integer products of operands whose bits are spread four
// apart ("holes"): a product of two such operands has at most 8 terms at any
// bit position, so its sums never carry into the next position of the same
// residue class, and masking keeps exactly the XOR of the terms.  The
// 128x128 product is two levels of Karatsuba over those 32-bit products
// (9 multiplies of 32 bits), then a two-step reduction that cancels the low
// 128 bits with multiples of P (x^128 = x^127 + x^126 + x^121 + 1).
#pragma once
#include <cstdint>

namespace bf {

__device__ __forceinline__ uint4 gf_add(uint4 a, uint4 b) {
  return make_uint4(a.x ^ b.x, a.y ^ b.y, a.z ^ b.z, a.w ^ b.w);
}

__device__ __forceinline__ bool gf_is_zero(uint4 a) { return (a.x | a.y | a.z | a.w) == 0; }

__device__ __forceinline__ uint64_t mulw(uint32_t a, uint32_t b) { return (uint64_t)a * b; }
__device__ __forceinline__ uint64_t madw(uint32_t a, uint32_t b, uint64_t c) { return (uint64_t)a * b + c; }

// Carry-less 32 x 32 -> 64.  a_i / b_i keep the bits of residue i mod 4; the
// product a_i * b_j only has terms at positions of residue i + j, at most 8
// per position.  Two products of the same residue may be ADDED (one integer
// multiply-add, no XOR) whenever their combined count stays <= 15 at every
// position, which holds for the pairs grouped below (checked exhaustively
// over positions with all-ones operands, the worst case); the remaining
// terms are XORed.
__device__ __forceinline__ uint64_t clmul32(uint32_t a, uint32_t b) {
  const uint32_t m0 = 0x11111111u, m1 = 0x22222222u, m2 = 0x44444444u, m3 = 0x88888888u;
  const uint32_t a0 = a & m0, a1 = a & m1, a2 = a & m2, a3 = a & m3;
  const uint32_t b0 = b & m0, b1 = b & m1, b2 = b & m2, b3 = b & m3;
  const uint64_t z0 = madw(a1, b3, mulw(a0, b0)) ^ mulw(a2, b2) ^ mulw(a3, b1);
  const uint64_t z1 = madw(a2, b3, mulw(a0, b1)) ^ madw(a3, b2, mulw(a1, b0));
  const uint64_t z2 = madw(a3, b3, mulw(a0, b2)) ^ mulw(a1, b1) ^ mulw(a2, b0);
  const uint64_t z3 = mulw(a0, b3) ^ mulw(a1, b2) ^ mulw(a2, b1) ^ mulw(a3, b0);
  return (z0 & 0x1111111111111111ull) | (z1 & 0x2222222222222222ull) | (z2 & 0x4444444444444444ull) |
         (z3 & 0x8888888888888888ull);
}

// The same 32 x 32 product with its work moved from the wide multiplies to
// the ALU: one Karatsuba level over 16-bit halves, each 16 x 16 product
// from nine 32-bit integer multiplies (IMAD, whose throughput is about 2.5
// times IMAD.WIDE's) of operands whose bits are three apart.  A product of
// two such operands has at most 6 terms at any position (a residue class of
// 16 bits has 5 or 6 of them), a count that fits the three bits up to the
// next position of its class, so masking keeps the XOR of the terms; the
// results fit 32 bits.  The ALU carries more (operand splits and masks, Karatsuba
// sums), so kernels bound by the multiplier take a few of these per field
// product and the rest from clmul32.
__device__ __forceinline__ uint32_t clmul16(uint32_t a, uint32_t b) {
  const uint32_t a0 = a & 0x9249u, a1 = a & 0x2492u, a2 = a & 0x4924u;
  const uint32_t b0 = b & 0x9249u, b1 = b & 0x2492u, b2 = b & 0x4924u;
  const uint32_t z0 = (a0 * b0) ^ (a1 * b2) ^ (a2 * b1);
  const uint32_t z1 = (a0 * b1) ^ (a1 * b0) ^ (a2 * b2);
  const uint32_t z2 = (a0 * b2) ^ (a2 * b0) ^ (a1 * b1);
  return (z0 & 0x49249249u) | (z1 & 0x92492492u) | (z2 & 0x24924924u);
}

__device__ __forceinline__ uint64_t clmul32_h3(uint32_t a, uint32_t b) {
  const uint32_t al = a & 0xffffu, ah = a >> 16, bl = b & 0xffffu, bh = b >> 16;
  const uint32_t l = clmul16(al, bl), h = clmul16(ah, bh);
  const uint32_t m = clmul16(al ^ ah, bl ^ bh) ^ l ^ h;
  return ((uint64_t)h << 32) ^ ((uint64_t)m << 16) ^ (uint64_t)l;
}

// Product number j of a field product: the first H of the nine from
// clmul32_h3, the rest from clmul32.
template <int H>
__device__ __forceinline__ uint64_t clmul32_sel(uint32_t a, uint32_t b, int j) {
  return j < H ? clmul32_h3(a, b) : clmul32(a, b);
}

// Carry-less 64 x 64 -> 128 by one Karatsuba level (products j0 .. j0+2).
template <int H>
__device__ __forceinline__ void clmul64_mix(uint64_t a, uint64_t b, uint64_t& lo, uint64_t& hi, int j0) {
  const uint32_t a0 = (uint32_t)a, a1 = (uint32_t)(a >> 32);
  const uint32_t b0 = (uint32_t)b, b1 = (uint32_t)(b >> 32);
  const uint64_t p0 = clmul32_sel<H>(a0, b0, j0);
  const uint64_t p2 = clmul32_sel<H>(a1, b1, j0 + 1);
  const uint64_t p1 = clmul32_sel<H>(a0 ^ a1, b0 ^ b1, j0 + 2) ^ p0 ^ p2;
  lo = p0 ^ (p1 << 32);
  hi = p2 ^ (p1 >> 32);
}

// Carry-less 64 x 64 -> 128 by one Karatsuba level.
__device__ __forceinline__ void clmul64(uint64_t a, uint64_t b, uint64_t& lo, uint64_t& hi) {
  const uint32_t a0 = (uint32_t)a, a1 = (uint32_t)(a >> 32);
  const uint32_t b0 = (uint32_t)b, b1 = (uint32_t)(b >> 32);
  const uint64_t p0 = clmul32(a0, b0);
  const uint64_t p2 = clmul32(a1, b1);
  const uint64_t p1 = clmul32(a0 ^ a1, b0 ^ b1) ^ p0 ^ p2;
  lo = p0 ^ (p1 << 32);
  hi = p2 ^ (p1 >> 32);
}

// Montgomery reduction of a 256-bit carry-less product c0 (low) .. c3: the
// field element c x^-128 mod P.  It is GF(2)-linear, so a sum of products
// may be reduced once.
__device__ __forceinline__ uint4 gf_reduce256(uint64_t c0, uint64_t c1, uint64_t c2, uint64_t c3) {
  // cancel bits 0..63:   + c0 * P
  c1 ^= (c0 << 63) ^ (c0 << 62) ^ (c0 << 57);
  c2 ^= c0 ^ (c0 >> 1) ^ (c0 >> 2) ^ (c0 >> 7);
  // cancel bits 64..127: + c1 * x^64 * P
  c2 ^= (c1 << 63) ^ (c1 << 62) ^ (c1 << 57);
  c3 ^= c1 ^ (c1 >> 1) ^ (c1 >> 2) ^ (c1 >> 7);
  return make_uint4((uint32_t)c2, (uint32_t)(c2 >> 32), (uint32_t)c3, (uint32_t)(c3 >> 32));
}

// Montgomery reduction of the 256-bit carry-less product given as three
// 128-bit Karatsuba parts: low = a0 b0, high = a1 b1, mid = (a0+a1)(b0+b1).
__device__ __forceinline__ uint4 gf_karatsuba_reduce(uint64_t l0, uint64_t l1, uint64_t h0, uint64_t h1,
                                                     uint64_t m0, uint64_t m1) {
  m0 ^= l0 ^ h0;
  m1 ^= l1 ^ h1;
  return gf_reduce256(l0, l1 ^ m0, h0 ^ m1, h1);
}

// Montgomery product a*b*x^-128 mod P.
__device__ __forceinline__ uint4 gf_mul(uint4 a, uint4 b) {
  const uint64_t a0 = ((uint64_t)a.y << 32) | a.x, a1 = ((uint64_t)a.w << 32) | a.z;
  const uint64_t b0 = ((uint64_t)b.y << 32) | b.x, b1 = ((uint64_t)b.w << 32) | b.z;
  uint64_t l0, l1, h0, h1, m0, m1;
  clmul64(a0, b0, l0, l1);
  clmul64(a1, b1, h0, h1);
  clmul64(a0 ^ a1, b0 ^ b1, m0, m1);
  return gf_karatsuba_reduce(l0, l1, h0, h1, m0, m1);
}

// One operand of many products, split once: the nine 32-bit words that
// gf_mul's Karatsuba tree multiplies (low half, high half, their sum; in each
// the two words and their sum), each already split into its four residue
// classes mod 4 (the clmul32 masks), 36 words in all.
struct GfPrep {
  uint32_t m[36];
};
__device__ __forceinline__ void gf_prepare(uint4 b, uint32_t* m) {
  const uint32_t w[9] = {b.x, b.y, b.x ^ b.y, b.z, b.w, b.z ^ b.w, b.x ^ b.z, b.y ^ b.w, b.x ^ b.z ^ b.y ^ b.w};
#pragma unroll
  for (int j = 0; j < 9; ++j) {
    m[4 * j + 0] = w[j] & 0x11111111u;
    m[4 * j + 1] = w[j] & 0x22222222u;
    m[4 * j + 2] = w[j] & 0x44444444u;
    m[4 * j + 3] = w[j] & 0x88888888u;
  }
}
// clmul32(a, b) with b given split (gf_prepare's four words of one product).
__device__ __forceinline__ uint64_t clmul32_prep(uint32_t a, uint32_t b0, uint32_t b1, uint32_t b2, uint32_t b3) {
  const uint32_t a0 = a & 0x11111111u, a1 = a & 0x22222222u, a2 = a & 0x44444444u, a3 = a & 0x88888888u;
  const uint64_t z0 = madw(a1, b3, mulw(a0, b0)) ^ mulw(a2, b2) ^ mulw(a3, b1);
  const uint64_t z1 = madw(a2, b3, mulw(a0, b1)) ^ madw(a3, b2, mulw(a1, b0));
  const uint64_t z2 = madw(a3, b3, mulw(a0, b2)) ^ mulw(a1, b1) ^ mulw(a2, b0);
  const uint64_t z3 = mulw(a0, b3) ^ mulw(a1, b2) ^ mulw(a2, b1) ^ mulw(a3, b0);
  return (z0 & 0x1111111111111111ull) | (z1 & 0x2222222222222222ull) | (z2 & 0x4444444444444444ull) |
         (z3 & 0x8888888888888888ull);
}
// c ^= the unreduced 256-bit carry-less product a * b for a prepared b (its
// 36 words at m, read as nine uint4); gf_reduce256(c) of a sum of these is
// the sum of the gf_mul products.
__device__ __forceinline__ void gf_clmul_acc(uint4 a, const uint4* m, uint64_t c[4]) {
  const uint32_t x[9] = {a.x, a.y, a.x ^ a.y, a.z, a.w, a.z ^ a.w, a.x ^ a.z, a.y ^ a.w, a.x ^ a.z ^ a.y ^ a.w};
  uint64_t q[9];
#pragma unroll
  for (int j = 0; j < 9; ++j) {
    const uint4 b = m[j];
    q[j] = clmul32_prep(x[j], b.x, b.y, b.z, b.w);
  }
  uint64_t lo[3], hi[3];
#pragma unroll
  for (int t = 0; t < 3; ++t) {  // 64 x 64 Karatsuba of each half
    const uint64_t p0 = q[3 * t], p2 = q[3 * t + 1], p1 = q[3 * t + 2] ^ p0 ^ p2;
    lo[t] = p0 ^ (p1 << 32);
    hi[t] = p2 ^ (p1 >> 32);
  }
  // 128 x 128 Karatsuba: low = lo[0]:hi[0], high = lo[1]:hi[1], mid = lo[2]:hi[2]
  const uint64_t m0 = lo[2] ^ lo[0] ^ lo[1], m1 = hi[2] ^ hi[0] ^ hi[1];
  c[0] ^= lo[0];
  c[1] ^= hi[0] ^ m0;
  c[2] ^= lo[1] ^ m1;
  c[3] ^= hi[1];
}

// c ^= the unreduced product a * b (both operands split here).
__device__ __forceinline__ void gf_clmul_acc(uint4 a, uint4 b, uint64_t c[4]) {
  uint32_t m[36];
  gf_prepare(b, m);
  gf_clmul_acc(a, reinterpret_cast<const uint4*>(m), c);
}

// gf_mul with H (0..9) of its nine 32 x 32 products from clmul32_h3: the
// same value, with part of the multiplier work moved to the ALU pipe.
template <int H>
__device__ __forceinline__ uint4 gf_mul_mix(uint4 a, uint4 b) {
  const uint64_t a0 = ((uint64_t)a.y << 32) | a.x, a1 = ((uint64_t)a.w << 32) | a.z;
  const uint64_t b0 = ((uint64_t)b.y << 32) | b.x, b1 = ((uint64_t)b.w << 32) | b.z;
  uint64_t l0, l1, h0, h1, m0, m1;
  clmul64_mix<H>(a0, b0, l0, l1, 0);
  clmul64_mix<H>(a1, b1, h0, h1, 3);
  clmul64_mix<H>(a0 ^ a1, b0 ^ b1, m0, m1, 6);
  return gf_karatsuba_reduce(l0, l1, h0, h1, m0, m1);
}

// The 32x32 carry-less product number j (0..8) of gf_mul's Karatsuba tree:
// 64-bit pair t = j / 3 (low, high, sum halves), 32-bit pair u = j % 3.
__device__ __forceinline__ uint64_t gf_mul_part(uint4 a, uint4 b, int j) {
  const int t = j / 3, u = j % 3;
  const uint32_t ax = t == 0 ? a.x : t == 1 ? a.z : a.x ^ a.z;
  const uint32_t ay = t == 0 ? a.y : t == 1 ? a.w : a.y ^ a.w;
  const uint32_t bx = t == 0 ? b.x : t == 1 ? b.z : b.x ^ b.z;
  const uint32_t by = t == 0 ? b.y : t == 1 ? b.w : b.y ^ b.w;
  const uint32_t x = u == 0 ? ax : u == 1 ? ay : ax ^ ay;
  const uint32_t y = u == 0 ? bx : u == 1 ? by : bx ^ by;
  return clmul32(x, y);
}

// Combines the nine parts (as gf_mul's clmul64 calls do) and reduces.
__device__ __forceinline__ uint4 gf_mul_combine(const uint64_t q[9]) {
  uint64_t lo[3], hi[3];
#pragma unroll
  for (int t = 0; t < 3; ++t) {
    const uint64_t p0 = q[3 * t], p2 = q[3 * t + 1], p1 = q[3 * t + 2] ^ p0 ^ p2;
    lo[t] = p0 ^ (p1 << 32);
    hi[t] = p2 ^ (p1 >> 32);
  }
  return gf_karatsuba_reduce(lo[0], hi[0], lo[1], hi[1], lo[2], hi[2]);
}

__device__ __forceinline__ uint64_t shfl64(uint64_t v, int src) {
  const uint32_t lo = __shfl_sync(0xffffffffu, (uint32_t)v, src);
  const uint32_t hi = __shfl_sync(0xffffffffu, (uint32_t)(v >> 32), src);
  return ((uint64_t)hi << 32) | lo;
}

// Two products a1*b1 and a2*b2 by one warp, for latency-bound scalar work:
// lanes 0..8 and 9..17 each take one 32x32 part, every lane gathers the
// parts and combines them, so the results are the same in all lanes.  The
// operands must be the same in all lanes.  All 32 lanes call this.
__device__ __forceinline__ void gf_mul_warp2(uint4 a1, uint4 b1, uint4 a2, uint4 b2, uint4& r1, uint4& r2) {
  const int lane = threadIdx.x & 31;
  const bool second = lane >= 9;
  const int j = second ? lane - 9 : lane;
  uint64_t part = 0;
  if (lane < 18) part = gf_mul_part(second ? a2 : a1, second ? b2 : b1, j);
  uint64_t q1[9], q2[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    q1[k] = shfl64(part, k);
    q2[k] = shfl64(part, 9 + k);
  }
  r1 = gf_mul_combine(q1);
  r2 = gf_mul_combine(q2);
}

__device__ __forceinline__ uint4 gf_mul_warp(uint4 a, uint4 b) {
  uint4 r, unused;
  gf_mul_warp2(a, b, a, b, r, unused);
  return r;
}

// XOR-reduce four words across a warp.
__device__ __forceinline__ uint4 warp_xor(uint4 v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v.x ^= __shfl_xor_sync(0xffffffffu, v.x, o);
    v.y ^= __shfl_xor_sync(0xffffffffu, v.y, o);
    v.z ^= __shfl_xor_sync(0xffffffffu, v.z, o);
    v.w ^= __shfl_xor_sync(0xffffffffu, v.w, o);
  }
  return v;
}

// XOR-reduce over a block whose size is a multiple of 32 and at most 1024;
// the result is valid in thread 0.  `scratch` holds 32 elements.
__device__ __forceinline__ uint4 block_xor(uint4 v, uint4* scratch) {
  v = warp_xor(v);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) scratch[warp] = v;
  __syncthreads();
  const int nw = blockDim.x >> 5;
  v = (threadIdx.x < nw) ? scratch[threadIdx.x] : make_uint4(0, 0, 0, 0);
  if (warp == 0) v = warp_xor(v);
  return v;
}

// Exact XOR accumulation into a 4-word global accumulator.
__device__ __forceinline__ void atomic_xor4(uint32_t* acc, uint4 v) {
  if (v.x) atomicXor(acc + 0, v.x);
  if (v.y) atomicXor(acc + 1, v.y);
  if (v.z) atomicXor(acc + 2, v.z);
  if (v.w) atomicXor(acc + 3, v.w);
}

}  // namespace bf
