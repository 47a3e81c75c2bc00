// Device arithmetic in BabyBear (p = 15 * 2^27 + 1) and its quintic
// extension E = F[X] / (X^5 - 2) — the field pair of the reference's prime
// benches, Basefold<BabyBear, BinomialExtensionField<BabyBear, 5>, ...>
// (poly-commit/benches/poly-commit.rs:114-123, poly-commit/src/basefold.rs:
// 470-478).
//
// On the device an element is held in Montgomery form a R mod p, R = 2^32:
// a product is one 32 x 32 -> 64 multiply, one low multiply by -p^-1 and one
// multiply-add of p, all on the integer multiplier, plus a conditional
// subtraction.  Values cross the C ABI, the Merkle leaves and the transcript
// in canonical form (bincode of a BabyBear: its canonical value, 4 bytes
// little-endian), converted at those edges.
#pragma once
#include <cstdint>

namespace bb {

constexpr uint32_t P = 2013265921u;        // 0x78000001
constexpr uint32_t P_INV = 0x88000001u;      // p^-1 mod 2^32
constexpr uint32_t R2 = 0x45dddde3u;        // R^2 mod p (to Montgomery form)
constexpr uint32_t MONT_ONE = 0x0ffffffeu;  // R mod p
constexpr uint32_t MONT_INV2 = 0x07ffffffu; // 2^-1 R mod p
constexpr uint32_t W = 2;                   // X^5 = W

__host__ __device__ __forceinline__ uint32_t umin(uint32_t a, uint32_t b) { return a < b ? a : b; }
// a + b mod p for a, b < p: with s = a + b < 2^32, s - p wraps above s
// exactly when s < p, so the smaller of the two is the reduced sum.
__host__ __device__ __forceinline__ uint32_t add(uint32_t a, uint32_t b) {
  const uint32_t s = a + b;
  return umin(s, s - P);
}
// a - b mod p: d = a - b wraps above 2^31 > p when a < b, and then d + p
// wraps back into [0, p).
__host__ __device__ __forceinline__ uint32_t sub(uint32_t a, uint32_t b) {
  const uint32_t d = a - b;
  return umin(d, d + P);
}
// Montgomery product a b R^-1 mod p of a, b < p (R = 2^32): with t = a b and
// m = t p^-1 mod R, m p has the low word of t, so (t - m p) / R is
// hi(t) - hi(m p), in (-p, p); a negative difference wraps and gets p added.
__host__ __device__ __forceinline__ uint32_t mul(uint32_t a, uint32_t b) {
  const uint64_t t = (uint64_t)a * b;
  const uint32_t m = (uint32_t)t * P_INV;
  const uint32_t mh = (uint32_t)(((uint64_t)m * P) >> 32);
  const uint32_t d = (uint32_t)(t >> 32) - mh;
  return umin(d, d + P);
}
// Shoup product a w mod p for any 32-bit a and a fixed w < p, given
// ws = floor(w 2^32 / p): q = hi(a ws) is below a w / p by less than 2, so
// a w - q p (mod 2^32) lies in [0, 2p).  One high multiply instead of the
// Montgomery product's wide and high ones; with a in Montgomery form and w
// canonical, the product stays in Montgomery form.
__host__ __device__ __forceinline__ uint32_t shoup_quot(uint32_t w) { return (uint32_t)(((uint64_t)w << 32) / P); }
#ifdef __CUDACC__
__device__ __forceinline__ uint32_t mul_shoup(uint32_t a, uint2 f) {  // f = (w, shoup_quot(w))
  const uint32_t r = a * f.x - __umulhi(a, f.y) * P;
  return umin(r, r - P);
}
#endif
__host__ __device__ __forceinline__ uint32_t to_mont(uint32_t a) { return mul(a, R2); }
__host__ __device__ __forceinline__ uint32_t from_mont(uint32_t a) { return mul(a, 1u); }

// Extension element: coefficients of 1, X, .., X^4, each in Montgomery form.
struct E5 {
  uint32_t c[5];
};
__host__ __device__ __forceinline__ E5 e_zero() { return E5{{0, 0, 0, 0, 0}}; }
__host__ __device__ __forceinline__ E5 e_from(uint32_t f) { return E5{{f, 0, 0, 0, 0}}; }
__host__ __device__ __forceinline__ E5 e_add(const E5& a, const E5& b) {
  E5 r;
  for (int i = 0; i < 5; ++i) r.c[i] = add(a.c[i], b.c[i]);
  return r;
}
__host__ __device__ __forceinline__ E5 e_sub(const E5& a, const E5& b) {
  E5 r;
  for (int i = 0; i < 5; ++i) r.c[i] = sub(a.c[i], b.c[i]);
  return r;
}
__host__ __device__ __forceinline__ E5 e_scale(const E5& a, uint32_t f) {
  E5 r;
  for (int i = 0; i < 5; ++i) r.c[i] = mul(a.c[i], f);
  return r;
}
// (sum_i a_i X^i)(sum_j b_j X^j) with X^5 = 2: coefficient k takes the
// products with i + j = k and twice those with i + j = k + 5.
__host__ __device__ __forceinline__ E5 e_mul(const E5& a, const E5& b) {
  uint32_t lo[5] = {0, 0, 0, 0, 0}, hi[4] = {0, 0, 0, 0};
  for (int i = 0; i < 5; ++i)
    for (int j = 0; j < 5; ++j) {
      const uint32_t t = mul(a.c[i], b.c[j]);
      if (i + j < 5)
        lo[i + j] = add(lo[i + j], t);
      else
        hi[i + j - 5] = add(hi[i + j - 5], t);
    }
  E5 r;
  for (int k = 0; k < 5; ++k) r.c[k] = k < 4 ? add(lo[k], add(hi[k], hi[k])) : lo[k];
  return r;
}

}  // namespace bb
