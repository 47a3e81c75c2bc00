// Host-side scalar arithmetic of the prover: the POLYVAL field for the
// per-round sumcheck scalars, Keccak-256 for the Fiat–Shamir transcript and
// the transcript itself.  Only O(num_vars) scalars and a few hundred bytes
// per round are handled here; every array of the path stays on the GPU.
#pragma once
#include <cstdint>
#include <cstring>
#include <vector>
#include <string>

namespace bfh {

typedef unsigned __int128 u128;

static inline u128 mk(uint64_t lo, uint64_t hi) { return ((u128)hi << 64) | lo; }

// Carry-less 32x32 -> 64 with integer products of operands whose bits are
// four apart (the same construction as the device multiply).
static inline uint64_t clmul32(uint32_t a, uint32_t b) {
  const uint32_t m[4] = {0x11111111u, 0x22222222u, 0x44444444u, 0x88888888u};
  const uint64_t M[4] = {0x1111111111111111ull, 0x2222222222222222ull, 0x4444444444444444ull,
                         0x8888888888888888ull};
  uint64_t a_[4], b_[4], z[4] = {0, 0, 0, 0};
  for (int i = 0; i < 4; ++i) {
    a_[i] = a & m[i];
    b_[i] = b & m[i];
  }
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) z[(i + j) & 3] ^= a_[i] * b_[j];
  return (z[0] & M[0]) | (z[1] & M[1]) | (z[2] & M[2]) | (z[3] & M[3]);
}

static inline void clmul64(uint64_t a, uint64_t b, uint64_t& lo, uint64_t& hi) {
  uint32_t a0 = (uint32_t)a, a1 = (uint32_t)(a >> 32), b0 = (uint32_t)b, b1 = (uint32_t)(b >> 32);
  uint64_t p0 = clmul32(a0, b0), p2 = clmul32(a1, b1), p1 = clmul32(a0 ^ a1, b0 ^ b1) ^ p0 ^ p2;
  lo = p0 ^ (p1 << 32);
  hi = p2 ^ (p1 >> 32);
}

// a*b*x^-128 mod x^128 + x^127 + x^126 + x^121 + 1
static inline u128 mul(u128 a, u128 b) {
  uint64_t a0 = (uint64_t)a, a1 = (uint64_t)(a >> 64), b0 = (uint64_t)b, b1 = (uint64_t)(b >> 64);
  uint64_t l0, l1, h0, h1, m0, m1;
  clmul64(a0, b0, l0, l1);
  clmul64(a1, b1, h0, h1);
  clmul64(a0 ^ a1, b0 ^ b1, m0, m1);
  m0 ^= l0 ^ h0;
  m1 ^= l1 ^ h1;
  uint64_t c0 = l0, c1 = l1 ^ m0, c2 = h0 ^ m1, c3 = h1;
  c1 ^= (c0 << 63) ^ (c0 << 62) ^ (c0 << 57);
  c2 ^= c0 ^ (c0 >> 1) ^ (c0 >> 2) ^ (c0 >> 7);
  c2 ^= (c1 << 63) ^ (c1 << 62) ^ (c1 << 57);
  c3 ^= c1 ^ (c1 >> 1) ^ (c1 >> 2) ^ (c1 >> 7);
  return mk(c2, c3);
}

// Montgomery form of 1: x^128 mod P (the reference's Polyval::ONE).
static inline u128 one() { return mk(1, 0xc200000000000000ull); }
static inline u128 sq(u128 a) { return mul(a, a); }

// x^(2^128 - 2) = prod_{k=1..127} x^(2^k); zero maps to zero.
static inline u128 inv(u128 a) {
  u128 r = one(), p = a;
  for (int k = 1; k < 128; ++k) {
    p = sq(p);
    r = mul(r, p);
  }
  return r;
}

// Inverses of all entries with one field inversion (prefix products).
// Returns false when an entry is zero.
static inline bool batch_inverse(const std::vector<u128>& v, std::vector<u128>& out) {
  size_t n = v.size();
  out.assign(n, 0);
  if (n == 0) return true;
  std::vector<u128> pre(n);
  u128 acc = one();
  for (size_t i = 0; i < n; ++i) {
    if (v[i] == 0) return false;
    pre[i] = acc;
    acc = mul(acc, v[i]);
  }
  u128 ia = inv(acc);
  for (size_t i = n; i-- > 0;) {
    out[i] = mul(ia, pre[i]);
    ia = mul(ia, v[i]);
  }
  return true;
}

static inline u128 load(const uint8_t* p) {
  u128 v;
  std::memcpy(&v, p, 16);
  return v;
}
static inline void store(uint8_t* p, u128 v) { std::memcpy(p, &v, 16); }

// ---- Merkle digests as the device trees store them ----
// The device keeps tree digests with every 64-bit lane bit-interleaved (even
// bits, odd bits); this turns such a digest back into its 32 bytes.
inline uint32_t bi_shuffle32_host(uint32_t x) {
  uint32_t t;
  t = (x ^ (x >> 8)) & 0x0000FF00u;
  x ^= t ^ (t << 8);
  t = (x ^ (x >> 4)) & 0x00F000F0u;
  x ^= t ^ (t << 4);
  t = (x ^ (x >> 2)) & 0x0C0C0C0Cu;
  x ^= t ^ (t << 2);
  t = (x ^ (x >> 1)) & 0x22222222u;
  x ^= t ^ (t << 1);
  return x;
}
inline void digest_from_interleaved(const uint8_t in[32], uint8_t out[32]) {
  for (int l = 0; l < 4; ++l) {
    uint32_t e, o;
    std::memcpy(&e, in + 8 * l, 4);
    std::memcpy(&o, in + 8 * l + 4, 4);
    const uint32_t lo = bi_shuffle32_host((e & 0xFFFFu) | (o << 16));
    const uint32_t hi = bi_shuffle32_host((e >> 16) | (o & 0xFFFF0000u));
    std::memcpy(out + 8 * l, &lo, 4);
    std::memcpy(out + 8 * l + 4, &hi, 4);
  }
}

// ---- Keccak-256 (FIPS 202 permutation, original Keccak padding 0x01) ----
static const uint64_t kRC[24] = {
    0x0000000000000001ull, 0x0000000000008082ull, 0x800000000000808aull, 0x8000000080008000ull,
    0x000000000000808bull, 0x0000000080000001ull, 0x8000000080008081ull, 0x8000000000008009ull,
    0x000000000000008aull, 0x0000000000000088ull, 0x0000000080008009ull, 0x000000008000000aull,
    0x000000008000808bull, 0x800000000000008bull, 0x8000000000008089ull, 0x8000000000008003ull,
    0x8000000000008002ull, 0x8000000000000080ull, 0x000000000000800aull, 0x800000008000000aull,
    0x8000000080008081ull, 0x8000000000008080ull, 0x0000000080000001ull, 0x8000000080008008ull};
static const int kRho[25] = {0, 1, 62, 28, 27, 36, 44, 6, 55, 20, 3, 10, 43, 25, 39, 41, 45, 15, 21, 8, 18, 2, 61, 56, 14};

static inline uint64_t rotl(uint64_t v, int r) { return r ? (v << r) | (v >> (64 - r)) : v; }

// Keccak-f[1600] on 25 local lanes (a<x><y> = A[x + 5y]), one round per
// iteration written out: theta (column parities c, d = c[x-1] ^ rot(c[x+1], 1)),
// rho and pi (b[y][2x+3y] = rot(a[x][y] ^ d[x], r[x][y])), chi, iota.
static inline void keccak_f(uint64_t A[25]) {
  uint64_t a00 = A[0], a10 = A[1], a20 = A[2], a30 = A[3], a40 = A[4], a01 = A[5], a11 = A[6], a21 = A[7], a31 = A[8], a41 = A[9], a02 = A[10], a12 = A[11], a22 = A[12], a32 = A[13], a42 = A[14], a03 = A[15], a13 = A[16], a23 = A[17], a33 = A[18], a43 = A[19], a04 = A[20], a14 = A[21], a24 = A[22], a34 = A[23], a44 = A[24];
  for (int ir = 0; ir < 24; ++ir) {
    const uint64_t c0 = a00 ^ a01 ^ a02 ^ a03 ^ a04, c1 = a10 ^ a11 ^ a12 ^ a13 ^ a14,
                   c2 = a20 ^ a21 ^ a22 ^ a23 ^ a24, c3 = a30 ^ a31 ^ a32 ^ a33 ^ a34,
                   c4 = a40 ^ a41 ^ a42 ^ a43 ^ a44;
    const uint64_t d0 = c4 ^ rotl(c1, 1);
    const uint64_t d1 = c0 ^ rotl(c2, 1);
    const uint64_t d2 = c1 ^ rotl(c3, 1);
    const uint64_t d3 = c2 ^ rotl(c4, 1);
    const uint64_t d4 = c3 ^ rotl(c0, 1);
    const uint64_t b00 = (a00 ^ d0);
    const uint64_t b10 = rotl(a11 ^ d1, 44);
    const uint64_t b20 = rotl(a22 ^ d2, 43);
    const uint64_t b30 = rotl(a33 ^ d3, 21);
    const uint64_t b40 = rotl(a44 ^ d4, 14);
    const uint64_t b01 = rotl(a30 ^ d3, 28);
    const uint64_t b11 = rotl(a41 ^ d4, 20);
    const uint64_t b21 = rotl(a02 ^ d0, 3);
    const uint64_t b31 = rotl(a13 ^ d1, 45);
    const uint64_t b41 = rotl(a24 ^ d2, 61);
    const uint64_t b02 = rotl(a10 ^ d1, 1);
    const uint64_t b12 = rotl(a21 ^ d2, 6);
    const uint64_t b22 = rotl(a32 ^ d3, 25);
    const uint64_t b32 = rotl(a43 ^ d4, 8);
    const uint64_t b42 = rotl(a04 ^ d0, 18);
    const uint64_t b03 = rotl(a40 ^ d4, 27);
    const uint64_t b13 = rotl(a01 ^ d0, 36);
    const uint64_t b23 = rotl(a12 ^ d1, 10);
    const uint64_t b33 = rotl(a23 ^ d2, 15);
    const uint64_t b43 = rotl(a34 ^ d3, 56);
    const uint64_t b04 = rotl(a20 ^ d2, 62);
    const uint64_t b14 = rotl(a31 ^ d3, 55);
    const uint64_t b24 = rotl(a42 ^ d4, 39);
    const uint64_t b34 = rotl(a03 ^ d0, 41);
    const uint64_t b44 = rotl(a14 ^ d1, 2);
    a00 = b00 ^ (~b10 & b20);
    a10 = b10 ^ (~b20 & b30);
    a20 = b20 ^ (~b30 & b40);
    a30 = b30 ^ (~b40 & b00);
    a40 = b40 ^ (~b00 & b10);
    a01 = b01 ^ (~b11 & b21);
    a11 = b11 ^ (~b21 & b31);
    a21 = b21 ^ (~b31 & b41);
    a31 = b31 ^ (~b41 & b01);
    a41 = b41 ^ (~b01 & b11);
    a02 = b02 ^ (~b12 & b22);
    a12 = b12 ^ (~b22 & b32);
    a22 = b22 ^ (~b32 & b42);
    a32 = b32 ^ (~b42 & b02);
    a42 = b42 ^ (~b02 & b12);
    a03 = b03 ^ (~b13 & b23);
    a13 = b13 ^ (~b23 & b33);
    a23 = b23 ^ (~b33 & b43);
    a33 = b33 ^ (~b43 & b03);
    a43 = b43 ^ (~b03 & b13);
    a04 = b04 ^ (~b14 & b24);
    a14 = b14 ^ (~b24 & b34);
    a24 = b24 ^ (~b34 & b44);
    a34 = b34 ^ (~b44 & b04);
    a44 = b44 ^ (~b04 & b14);
    a00 ^= kRC[ir];

  }
  A[0] = a00;
  A[1] = a10;
  A[2] = a20;
  A[3] = a30;
  A[4] = a40;
  A[5] = a01;
  A[6] = a11;
  A[7] = a21;
  A[8] = a31;
  A[9] = a41;
  A[10] = a02;
  A[11] = a12;
  A[12] = a22;
  A[13] = a32;
  A[14] = a42;
  A[15] = a03;
  A[16] = a13;
  A[17] = a23;
  A[18] = a33;
  A[19] = a43;
  A[20] = a04;
  A[21] = a14;
  A[22] = a24;
  A[23] = a34;
  A[24] = a44;
}

static inline void keccak256(const uint8_t* msg, size_t len, uint8_t out[32]) {
  uint64_t A[25] = {0};
  const size_t rate = 136;
  while (len >= rate) {
    for (int i = 0; i < 17; ++i) {
      uint64_t v;
      std::memcpy(&v, msg + 8 * i, 8);
      A[i] ^= v;
    }
    keccak_f(A);
    msg += rate;
    len -= rate;
  }
  uint8_t block[136] = {0};
  if (len) std::memcpy(block, msg, len);
  block[len] ^= 0x01;
  block[rate - 1] ^= 0x80;
  for (int i = 0; i < 17; ++i) {
    uint64_t v;
    std::memcpy(&v, block + 8 * i, 8);
    A[i] ^= v;
  }
  keccak_f(A);
  std::memcpy(out, A, 32);
}

// ---- Fiat–Shamir transcript -----------------------------------------------
// The reference's GenericChallenger<Polyval, Keccak256Hash>
// (p3/src/challenger.rs) over Plonky3's HashChallenger<u8, _, 32>:
// observing appends bytes to the input buffer and empties the output buffer;
// sampling a byte first (if the output buffer is empty) hashes the input
// buffer and makes the 32-byte digest both the output and the new input
// buffer, then pops the LAST output byte.  A field element is 16 popped bytes
// read little-endian; sample_bits pops 8 bytes as a little-endian usize.
struct Challenger {
  std::vector<uint8_t> in, out;
  void observe(const uint8_t* p, size_t n) {
    out.clear();
    in.insert(in.end(), p, p + n);
  }
  void observe_elem(u128 v) {
    uint8_t b[16];
    store(b, v);
    observe(b, 16);
  }
  uint8_t sample_byte() {
    if (out.empty()) {
      uint8_t d[32];
      keccak256(in.data(), in.size(), d);
      out.assign(d, d + 32);
      in.assign(d, d + 32);
    }
    uint8_t b = out.back();
    out.pop_back();
    return b;
  }
  u128 sample_elem() {
    uint8_t b[16];
    for (int i = 0; i < 16; ++i) b[i] = sample_byte();
    return load(b);
  }
  uint64_t sample_bits(int bits) {
    uint64_t v = 0;
    for (int i = 0; i < 8; ++i) v |= (uint64_t)sample_byte() << (8 * i);
    return bits >= 64 ? v : (v & (((uint64_t)1 << bits) - 1));
  }
  // [u64 in_len][in][u64 out_len][out]
  std::vector<uint8_t> blob() const {
    std::vector<uint8_t> b(16 + in.size() + out.size());
    uint64_t li = in.size(), lo = out.size();
    std::memcpy(b.data(), &li, 8);
    if (li) std::memcpy(b.data() + 8, in.data(), li);
    std::memcpy(b.data() + 8 + li, &lo, 8);
    if (lo) std::memcpy(b.data() + 16 + li, out.data(), lo);
    return b;
  }
  bool from_blob(const uint8_t* p, size_t n) {
    if (n < 16) return false;
    uint64_t li, lo;
    std::memcpy(&li, p, 8);
    if (li > n - 16) return false;
    std::memcpy(&lo, p + 8 + li, 8);
    if (n != 16 + li + lo) return false;
    in.assign(p + 8, p + 8 + li);
    out.assign(p + 16 + li, p + 16 + li + lo);
    return true;
  }
};

}  // namespace bfh
