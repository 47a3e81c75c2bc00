// Device Keccak-f[1600] and the fixed-length Keccak-256 digests of the
// Basefold Merkle trees.
//
// The reference hashes with Plonky3's Keccak256Hash over tiny-keccak 2.0.2
// `Keccak::v256` (original Keccak padding: 0x01 after the message, 0x80 in
// the last byte of the 136-byte rate).  Every message on the hot path fits
// one block: a codeword leaf is one 16-byte field element, a folded-codeword
// leaf is two elements (32 bytes), an inner node is left || right (64 bytes)
// (p3/src/symmetric.rs:11-26, p3/src/merkle_tree.rs:8-21).
//
// Lanes are 64-bit words kept as uint2 (x = low 32 bits); every rotation is
// two funnel shifts.  Constants are FIPS 202's round constants and rho
// offsets (checked against the spec's LFSR and lane walk by the tests).
//
// The Merkle-tree hashes run on bit-interleaved lanes instead: a lane is
// (even bits, odd bits), so a 64-bit rotation by an even amount is two
// 32-bit rotations, by an odd amount two with the halves swapped, and by one
// (theta) a single funnel shift — 6 fewer ALU instructions per round
// (measured on GB300: 4.67 vs 4.51 G permutations/s).  Digests stored in
// the trees stay interleaved, so a node hash reads its children as they are;
// only what leaves the trees (roots to the transcript and the host, query
// paths) is converted back to bytes.
#pragma once
#include <cstdint>

namespace bf {

__constant__ uint2 c_keccak_rc[24] = {
    {0x00000001u, 0x00000000u}, {0x00008082u, 0x00000000u}, {0x0000808au, 0x80000000u},
    {0x80008000u, 0x80000000u}, {0x0000808bu, 0x00000000u}, {0x80000001u, 0x00000000u},
    {0x80008081u, 0x80000000u}, {0x00008009u, 0x80000000u}, {0x0000008au, 0x00000000u},
    {0x00000088u, 0x00000000u}, {0x80008009u, 0x00000000u}, {0x8000000au, 0x00000000u},
    {0x8000808bu, 0x00000000u}, {0x0000008bu, 0x80000000u}, {0x00008089u, 0x80000000u},
    {0x00008003u, 0x80000000u}, {0x00008002u, 0x80000000u}, {0x00000080u, 0x80000000u},
    {0x0000800au, 0x00000000u}, {0x8000000au, 0x80000000u}, {0x80008081u, 0x80000000u},
    {0x00008080u, 0x80000000u}, {0x80000001u, 0x00000000u}, {0x80008008u, 0x80000000u},
};

__device__ __forceinline__ uint2 kx2(uint2 a, uint2 b) { return make_uint2(a.x ^ b.x, a.y ^ b.y); }
__device__ __forceinline__ uint2 kx3(uint2 a, uint2 b, uint2 c) {
  return make_uint2(a.x ^ b.x ^ c.x, a.y ^ b.y ^ c.y);
}
__device__ __forceinline__ uint2 kx5(uint2 a, uint2 b, uint2 c, uint2 d, uint2 e) {
  return make_uint2(a.x ^ b.x ^ c.x ^ d.x ^ e.x, a.y ^ b.y ^ c.y ^ d.y ^ e.y);
}
// a ^ (~b & c)
__device__ __forceinline__ uint2 kchi(uint2 a, uint2 b, uint2 c) {
  return make_uint2(a.x ^ (~b.x & c.x), a.y ^ (~b.y & c.y));
}
// 64-bit rotation by R in two funnel shifts.  (Measured on GB300: funnel
// shifts, LOP3 and IADD3 all issue at half rate on the ALU pipe; a rotation
// rebuilt from integer multiplies needs the quarter-rate IMAD.HI/IMAD.WIDE
// forms and was slower, so rotations stay on the ALU pipe.)
template <int R>
__device__ __forceinline__ uint2 krol(uint2 v) {
  if constexpr (R == 0) {
    return v;
  } else if constexpr (R < 32) {
    return make_uint2(__funnelshift_l(v.y, v.x, R), __funnelshift_l(v.x, v.y, R));
  } else if constexpr (R == 32) {
    return make_uint2(v.y, v.x);
  } else {
    return make_uint2(__funnelshift_l(v.x, v.y, R - 32), __funnelshift_l(v.y, v.x, R - 32));
  }
}

// ---- bit-interleaved lanes --------------------------------------------------
// Even bits of each 32-bit word to its low half, odd bits to its high half
// (an inverse perfect shuffle), and back.
__host__ __device__ __forceinline__ uint32_t bi_unshuffle32(uint32_t x) {
  uint32_t t;
  t = (x ^ (x >> 1)) & 0x22222222u;
  x ^= t ^ (t << 1);
  t = (x ^ (x >> 2)) & 0x0C0C0C0Cu;
  x ^= t ^ (t << 2);
  t = (x ^ (x >> 4)) & 0x00F000F0u;
  x ^= t ^ (t << 4);
  t = (x ^ (x >> 8)) & 0x0000FF00u;
  x ^= t ^ (t << 8);
  return x;
}
__host__ __device__ __forceinline__ uint32_t bi_shuffle32(uint32_t x) {
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
// 64-bit lane (x = low word) -> (even bits, odd bits), and back.
__device__ __forceinline__ uint2 bi_from_lane(uint2 v) {
  const uint32_t lo = bi_unshuffle32(v.x), hi = bi_unshuffle32(v.y);
  return make_uint2(__byte_perm(lo, hi, 0x5410), __byte_perm(lo, hi, 0x7632));
}
__device__ __forceinline__ uint2 bi_to_lane(uint2 v) {
  return make_uint2(bi_shuffle32(__byte_perm(v.x, v.y, 0x5410)), bi_shuffle32(__byte_perm(v.x, v.y, 0x7632)));
}

// FIPS 202 round constants, bit-interleaved (even bits, odd bits).
__constant__ uint2 c_keccak_rc_bi[24] = {
    {0x00000001u, 0x00000000u}, {0x00000000u, 0x00000089u}, {0x00000000u, 0x8000008bu},
    {0x00000000u, 0x80008080u}, {0x00000001u, 0x0000008bu}, {0x00000001u, 0x00008000u},
    {0x00000001u, 0x80008088u}, {0x00000001u, 0x80000082u}, {0x00000000u, 0x0000000bu},
    {0x00000000u, 0x0000000au}, {0x00000001u, 0x00008082u}, {0x00000000u, 0x00008003u},
    {0x00000001u, 0x0000808bu}, {0x00000001u, 0x8000000bu}, {0x00000001u, 0x8000008au},
    {0x00000001u, 0x80000081u}, {0x00000000u, 0x80000081u}, {0x00000000u, 0x80000008u},
    {0x00000000u, 0x00000083u}, {0x00000000u, 0x80008003u}, {0x00000001u, 0x80008088u},
    {0x00000000u, 0x80000088u}, {0x00000001u, 0x00008000u}, {0x00000000u, 0x80008082u},
};

__device__ __forceinline__ uint32_t rotl32(uint32_t x, int k) { return __funnelshift_l(x, x, k); }
// 64-bit rotation by R of an interleaved lane.
template <int R>
__device__ __forceinline__ uint2 krol_bi(uint2 v) {
  if constexpr (R == 0) {
    return v;
  } else if constexpr ((R & 1) == 0) {
    return make_uint2(rotl32(v.x, R / 2), rotl32(v.y, R / 2));
  } else if constexpr (R == 1) {
    return make_uint2(rotl32(v.y, 1), v.x);
  } else {
    return make_uint2(rotl32(v.y, (R + 1) / 2), rotl32(v.x, (R - 1) / 2));
  }
}

template <int R, bool BI>
__device__ __forceinline__ uint2 krot(uint2 v) {
  if constexpr (BI)
    return krol_bi<R>(v);
  else
    return krol<R>(v);
}

// One round: theta, rho and pi into b[], chi back into s[], iota.  BI: the
// lanes are bit-interleaved.
template <bool BI = false>
__device__ __forceinline__ void keccak_round(uint2 s[25], uint2 rc) {
  uint2 C[5], D[5], b[25];
#pragma unroll
  for (int x = 0; x < 5; ++x) C[x] = kx5(s[x], s[x + 5], s[x + 10], s[x + 15], s[x + 20]);
#pragma unroll
  for (int x = 0; x < 5; ++x) D[x] = krot<1, BI>(C[(x + 1) % 5]);
#pragma unroll
  for (int i = 0; i < 25; ++i) s[i] = kx3(s[i], C[(i + 4) % 5], D[i % 5]);
  // b[y + 5 ((2x + 3y) mod 5)] = rot(s[x + 5y], r[x, y])
  b[0] = s[0];
  b[10] = krot<1, BI>(s[1]);
  b[20] = krot<62, BI>(s[2]);
  b[5] = krot<28, BI>(s[3]);
  b[15] = krot<27, BI>(s[4]);
  b[16] = krot<36, BI>(s[5]);
  b[1] = krot<44, BI>(s[6]);
  b[11] = krot<6, BI>(s[7]);
  b[21] = krot<55, BI>(s[8]);
  b[6] = krot<20, BI>(s[9]);
  b[7] = krot<3, BI>(s[10]);
  b[17] = krot<10, BI>(s[11]);
  b[2] = krot<43, BI>(s[12]);
  b[12] = krot<25, BI>(s[13]);
  b[22] = krot<39, BI>(s[14]);
  b[23] = krot<41, BI>(s[15]);
  b[8] = krot<45, BI>(s[16]);
  b[18] = krot<15, BI>(s[17]);
  b[3] = krot<21, BI>(s[18]);
  b[13] = krot<8, BI>(s[19]);
  b[14] = krot<18, BI>(s[20]);
  b[24] = krot<2, BI>(s[21]);
  b[9] = krot<61, BI>(s[22]);
  b[19] = krot<56, BI>(s[23]);
  b[4] = krot<14, BI>(s[24]);
#pragma unroll
  for (int y = 0; y < 25; y += 5) {
#pragma unroll
    for (int x = 0; x < 5; ++x) s[y + x] = kchi(b[y + x], b[y + (x + 1) % 5], b[y + (x + 2) % 5]);
  }
  s[0] = kx2(s[0], rc);
}

// Last round when only the 32-byte digest (lanes 0..3) is wanted: theta is
// still needed in full, but rho/pi/chi only for the five lanes of row y = 0.
template <bool BI = false>
__device__ __forceinline__ void keccak_round_digest(uint2 s[25], uint2 rc) {
  uint2 C[5], D[5];
#pragma unroll
  for (int x = 0; x < 5; ++x) C[x] = kx5(s[x], s[x + 5], s[x + 10], s[x + 15], s[x + 20]);
#pragma unroll
  for (int x = 0; x < 5; ++x) D[x] = krot<1, BI>(C[(x + 1) % 5]);
  // row y = 0 of b takes lanes 0, 6, 12, 18, 24
  const uint2 b0 = kx3(s[0], C[4], D[0]);
  const uint2 b1 = krot<44, BI>(kx3(s[6], C[0], D[1]));
  const uint2 b2 = krot<43, BI>(kx3(s[12], C[1], D[2]));
  const uint2 b3 = krot<21, BI>(kx3(s[18], C[2], D[3]));
  const uint2 b4 = krot<14, BI>(kx3(s[24], C[3], D[4]));
  s[0] = kx2(kchi(b0, b1, b2), rc);
  s[1] = kchi(b1, b2, b3);
  s[2] = kchi(b2, b3, b4);
  s[3] = kchi(b3, b4, b0);
}

template <bool BI>
__device__ __forceinline__ uint2 keccak_rc(int r) {
  return BI ? c_keccak_rc_bi[r] : c_keccak_rc[r];
}

// Full permutation.  The first round is peeled so that the compiler folds
// the lanes a fixed-length message leaves constant (zero or padding).
template <bool BI = false>
__device__ __forceinline__ void keccak_f1600(uint2 s[25]) {
  keccak_round<BI>(s, keccak_rc<BI>(0));
#pragma unroll 2
  for (int r = 1; r < 23; ++r) keccak_round<BI>(s, keccak_rc<BI>(r));
  keccak_round<BI>(s, keccak_rc<BI>(23));
}

// Permutation whose output is only read in lanes 0..3.
template <bool BI = false>
__device__ __forceinline__ void keccak_f1600_digest(uint2 s[25]) {
  keccak_round<BI>(s, keccak_rc<BI>(0));
#pragma unroll 2
  for (int r = 1; r < 23; ++r) keccak_round<BI>(s, keccak_rc<BI>(r));
  keccak_round_digest<BI>(s, keccak_rc<BI>(23));
}

// Absorb `nlanes` message lanes (already in s[0..nlanes)), pad and permute.
// The digest is lanes 0..3 (32 bytes, little-endian).  The padding bits (bit
// 0 of lane nlanes, bit 63 of lane 16) sit at the same word and bit in the
// interleaved form (even bit 0; odd bit 31).
template <bool BI = false>
__device__ __forceinline__ void keccak256_lanes(uint2 s[25], int nlanes) {
#pragma unroll
  for (int i = 0; i < 25; ++i)
    if (i >= nlanes) s[i] = make_uint2(0, 0);
  // nlanes <= 16 here, so the 0x01 byte and the final 0x80 byte never share a lane.
#pragma unroll
  for (int i = 0; i < 17; ++i)
    if (i == nlanes) s[i].x ^= 0x01u;
  s[16].y ^= 0x80000000u;
  keccak_f1600_digest<BI>(s);
}

struct Digest {
  uint4 lo, hi;  // bytes 0..15, 16..31
};

__device__ __forceinline__ Digest digest_from_state(const uint2 s[25]) {
  Digest d;
  d.lo = make_uint4(s[0].x, s[0].y, s[1].x, s[1].y);
  d.hi = make_uint4(s[2].x, s[2].y, s[3].x, s[3].y);
  return d;
}

// ---- Merkle-tree hashes: digests are returned (and stored) interleaved ----

// keccak256 of one 16-byte field element.
__device__ __forceinline__ Digest hash_elem(uint4 e) {
  uint2 s[25];
  s[0] = bi_from_lane(make_uint2(e.x, e.y));
  s[1] = bi_from_lane(make_uint2(e.z, e.w));
  keccak256_lanes<true>(s, 2);
  return digest_from_state(s);
}

// keccak256 of two field elements (32 bytes).
__device__ __forceinline__ Digest hash_pair(uint4 a, uint4 b) {
  uint2 s[25];
  s[0] = bi_from_lane(make_uint2(a.x, a.y));
  s[1] = bi_from_lane(make_uint2(a.z, a.w));
  s[2] = bi_from_lane(make_uint2(b.x, b.y));
  s[3] = bi_from_lane(make_uint2(b.z, b.w));
  keccak256_lanes<true>(s, 4);
  return digest_from_state(s);
}

// keccak256(left || right), 64 bytes, of two interleaved digests: their
// lanes are the message lanes in interleaved form as they are.
__device__ __forceinline__ Digest hash_node(const Digest& l, const Digest& r) {
  uint2 s[25];
  s[0] = make_uint2(l.lo.x, l.lo.y);
  s[1] = make_uint2(l.lo.z, l.lo.w);
  s[2] = make_uint2(l.hi.x, l.hi.y);
  s[3] = make_uint2(l.hi.z, l.hi.w);
  s[4] = make_uint2(r.lo.x, r.lo.y);
  s[5] = make_uint2(r.lo.z, r.lo.w);
  s[6] = make_uint2(r.hi.x, r.hi.y);
  s[7] = make_uint2(r.hi.z, r.hi.w);
  keccak256_lanes<true>(s, 8);
  return digest_from_state(s);
}

// A digest computed on standard lanes, interleaved for storage in a tree.
__device__ __forceinline__ Digest digest_interleaved(const Digest& d) {
  const uint2 l0 = bi_from_lane(make_uint2(d.lo.x, d.lo.y)), l1 = bi_from_lane(make_uint2(d.lo.z, d.lo.w));
  const uint2 l2 = bi_from_lane(make_uint2(d.hi.x, d.hi.y)), l3 = bi_from_lane(make_uint2(d.hi.z, d.hi.w));
  Digest o;
  o.lo = make_uint4(l0.x, l0.y, l1.x, l1.y);
  o.hi = make_uint4(l2.x, l2.y, l3.x, l3.y);
  return o;
}

// An interleaved digest as its 32 bytes (four little-endian lanes).
__device__ __forceinline__ Digest digest_bytes(const Digest& d) {
  const uint2 l0 = bi_to_lane(make_uint2(d.lo.x, d.lo.y)), l1 = bi_to_lane(make_uint2(d.lo.z, d.lo.w));
  const uint2 l2 = bi_to_lane(make_uint2(d.hi.x, d.hi.y)), l3 = bi_to_lane(make_uint2(d.hi.z, d.hi.w));
  Digest o;
  o.lo = make_uint4(l0.x, l0.y, l1.x, l1.y);
  o.hi = make_uint4(l2.x, l2.y, l3.x, l3.y);
  return o;
}

// ---------------------------------------------------------------------------
// Keccak-f[1600] spread over a warp, for latency-bound hashing (the top
// levels of a Merkle tree, the transcript): lane j < 25 holds state word
// A[x][y], j = x + 5y; lanes 25..31 only take part in the shuffles.  One
// round is nine 64-bit shuffles (theta column sums and neighbours, pi, chi)
// and a per-lane rotation.  Measured on GB300: 2.9 us per permutation on one
// warp, against 4.25 us for one thread (whose ~4450 instructions issue at
// the half-rate ALU pipe's pace) — so it pays only when each warp has a
// single permutation to do (a level of at most as many nodes as warps).
struct WarpKeccak {
  int lane, x, y;
  int col[4];      // theta: the other four lanes of this column
  int xm1, xp1;    // theta: lanes of columns x-1, x+1 in this row
  int pi_src;      // pi: B[x][y] = A[x'][y'] with x = y', y = 2x' + 3y'
  int chi1, chi2;  // chi: lanes of columns x+1, x+2 in this row
  int rho;         // rotation of this lane

  __device__ __forceinline__ WarpKeccak() {
    lane = threadIdx.x & 31;
    const int j = lane < 25 ? lane : 0;
    x = j % 5;
    y = j / 5;
#pragma unroll
    for (int k = 0; k < 4; ++k) col[k] = x + 5 * ((y + 1 + k) % 5);
    xm1 = (x + 4) % 5 + 5 * y;
    xp1 = (x + 1) % 5 + 5 * y;
    // lane (X, Y) receives A[x'][y'] with y' = X, x' = 3 (Y - 3X) mod 5
    const int xs = (3 * ((y - 3 * x) % 5 + 5)) % 5;
    pi_src = xs + 5 * x;
    chi1 = (x + 1) % 5 + 5 * y;
    chi2 = (x + 2) % 5 + 5 * y;
    // rotation of A[x][y] (FIPS 202 rho offsets), applied before pi moves it
    constexpr int kRho[25] = {0,  1,  62, 28, 27, 36, 44, 6,  55, 20, 3,  10, 43,
                              25, 39, 41, 45, 15, 21, 8,  18, 2,  61, 56, 14};
    int r = 0;
#pragma unroll
    for (int k = 0; k < 25; ++k)
      if (k == j) r = kRho[k];
    rho = r;
  }

  static __device__ __forceinline__ uint2 shfl(uint2 v, int src) {
    return make_uint2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
  }
  static __device__ __forceinline__ uint2 rolv(uint2 v, int r) {
    if (r & 32) v = make_uint2(v.y, v.x);
    const int s = r & 31;
    return make_uint2(__funnelshift_l(v.y, v.x, s), __funnelshift_l(v.x, v.y, s));
  }
  // the same on an interleaved lane
  static __device__ __forceinline__ uint2 rolv_bi(uint2 v, int r) {
    if (r & 1) return make_uint2(rotl32(v.y, (r + 1) >> 1), rotl32(v.x, r >> 1));
    return make_uint2(rotl32(v.x, r >> 1), rotl32(v.y, r >> 1));
  }

  // All 32 lanes call this; `a` is this lane's word (interleaved when BI).
  template <bool BI>
  __device__ __forceinline__ uint2 permute(uint2 a) const {
#pragma unroll 1
    for (int r = 0; r < 24; ++r) {
      const uint2 c1 = shfl(a, col[0]), c2 = shfl(a, col[1]), c3 = shfl(a, col[2]), c4 = shfl(a, col[3]);
      const uint2 c = kx5(a, c1, c2, c3, c4);  // C[x]
      const uint2 cm = shfl(c, xm1), cp = shfl(c, xp1);
      a = kx3(a, cm, krot<1, BI>(cp));         // theta
      a = BI ? rolv_bi(a, rho) : rolv(a, rho);  // rho
      const uint2 b = shfl(a, pi_src);         // pi
      const uint2 b1 = shfl(b, chi1), b2 = shfl(b, chi2);
      a = kchi(b, b1, b2);                     // chi
      if (lane == 0) a = kx2(a, keccak_rc<BI>(r));  // iota
    }
    return a;
  }
};

// keccak256(left || right) of node `s` by one warp: lanes 0..7 read the 64
// message bytes, lanes 0..3 write the digest.
__device__ __forceinline__ void warp_hash_node(const WarpKeccak& wk, const uint4* cur, size_t s, size_t h, uint4* nxt) {
  const uint2* left = reinterpret_cast<const uint2*>(cur + 2 * s);
  const uint2* right = reinterpret_cast<const uint2*>(cur + 2 * (s + h));
  uint2 a = make_uint2(0, 0);
  if (wk.lane < 4) a = left[wk.lane];
  else if (wk.lane < 8) a = right[wk.lane - 4];
  if (wk.lane == 8) a.x ^= 0x01u;         // pad10*1 after 64 bytes
  if (wk.lane == 16) a.y ^= 0x80000000u;  // last byte of the 136-byte rate
  a = wk.permute<true>(a);  // interleaved digests in, interleaved digest out
  if (wk.lane < 4) reinterpret_cast<uint2*>(nxt + 2 * s)[wk.lane] = a;
}

// keccak256 of matrix rows of `words` 32-bit words, one lane per row, the
// 32 rows [r0, r0 + 32) per warp.  The 136-byte rate is 34 words, so every
// block of every row starts on a word: the warp stages the current block of
// its rows in shared memory (`st`: 32 x kStagePitch words) with loads whose
// 32 lanes read one 128-byte row run (8 in flight per lane), then each lane
// absorbs its row.  word_at(row, i) returns word i of a row (rows < `rows`,
// i < `words`); the 0x01 pad word follows the message and 0x80 ends the
// last block.  The row is absorbed and permuted on plain lanes (interleaving
// 17 message lanes per block would cost more than the interleaved rounds
// save); only the four digest lanes are interleaved, the trees' form.
constexpr int kRateWords = 34;
constexpr int kStagePitch = 35;  // odd pitch: lane r reads word r * 35 + i without bank conflicts
template <class WordAt>
__device__ __forceinline__ Digest keccak_rows_warp(uint32_t* st, size_t r0, size_t rows, uint32_t words,
                                                   const WordAt& word_at) {
  const uint32_t lane = threadIdx.x & 31u;
  uint2 s[25];
#pragma unroll
  for (int i = 0; i < 25; ++i) s[i] = make_uint2(0, 0);
  const uint32_t nblk = words / kRateWords + 1;
  for (uint32_t blk = 0; blk < nblk; ++blk) {
    auto pad = [&](uint32_t i, uint32_t v) {
      const uint32_t col = blk * kRateWords + i;
      uint32_t o = col < words ? v : (col == words ? 0x01u : 0u);
      if (blk == nblk - 1 && i == kRateWords - 1) o |= 0x80000000u;
      return o;
    };
    const uint32_t col = blk * kRateWords + lane;  // words 0..31 of the block: lane = word
#pragma unroll 1
    for (int h = 0; h < 32; h += 8) {
      uint32_t raw[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) raw[k] = (col < words && r0 + h + k < rows) ? word_at(r0 + h + k, col) : 0u;
#pragma unroll
      for (int k = 0; k < 8; ++k) st[(h + k) * kStagePitch + lane] = pad(lane, raw[k]);
    }
#pragma unroll
    for (int i = 32; i < kRateWords; ++i) {  // words 32, 33: lane = row
      const uint32_t c2 = blk * kRateWords + i;
      const uint32_t v = (c2 < words && r0 + lane < rows) ? word_at(r0 + lane, c2) : 0u;
      st[lane * kStagePitch + i] = pad(i, v);
    }
    __syncwarp();
#pragma unroll
    for (int k = 0; k < 17; ++k) {
      s[k].x ^= st[lane * kStagePitch + 2 * k];
      s[k].y ^= st[lane * kStagePitch + 2 * k + 1];
    }
    __syncwarp();
    if (blk + 1 < nblk)
      keccak_f1600<false>(s);
    else
      keccak_f1600_digest<false>(s);
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) s[i] = bi_from_lane(s[i]);
  return digest_from_state(s);
}

__device__ __forceinline__ Digest load_digest(const uint4* p, size_t i) {
  Digest d;
  d.lo = p[2 * i];
  d.hi = p[2 * i + 1];
  return d;
}
__device__ __forceinline__ void store_digest(uint4* p, size_t i, const Digest& d) {
  p[2 * i] = d.lo;
  p[2 * i + 1] = d.hi;
}

}  // namespace bf
