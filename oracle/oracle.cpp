// ORACLE — test infrastructure only.
//
// CPU restatement of han0110/learn-zkp's Basefold prover path over the binary
// field POLYVAL with the binary Reed–Solomon code.  It exists to check the CUDA
// library: only the tests, the smoke check and the CPU-baseline leg of the
// benchmark may load it.  It is never part of the product path.
//
// Parity status.  The reference (Rust, Plonky3@784b7dd) cannot be compiled in
// this environment (no cargo/rustc, no vendored crates), and its own tests hold
// no golden vectors.  This restatement is pinned against:
//   * the reference's own constants read out of its sources (the x^256 mod P
//     constant of p3/src/polyval/portable.rs:12 and the nibble table of
//     portable.rs:169-376), see tests/golden/make_golden.py;
//   * the RFC 8452 POLYVAL known-answer vector and FIPS 202 (SHA3-256 from
//     Python hashlib) for the Keccak-f[1600] permutation;
//   * the reference's definitional test of the additive NTT
//     (p3/src/field/binary.rs:149-203), restated here as
//     orc_ntt_forward_definition.
// The Plonky3 behaviour this file restates (HashChallenger, MerkleTreeMmcs,
// bincode layout) is written from its published semantics and is NOT pinned
// by any byte-level vector.
//
// Field elements travel across the C interface as 16 raw little-endian bytes
// (the Montgomery-form u128 that Polyval stores, p3/src/polyval.rs:30-34).

#include <cstdint>
#include <cstring>
#include <cmath>
#include <vector>
#include <thread>
#include <algorithm>
#include <functional>
#include <cstdlib>

#if defined(__aarch64__) && defined(ORACLE_PMULL)
#include <arm_neon.h>
#endif

typedef unsigned __int128 u128;

namespace orc {

// ---------------------------------------------------------------------------
// Threading: rayon-style data parallelism over index ranges.
// ---------------------------------------------------------------------------
static int g_threads = 0;

static int num_threads() {
  if (g_threads > 0) return g_threads;
  const char* e = std::getenv("ORACLE_THREADS");
  int n = e ? std::atoi(e) : 0;
  if (n <= 0) n = (int)std::thread::hardware_concurrency();
  if (n <= 0) n = 1;
  g_threads = n;
  return n;
}

// f(begin, end) over [0, n) split into contiguous chunks.
static void parallel_for(size_t n, const std::function<void(size_t, size_t)>& f,
                         size_t grain = 1024) {
  int nt = num_threads();
  if (nt <= 1 || n <= grain) {
    f(0, n);
    return;
  }
  size_t chunks = std::min<size_t>((size_t)nt, (n + grain - 1) / grain);
  std::vector<std::thread> ts;
  ts.reserve(chunks);
  size_t per = (n + chunks - 1) / chunks;
  for (size_t c = 0; c < chunks; ++c) {
    size_t b = c * per, e = std::min(n, b + per);
    if (b >= e) break;
    ts.emplace_back([&f, b, e]() { f(b, e); });
  }
  for (auto& t : ts) t.join();
}

// ---------------------------------------------------------------------------
// POLYVAL field (p3/src/polyval.rs, p3/src/polyval/portable.rs).
//
// An element is the raw u128 `value` of Polyval; bit i is the coefficient of
// x^i.  Multiplication is the POLYVAL "dot" of RFC 8452 section 3:
// a*b*x^-128 mod P, P = x^128 + x^127 + x^126 + x^121 + 1
// (portable.rs:20-28).  Addition is XOR (polyval.rs:183-191).
// ---------------------------------------------------------------------------

static inline u128 mk(uint64_t lo, uint64_t hi) { return ((u128)hi << 64) | lo; }

// Carry-less 64x64 -> 128 product.
static inline u128 clmul64(uint64_t a, uint64_t b) {
#if defined(__aarch64__) && defined(ORACLE_PMULL)
  poly128_t r = vmull_p64((poly64_t)a, (poly64_t)b);
  u128 out;
  std::memcpy(&out, &r, 16);
  return out;
#else
  // 4-bit window: tab[k] = a*k as polynomials, k < 16.
  u128 tab[16];
  tab[0] = 0;
  tab[1] = a;
  for (int k = 2; k < 16; ++k) tab[k] = (k & 1) ? (tab[k - 1] ^ (u128)a) : (tab[k >> 1] << 1);
  u128 r = 0;
  for (int i = 15; i >= 0; --i) r = (r << 4) ^ tab[(b >> (4 * i)) & 15];
  return r;
#endif
}

// Montgomery product a*b*x^-128 mod P.  The 256-bit carry-less product is
// reduced by cancelling its low 128 bits with multiples of P
// (P = 1 + x^121 + x^126 + x^127 + x^128), 64 bits at a time.
static inline u128 mul(u128 a, u128 b) {
  uint64_t a0 = (uint64_t)a, a1 = (uint64_t)(a >> 64);
  uint64_t b0 = (uint64_t)b, b1 = (uint64_t)(b >> 64);
  u128 lo = clmul64(a0, b0);
  u128 hi = clmul64(a1, b1);
  u128 mid = clmul64(a0 ^ a1, b0 ^ b1) ^ lo ^ hi;
  uint64_t c0 = (uint64_t)lo;
  uint64_t c1 = (uint64_t)(lo >> 64) ^ (uint64_t)mid;
  uint64_t c2 = (uint64_t)hi ^ (uint64_t)(mid >> 64);
  uint64_t c3 = (uint64_t)(hi >> 64);
  c1 ^= (c0 << 63) ^ (c0 << 62) ^ (c0 << 57);
  c2 ^= c0 ^ (c0 >> 1) ^ (c0 >> 2) ^ (c0 >> 7);
  c2 ^= (c1 << 63) ^ (c1 << 62) ^ (c1 << 57);
  c3 ^= c1 ^ (c1 >> 1) ^ (c1 >> 2) ^ (c1 >> 7);
  return mk(c2, c3);
}

static inline u128 add(u128 a, u128 b) { return a ^ b; }
static inline u128 sq(u128 a) { return mul(a, a); }

// x * v mod P (plain polynomial arithmetic, no Montgomery factor).
static inline u128 mul_x(u128 v) {
  bool carry = (v >> 127) & 1;
  v <<= 1;
  if (carry) v ^= mk(1, 0) ^ ((u128)1 << 121) ^ ((u128)1 << 126) ^ ((u128)1 << 127);
  return v;
}

// x^k mod P
static u128 x_pow(int k) {
  u128 v = 1;
  for (int i = 0; i < k; ++i) v = mul_x(v);
  return v;
}

// Montgomery constants: R = x^128 mod P is the Montgomery form of 1
// (Polyval::ONE, polyval.rs:85); R2 = x^256 mod P converts canonical values
// into Montgomery form (portable.rs:10-13).
static u128 g_one = 0, g_r2 = 0;
static void init_consts() {
  if (g_one) return;
  g_one = x_pow(128);
  g_r2 = x_pow(256);
}
static inline u128 one() { init_consts(); return g_one; }
static inline u128 from_canonical(u128 v) { init_consts(); return mul(v, g_r2); }
static inline u128 to_canonical(u128 v) { return mul(v, 1); }
// Polyval::basis(i) = from_canonical(1 << i) (polyval.rs:167-172).
static inline u128 basis(int i) { return from_canonical((u128)1 << i); }

// Inverse: a^(2^128 - 2) = prod_{k=1..127} a^(2^k) (Fermat).  Zero maps to
// zero, like invert_or_zero (portable.rs:113).
static u128 inv(u128 a) {
  u128 r = one();
  u128 p = a;
  for (int k = 1; k < 128; ++k) {
    p = sq(p);
    r = mul(r, p);
  }
  return r;
}

// Definition-level product, independent of the fast path above: the plain
// product mod P by shift-and-add, then times x^-128 (x^-1 applied 128 times).
static u128 mul_definition(u128 a, u128 b) {
  u128 acc = 0, sh = a;
  for (int i = 0; i < 128; ++i) {
    if ((b >> i) & 1) acc ^= sh;
    sh = mul_x(sh);
  }
  // divide by x 128 times: v/x = (v + v0*P)/x
  u128 pl = mk(1, 0) ^ ((u128)1 << 121) ^ ((u128)1 << 126) ^ ((u128)1 << 127);
  for (int i = 0; i < 128; ++i) {
    bool low = acc & 1;
    if (low) {
      acc ^= pl;  // acc + P without the x^128 term; the x^128 term enters as the carried-in top bit
      acc >>= 1;
      acc |= (u128)1 << 127;
    } else {
      acc >>= 1;
    }
  }
  return acc;
}

static inline u128 load(const uint8_t* p) {
  u128 v;
  std::memcpy(&v, p, 16);  // little-endian hosts only (x86_64, aarch64)
  return v;
}
static inline void store(uint8_t* p, u128 v) { std::memcpy(p, &v, 16); }

// ---------------------------------------------------------------------------
// Keccak-f[1600] and Keccak-256 (FIPS 202; original Keccak padding 0x01 as
// used by tiny-keccak 2.0.2 `Keccak::v256`, reached through Plonky3's
// Keccak256Hash).
// ---------------------------------------------------------------------------
struct KeccakTables {
  uint64_t rc[24];
  int rho[25];
};

// Round constants from the rc(t) LFSR of FIPS 202 section 3.2.5 and rho
// offsets from the (x, y) walk of section 3.2.2, evaluated at compile time.
static constexpr KeccakTables make_keccak_tables() {
  KeccakTables t{};
  for (int ir = 0; ir < 24; ++ir) {
    uint64_t rc = 0;
    for (int j = 0; j <= 6; ++j) {
      int tt = (j + 7 * ir) % 255;
      unsigned R = 0x01;
      for (int i = 1; i <= tt; ++i) {
        unsigned r8 = (R >> 7) & 1;
        R = (R << 1) & 0xff;
        if (r8) R ^= 0x71;  // R[0], R[4], R[5], R[6] ^= R[8]
      }
      if (R & 1) rc |= (uint64_t)1 << ((1u << j) - 1);
    }
    t.rc[ir] = rc;
  }
  t.rho[0] = 0;
  int x = 1, y = 0;
  for (int s = 0; s < 24; ++s) {
    t.rho[x + 5 * y] = ((s + 1) * (s + 2) / 2) % 64;
    int nx = y, ny = (2 * x + 3 * y) % 5;
    x = nx;
    y = ny;
  }
  return t;
}
static constexpr KeccakTables KT = make_keccak_tables();

static inline uint64_t rotl(uint64_t v, int r) { return r ? (v << r) | (v >> (64 - r)) : v; }

static void keccak_f(uint64_t A[25]) {
  for (int ir = 0; ir < 24; ++ir) {
    uint64_t C[5], B[25];
#pragma GCC unroll 5
    for (int x = 0; x < 5; ++x) C[x] = A[x] ^ A[x + 5] ^ A[x + 10] ^ A[x + 15] ^ A[x + 20];
#pragma GCC unroll 25
    for (int i = 0; i < 25; ++i) A[i] ^= C[(i + 4) % 5] ^ rotl(C[(i + 1) % 5], 1);
    // rho and pi: B[y, 2x+3y] = rot(A[x, y], r[x, y])
#pragma GCC unroll 25
    for (int i = 0; i < 25; ++i) {
      const int x = i % 5, y = i / 5;
      B[y + 5 * ((2 * x + 3 * y) % 5)] = rotl(A[i], KT.rho[i]);
    }
#pragma GCC unroll 25
    for (int i = 0; i < 25; ++i) {
      const int x = i % 5, y5 = i - x;
      A[i] = B[i] ^ ((~B[y5 + (x + 1) % 5]) & B[y5 + (x + 2) % 5]);
    }
    A[0] ^= KT.rc[ir];
  }
}

// Sponge with rate 136 bytes and 32-byte output; `pad` is the first padding
// byte (0x01 Keccak, 0x06 SHA3).
static void sponge256(const uint8_t* msg, size_t len, uint8_t pad, uint8_t out[32]) {
  uint64_t A[25] = {0};
  const size_t rate = 136;
  uint8_t block[136];
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
  std::memset(block, 0, rate);
  std::memcpy(block, msg, len);
  block[len] ^= pad;
  block[rate - 1] ^= 0x80;
  for (int i = 0; i < 17; ++i) {
    uint64_t v;
    std::memcpy(&v, block + 8 * i, 8);
    A[i] ^= v;
  }
  keccak_f(A);
  std::memcpy(out, A, 32);
}

static inline void keccak256(const uint8_t* msg, size_t len, uint8_t out[32]) {
  sponge256(msg, len, 0x01, out);
}

struct Digest {
  uint8_t b[32];
};

// ---------------------------------------------------------------------------
// Additive NTT (p3/src/field/binary.rs).
// ---------------------------------------------------------------------------
static size_t reverse_bits_len(size_t x, int bits) {
  if (bits == 0) return 0;
  uint64_t v = x;
  v = ((v >> 1) & 0x5555555555555555ull) | ((v & 0x5555555555555555ull) << 1);
  v = ((v >> 2) & 0x3333333333333333ull) | ((v & 0x3333333333333333ull) << 2);
  v = ((v >> 4) & 0x0f0f0f0f0f0f0f0full) | ((v & 0x0f0f0f0f0f0f0f0full) << 4);
  v = ((v >> 8) & 0x00ff00ff00ff00ffull) | ((v & 0x00ff00ff00ff00ffull) << 8);
  v = ((v >> 16) & 0x0000ffff0000ffffull) | ((v & 0x0000ffff0000ffffull) << 16);
  v = (v >> 32) | (v << 32);
  return (size_t)(v >> (64 - bits));
}

// AddtiveNtt::new (binary.rs:23-53).  Returns `twiddles` in the reference's
// order: twiddles[t] is the table of stage log_n-1-t and has 2^t entries.
static std::vector<std::vector<u128>> ntt_twiddles(int log_n) {
  std::vector<std::vector<u128>> rev_tables;
  if (log_n == 0) return rev_tables;
  u128 w_beta_i = basis(0);
  std::vector<u128> w_betas;
  for (int i = 1; i < log_n; ++i) w_betas.push_back(basis(i));
  while (true) {
    u128 inv_i = inv(w_beta_i);
    std::vector<u128> tab((size_t)1 << w_betas.size(), 0);
    for (size_t j = 0; j < w_betas.size(); ++j) {
      u128 wb = mul(w_betas[j], inv_i);
      size_t h = (size_t)1 << j;
      for (size_t k = 0; k < h; ++k) tab[h + k] = tab[k] ^ wb;
    }
    rev_tables.push_back(std::move(tab));
    if (w_betas.empty()) break;
    // W_{i+1}(x) = W_i(x)^2 + W_i(x) W_i(beta_i)
    u128 wbi = w_beta_i;
    auto q = [wbi](u128 w) { return sq(w) ^ mul(w, wbi); };
    u128 first = q(w_betas[0]);
    std::vector<u128> rest;
    for (size_t j = 1; j < w_betas.size(); ++j) rest.push_back(q(w_betas[j]));
    w_beta_i = first;
    w_betas = rest;
  }
  std::reverse(rev_tables.begin(), rev_tables.end());
  return rev_tables;
}

// One layer (binary.rs:126-137) over a row-major matrix of `width` columns:
// chunks of 2<<i rows, chunk k uses tw[k].
static void ntt_layer(u128* data, size_t width, size_t height, int i, const u128* tw, bool inverse) {
  size_t half = (size_t)1 << i;
  size_t nchunks = height / (2 * half);
  parallel_for(nchunks * half, [&](size_t b, size_t e) {
    for (size_t idx = b; idx < e; ++idx) {
      size_t k = idx / half, r = idx % half;
      u128 t = tw[k];
      u128* lo = data + (k * 2 * half + r) * width;
      u128* hi = lo + half * width;
      for (size_t c = 0; c < width; ++c) {
        if (inverse) {
          hi[c] ^= lo[c];
          lo[c] ^= mul(hi[c], t);
        } else {
          lo[c] ^= mul(hi[c], t);
          hi[c] ^= lo[c];
        }
      }
    }
  }, 256);
}

// forward_batch_inplace / backward_batch_inplace (binary.rs:98-123) with a
// list of (possibly coset-restricted) tables: tables[t] belongs to layer
// log_n-1-t.
static void ntt_forward(u128* data, size_t width, int log_n, const std::vector<const u128*>& tables) {
  size_t height = (size_t)1 << log_n;
  for (int t = 0; t < log_n; ++t) ntt_layer(data, width, height, log_n - 1 - t, tables[t], false);
}
static void ntt_backward(u128* data, size_t width, int log_n, const std::vector<const u128*>& tables) {
  size_t height = (size_t)1 << log_n;
  for (int i = 0; i < log_n; ++i) ntt_layer(data, width, height, i, tables[log_n - 1 - i], true);
}

// The reference's definitional forward transform (binary.rs:149-192): the
// evaluation matrix of the novel polynomial basis built from normalised
// subspace polynomials on the points u = 0 .. 2^log_n - 1 (canonical
// integers mapped into the field).
static std::vector<u128> ntt_forward_definition(int log_n, const std::vector<u128>& data) {
  auto u = [](int i) {
    std::vector<u128> v;
    for (size_t k = 0; k < ((size_t)1 << i); ++k) v.push_back(from_canonical(k));
    return v;
  };
  auto w_beta = [&](int i) {  // prod_{u in U_i} (basis(i) - u)
    u128 p = one();
    for (u128 x : u(i)) p = mul(p, basis(i) ^ x);
    return p;
  };
  auto q = [&](int i, u128 x) {
    u128 wi = w_beta(i), wi1 = w_beta(i + 1);
    return mul(mul(mul(sq(wi), inv(wi1)), x), x ^ one());
  };
  std::function<std::vector<u128>(int, std::vector<u128>, u128)> recurse =
      [&](int i, std::vector<u128> s, u128 x) -> std::vector<u128> {
    if (s.size() == 1) return {one()};
    std::vector<u128> ns;
    for (u128 v : s) {
      u128 w = q(i, v);
      if (ns.empty() || ns.back() != w) ns.push_back(w);  // Itertools::dedup (consecutive)
    }
    std::vector<u128> sub = recurse(i + 1, ns, q(i, x));
    std::vector<u128> out;
    for (u128 v : sub) {
      out.push_back(v);
      out.push_back(mul(v, x));
    }
    return out;
  };
  std::vector<u128> pts = u(log_n);
  std::vector<u128> out;
  for (u128 x : pts) {
    std::vector<u128> row = recurse(0, pts, x);
    u128 acc = 0;
    for (size_t k = 0; k < row.size(); ++k) acc ^= mul(row[k], data[k]);
    out.push_back(acc);
  }
  return out;
}

// ---------------------------------------------------------------------------
// Binary Reed–Solomon code (poly-commit/src/basefold/code/binary_reed_solomon.rs).
// ---------------------------------------------------------------------------
struct Code {
  int lambda, log2_c, d;
  std::vector<std::vector<u128>> tw;  // AddtiveNtt::new(log2_c + d)
  Code(int lambda_, int log2_c_, int d_) : lambda(lambda_), log2_c(log2_c_), d(d_) {
    tw = ntt_twiddles(log2_c + d);
  }
  size_t c() const { return (size_t)1 << log2_c; }
  size_t k_d() const { return (size_t)1 << d; }  // log2_k_0 = 0 (:47-49)
  size_t n_d() const { return c() * k_d(); }
  size_t n_0() const { return c(); }
  size_t n_i(int i) const { return n_0() << i; }
  int log2_n_d() const { return log2_c + d; }
  // Formula 8 of 2024/504 (:55-59); a non-finite or non-positive quotient
  // saturates to 0 like Rust's float-to-usize cast.
  size_t num_queries() const {
    double delta = (1.0 + 1.0 / (double)c()) / 2.0;
    double q = std::ceil((double)lambda / -std::log2(delta));
    if (!(q > 0) || !std::isfinite(q)) return 0;
    return (size_t)q;
  }
  // twiddle_bo(i).nth(j) = twiddles[log2_c + i][rev(j)] (:29-35)
  u128 twiddle_bo(int i, size_t j) const {
    const std::vector<u128>& t = tw[log2_c + i];
    int bits = 0;
    while (((size_t)1 << bits) < t.size()) ++bits;
    return t[reverse_bits_len(j, bits)];
  }
  // encode_batch (:67-82)
  std::vector<u128> encode_batch(const std::vector<u128>& m, size_t width) const {
    std::vector<u128> out = encode_batch_unpermuted(m, width);
    size_t nd = n_d();
    std::vector<u128> res(nd * width);
    int lb = log2_n_d();
    for (size_t r = 0; r < nd; ++r)
      for (size_t c0 = 0; c0 < width; ++c0) res[r * width + c0] = out[reverse_bits_len(r, lb) * width + c0];
    return res;
  }
  // encode_batch before its final bit_reverse_rows (:80-81): row r of the
  // codeword is row reverse_bits_len(r, log2_n_d) of this matrix.
  std::vector<u128> encode_batch_unpermuted(const std::vector<u128>& m, size_t width) const {
    size_t kd = k_d();
    std::vector<u128> out(n_d() * width, 0);
    for (size_t r = 0; r < kd; ++r)  // bit_reverse_rows
      for (size_t c0 = 0; c0 < width; ++c0) out[r * width + c0] = m[reverse_bits_len(r, d) * width + c0];
    size_t len = width * kd;  // pad_to_height + copy_within
    for (size_t i = 1; i < c(); ++i) std::copy(out.begin(), out.begin() + len, out.begin() + i * len);
    for (size_t j = 0; j < c(); ++j) {  // coset NTTs (binary.rs:55-68)
      std::vector<const u128*> tabs;
      for (size_t t = log2_c; t < tw.size(); ++t) {
        size_t part = tw[t].size() >> log2_c;
        tabs.push_back(tw[t].data() + j * part);
      }
      ntt_forward(out.data() + j * len, width, d, tabs);
    }
    return out;
  }
  // interpolate (:103-109)
  static u128 interpolate_raw(u128 t, u128 lo, u128 hi, u128 r) {
    hi ^= lo;
    lo ^= mul(hi, t);
    return lo ^ mul(hi ^ lo, r);
  }
  u128 interpolate(int i, size_t j, u128 lo, u128 hi, u128 r) const {
    return interpolate_raw(twiddle_bo(i, j), lo, hi, r);
  }
  // fold (:88-96)
  void fold(int i, std::vector<u128>& w, u128 r) const {
    size_t mid = w.size() / 2;
    const std::vector<u128>& t = tw[log2_c + i];
    int bits = log2_c + i;
    parallel_for(mid, [&](size_t b, size_t e) {
      for (size_t j = b; j < e; ++j) w[j] = interpolate_raw(t[reverse_bits_len(j, bits)], w[j], w[j + mid], r);
    });
    w.resize(mid);
  }
};

// ---------------------------------------------------------------------------
// Merkle tree MMCS (p3/src/merkle_tree.rs:8-21 over Plonky3 MerkleTreeMmcs):
// leaf = keccak256(bincode(row)) = keccak256 of the row's raw 16-byte LE
// elements (p3/src/symmetric.rs:11-26); node = keccak256(left || right)
// (CompressionFunctionFromHasher<Keccak256Hash, 2, 32>).  Power-of-two heights.
// ---------------------------------------------------------------------------
struct MerkleTree {
  std::vector<std::vector<Digest>> layers;  // layers[0] = leaves
  std::vector<u128> rows;
  size_t width = 0;
  const Digest& root() const { return layers.back()[0]; }
  size_t height() const { return layers[0].size(); }
};

static MerkleTree merkle_commit(const std::vector<u128>& rows, size_t width) {
  MerkleTree t;
  t.rows = rows;
  t.width = width;
  size_t h = rows.size() / width;
  std::vector<Digest> leaves(h);
  parallel_for(h, [&](size_t b, size_t e) {
    for (size_t r = b; r < e; ++r)
      keccak256(reinterpret_cast<const uint8_t*>(rows.data() + r * width), 16 * width, leaves[r].b);
  }, 256);
  t.layers.push_back(std::move(leaves));
  while (t.layers.back().size() > 1) {
    const std::vector<Digest>& prev = t.layers.back();
    std::vector<Digest> next(prev.size() / 2);
    parallel_for(next.size(), [&](size_t b, size_t e) {
      uint8_t buf[64];
      for (size_t i = b; i < e; ++i) {
        std::memcpy(buf, prev[2 * i].b, 32);
        std::memcpy(buf + 32, prev[2 * i + 1].b, 32);
        keccak256(buf, 64, next[i].b);
      }
    }, 256);
    t.layers.push_back(std::move(next));
  }
  return t;
}

// open_batch: the row and the sibling path from the leaf up to below the root.
static std::vector<Digest> merkle_path(const MerkleTree& t, size_t index) {
  std::vector<Digest> p;
  for (size_t k = 0; k + 1 < t.layers.size(); ++k) p.push_back(t.layers[k][(index >> k) ^ 1]);
  return p;
}

// verify_batch for one matrix of the given height.
static bool merkle_verify(const Digest& root, size_t height, size_t index, const std::vector<u128>& row,
                          const std::vector<Digest>& path) {
  int log_h = 0;
  while (((size_t)1 << log_h) < height) ++log_h;
  if ((int)path.size() != log_h) return false;
  Digest cur;
  keccak256(reinterpret_cast<const uint8_t*>(row.data()), 16 * row.size(), cur.b);
  uint8_t buf[64];
  for (int k = 0; k < log_h; ++k) {
    if ((index >> k) & 1) {
      std::memcpy(buf, path[k].b, 32);
      std::memcpy(buf + 32, cur.b, 32);
    } else {
      std::memcpy(buf, cur.b, 32);
      std::memcpy(buf + 32, path[k].b, 32);
    }
    keccak256(buf, 64, cur.b);
  }
  return std::memcmp(cur.b, root.b, 32) == 0;
}

// ---------------------------------------------------------------------------
// Fiat–Shamir transcript: GenericChallenger<F, Keccak256Hash>
// (p3/src/challenger.rs) over Plonky3's HashChallenger<u8, H, 32>.
//   observe: clear the output buffer, append bytes to the input buffer.
//   sample:  if the output buffer is empty, hash the input buffer, make the
//            digest both the output buffer and the new input buffer; then pop
//            one byte from the END of the output buffer.
// A field element is 16 popped bytes read little-endian (challenger.rs:62-74,
// polyval.rs:71-77); sample_bits pops 8 bytes as a LE usize and masks
// (challenger.rs:76-83).
// ---------------------------------------------------------------------------
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
  void observe_digest(const Digest& d) { observe(d.b, 32); }
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
  size_t sample_bits(int bits) {
    uint64_t v = 0;
    for (int i = 0; i < 8; ++i) v |= (uint64_t)sample_byte() << (8 * i);
    uint64_t mask = bits >= 64 ? ~(uint64_t)0 : (((uint64_t)1 << bits) - 1);
    return (size_t)(v & mask);
  }
  // State blob used across the C interface:
  // [u64 LE in_len][in bytes][u64 LE out_len][out bytes].
  static bool from_blob(const uint8_t* p, size_t n, Challenger& c) {
    if (n < 16) return false;
    uint64_t li;
    std::memcpy(&li, p, 8);
    if (n < 16 + li) return false;
    uint64_t lo;
    std::memcpy(&lo, p + 8 + li, 8);
    if (n != 16 + li + lo) return false;
    c.in.assign(p + 8, p + 8 + li);
    c.out.assign(p + 16 + li, p + 16 + li + lo);
    return true;
  }
  std::vector<uint8_t> to_blob() const {
    std::vector<uint8_t> b(16 + in.size() + out.size());
    uint64_t li = in.size(), lo = out.size();
    std::memcpy(b.data(), &li, 8);
    if (li) std::memcpy(b.data() + 8, in.data(), li);
    std::memcpy(b.data() + 8 + li, &lo, 8);
    if (lo) std::memcpy(b.data() + 16 + li, out.data(), lo);
    return b;
  }
};

// ---------------------------------------------------------------------------
// Multilinear polynomials (p3/src/poly/multilinear.rs, poly/univariate.rs).
// ---------------------------------------------------------------------------
// eq_expand (:216-222): hi = lo * x_i; lo -= hi over the first 2<<i entries.
static void eq_expand(std::vector<u128>& evals, u128 x_i, int i) {
  size_t h = (size_t)1 << i;
  parallel_for(h, [&](size_t b, size_t e) {
    for (size_t k = b; k < e; ++k) {
      u128 hi = mul(evals[k], x_i);
      evals[h + k] = hi;
      evals[k] ^= hi;
    }
  });
}
// MultiPoly::eq (:41-64) for D = 1.
static std::vector<u128> eq_table(const std::vector<u128>& x, u128 scalar) {
  std::vector<u128> evals((size_t)1 << x.size(), 0);
  evals[0] = scalar;
  for (size_t i = 0; i < x.size(); ++i) eq_expand(evals, x[i], (int)i);
  return evals;
}
// fix_last_var (:183-198): lo += x (hi - lo), then truncate.
static void fix_last_var(std::vector<u128>& evals, u128 x) {
  size_t mid = evals.size() / 2;
  parallel_for(mid, [&](size_t b, size_t e) {
    for (size_t k = b; k < e; ++k) evals[k] ^= mul(x, evals[k + mid] ^ evals[k]);
  });
  evals.resize(mid);
}
// evaluate (:200-214): the top variable is the last coordinate.
static u128 evaluate(std::vector<u128> evals, const std::vector<u128>& x) {
  for (size_t k = x.size(); k-- > 0;) fix_last_var(evals, x[k]);
  return evals[0];
}
// eq_eval (:224-229): prod (2xy + 1 - x - y) = prod (1 + x + y) in char 2.
static u128 eq_eval(const u128* x, const u128* y, size_t n) {
  u128 p = one();
  for (size_t i = 0; i < n; ++i) p = mul(p, one() ^ x[i] ^ y[i]);
  return p;
}
// horner (univariate.rs:5-12)
static u128 horner(const std::vector<u128>& c, u128 x) {
  u128 acc = 0;
  for (size_t k = c.size(); k-- > 0;) acc = mul(acc, x) ^ c[k];
  return acc;
}

// ---------------------------------------------------------------------------
// Sumcheck (sumcheck/src/lib.rs, function/eval.rs, function/eval_impr.rs,
// function/quadratic.rs).
// ---------------------------------------------------------------------------
struct Subclaim {  // SumcheckSubclaim (lib.rs:18-48)
  u128 value = 0;
  std::vector<u128> r_rev;
  std::vector<u128> r() const { return std::vector<u128>(r_rev.rbegin(), r_rev.rend()); }
  void reduce(const std::vector<u128>& round_poly, u128 r_i) {
    value = horner(round_poly, r_i);
    r_rev.push_back(r_i);
  }
};

// EvalProver over EvalImprProver with HalfEq (eval.rs:27-116,
// eval_impr.rs:13-207), specialised to E = F = Polyval.
struct EvalProver {
  std::vector<u128> r, r_inv;           // EvalImpr
  std::vector<u128> one_minus_r_inv;    // HalfEq
  std::vector<u128> half_eq;            // HalfEq::poly
  std::vector<u128> poly;               // EvalImprProver::poly
  Subclaim inner_subclaim;              // EvalProver::inner_subclaim
  u128 inner_round_poly[2] = {0, 0};
  bool ok = true;

  EvalProver(const std::vector<u128>& point, std::vector<u128> p) : r(point), poly(std::move(p)) {
    for (u128 x : r) {
      if (x == 0) ok = false;  // batch_multiplicative_inverse assumes non-zero inputs
      r_inv.push_back(inv(x));
    }
    size_t n1 = r.empty() ? 0 : r.size() - 1;
    std::vector<u128> rlo(r.begin(), r.begin() + n1);
    for (u128 x : rlo) {
      if ((one() ^ x) == 0) ok = false;
      one_minus_r_inv.push_back(inv(one() ^ x));
    }
    half_eq = eq_table(rlo, one());
  }
  size_t num_vars() const { return r.size(); }
  u128 correcting_factor(int round) const {  // eval_impr.rs:83-90
    u128 p = one();
    for (size_t k = round; k < one_minus_r_inv.size(); ++k) p = mul(p, one_minus_r_inv[k]);
    return p;
  }
  u128 eval_1(int round, u128 claim, u128 eval_0) const {  // eval_impr.rs:41-43
    return mul(claim ^ mul(one() ^ r[round], eval_0), r_inv[round]);
  }
  u128 delta_scalar(int round, const Subclaim& sc) const {  // eval_impr.rs:45-51
    if ((size_t)round == (num_vars() == 0 ? 0 : num_vars() - 1)) return one();
    std::vector<u128> rr = sc.r();
    size_t n = std::min(r.size() - (round + 1), rr.size());
    return eq_eval(r.data() + round + 1, rr.data(), n);
  }
  // EvalImprProver::compute_round_poly (eval_impr.rs:187-197) then
  // EvalProver::compute_round_poly (eval.rs:89-106).
  std::vector<u128> compute_round_poly(int round, const Subclaim& outer) {
    const Subclaim& sc = ((size_t)round == num_vars() - 1) ? outer : inner_subclaim;
    size_t half = poly.size() / 2;
    size_t n = std::min(half, half_eq.size());
    // XOR sums are exact and order-free; split across threads.
    int nt = num_threads();
    std::vector<u128> parts((size_t)nt, 0);
    size_t per = (n + nt - 1) / nt;
    parallel_for((size_t)nt, [&](size_t b, size_t e) {
      for (size_t t = b; t < e; ++t) {
        u128 acc = 0;
        size_t lo = t * per, hi = std::min(n, lo + per);
        for (size_t k = lo; k < hi; ++k) acc ^= mul(half_eq[k], poly[k]);
        parts[t] = acc;
      }
    }, 1);
    u128 s = 0;
    for (u128 p : parts) s ^= p;
    u128 c0 = mul(correcting_factor(round), s);
    u128 c1 = eval_1(round, sc.value, c0) ^ c0;  // decompress_round_poly (:116-127)
    inner_round_poly[0] = c0;
    inner_round_poly[1] = c1;
    u128 scalar = delta_scalar(round, sc);
    u128 d0 = mul(scalar, one() ^ r[round]);           // delta (:53-58)
    u128 d1 = mul(scalar, r[round] ^ (one() ^ r[round]));
    return {mul(c0, d0), mul(c0, d1) ^ mul(c1, d0), mul(c1, d1)};
  }
  void fix_last(u128 x) {  // eval.rs:108-111
    fix_last_var(poly, x);
    half_eq.resize(half_eq.size() / 2);  // HalfEq::halve
    inner_subclaim.reduce({inner_round_poly[0], inner_round_poly[1]}, x);
  }
};

// prove_sumcheck_round (lib.rs:81-103) for EvalProver; returns compressed.
static std::vector<u128> prove_eval_round(EvalProver& p, Subclaim& sc, int round, Challenger& ch) {
  std::vector<u128> rp = p.compute_round_poly(round, sc);
  std::vector<u128> comp = {rp[0], rp[2]};  // Eval::compress_round_poly (eval.rs:64-66)
  for (u128 v : comp) ch.observe_elem(v);
  u128 r_i = ch.sample_elem();
  p.fix_last(r_i);
  sc.reduce(rp, r_i);
  return comp;
}

// ---------------------------------------------------------------------------
// Basefold (poly-commit/src/basefold.rs).
// ---------------------------------------------------------------------------
struct Proof {
  std::vector<std::vector<u128>> round_polys;
  std::vector<u128> final_poly;
  std::vector<Digest> pi_comms;
  struct Ext {
    u128 sibling;
    std::vector<Digest> path;
  };
  struct Opening {
    std::vector<u128> leaves;
    std::vector<Digest> path;
    std::vector<Ext> ext;
  };
  std::vector<Opening> openings;
};

// bincode 1.3 legacy layout: fixint LE, u64 length before each Vec, arrays and
// tuples without prefix, PhantomData empty (basefold.rs:49-66, lib.rs:50-54).
struct Writer {
  std::vector<uint8_t> b;
  void u64(uint64_t v) { for (int i = 0; i < 8; ++i) b.push_back((v >> (8 * i)) & 0xff); }
  void elem(u128 v) {
    uint8_t t[16];
    store(t, v);
    b.insert(b.end(), t, t + 16);
  }
  void digest(const Digest& d) { b.insert(b.end(), d.b, d.b + 32); }
};
struct Reader {
  const uint8_t* p;
  size_t n, off = 0;
  bool ok = true;
  uint64_t u64() {
    if (off + 8 > n) { ok = false; return 0; }
    uint64_t v;
    std::memcpy(&v, p + off, 8);
    off += 8;
    return v;
  }
  u128 elem() {
    if (off + 16 > n) { ok = false; return 0; }
    u128 v = load(p + off);
    off += 16;
    return v;
  }
  Digest digest() {
    Digest d{};
    if (off + 32 > n) { ok = false; return d; }
    std::memcpy(d.b, p + off, 32);
    off += 32;
    return d;
  }
  bool len(uint64_t& v, uint64_t limit) {
    v = u64();
    if (v > limit) ok = false;
    return ok;
  }
};

static std::vector<uint8_t> serialize(const Proof& pf) {
  Writer w;
  w.u64(pf.round_polys.size());
  for (auto& rp : pf.round_polys) {
    w.u64(rp.size());
    for (u128 v : rp) w.elem(v);
  }
  w.u64(pf.final_poly.size());
  for (u128 v : pf.final_poly) w.elem(v);
  w.u64(pf.pi_comms.size());
  for (auto& d : pf.pi_comms) w.digest(d);
  w.u64(pf.openings.size());
  for (auto& o : pf.openings) {
    w.u64(o.leaves.size());
    for (u128 v : o.leaves) w.elem(v);
    w.u64(o.path.size());
    for (auto& d : o.path) w.digest(d);
    w.u64(o.ext.size());
    for (auto& e : o.ext) {
      w.elem(e.sibling);
      w.u64(e.path.size());
      for (auto& d : e.path) w.digest(d);
    }
  }
  return w.b;
}

static bool deserialize(const uint8_t* p, size_t n, Proof& pf) {
  Reader r{p, n};
  const uint64_t LIM = (uint64_t)1 << 26;
  uint64_t a;
  if (!r.len(a, 64)) return false;
  pf.round_polys.resize(a);
  for (auto& rp : pf.round_polys) {
    uint64_t b;
    if (!r.len(b, 16)) return false;
    rp.resize(b);
    for (auto& v : rp) v = r.elem();
  }
  if (!r.len(a, LIM)) return false;
  pf.final_poly.resize(a);
  for (auto& v : pf.final_poly) v = r.elem();
  if (!r.len(a, 64)) return false;
  pf.pi_comms.resize(a);
  for (auto& d : pf.pi_comms) d = r.digest();
  if (!r.len(a, 1 << 16)) return false;
  pf.openings.resize(a);
  for (auto& o : pf.openings) {
    uint64_t b;
    if (!r.len(b, 1 << 16)) return false;
    o.leaves.resize(b);
    for (auto& v : o.leaves) v = r.elem();
    if (!r.len(b, 64)) return false;
    o.path.resize(b);
    for (auto& d : o.path) d = r.digest();
    if (!r.len(b, 64)) return false;
    o.ext.resize(b);
    for (auto& e : o.ext) {
      e.sibling = r.elem();
      uint64_t c;
      if (!r.len(c, 64)) return false;
      e.path.resize(c);
      for (auto& d : e.path) d = r.digest();
    }
  }
  return r.ok && r.off == n;
}

struct CommitmentData {
  MerkleTree codewords;
  std::vector<u128> data;  // row-major k_d x width
  size_t width;
};

// commit (basefold.rs:112-120)
static CommitmentData commit(const Code& code, const std::vector<u128>& data, size_t width) {
  CommitmentData cd;
  std::vector<u128> cw = code.encode_batch(data, width);
  cd.codewords = merkle_commit(cw, width);
  cd.data = data;
  cd.width = width;
  return cd;
}

// eval (basefold.rs:126-131): one value per column.
static std::vector<u128> eval(const std::vector<u128>& data, size_t width, const std::vector<u128>& point) {
  size_t h = data.size() / width;
  std::vector<u128> out;
  for (size_t c = 0; c < width; ++c) {
    std::vector<u128> col(h);
    for (size_t r = 0; r < h; ++r) col[r] = data[r * width + c];
    out.push_back(evaluate(col, point));
  }
  return out;
}

// sample_random_scalars_by_eq (basefold.rs:398-408)
static std::vector<u128> sample_scalars_by_eq(size_t n, Challenger& ch) {
  int log_n = 0;
  while (((size_t)1 << log_n) < n) ++log_n;
  std::vector<u128> r;
  for (int i = 0; i < log_n; ++i) r.push_back(ch.sample_elem());
  std::vector<u128> eq = eq_table(r, one());
  eq.resize(n);
  return eq;
}

static u128 dot(const u128* a, const u128* b, size_t n) {
  u128 acc = 0;
  for (size_t i = 0; i < n; ++i) acc ^= mul(a[i], b[i]);
  return acc;
}

// open (basefold.rs:133-232) for one evaluation point; `has_eval` false
// reproduces the empty-evals early return.
static Proof open(const Code& code, const CommitmentData& cd, bool has_eval, const std::vector<u128>& point,
                  const std::vector<u128>& values, Challenger& ch, bool& ok) {
  Proof pf;
  ok = true;
  if (!has_eval) return pf;
  size_t w = cd.width;
  size_t kd = code.k_d();
  const std::vector<u128>& cw = cd.codewords.rows;
  std::vector<u128> poly, pi;
  u128 claim;
  std::vector<u128> scalars;
  if (w == 1) {
    poly = cd.data;
    claim = values[0];
    pi = cw;
  } else {
    scalars = sample_scalars_by_eq(w, ch);
    poly.resize(kd);
    parallel_for(kd, [&](size_t b, size_t e) {
      for (size_t r = b; r < e; ++r) poly[r] = dot(scalars.data(), cd.data.data() + r * w, w);
    });
    claim = dot(scalars.data(), values.data(), w);
    pi.resize(code.n_d());
    parallel_for(code.n_d(), [&](size_t b, size_t e) {
      for (size_t r = b; r < e; ++r) pi[r] = dot(scalars.data(), cw.data() + r * w, w);
    });
  }
  EvalProver prover(point, poly);
  if (!prover.ok) ok = false;
  Subclaim sc;
  sc.value = claim;
  std::vector<MerkleTree> pi_trees;
  // prove_interleaved_folding_sumcheck (basefold.rs:335-369)
  for (int i = code.d - 1; i >= 0; --i) {
    size_t half = pi.size() / 2;
    std::vector<u128> pairs(pi.size());
    for (size_t j = 0; j < half; ++j) {
      pairs[2 * j] = pi[j];
      pairs[2 * j + 1] = pi[j + half];
    }
    pi_trees.push_back(merkle_commit(pairs, 2));
    ch.observe_digest(pi_trees.back().root());
    pf.round_polys.push_back(prove_eval_round(prover, sc, i, ch));
    u128 r_i = sc.r_rev.back();
    code.fold(i, pi, r_i);
  }
  pf.final_poly = prover.poly;  // into_ext_poly
  for (u128 v : pf.final_poly) ch.observe_elem(v);
  std::vector<size_t> idxs;
  for (size_t q = 0; q < code.num_queries(); ++q) idxs.push_back(ch.sample_bits(code.log2_n_d()));
  for (size_t idx : idxs) {
    Proof::Opening o;
    o.leaves.assign(cw.begin() + idx * w, cw.begin() + (idx + 1) * w);
    o.path = merkle_path(cd.codewords, idx);
    for (int k = 0; k < code.d; ++k) {
      int i = code.d - 1 - k;
      size_t ni = code.n_i(i);
      size_t sib = ((idx / ni) & 1) ^ 1;
      size_t ii = idx % ni;
      Proof::Ext e;
      e.sibling = pi_trees[k].rows[2 * ii + sib];
      e.path = merkle_path(pi_trees[k], ii);
      o.ext.push_back(e);
    }
    pf.openings.push_back(o);
  }
  for (auto& t : pi_trees) pf.pi_comms.push_back(t.root());
  return pf;
}

// verify (basefold.rs:234-324).  0 = ok, 1 = InvalidFinalPoly,
// 2 = InvalidQuery, 3 = Mmcs, 4 = malformed proof.
static int verify(const Code& code, const Digest& comm, bool has_eval, const std::vector<u128>& point,
                  const std::vector<u128>& values, const Proof& pf, Challenger& ch) {
  if (!has_eval) return 0;
  size_t w = values.size();
  std::vector<u128> scalars;
  u128 claim;
  if (w == 1) {
    scalars = {one()};
    claim = values[0];
  } else {
    scalars = sample_scalars_by_eq(w, ch);
    claim = dot(scalars.data(), values.data(), w);
  }
  if (pf.round_polys.size() != (size_t)code.d || pf.pi_comms.size() != (size_t)code.d) return 4;
  Subclaim sc;
  sc.value = claim;
  // verify_interleaved_folding_sumcheck (basefold.rs:371-396)
  for (int k = 0; k < code.d; ++k) {
    int round = code.d - 1 - k;
    ch.observe_digest(pf.pi_comms[k]);
    const std::vector<u128>& comp = pf.round_polys[k];
    if (comp.size() != 2) return 4;
    for (u128 v : comp) ch.observe_elem(v);
    // Eval::decompress_round_poly (eval.rs:68-79): c1 = claim - 2 c0 - c2
    u128 c1 = sc.value ^ comp[1];
    std::vector<u128> rp = {comp[0], c1, comp[1]};
    u128 r_i = ch.sample_elem();
    sc.reduce(rp, r_i);
    (void)round;
  }
  std::vector<u128> r = sc.r();
  for (u128 v : pf.final_poly) ch.observe_elem(v);
  if (pf.final_poly.size() != 1) return 4;
  // point_lo = point[..0]: evaluate(final_poly, []) = final_poly[0]
  if (mul(pf.final_poly[0], eq_eval(point.data(), r.data(), point.size())) != sc.value) return 1;
  std::vector<u128> pi0(code.c(), pf.final_poly[0]);  // encode0
  std::vector<size_t> idxs;
  for (size_t q = 0; q < code.num_queries(); ++q) idxs.push_back(ch.sample_bits(code.log2_n_d()));
  if (pf.openings.size() != idxs.size()) return 4;
  for (size_t q = 0; q < idxs.size(); ++q) {
    size_t idx = idxs[q];
    const Proof::Opening& o = pf.openings[q];
    if (o.leaves.size() != w || o.ext.size() != (size_t)code.d) return 4;
    if (!merkle_verify(comm, code.n_d(), idx, o.leaves, o.path)) return 3;
    u128 folded = dot(scalars.data(), o.leaves.data(), w);
    for (int k = 0; k < code.d; ++k) {
      int i = code.d - 1 - k;
      size_t ni = code.n_i(i);
      size_t sib = ((idx / ni) & 1) ^ 1;
      size_t ii = idx % ni;
      std::vector<u128> vals(2, folded);
      vals[sib] = o.ext[k].sibling;
      if (!merkle_verify(pf.pi_comms[k], ni, ii, vals, o.ext[k].path)) return 3;
      folded = code.interpolate(i, ii, vals[0], vals[1], r[i]);
    }
    if (pi0[idx % code.n_0()] != folded) return 2;
  }
  return 0;
}

// ---------------------------------------------------------------------------
// Standalone product sumcheck (sumcheck/src/lib.rs:56-79 with
// function/quadratic.rs:84-134).  k = 2 is Quadratic with one pair
// (ONE, 0, 1).  k = 3 is this project's product-of-three extension, which
// the reference does not have: round polynomial coefficients c0..c3 of
// sum_b prod_k (lo_k + X (hi_k - lo_k)), compressed by dropping c1 (the way
// function/batch.rs:70-74 compresses), c1 = claim - 2 c0 - c2 - c3.
// ---------------------------------------------------------------------------
struct SumcheckOut {
  std::vector<std::vector<u128>> round_polys;  // compressed
  std::vector<u128> r;                         // challenges in round order (n-1 first)
  std::vector<u128> final_evals;               // each poly at the challenge point
  u128 final_claim = 0;
};

static SumcheckOut prove_product_sumcheck(int k, std::vector<std::vector<u128>> polys, u128 claim, Challenger& ch) {
  SumcheckOut out;
  int n = 0;
  while (((size_t)1 << n) < polys[0].size()) ++n;
  Subclaim sc;
  sc.value = claim;
  if (n == 0) {
    for (auto& p : polys) out.final_evals.push_back(p[0]);
    out.final_claim = claim;
    return out;
  }
  ch.observe_elem(claim);
  for (int round = n - 1; round >= 0; --round) {
    size_t half = polys[0].size() / 2;
    int nt = num_threads();
    std::vector<std::vector<u128>> parts((size_t)nt, std::vector<u128>(4, 0));
    size_t per = (half + nt - 1) / nt;
    parallel_for((size_t)nt, [&](size_t b, size_t e) {
      for (size_t t = b; t < e; ++t) {
        u128 s0 = 0, s2 = 0, s3 = 0;
        size_t lo = t * per, hi = std::min(half, lo + per);
        for (size_t i = lo; i < hi; ++i) {
          if (k == 2) {
            const u128 f0 = polys[0][i], f1 = polys[0][i + half], g0 = polys[1][i], g1 = polys[1][i + half];
            s0 ^= mul(f0, g0);
            s2 ^= mul(f1 ^ f0, g1 ^ g0);
          } else {
            u128 a0 = polys[0][i], b0 = polys[0][i + half] ^ a0;
            u128 a1 = polys[1][i], b1 = polys[1][i + half] ^ a1;
            u128 a2 = polys[2][i], b2 = polys[2][i + half] ^ a2;
            s0 ^= mul(a0, mul(a1, a2));
            s2 ^= mul(b0, mul(b1, a2) ^ mul(a1, b2)) ^ mul(a0, mul(b1, b2));
            s3 ^= mul(b0, mul(b1, b2));
          }
        }
        parts[t][0] = s0;
        parts[t][2] = s2;
        parts[t][3] = s3;
      }
    }, 1);
    u128 c0 = 0, c2 = 0, c3 = 0;
    for (auto& p : parts) {
      c0 ^= p[0];
      c2 ^= p[2];
      c3 ^= p[3];
    }
    std::vector<u128> rp, comp;
    if (k == 2) {
      // Quadratic: pair scalar ONE (quadratic.rs:118), decompress (:68-79)
      c0 = mul(c0, one());
      c2 = mul(c2, one());
      comp = {c0, c2};
      rp = {c0, sc.value ^ c2, c2};
    } else {
      comp = {c0, c2, c3};
      rp = {c0, sc.value ^ c2 ^ c3, c2, c3};
    }
    for (u128 v : comp) ch.observe_elem(v);
    u128 r_i = ch.sample_elem();
    for (auto& p : polys) fix_last_var(p, r_i);
    sc.reduce(rp, r_i);
    out.round_polys.push_back(comp);
    out.r.push_back(r_i);
  }
  for (auto& p : polys) out.final_evals.push_back(p[0]);
  out.final_claim = sc.value;
  return out;
}

// verify_sumcheck (lib.rs:111-148) for the product functions.
static bool verify_product_sumcheck(int k, int n, u128 claim, const std::vector<std::vector<u128>>& comp,
                                    Challenger& ch, SumcheckOut& out) {
  Subclaim sc;
  sc.value = claim;
  if (n == 0) {
    out.final_claim = claim;
    return true;
  }
  ch.observe_elem(claim);
  if ((int)comp.size() != n) return false;
  for (int i = 0; i < n; ++i) {
    if ((int)comp[i].size() != k) return false;
    for (u128 v : comp[i]) ch.observe_elem(v);
    std::vector<u128> rp;
    if (k == 2)
      rp = {comp[i][0], sc.value ^ comp[i][1], comp[i][1]};
    else
      rp = {comp[i][0], sc.value ^ comp[i][1] ^ comp[i][2], comp[i][1], comp[i][2]};
    u128 r_i = ch.sample_elem();
    sc.reduce(rp, r_i);
    out.r.push_back(r_i);
  }
  out.final_claim = sc.value;
  return true;
}

}  // namespace orc

// ===========================================================================
// C interface (loaded by the tests through ctypes).  Status: 0 ok, <0 error.
// ===========================================================================
using namespace orc;

static std::vector<u128> load_vec(const uint8_t* p, size_t n) {
  std::vector<u128> v(n);
  for (size_t i = 0; i < n; ++i) v[i] = load(p + 16 * i);
  return v;
}
static void store_vec(uint8_t* p, const std::vector<u128>& v) {
  for (size_t i = 0; i < v.size(); ++i) store(p + 16 * i, v[i]);
}

extern "C" {

// The oracle's thread count, shared with the prime-field oracle.
int orc_num_threads() { return num_threads(); }

int orc_set_threads(int n) {
  g_threads = n > 0 ? n : 0;
  return num_threads();
}

void orc_gf_mul(const uint8_t* a, const uint8_t* b, uint8_t* out, size_t n) {
  parallel_for(n, [&](size_t s, size_t e) {
    for (size_t i = s; i < e; ++i) store(out + 16 * i, mul(load(a + 16 * i), load(b + 16 * i)));
  });
}
void orc_gf_mul_definition(const uint8_t* a, const uint8_t* b, uint8_t* out, size_t n) {
  for (size_t i = 0; i < n; ++i) store(out + 16 * i, mul_definition(load(a + 16 * i), load(b + 16 * i)));
}
void orc_gf_inv(const uint8_t* a, uint8_t* out, size_t n) {
  for (size_t i = 0; i < n; ++i) store(out + 16 * i, inv(load(a + 16 * i)));
}
void orc_from_canonical(const uint8_t* a, uint8_t* out, size_t n) {
  for (size_t i = 0; i < n; ++i) store(out + 16 * i, from_canonical(load(a + 16 * i)));
}
void orc_to_canonical(const uint8_t* a, uint8_t* out, size_t n) {
  for (size_t i = 0; i < n; ++i) store(out + 16 * i, to_canonical(load(a + 16 * i)));
}
// out[0] = x^128 mod P (ONE), out[1] = x^256 mod P (R2)
void orc_field_consts(uint8_t* out) {
  store(out, one());
  init_consts();
  store(out + 16, g_r2);
}
// Polyval "dot-product" chain of RFC 8452: S_j = dot(S_{j-1} + X_j, H)
void orc_polyval_rfc(const uint8_t* h, const uint8_t* xs, size_t n, uint8_t* out) {
  u128 H = load(h), S = 0;
  for (size_t j = 0; j < n; ++j) S = mul(S ^ load(xs + 16 * j), H);
  store(out, S);
}

void orc_keccak_f(uint64_t* st) { keccak_f(st); }
void orc_keccak_consts(uint64_t* rc24, int* rho25) {
  std::memcpy(rc24, KT.rc, sizeof(KT.rc));
  std::memcpy(rho25, KT.rho, sizeof(KT.rho));
}
void orc_keccak256(const uint8_t* msg, size_t len, uint8_t* out) { keccak256(msg, len, out); }
void orc_sha3_256(const uint8_t* msg, size_t len, uint8_t* out) { sponge256(msg, len, 0x06, out); }

// All stage tables of AddtiveNtt::new(log_n), concatenated in the
// reference's `twiddles` order (2^log_n - 1 elements).
int orc_ntt_twiddles(int log_n, uint8_t* out) {
  if (log_n < 0 || log_n > 26) return -1;
  auto tw = ntt_twiddles(log_n);
  size_t off = 0;
  for (auto& t : tw) {
    store_vec(out + 16 * off, t);
    off += t.size();
  }
  return 0;
}
int orc_ntt_forward(int log_n, size_t width, uint8_t* data) {
  if (log_n < 0 || log_n > 26) return -1;
  auto tw = ntt_twiddles(log_n);
  std::vector<const u128*> tabs;
  for (auto& t : tw) tabs.push_back(t.data());
  std::vector<u128> v = load_vec(data, width << log_n);
  ntt_forward(v.data(), width, log_n, tabs);
  store_vec(data, v);
  return 0;
}
int orc_ntt_backward(int log_n, size_t width, uint8_t* data) {
  if (log_n < 0 || log_n > 26) return -1;
  auto tw = ntt_twiddles(log_n);
  std::vector<const u128*> tabs;
  for (auto& t : tw) tabs.push_back(t.data());
  std::vector<u128> v = load_vec(data, width << log_n);
  ntt_backward(v.data(), width, log_n, tabs);
  store_vec(data, v);
  return 0;
}
int orc_ntt_forward_definition(int log_n, uint8_t* data) {
  if (log_n < 0 || log_n > 12) return -1;
  std::vector<u128> v = load_vec(data, (size_t)1 << log_n);
  store_vec(data, ntt_forward_definition(log_n, v));
  return 0;
}

size_t orc_num_queries(int lambda, int log2_c) {
  Code code(lambda, log2_c, 0);
  return code.num_queries();
}

int orc_encode(int n, int log2_c, size_t width, const uint8_t* data, uint8_t* out) {
  if (n < 0 || log2_c < 0 || n + log2_c > 28) return -1;
  Code code(128, log2_c, n);
  store_vec(out, code.encode_batch(load_vec(data, width << n), width));
  return 0;
}

// Merkle root of a row-major matrix; `layers_out` (optional) receives every
// layer, leaves first.
int orc_merkle_commit(const uint8_t* rows, size_t height, size_t width, uint8_t* root, uint8_t* layers_out) {
  if (height == 0 || (height & (height - 1))) return -1;
  MerkleTree t = merkle_commit(load_vec(rows, height * width), width);
  std::memcpy(root, t.root().b, 32);
  if (layers_out) {
    size_t off = 0;
    for (auto& l : t.layers)
      for (auto& d : l) {
        std::memcpy(layers_out + off, d.b, 32);
        off += 32;
      }
  }
  return 0;
}

int orc_commit(int n, int log2_c, size_t width, const uint8_t* data, uint8_t* root) {
  if (n < 0 || log2_c < 0 || n + log2_c > 28 || width == 0) return -1;
  Code code(128, log2_c, n);
  CommitmentData cd = commit(code, load_vec(data, width << n), width);
  std::memcpy(root, cd.codewords.root().b, 32);
  return 0;
}

// The root of orc_commit computed in bounded memory, for the largest
// commits (2^28-row codewords): the codeword is hashed in subtrees of at most
// 2^14 leaves, each on one thread with its own scratch, and only the subtree
// roots are kept; leaf r reads codeword row r through the bit reversal that
// encode_batch applies last.  Same tree and root as merkle_commit.
int orc_commit_root(int n, int log2_c, size_t width, const uint8_t* data, uint8_t* root) {
  if (n < 0 || log2_c < 0 || n + log2_c > 28 || width == 0) return -1;
  Code code(128, log2_c, n);
  const std::vector<u128> cw = code.encode_batch_unpermuted(load_vec(data, width << n), width);
  const size_t h = code.n_d();
  const int lb = code.log2_n_d();
  const size_t sub = std::min<size_t>(h, (size_t)1 << 14);
  std::vector<Digest> tops(h / sub);
  parallel_for(tops.size(), [&](size_t b, size_t e) {
    std::vector<Digest> lv(sub);
    std::vector<u128> row(width);
    uint8_t buf[64];
    for (size_t t = b; t < e; ++t) {
      for (size_t i = 0; i < sub; ++i) {
        const size_t src = reverse_bits_len(t * sub + i, lb) * width;
        for (size_t c0 = 0; c0 < width; ++c0) row[c0] = cw[src + c0];
        keccak256(reinterpret_cast<const uint8_t*>(row.data()), 16 * width, lv[i].b);
      }
      for (size_t m = sub; m > 1; m >>= 1)
        for (size_t i = 0; i < m / 2; ++i) {
          std::memcpy(buf, lv[2 * i].b, 32);
          std::memcpy(buf + 32, lv[2 * i + 1].b, 32);
          keccak256(buf, 64, lv[i].b);
        }
      tops[t] = lv[0];
    }
  }, 1);
  uint8_t buf[64];
  for (size_t m = tops.size(); m > 1; m >>= 1)
    for (size_t i = 0; i < m / 2; ++i) {
      std::memcpy(buf, tops[2 * i].b, 32);
      std::memcpy(buf + 32, tops[2 * i + 1].b, 32);
      keccak256(buf, 64, tops[i].b);
    }
  std::memcpy(root, tops[0].b, 32);
  return 0;
}

int orc_eval(int n, size_t width, const uint8_t* data, const uint8_t* point, uint8_t* values) {
  if (n < 0 || n > 28 || width == 0) return -1;
  store_vec(values, eval(load_vec(data, width << n), width, load_vec(point, n)));
  return 0;
}

// Challenger helpers: state blobs (see Challenger::from_blob).
int orc_challenger_sample(const uint8_t* blob, size_t blob_len, int kind, size_t count, int bits, uint8_t* out,
                          uint8_t* blob_out, size_t* blob_out_len) {
  Challenger ch;
  if (!Challenger::from_blob(blob, blob_len, ch)) return -1;
  for (size_t i = 0; i < count; ++i) {
    if (kind == 0) {
      store(out + 16 * i, ch.sample_elem());
    } else {
      uint64_t v = ch.sample_bits(bits);
      std::memcpy(out + 8 * i, &v, 8);
    }
  }
  if (blob_out) {
    auto b = ch.to_blob();
    if (*blob_out_len < b.size()) return -2;
    std::memcpy(blob_out, b.data(), b.size());
    *blob_out_len = b.size();
  }
  return 0;
}

// The reference's harness up to `open` (poly-commit/src/lib.rs:64-105):
// commit, observe the root, evaluate at `point`, observe the values.
// Outputs the root, the values and the challenger blob handed to open.
int orc_harness_prepare(int n, int log2_c, size_t width, const uint8_t* data, const uint8_t* point, uint8_t* root,
                        uint8_t* values, uint8_t* blob_out, size_t* blob_len) {
  if (n < 0 || log2_c < 0 || n + log2_c > 28 || width == 0) return -1;
  Code code(128, log2_c, n);
  std::vector<u128> d = load_vec(data, width << n);
  CommitmentData cd = commit(code, d, width);
  std::memcpy(root, cd.codewords.root().b, 32);
  std::vector<u128> vals = eval(d, width, load_vec(point, n));
  store_vec(values, vals);
  Challenger ch;
  ch.observe_digest(cd.codewords.root());
  for (u128 v : vals) ch.observe_elem(v);
  auto b = ch.to_blob();
  if (*blob_len < b.size()) return -2;
  std::memcpy(blob_out, b.data(), b.size());
  *blob_len = b.size();
  return 0;
}

// open: writes the bincode proof.  n_evals is 0 or 1.
int orc_open(int n, int log2_c, size_t width, const uint8_t* data, const uint8_t* point, const uint8_t* values,
             int n_evals, const uint8_t* blob, size_t blob_len, uint8_t* proof_out, size_t cap, size_t* proof_len) {
  if (n < 0 || log2_c < 0 || n + log2_c > 28 || width == 0 || n_evals < 0 || n_evals > 1) return -1;
  Challenger ch;
  if (!Challenger::from_blob(blob, blob_len, ch)) return -1;
  Code code(128, log2_c, n);
  CommitmentData cd = commit(code, load_vec(data, width << n), width);
  bool ok;
  Proof pf = open(code, cd, n_evals == 1, load_vec(point, n_evals ? n : 0), load_vec(values, n_evals ? width : 0),
                  ch, ok);
  if (!ok) return -3;
  std::vector<uint8_t> b = serialize(pf);
  *proof_len = b.size();
  if (cap < b.size()) return -2;
  std::memcpy(proof_out, b.data(), b.size());
  return 0;
}

// One full prover step of the reference's harness, timed as the CPU
// baseline: commit, observe the root, evaluate, observe the values, open.
int orc_commit_eval_open(int n, int log2_c, const uint8_t* data, const uint8_t* point, uint8_t* root,
                         uint8_t* proof_out, size_t cap, size_t* proof_len) {
  if (n < 0 || log2_c < 0 || n + log2_c > 28) return -1;
  Code code(128, log2_c, n);
  std::vector<u128> d = load_vec(data, (size_t)1 << n);
  std::vector<u128> pt = load_vec(point, n);
  CommitmentData cd = commit(code, d, 1);
  std::memcpy(root, cd.codewords.root().b, 32);
  Challenger ch;
  ch.observe_digest(cd.codewords.root());
  std::vector<u128> vals = eval(d, 1, pt);
  for (u128 v : vals) ch.observe_elem(v);
  bool ok;
  Proof pf = open(code, cd, true, pt, vals, ch, ok);
  if (!ok) return -3;
  std::vector<uint8_t> b = serialize(pf);
  *proof_len = b.size();
  if (cap < b.size()) return -2;
  std::memcpy(proof_out, b.data(), b.size());
  return 0;
}

int orc_verify(int n, int log2_c, size_t width, const uint8_t* root, const uint8_t* point, const uint8_t* values,
               int n_evals, const uint8_t* blob, size_t blob_len, const uint8_t* proof, size_t proof_len) {
  if (n < 0 || log2_c < 0 || n + log2_c > 28 || width == 0) return -1;
  Challenger ch;
  if (!Challenger::from_blob(blob, blob_len, ch)) return -1;
  Proof pf;
  if (!deserialize(proof, proof_len, pf)) return 4;
  Code code(128, log2_c, n);
  Digest comm;
  std::memcpy(comm.b, root, 32);
  return verify(code, comm, n_evals == 1, load_vec(point, n_evals ? n : 0), load_vec(values, n_evals ? width : 0),
                pf, ch);
}

// Standalone product sumcheck.  polys: k arrays of 2^n elements back to back.
// out layout: n compressed round polynomials (k elements each), then the n
// challenges (round n-1 first), then k final evaluations, then the final
// subclaim.
int orc_sumcheck_prove(int k, int n, const uint8_t* polys, const uint8_t* claim, const uint8_t* blob, size_t blob_len,
                       uint8_t* out) {
  if ((k != 2 && k != 3) || n < 0 || n > 28) return -1;
  Challenger ch;
  if (!Challenger::from_blob(blob, blob_len, ch)) return -1;
  std::vector<std::vector<u128>> ps;
  size_t N = (size_t)1 << n;
  for (int i = 0; i < k; ++i) ps.push_back(load_vec(polys + 16 * N * i, N));
  SumcheckOut o = prove_product_sumcheck(k, ps, load(claim), ch);
  size_t off = 0;
  for (auto& rp : o.round_polys)
    for (u128 v : rp) store(out + 16 * off++, v);
  for (u128 v : o.r) store(out + 16 * off++, v);
  for (u128 v : o.final_evals) store(out + 16 * off++, v);
  store(out + 16 * off++, o.final_claim);
  return 0;
}

// Verify a product sumcheck transcript; returns 0 when the final subclaim
// equals prod_k final_evals[k] (the reference's run_sumcheck identity,
// sumcheck/src/lib.rs:160-182), 1 when it does not, <0 on bad input.
int orc_sumcheck_verify(int k, int n, const uint8_t* claim, const uint8_t* round_polys, const uint8_t* final_evals,
                        const uint8_t* blob, size_t blob_len, uint8_t* r_out) {
  if ((k != 2 && k != 3) || n < 0 || n > 28) return -1;
  Challenger ch;
  if (!Challenger::from_blob(blob, blob_len, ch)) return -1;
  std::vector<std::vector<u128>> comp(n);
  for (int i = 0; i < n; ++i) comp[i] = load_vec(round_polys + 16 * (size_t)k * i, k);
  SumcheckOut o;
  if (!verify_product_sumcheck(k, n, load(claim), comp, ch, o)) return -2;
  if (r_out) store_vec(r_out, o.r);
  u128 p = one();
  for (int i = 0; i < k; ++i) p = mul(p, load(final_evals + 16 * i));
  if (k == 2) p = mul(p, one());  // pair scalar ONE (quadratic.rs:57-62)
  return p == o.final_claim ? 0 : 1;
}

}  // extern "C"
