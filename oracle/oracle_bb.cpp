// ORACLE — test infrastructure only.
//
// CPU restatement of han0110/learn-zkp's Basefold over the prime field
// BabyBear (p = 15 * 2^27 + 1) with the extension E = BinomialExtensionField<
// BabyBear, 5> and the multiplicative Reed–Solomon code
// (poly-commit/src/basefold/code/reed_solomon.rs), width 1.  It exists to
// check the CUDA library's prime-field path: only the tests may load it.
//
// Parity status: unpinned against Plonky3@784b7dd, whose source is not in
// this environment.  From that dependency it restates, as published:
//   * BabyBear arithmetic and its two-adic generator 0x1a427a41 (= 31^15,
//     the multiplicative generator 31 raised to the odd part of p - 1), with
//     two_adic_generator(bits) = 0x1a427a41^(2^(27 - bits));
//   * the quintic extension as F[X] / (X^5 - 2) (2 is not a fifth power
//     mod p, checked by the tests);
//   * Radix2DitParallel::dft_batch as the natural-order evaluation of the
//     coefficient vector on the subgroup of order n;
//   * bincode of a BabyBear as its canonical value, 4 bytes little-endian,
//     and of an extension element as its five coefficients.
// Everything else follows the reference's own sources, cited per function.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

extern "C" void orc_keccak256(const uint8_t* msg, size_t len, uint8_t* out);
extern "C" int orc_num_threads();

namespace orb {

// f(begin, end) over [0, n) in contiguous chunks on the oracle's threads.
template <class F>
static void parallel_for(size_t n, const F& f, size_t grain = 256) {
  const int nt = orc_num_threads();
  if (nt <= 1 || n <= grain) {
    f((size_t)0, n);
    return;
  }
  const size_t chunks = std::min<size_t>((size_t)nt, (n + grain - 1) / grain);
  const size_t per = (n + chunks - 1) / chunks;
  std::vector<std::thread> ts;
  for (size_t c = 0; c < chunks; ++c) {
    const size_t b = c * per, e = std::min(n, b + per);
    if (b < e) ts.emplace_back([&f, b, e]() { f(b, e); });
  }
  for (auto& t : ts) t.join();
}

// ---------------------------------------------------------------------------
// BabyBear (canonical u32 in [0, p)).
// ---------------------------------------------------------------------------
constexpr uint32_t P = 2013265921u;
constexpr uint32_t W = 2;  // X^5 = W in the quintic extension
inline uint32_t fadd(uint32_t a, uint32_t b) {
  uint32_t s = a + b;
  return s >= P ? s - P : s;
}
inline uint32_t fsub(uint32_t a, uint32_t b) { return a >= b ? a - b : a + P - b; }
inline uint32_t fmul(uint32_t a, uint32_t b) { return (uint32_t)((uint64_t)a * b % P); }
inline uint32_t fpow(uint32_t a, uint64_t e) {
  uint32_t r = 1;
  while (e) {
    if (e & 1) r = fmul(r, a);
    a = fmul(a, a);
    e >>= 1;
  }
  return r;
}
inline uint32_t finv(uint32_t a) { return fpow(a, P - 2); }
constexpr uint32_t INV2 = (P + 1) / 2;
// TwoAdicField::two_adic_generator(bits) of Plonky3's BabyBear.
inline uint32_t two_adic_generator(int bits) {
  uint32_t g = 0x1a427a41u;
  for (int k = bits; k < 27; ++k) g = fmul(g, g);
  return g;
}

// ---------------------------------------------------------------------------
// E = F[X] / (X^5 - W).
// ---------------------------------------------------------------------------
struct E {
  uint32_t c[5] = {0, 0, 0, 0, 0};
  static E from(uint32_t f) {
    E e;
    e.c[0] = f;
    return e;
  }
  static E one() { return from(1); }
  bool operator==(const E& o) const { return std::memcmp(c, o.c, sizeof(c)) == 0; }
  bool operator!=(const E& o) const { return !(*this == o); }
  bool is_zero() const { return (c[0] | c[1] | c[2] | c[3] | c[4]) == 0; }
};
inline E eadd(const E& a, const E& b) {
  E r;
  for (int i = 0; i < 5; ++i) r.c[i] = fadd(a.c[i], b.c[i]);
  return r;
}
inline E esub(const E& a, const E& b) {
  E r;
  for (int i = 0; i < 5; ++i) r.c[i] = fsub(a.c[i], b.c[i]);
  return r;
}
inline E emul(const E& a, const E& b) {
  uint64_t acc[9] = {0};
  for (int i = 0; i < 5; ++i)
    for (int j = 0; j < 5; ++j) acc[i + j] = (acc[i + j] + (uint64_t)a.c[i] * b.c[j]) % P;
  E r;
  for (int k = 0; k < 5; ++k) r.c[k] = (uint32_t)((acc[k] + (k + 5 < 9 ? acc[k + 5] * W : 0)) % P);
  return r;
}
inline E escale(const E& a, uint32_t f) {
  E r;
  for (int i = 0; i < 5; ++i) r.c[i] = fmul(a.c[i], f);
  return r;
}
inline E edouble(const E& a) { return eadd(a, a); }
// Inverse by the extended Euclidean algorithm over F[X] modulo X^5 - W.
static E einv(const E& a) {
  using Poly = std::vector<uint32_t>;  // low degree first
  auto trim = [](Poly& p) {
    while (!p.empty() && p.back() == 0) p.pop_back();
  };
  auto sub_scaled = [](Poly& p, const Poly& q, uint32_t s, size_t shift) {  // p -= s X^shift q
    if (p.size() < q.size() + shift) p.resize(q.size() + shift, 0);
    for (size_t i = 0; i < q.size(); ++i) p[i + shift] = fsub(p[i + shift], fmul(s, q[i]));
  };
  Poly r0 = {P - W, 0, 0, 0, 0, 1}, r1(a.c, a.c + 5);  // X^5 - W, a
  Poly s0 = {}, s1 = {1};
  trim(r1);
  if (r1.empty()) return E();  // zero has no inverse (batch_multiplicative_inverse's caller checks)
  while (r1.size() > 1) {
    // r0 = q r1 + rem; s0 -= q s1
    Poly rem = r0, q;
    q.assign(rem.size() >= r1.size() ? rem.size() - r1.size() + 1 : 0, 0);
    const uint32_t lead_inv = finv(r1.back());
    while (rem.size() >= r1.size()) {
      const size_t shift = rem.size() - r1.size();
      const uint32_t f = fmul(rem.back(), lead_inv);
      q[shift] = f;
      sub_scaled(rem, r1, f, shift);
      rem.pop_back();
      trim(rem);
    }
    Poly s = s0;
    for (size_t i = 0; i < q.size(); ++i)
      if (q[i]) sub_scaled(s, s1, q[i], i);
    trim(s);
    r0 = r1;
    r1 = rem;
    s0 = s1;
    s1 = s;
    if (r1.empty()) return E();  // not reached for a field
  }
  const uint32_t k = finv(r1[0]);
  E r;
  for (size_t i = 0; i < s1.size() && i < 5; ++i) r.c[i] = fmul(s1[i], k);
  return r;
}

// ---------------------------------------------------------------------------
// Bytes (bincode): a BabyBear is 4 bytes LE (canonical), an E five of them.
// ---------------------------------------------------------------------------
inline void put_u32(std::vector<uint8_t>& b, uint32_t v) {
  for (int i = 0; i < 4; ++i) b.push_back((uint8_t)(v >> (8 * i)));
}
inline void put_u64(std::vector<uint8_t>& b, uint64_t v) {
  for (int i = 0; i < 8; ++i) b.push_back((uint8_t)(v >> (8 * i)));
}
inline void put_e(std::vector<uint8_t>& b, const E& e) {
  for (int i = 0; i < 5; ++i) put_u32(b, e.c[i]);
}
inline uint32_t ld_u32(const uint8_t* p) {
  uint32_t v;
  std::memcpy(&v, p, 4);
  return v;
}
inline E ld_e(const uint8_t* p) {
  E e;
  for (int i = 0; i < 5; ++i) e.c[i] = ld_u32(p + 4 * i);
  return e;
}

struct Digest {
  uint8_t b[32];
};

// HashChallenger<u8, Keccak256Hash, 32> under GenericChallenger<BabyBear, _>
// (p3/src/challenger.rs:51-83): observe appends bincode bytes; sample pops
// from the end of the last digest, hashing the input when it is empty.
struct Challenger {
  std::vector<uint8_t> in, out;
  void observe(const uint8_t* p, size_t n) {
    out.clear();
    in.insert(in.end(), p, p + n);
  }
  void observe_f(uint32_t f) {
    std::vector<uint8_t> b;
    put_u32(b, f);
    observe(b.data(), 4);
  }
  // observe_ext_slice (challenger.rs:10-13): each coefficient on its own
  void observe_e(const E& e) {
    for (int i = 0; i < 5; ++i) observe_f(e.c[i]);
  }
  uint8_t sample_byte() {
    if (out.empty()) {
      uint8_t d[32];
      orc_keccak256(in.data(), in.size(), d);
      out.assign(d, d + 32);
      in.assign(d, d + 32);
    }
    uint8_t b = out.back();
    out.pop_back();
    return b;
  }
  // FromUniformBytes for BabyBear (p3/src/field/from_uniform_bytes.rs:37-45):
  // 4 sampled bytes LE, shifted right by one, rejected when >= p.
  uint32_t sample_f() {
    while (true) {
      uint8_t b[4];
      for (int i = 0; i < 4; ++i) b[i] = sample_byte();
      const uint32_t v = ld_u32(b) >> 1;
      if (v < P) return v;
    }
  }
  // CanSample<E> (challenger.rs:62-74): the five coefficients in order.
  E sample_e() {
    E e;
    for (int i = 0; i < 5; ++i) e.c[i] = sample_f();
    return e;
  }
  uint64_t sample_bits(int bits) {
    uint64_t v = 0;
    for (int i = 0; i < 8; ++i) v |= (uint64_t)sample_byte() << (8 * i);
    return bits >= 64 ? v : (v & (((uint64_t)1 << bits) - 1));
  }
  static bool from_blob(const uint8_t* p, size_t n, Challenger& c) {
    if (n < 16) return false;
    uint64_t li;
    std::memcpy(&li, p, 8);
    if (n < 16 + li) return false;
    uint64_t lo;
    std::memcpy(&lo, p + 8 + li, 8);
    if (n < 16 + li + lo) return false;
    c.in.assign(p + 8, p + 8 + li);
    c.out.assign(p + 16 + li, p + 16 + li + lo);
    return true;
  }
  std::vector<uint8_t> to_blob() const {
    std::vector<uint8_t> b;
    put_u64(b, in.size());
    b.insert(b.end(), in.begin(), in.end());
    put_u64(b, out.size());
    b.insert(b.end(), out.begin(), out.end());
    return b;
  }
};

static size_t brev(size_t x, int bits) {
  size_t r = 0;
  for (int i = 0; i < bits; ++i) r |= ((x >> i) & 1) << (bits - 1 - i);
  return r;
}

// ---------------------------------------------------------------------------
// Radix2DitParallel::dft_batch (width 1): natural-order evaluations of the
// coefficient vector on the subgroup generated by two_adic_generator(log n).
// ---------------------------------------------------------------------------
static std::vector<uint32_t> dft(std::vector<uint32_t> a) {
  const size_t n = a.size();
  int L = 0;
  while (((size_t)1 << L) < n) ++L;
  std::vector<uint32_t> x(n);
  for (size_t i = 0; i < n; ++i) x[i] = a[brev(i, L)];
  for (int s = 0; s < L; ++s) {  // butterflies of half-size h = 2^s
    const size_t h = (size_t)1 << s;
    const uint32_t wm = two_adic_generator(s + 1);
    for (size_t blk = 0; blk < n; blk += 2 * h) {
      uint32_t w = 1;
      for (size_t j = 0; j < h; ++j) {
        const uint32_t u = x[blk + j], v = fmul(x[blk + j + h], w);
        x[blk + j] = fadd(u, v);
        x[blk + j + h] = fsub(u, v);
        w = fmul(w, wm);
      }
    }
  }
  return x;
}

// The definitional DFT (for the tests): w_j = sum_k a_k g^(jk).
static std::vector<uint32_t> dft_definition(const std::vector<uint32_t>& a) {
  const size_t n = a.size();
  int L = 0;
  while (((size_t)1 << L) < n) ++L;
  const uint32_t g = two_adic_generator(L);
  std::vector<uint32_t> out(n);
  for (size_t j = 0; j < n; ++j) {
    uint32_t acc = 0, gj = fpow(g, j), p = 1;
    for (size_t k = 0; k < n; ++k) {
      acc = fadd(acc, fmul(a[k], p));
      p = fmul(p, gj);
    }
    out[j] = acc;
  }
  return out;
}

// ---------------------------------------------------------------------------
// The two prime-field RandomFoldableCodes (code.rs:16-91): ReedSolomonCode
// (reed_solomon.rs, log2_k_0 = 0) and GenericRandomFoldableCode with
// reed_solomon_g_0_with_random_ts (generic.rs), whose random t's come from
// the caller's RNG and are given here as arrays.
// ---------------------------------------------------------------------------
struct Code {
  int lambda, log2_c, log2_k0 = 0, d;
  bool generic = false;
  std::vector<std::vector<uint32_t>> ts;            // generic: ts[i] has n_i entries
  std::vector<std::vector<uint32_t>> t_inv_halves;  // per i: (2 t_i[j])^-1, j < n_i
  // ReedSolomonCode::new (reed_solomon.rs:20-38): t_i[j] = g_i^j with
  // g_i = two_adic_generator(log2_c + i + 1)
  Code(int lambda_, int log2_c_, int d_) : lambda(lambda_), log2_c(log2_c_), d(d_) {
    for (int i = 0; i < d; ++i) {
      const uint32_t g = two_adic_generator(log2_c + i + 1);
      std::vector<uint32_t> t((size_t)1 << (log2_c + i));
      uint32_t p = 1;
      for (auto& v : t) {
        v = finv(fadd(p, p));
        p = fmul(p, g);
      }
      t_inv_halves.push_back(std::move(t));
    }
  }
  // reed_solomon_g_0_with_random_ts (generic.rs:43-71) with the random
  // vectors given: ts_flat holds ts[0], ts[1], .., ts[d-1] back to back.
  Code(int lambda_, int log2_c_, int log2_k0_, int d_, const uint32_t* ts_flat)
      : lambda(lambda_), log2_c(log2_c_), log2_k0(log2_k0_), d(d_), generic(true) {
    size_t off = 0;
    for (int i = 0; i < d; ++i) {
      std::vector<uint32_t> t(ts_flat + off, ts_flat + off + n_i(i)), inv(n_i(i));
      off += n_i(i);
      for (size_t j = 0; j < t.size(); ++j) inv[j] = finv(fadd(t[j], t[j]));
      ts.push_back(std::move(t));
      t_inv_halves.push_back(std::move(inv));
    }
  }
  size_t c() const { return (size_t)1 << log2_c; }
  size_t k0() const { return (size_t)1 << log2_k0; }
  size_t n0() const { return c() * k0(); }
  size_t n_d() const { return n0() << d; }
  size_t n_i(int i) const { return n0() << i; }
  int log2_n_d() const { return log2_c + log2_k0 + d; }
  // Appendix C of ePrint 2023/1705 as generic.rs:24-39 computes it, with
  // F::bits() = 31 for BabyBear.
  static double z_c(double lambda, double log2_f, size_t c, int i, int log2_n_i) {
    if (i == 0) return 1.0 / (double)c;
    return z_c(lambda, log2_f, c, i - 1, log2_n_i - 1) * (log2_f / (log2_f - 1.001)) +
           1.0 / (log2_f - 1.001) *
               ((2.0 * (double)(log2_n_i - 1) + lambda) / (double)((uint64_t)1 << log2_n_i) + 0.6);
  }
  // num_queries (reed_solomon.rs:58-64, generic.rs:99-103): unique decoding,
  // delta = 1 - distance / 3; Rust's saturating cast maps -inf, NaN and
  // negatives to 0.
  size_t num_queries() const {
    const double rel = generic ? 1.0 - z_c((double)lambda, 31.0, c(), d, log2_n_d()) : 1.0 - 1.0 / (double)c();
    const double delta = 1.0 - rel / 3.0;
    const double q = std::ceil((double)lambda / -std::log2(delta));
    if (!(q > 0)) return 0;
    if (!std::isfinite(q) || q >= 1.8446744073709552e19) return SIZE_MAX;
    return (size_t)q;
  }
  // encode_batch of one column of k_0 << d entries.
  std::vector<uint32_t> encode(const std::vector<uint32_t>& m) const {
    if (!generic) {  // reed_solomon.rs:71-75: bit_reverse_rows, pad_to_height(n_d), dft_batch
      std::vector<uint32_t> a(n_d(), 0);
      for (size_t r = 0; r < m.size(); ++r) a[r] = m[brev(r, d)];
      return dft(a);
    }
    // generic.rs:118-140: every k_0-chunk times G_0 (g_0[i][j] = i^j), then
    // the butterflies (l, r) -> (l + t r, l - t r) of ts[i-1] on the halves of
    // every n_i-chunk, i = 1..d
    std::vector<uint32_t> w(n_d(), 0);
    for (size_t b = 0; b < ((size_t)1 << d); ++b)
      for (size_t i = 0; i < n0(); ++i) {
        uint32_t acc = 0, pw = 1;
        for (size_t j = 0; j < k0(); ++j) {
          acc = fadd(acc, fmul(pw, m[b * k0() + j]));
          pw = fmul(pw, (uint32_t)i);
        }
        w[b * n0() + i] = acc;
      }
    for (int i = 1; i <= d; ++i) {
      const size_t ni = n_i(i), half = ni / 2;
      for (size_t base = 0; base < w.size(); base += ni)
        for (size_t k = 0; k < half; ++k) {
          const uint32_t l = w[base + k], r = fmul(w[base + half + k], ts[i - 1][k]);
          w[base + k] = fadd(l, r);
          w[base + half + k] = fsub(l, r);
        }
    }
    return w;
  }
  // encode0 (reed_solomon.rs:66-70, generic.rs:105-110): w = m G_0
  std::vector<E> encode0(const std::vector<E>& m) const {
    if (!generic) return std::vector<E>(c(), m[0]);
    std::vector<E> w(n0());
    for (size_t i = 0; i < n0(); ++i) {
      uint32_t pw = 1;
      for (size_t j = 0; j < m.size(); ++j) {
        w[i] = eadd(w[i], escale(m[j], pw));
        pw = fmul(pw, (uint32_t)i);
      }
    }
    return w;
  }
  // interpolate (code.rs:86-91)
  E interpolate(int i, size_t j, const E& lo, const E& hi, const E& r) const {
    const E l = escale(eadd(lo, hi), INV2);
    const E h = escale(esub(lo, hi), t_inv_halves[i][j]);
    return eadd(l, emul(esub(h, l), r));
  }
  // fold (code.rs:66-77)
  void fold(int i, std::vector<E>& w, const E& r) const {
    const size_t mid = w.size() / 2;
    parallel_for(mid, [&](size_t b, size_t e) {
      for (size_t j = b; j < e; ++j) w[j] = interpolate(i, j, w[j], w[j + mid], r);
    });
    w.resize(mid);
  }
};

// ---------------------------------------------------------------------------
// Merkle trees (MerkleTreeMmcs over GenericHasher<Keccak256Hash>): leaf =
// keccak256 of the row's bincode, node = keccak256(left || right).
// ---------------------------------------------------------------------------
struct Tree {
  std::vector<std::vector<Digest>> layers;
  const Digest& root() const { return layers.back()[0]; }
  std::vector<Digest> path(size_t idx) const {
    std::vector<Digest> p;
    for (size_t k = 0; k + 1 < layers.size(); ++k) {
      p.push_back(layers[k][idx ^ 1]);
      idx >>= 1;
    }
    return p;
  }
};
static Digest hash_bytes(const std::vector<uint8_t>& b) {
  Digest d;
  orc_keccak256(b.data(), b.size(), d.b);
  return d;
}
static Digest hash_node(const Digest& l, const Digest& r) {
  uint8_t buf[64];
  std::memcpy(buf, l.b, 32);
  std::memcpy(buf + 32, r.b, 32);
  Digest d;
  orc_keccak256(buf, 64, d.b);
  return d;
}
static Tree build_tree(std::vector<Digest> leaves) {
  Tree t;
  t.layers.push_back(std::move(leaves));
  while (t.layers.back().size() > 1) {
    const auto& prev = t.layers.back();
    std::vector<Digest> next(prev.size() / 2);
    parallel_for(next.size(), [&](size_t b, size_t e) {
      for (size_t i = b; i < e; ++i) next[i] = hash_node(prev[2 * i], prev[2 * i + 1]);
    });
    t.layers.push_back(std::move(next));
  }
  return t;
}
static Digest leaf_row(const uint32_t* row, size_t w) {
  std::vector<uint8_t> b;
  for (size_t c = 0; c < w; ++c) put_u32(b, row[c]);
  return hash_bytes(b);
}
// ExtensionMmcs row of the pi commit (basefold.rs:350-355): two E, flattened
static Digest leaf_pair(const E& a, const E& b) {
  std::vector<uint8_t> buf;
  put_e(buf, a);
  put_e(buf, b);
  return hash_bytes(buf);
}
static bool verify_path(const Digest& root, Digest leaf, size_t idx, const std::vector<Digest>& path,
                        size_t height) {
  size_t h = 0;
  while (((size_t)1 << h) < height) ++h;
  if (path.size() != h) return false;
  for (const Digest& s : path) {
    leaf = (idx & 1) ? hash_node(s, leaf) : hash_node(leaf, s);
    idx >>= 1;
  }
  return std::memcmp(leaf.b, root.b, 32) == 0;
}

// ---------------------------------------------------------------------------
// Multilinear polynomials (p3/src/poly/multilinear.rs) and sumcheck
// (sumcheck/src/lib.rs, function/eval.rs, function/eval_impr.rs).
// ---------------------------------------------------------------------------
// eq_expand (:216-222)
static std::vector<E> eq_table(const std::vector<E>& x, const E& scalar) {
  std::vector<E> ev((size_t)1 << x.size());
  ev[0] = scalar;
  for (size_t i = 0; i < x.size(); ++i) {
    const size_t h = (size_t)1 << i;
    for (size_t k = 0; k < h; ++k) {
      ev[h + k] = emul(ev[k], x[i]);
      ev[k] = esub(ev[k], ev[h + k]);
    }
  }
  return ev;
}
// fix_last_var (:183-198): lo += x (hi - lo)
static void fix_last_var(std::vector<E>& ev, const E& x) {
  const size_t mid = ev.size() / 2;
  for (size_t k = 0; k < mid; ++k) ev[k] = eadd(ev[k], emul(x, esub(ev[k + mid], ev[k])));
  ev.resize(mid);
}
static E evaluate(std::vector<E> ev, const std::vector<E>& x) {
  for (size_t k = x.size(); k-- > 0;) fix_last_var(ev, x[k]);
  return ev[0];
}
// eq_eval (:224-229): prod (2 x y + 1 - x - y), zipped to the shorter
static E eq_eval(const E* x, const E* y, size_t n) {
  E p = E::one();
  for (size_t i = 0; i < n; ++i) p = emul(p, esub(esub(eadd(edouble(emul(x[i], y[i])), E::one()), x[i]), y[i]));
  return p;
}
// horner (univariate.rs:5-12)
static E horner(const std::vector<E>& c, const E& x) {
  E acc;
  for (size_t k = c.size(); k-- > 0;) acc = eadd(emul(acc, x), c[k]);
  return acc;
}

struct Subclaim {  // SumcheckSubclaim (lib.rs:18-48)
  E value;
  std::vector<E> r_rev;
  std::vector<E> r() const { return std::vector<E>(r_rev.rbegin(), r_rev.rend()); }
  void reduce(const std::vector<E>& rp, const E& x) {
    value = horner(rp, x);
    r_rev.push_back(x);
  }
};

// EvalProver over EvalImprProver and HalfEq (eval.rs:27-116, eval_impr.rs:13-207).
struct EvalProver {
  std::vector<E> r, r_inv, one_minus_r_inv, half_eq, poly;
  Subclaim inner;
  E inner_rp[2];
  bool ok = true;
  EvalProver(const std::vector<E>& point, std::vector<E> p) : r(point), poly(std::move(p)) {
    for (const E& x : r) {
      if (x.is_zero()) ok = false;
      r_inv.push_back(einv(x));
    }
    const size_t n1 = r.empty() ? 0 : r.size() - 1;
    std::vector<E> rlo(r.begin(), r.begin() + n1);
    for (const E& x : rlo) {
      const E d = esub(E::one(), x);
      if (d.is_zero()) ok = false;
      one_minus_r_inv.push_back(einv(d));
    }
    half_eq = eq_table(rlo, E::one());
  }
  size_t num_vars() const { return r.size(); }
  E correcting_factor(int round) const {  // eval_impr.rs:83-90
    E p = E::one();
    for (size_t k = round; k < one_minus_r_inv.size(); ++k) p = emul(p, one_minus_r_inv[k]);
    return p;
  }
  E eval_1(int round, const E& claim, const E& e0) const {  // eval_impr.rs:41-43
    return emul(esub(claim, emul(esub(E::one(), r[round]), e0)), r_inv[round]);
  }
  E delta_scalar(int round, const Subclaim& sc) const {  // eval_impr.rs:45-51
    if ((size_t)round == (num_vars() == 0 ? 0 : num_vars() - 1)) return E::one();
    const std::vector<E> rr = sc.r();
    const size_t n = std::min(r.size() - (round + 1), rr.size());
    return eq_eval(r.data() + round + 1, rr.data(), n);
  }
  std::vector<E> compute_round_poly(int round, const Subclaim& outer) {
    const Subclaim& sc = ((size_t)round == num_vars() - 1) ? outer : inner;
    const size_t half = poly.size() / 2, n = std::min(half, half_eq.size());
    E s;
    for (size_t k = 0; k < n; ++k) s = eadd(s, emul(half_eq[k], poly[k]));
    const E c0 = emul(correcting_factor(round), s);
    const E c1 = esub(eval_1(round, sc.value, c0), c0);  // eval_impr.rs:150-162
    inner_rp[0] = c0;
    inner_rp[1] = c1;
    const E scalar = delta_scalar(round, sc);  // delta (eval_impr.rs:53-58)
    const E d0 = emul(scalar, esub(E::one(), r[round]));
    const E d1 = emul(scalar, esub(r[round], esub(E::one(), r[round])));
    return {emul(c0, d0), eadd(emul(c0, d1), emul(c1, d0)), emul(c1, d1)};
  }
  void fix_last(const E& x) {  // eval.rs:108-111
    fix_last_var(poly, x);
    half_eq.resize(half_eq.size() / 2);
    inner.reduce({inner_rp[0], inner_rp[1]}, x);
  }
};

// ---------------------------------------------------------------------------
// Basefold (poly-commit/src/basefold.rs), width 1.
// ---------------------------------------------------------------------------
struct Commitment {
  Tree tree;
  size_t w = 1;
  std::vector<uint32_t> cw;  // n_d rows of w, row-major
  const uint32_t* row(size_t q) const { return cw.data() + q * w; }
};
// A column of a row-major matrix.
static std::vector<uint32_t> column(const std::vector<uint32_t>& m, size_t w, size_t c) {
  std::vector<uint32_t> v(m.size() / w);
  for (size_t r = 0; r < v.size(); ++r) v[r] = m[r * w + c];
  return v;
}
// commit (:112-120): encode_batch column by column, leaf = row bincode
static Commitment commit(const Code& code, const std::vector<uint32_t>& data, size_t w) {
  Commitment cm;
  cm.w = w;
  cm.cw.assign(code.n_d() * w, 0);
  parallel_for(w, [&](size_t b, size_t e) {  // columns are independent
    for (size_t c = b; c < e; ++c) {
      const std::vector<uint32_t> col = code.encode(column(data, w, c));
      for (size_t q = 0; q < col.size(); ++q) cm.cw[q * w + c] = col[q];
    }
  }, 1);
  std::vector<Digest> leaves(code.n_d());
  parallel_for(leaves.size(), [&](size_t b, size_t e) {
    for (size_t q = b; q < e; ++q) leaves[q] = leaf_row(cm.row(q), w);
  });
  cm.tree = build_tree(std::move(leaves));
  return cm;
}
// eval (:126-131): every column's multilinear extension at the point
static std::vector<E> eval(const std::vector<uint32_t>& data, size_t w, const std::vector<E>& point) {
  std::vector<E> out(w);
  parallel_for(w, [&](size_t b, size_t e) {
    for (size_t c = b; c < e; ++c) {
      std::vector<E> ev(data.size() / w);
      for (size_t i = 0; i < ev.size(); ++i) ev[i] = E::from(data[i * w + c]);
      out[c] = evaluate(ev, point);
    }
  }, 1);
  return out;
}
// dot_product of extension scalars with a base-field row
static E dot_row(const std::vector<E>& s, const uint32_t* row, size_t w) {
  E acc;
  for (size_t c = 0; c < w; ++c) acc = eadd(acc, escale(s[c], row[c]));
  return acc;
}
// sample_random_scalars_by_eq (:398-408): eq of ceil(log2 n) sampled points,
// truncated to n
static std::vector<E> scalars_by_eq(size_t n, Challenger& ch) {
  int log_n = 0;
  while (((size_t)1 << log_n) < n) ++log_n;
  std::vector<E> r(log_n);
  for (E& x : r) x = ch.sample_e();
  std::vector<E> s = eq_table(r, E::one());
  s.resize(n);
  return s;
}

// open (:133-232); returns the bincode of BasefoldProof, empty on failure
static std::vector<uint8_t> open(const Code& code, const Commitment& cm, const std::vector<uint32_t>& data,
                                 const std::vector<E>& point, const std::vector<E>& values, Challenger& ch) {
  const int d = code.d;
  const size_t w = cm.w, rows = data.size() / w;
  std::vector<E> pi(code.n_d()), poly(rows);
  E claim;
  if (w == 1) {
    for (size_t q = 0; q < pi.size(); ++q) pi[q] = E::from(cm.cw[q]);
    for (size_t i = 0; i < rows; ++i) poly[i] = E::from(data[i]);
    claim = values[0];
  } else {  // :160-176: rows combined with scalars sampled by eq
    const std::vector<E> s = scalars_by_eq(w, ch);
    parallel_for(rows, [&](size_t b, size_t e) {
      for (size_t i = b; i < e; ++i) poly[i] = dot_row(s, data.data() + i * w, w);
    });
    for (size_t c = 0; c < w; ++c) claim = eadd(claim, emul(s[c], values[c]));
    parallel_for(pi.size(), [&](size_t b, size_t e) {
      for (size_t q = b; q < e; ++q) pi[q] = dot_row(s, cm.row(q), w);
    });
  }
  EvalProver pr(point, poly);
  if (!pr.ok) return {};
  Subclaim sc;
  sc.value = claim;
  std::vector<Tree> pi_trees;
  std::vector<std::vector<E>> pi_vals;  // the matrix committed each round (pairs)
  std::vector<std::vector<E>> comp;
  for (int i = d - 1; i >= 0; --i) {  // prove_interleaved_folding_sumcheck (:335-369)
    const size_t mid = pi.size() / 2;
    std::vector<Digest> leaves(mid);
    parallel_for(mid, [&](size_t b, size_t e) {
      for (size_t j = b; j < e; ++j) leaves[j] = leaf_pair(pi[j], pi[j + mid]);
    });
    pi_trees.push_back(build_tree(std::move(leaves)));
    pi_vals.push_back(pi);
    ch.observe(pi_trees.back().root().b, 32);
    const std::vector<E> rp = pr.compute_round_poly(i + code.log2_k0, sc);  // round i + log2_k_0 (:356-361)
    const std::vector<E> c = {rp[0], rp[2]};  // Eval::compress_round_poly
    for (const E& e : c) ch.observe_e(e);
    const E x = ch.sample_e();
    pr.fix_last(x);
    sc.reduce(rp, x);
    comp.push_back(c);
    code.fold(i, pi, x);
  }
  const std::vector<E> fin = pr.poly;  // into_ext_poly: the k_0 evaluations left
  for (const E& e : fin) ch.observe_e(e);
  if (code.encode0(fin) != pi) return {};  // debug_assert_eq!(encode0(final_poly), pi) (:189)
  const size_t Q = code.num_queries();
  std::vector<uint64_t> idx(Q);
  for (auto& v : idx) v = ch.sample_bits(code.log2_n_d());
  std::vector<uint8_t> b;
  put_u64(b, comp.size());
  for (const auto& c : comp) {
    put_u64(b, c.size());
    for (const E& e : c) put_e(b, e);
  }
  put_u64(b, fin.size());
  for (const E& e : fin) put_e(b, e);
  put_u64(b, pi_trees.size());
  for (const Tree& t : pi_trees) b.insert(b.end(), t.root().b, t.root().b + 32);
  put_u64(b, Q);
  for (uint64_t q : idx) {
    put_u64(b, w);
    for (size_t c = 0; c < w; ++c) put_u32(b, cm.row(q)[c]);
    const auto path = cm.tree.path(q);
    put_u64(b, path.size());
    for (const Digest& g : path) b.insert(b.end(), g.b, g.b + 32);
    put_u64(b, (uint64_t)d);
    for (int k = 0; k < d; ++k) {
      const int i = d - 1 - k;
      const size_t ni = code.n_i(i);
      const size_t sib = ((q / ni) & 1) ^ 1, j = q % ni;
      put_e(b, pi_vals[k][j + sib * ni]);  // row j holds (pi[j], pi[j + n_i])
      const auto p2 = pi_trees[k].path(j);
      put_u64(b, p2.size());
      for (const Digest& g : p2) b.insert(b.end(), g.b, g.b + 32);
    }
  }
  return b;
}

struct Reader {
  const uint8_t* p;
  size_t n, off = 0;
  bool ok = true;
  const uint8_t* take(size_t k) {
    if (off + k > n) {
      ok = false;
      return nullptr;
    }
    const uint8_t* r = p + off;
    off += k;
    return r;
  }
  uint64_t u64() {
    const uint8_t* q = take(8);
    uint64_t v = 0;
    if (q) std::memcpy(&v, q, 8);
    return v;
  }
  // a coefficient >= p does not decode (malformed), like a short read
  E e() {
    const uint8_t* q = take(20);
    if (!q) return E();
    const E v = ld_e(q);
    for (int i = 0; i < 5; ++i)
      if (v.c[i] >= P) ok = false;
    return v;
  }
  Digest dg() {
    Digest g{};
    const uint8_t* q = take(32);
    if (q) std::memcpy(g.b, q, 32);
    return g;
  }
};

// verify (:234-324): 0 ok, 1 InvalidFinalPoly, 2 InvalidQuery, 3 Mmcs, 4 malformed
static int verify(const Code& code, const Digest& root, const std::vector<E>& point, const std::vector<E>& values,
                  Challenger& ch, const uint8_t* proof, size_t len) {
  const int d = code.d;
  const size_t w = values.size();
  std::vector<E> scalars = {E::one()};
  E claim = values[0];
  if (w > 1) {  // :253-259
    scalars = scalars_by_eq(w, ch);
    claim = E();
    for (size_t c = 0; c < w; ++c) claim = eadd(claim, emul(scalars[c], values[c]));
  }
  Reader rd{proof, len};
  std::vector<std::vector<E>> comp(rd.u64());
  if (!rd.ok || comp.size() != (size_t)d) return 4;
  for (auto& c : comp) {
    c.resize(rd.u64());
    if (!rd.ok || c.size() != 2) return 4;
    for (E& e : c) e = rd.e();
  }
  if (!rd.ok || rd.u64() != code.k0()) return 4;
  std::vector<E> fin(code.k0());
  for (E& e : fin) e = rd.e();
  if (!rd.ok) return 4;
  std::vector<Digest> pi_comms(rd.u64());
  if (!rd.ok || pi_comms.size() != (size_t)d) return 4;
  for (Digest& g : pi_comms) g = rd.dg();
  Subclaim sc;
  sc.value = claim;
  for (int k = 0; k < d; ++k) {  // verify_interleaved_folding_sumcheck
    ch.observe(pi_comms[k].b, 32);
    for (const E& e : comp[k]) ch.observe_e(e);
    // Eval::decompress_round_poly: c1 = claim - 2 c0 - c2
    const E c1 = esub(esub(sc.value, edouble(comp[k][0])), comp[k][1]);
    const E x = ch.sample_e();
    sc.reduce({comp[k][0], c1, comp[k][1]}, x);
  }
  for (const E& e : fin) ch.observe_e(e);
  const std::vector<E> r = sc.r();
  // evaluate(final_poly, point_lo) * eq_eval(point_hi, r) (:271-275)
  const std::vector<E> point_lo(point.begin(), point.begin() + code.log2_k0);
  const size_t nhi = point.size() - code.log2_k0;
  if (emul(evaluate(fin, point_lo), eq_eval(point.data() + code.log2_k0, r.data(), std::min(nhi, r.size()))) !=
      sc.value)
    return 1;
  const std::vector<E> pi0 = code.encode0(fin);
  const size_t Q = code.num_queries();
  std::vector<uint64_t> idx(Q);
  for (auto& v : idx) v = ch.sample_bits(code.log2_n_d());
  if (rd.u64() != Q) return 4;
  for (size_t qi = 0; qi < Q; ++qi) {
    const uint64_t q = idx[qi];
    if (rd.u64() != w) return 4;
    const uint8_t* vp = rd.take(4 * w);
    if (!vp) return 4;
    std::vector<uint32_t> row(w);
    for (size_t c = 0; c < w; ++c) {
      row[c] = ld_u32(vp + 4 * c);
      if (row[c] >= P) return 4;
    }
    std::vector<Digest> path(rd.u64());
    if (!rd.ok || path.size() > 64) return 4;
    for (Digest& g : path) g = rd.dg();
    if (!rd.ok) return 4;
    if (!verify_path(root, leaf_row(row.data(), w), q, path, code.n_d())) return 3;
    E folded = dot_row(scalars, row.data(), w);
    if (rd.u64() != (uint64_t)d) return 4;
    for (int k = 0; k < d; ++k) {
      const int i = d - 1 - k;
      const size_t ni = code.n_i(i);
      const size_t sib = ((q / ni) & 1) ^ 1, j = q % ni;
      const E other = rd.e();
      if (!rd.ok) return 4;
      std::vector<Digest> p2(rd.u64());
      if (!rd.ok || p2.size() > 64) return 4;
      for (Digest& g : p2) g = rd.dg();
      if (!rd.ok) return 4;
      E vals[2] = {folded, folded};
      vals[sib] = other;
      if (!verify_path(pi_comms[k], leaf_pair(vals[0], vals[1]), j, p2, ni)) return 3;
      folded = code.interpolate(i, j, vals[0], vals[1], r[i]);  // r[i]: round i's challenge
    }
    if (folded != pi0[q % code.n0()]) return 2;  // pi_0[idx % n_0] (:316-318)
  }
  return rd.off == len ? 0 : 4;
}

}  // namespace orb

using namespace orb;

static std::vector<uint32_t> load_u32s(const uint8_t* p, size_t n) {
  std::vector<uint32_t> v(n);
  if (n) std::memcpy(v.data(), p, 4 * n);
  return v;
}
static std::vector<E> load_es(const uint8_t* p, size_t n) {
  std::vector<E> v(n);
  for (size_t i = 0; i < n; ++i) v[i] = ld_e(p + 20 * i);
  return v;
}
static void store_e(uint8_t* p, const E& e) { std::memcpy(p, e.c, 20); }

extern "C" {

// Field helpers for the tests: products and inverses of E, and the DFT.
void orc_bb_emul(const uint8_t* a, const uint8_t* b, uint8_t* out, size_t n) {
  for (size_t i = 0; i < n; ++i) store_e(out + 20 * i, emul(ld_e(a + 20 * i), ld_e(b + 20 * i)));
}
void orc_bb_einv(const uint8_t* a, uint8_t* out, size_t n) {
  for (size_t i = 0; i < n; ++i) store_e(out + 20 * i, einv(ld_e(a + 20 * i)));
}
int orc_bb_dft(int log_n, uint32_t* data, int definition) {
  if (log_n < 0 || log_n > 27) return -1;
  std::vector<uint32_t> a(data, data + ((size_t)1 << log_n));
  const std::vector<uint32_t> r = definition ? dft_definition(a) : dft(a);
  std::memcpy(data, r.data(), 4 * r.size());
  return 0;
}
// The code of a call: Reed–Solomon when ts is null (log2_k0 must be 0), else
// the generic random foldable code with the given t's (d = n - log2_k0).
static bool bad_size(int n, int log2_c, int log2_k0, size_t w) {
  return n < 0 || log2_c < 0 || log2_k0 < 0 || log2_k0 > n || n + log2_c > 27 || w == 0;
}
static Code make_code(int n, int log2_c, int log2_k0, const uint32_t* ts) {
  if (!ts) return Code(128, log2_c, n);
  return Code(128, log2_c, log2_k0, n - log2_k0, ts);
}
size_t orc_bb_num_queries(int lambda, int n, int log2_c, int log2_k0, int generic) {
  if (!generic) return Code(lambda, log2_c, 0).num_queries();
  const int d = n - log2_k0;
  std::vector<uint32_t> ts(((size_t)1 << (log2_c + log2_k0)) * (((size_t)1 << d) - 1) + 1, 1);
  Code code(lambda, log2_c, log2_k0, d, ts.data());
  return code.num_queries();
}
// Data is row-major, 2^n rows of `width` canonical BabyBears.
int orc_bb_encode(int n, int log2_c, int log2_k0, const uint32_t* ts, size_t width, const uint8_t* data,
                  uint8_t* out) {
  if (bad_size(n, log2_c, log2_k0, width) || (!ts && log2_k0)) return -1;
  const Code code = make_code(n, log2_c, log2_k0, ts);
  const Commitment cm = commit(code, load_u32s(data, width << n), width);
  std::memcpy(out, cm.cw.data(), 4 * cm.cw.size());
  return 0;
}
int orc_bb_commit(int n, int log2_c, int log2_k0, const uint32_t* ts, size_t width, const uint8_t* data,
                  uint8_t* root) {
  if (bad_size(n, log2_c, log2_k0, width) || (!ts && log2_k0)) return -1;
  const Code code = make_code(n, log2_c, log2_k0, ts);
  const Commitment cm = commit(code, load_u32s(data, width << n), width);
  std::memcpy(root, cm.tree.root().b, 32);
  return 0;
}
int orc_bb_eval(int n, size_t width, const uint8_t* data, const uint8_t* point, uint8_t* out) {
  if (bad_size(n, 0, 0, width)) return -1;
  const std::vector<E> v = eval(load_u32s(data, width << n), width, load_es(point, n));
  for (size_t c = 0; c < width; ++c) store_e(out + 20 * c, v[c]);
  return 0;
}
// The reference harness (poly-commit/src/lib.rs:80-100): commit, observe the
// root, evaluate at the point, observe the values; returns root, values and
// the challenger state.
int orc_bb_harness_prepare(int n, int log2_c, int log2_k0, const uint32_t* ts, size_t width, const uint8_t* data,
                           const uint8_t* point, uint8_t* root, uint8_t* values, uint8_t* blob, size_t* blob_len) {
  if (bad_size(n, log2_c, log2_k0, width) || (!ts && log2_k0)) return -1;
  const Code code = make_code(n, log2_c, log2_k0, ts);
  const std::vector<uint32_t> m = load_u32s(data, width << n);
  const Commitment cm = commit(code, m, width);
  Challenger ch;
  ch.observe(cm.tree.root().b, 32);
  const std::vector<E> v = eval(m, width, load_es(point, n));
  for (const E& e : v) ch.observe_e(e);
  std::memcpy(root, cm.tree.root().b, 32);
  for (size_t c = 0; c < width; ++c) store_e(values + 20 * c, v[c]);
  const std::vector<uint8_t> b = ch.to_blob();
  if (*blob_len < b.size()) return -2;
  std::memcpy(blob, b.data(), b.size());
  *blob_len = b.size();
  return 0;
}
int orc_bb_open(int n, int log2_c, int log2_k0, const uint32_t* ts, size_t width, const uint8_t* data,
                const uint8_t* point, const uint8_t* values, const uint8_t* blob, size_t blob_len, uint8_t* out,
                size_t cap, size_t* len) {
  if (bad_size(n, log2_c, log2_k0, width) || (!ts && log2_k0)) return -1;
  const Code code = make_code(n, log2_c, log2_k0, ts);
  Challenger ch;
  if (!Challenger::from_blob(blob, blob_len, ch)) return -1;
  const std::vector<uint32_t> m = load_u32s(data, width << n);
  const Commitment cm = commit(code, m, width);
  const std::vector<uint8_t> pf = open(code, cm, m, load_es(point, n), load_es(values, width), ch);
  if (pf.empty()) return -3;
  *len = pf.size();
  if (cap < pf.size()) return -2;
  std::memcpy(out, pf.data(), pf.size());
  return 0;
}
int orc_bb_verify(int n, int log2_c, int log2_k0, const uint32_t* ts, size_t width, const uint8_t* root,
                  const uint8_t* point, const uint8_t* values, const uint8_t* blob, size_t blob_len,
                  const uint8_t* proof, size_t len) {
  if (bad_size(n, log2_c, log2_k0, width) || (!ts && log2_k0)) return -1;
  const Code code = make_code(n, log2_c, log2_k0, ts);
  Challenger ch;
  if (!Challenger::from_blob(blob, blob_len, ch)) return -1;
  Digest r;
  std::memcpy(r.b, root, 32);
  return verify(code, r, load_es(point, n), load_es(values, width), ch, proof, len);
}

}  // extern "C"
