// Host-side scalars of the prime-field prover and verifier: BabyBear and its
// quintic extension E = F[X] / (X^5 - 2) in canonical form, the transcript's
// field sampling, the verifier's sumcheck algebra and the prover's per-point
// constants.  Only O(num_vars) values pass through here; every array stays
// on the GPU.
#pragma once
#include <cstdint>
#include <cstring>
#include <vector>

#include "bb.cuh"
#include "host_math.h"

namespace bbh {

constexpr uint32_t P = bb::P;

inline uint32_t fadd(uint32_t a, uint32_t b) {
  const uint32_t s = a + b;
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
inline uint32_t finv(uint32_t a) { return fpow(a, P - 2); }  // Fermat; a != 0
// TwoAdicField::two_adic_generator(bits): 31^((p - 1) / 2^27) squared
// 27 - bits times.
inline uint32_t two_adic_generator(int bits) {
  uint32_t g = 0x1a427a41u;
  for (int k = bits; k < 27; ++k) g = fmul(g, g);
  return g;
}

struct E {
  uint32_t c[5] = {0, 0, 0, 0, 0};
  static E from(uint32_t f) {
    E e;
    e.c[0] = f;
    return e;
  }
  static E one() { return from(1); }
  bool is_zero() const { return (c[0] | c[1] | c[2] | c[3] | c[4]) == 0; }
  bool operator==(const E& o) const { return std::memcmp(c, o.c, sizeof(c)) == 0; }
  bool operator!=(const E& o) const { return !(*this == o); }
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
inline E escale(const E& a, uint32_t f) {
  E r;
  for (int i = 0; i < 5; ++i) r.c[i] = fmul(a.c[i], f);
  return r;
}
inline E emul(const E& a, const E& b) {
  uint64_t t[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int i = 0; i < 5; ++i)
    for (int j = 0; j < 5; ++j) t[i + j] = (t[i + j] + (uint64_t)a.c[i] * b.c[j]) % P;
  E r;
  for (int k = 0; k < 5; ++k) r.c[k] = (uint32_t)((t[k] + (k < 4 ? 2 * t[k + 5] : 0)) % P);
  return r;
}
// Frobenius a -> a^p: X^p = z X with z = 2^((p - 1) / 5), so coefficient i
// is multiplied by z^i.  The inverse is phi(a) phi^2(a) phi^3(a) phi^4(a)
// divided by the norm a phi(a) .. phi^4(a), which lies in the base field.
inline E frobenius(const E& a, int k) {
  static const uint32_t z = fpow(2, (P - 1) / 5);
  const uint32_t zk = fpow(z, (uint64_t)k);
  E r;
  uint32_t f = 1;
  for (int i = 0; i < 5; ++i) {
    r.c[i] = fmul(a.c[i], f);
    f = fmul(f, zk);
  }
  return r;
}
inline E einv(const E& a) {  // a != 0
  E prod = frobenius(a, 1);
  for (int k = 2; k < 5; ++k) prod = emul(prod, frobenius(a, k));
  const uint32_t norm = emul(a, prod).c[0];
  return escale(prod, finv(norm));
}

// Inverses of every v[k] with one field inversion (prefix products, then
// back-substitution); false when some v[k] is 0.
inline bool batch_einv(const std::vector<E>& v, std::vector<E>& out) {
  out.assign(v.size(), E::one());
  if (v.empty()) return true;
  std::vector<E> pre(v.size());
  E acc = E::one();
  for (size_t k = 0; k < v.size(); ++k) {
    if (v[k].is_zero()) return false;
    pre[k] = acc;  // product of v[0 .. k)
    acc = emul(acc, v[k]);
  }
  E inv = einv(acc);  // (v[0] .. v[k])^-1 as k runs down
  for (size_t k = v.size(); k-- > 0;) {
    out[k] = emul(inv, pre[k]);
    inv = emul(inv, v[k]);
  }
  return true;
}

inline E load(const uint8_t* p) {
  E e;
  std::memcpy(e.c, p, 20);
  return e;
}
inline void store(uint8_t* p, const E& e) { std::memcpy(p, e.c, 20); }
inline bool canonical(const E& e) {
  for (int i = 0; i < 5; ++i)
    if (e.c[i] >= P) return false;
  return true;
}
inline bb::E5 to_dev(const E& e) {
  bb::E5 r;
  for (int i = 0; i < 5; ++i) r.c[i] = bb::to_mont(e.c[i]);
  return r;
}
inline E from_dev_sums(const unsigned long long s[5]) {  // Montgomery coefficient sums -> canonical
  E r;
  for (int i = 0; i < 5; ++i) r.c[i] = bb::from_mont((uint32_t)(s[i] % P));
  return r;
}
inline E from_canonical_sums(const unsigned long long s[5]) {
  E r;
  for (int i = 0; i < 5; ++i) r.c[i] = (uint32_t)(s[i] % P);
  return r;
}
inline bb::E5 to_dev2(const E& e) {  // e R^2 coefficient-wise: mul(e R^2, v) = e v R for canonical v
  bb::E5 r;
  for (int i = 0; i < 5; ++i) r.c[i] = bb::to_mont(bb::to_mont(e.c[i]));
  return r;
}

// MultiPoly::eq (p3/src/poly/multilinear.rs:41-64, 216-222) on the host.
inline std::vector<E> eq_table(const std::vector<E>& x, const E& scalar) {
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
// eq_eval (multilinear.rs:224-229): prod (2 x y + 1 - x - y) over the
// shorter of the two.
inline E eq_eval(const E* x, const E* y, size_t n) {
  E p = E::one();
  for (size_t i = 0; i < n; ++i) {
    const E xy = emul(x[i], y[i]);
    p = emul(p, esub(esub(eadd(eadd(xy, xy), E::one()), x[i]), y[i]));
  }
  return p;
}
inline E horner(const E* c, size_t n, const E& x) {  // univariate.rs:5-12
  E acc;
  for (size_t k = n; k-- > 0;) acc = eadd(emul(acc, x), c[k]);
  return acc;
}

// GenericChallenger<BabyBear, Keccak256Hash> over the byte transcript
// (p3/src/challenger.rs:51-83): a BabyBear is observed as its 4 canonical
// bytes; sampling one takes 4 popped bytes little-endian, shifted right by
// one, rejected while >= p (from_uniform_bytes.rs:37-45); an extension
// element is five of them (E::from_base_fn).
inline void observe_f(bfh::Challenger& ch, uint32_t f) {
  uint8_t b[4];
  std::memcpy(b, &f, 4);
  ch.observe(b, 4);
}
inline void observe_e(bfh::Challenger& ch, const E& e) {  // observe_ext_slice
  for (int i = 0; i < 5; ++i) observe_f(ch, e.c[i]);
}
inline uint32_t sample_f(bfh::Challenger& ch) {
  while (true) {
    uint32_t v = 0;
    for (int i = 0; i < 4; ++i) v |= (uint32_t)ch.sample_byte() << (8 * i);
    v >>= 1;
    if (v < P) return v;
  }
}
inline E sample_e(bfh::Challenger& ch) {
  E e;
  for (int i = 0; i < 5; ++i) e.c[i] = sample_f(ch);
  return e;
}
// sample_random_scalars_by_eq (poly-commit/src/basefold.rs:398-408).
inline std::vector<E> scalars_by_eq(size_t n, bfh::Challenger& ch) {
  int log_n = 0;
  while (((size_t)1 << log_n) < n) ++log_n;
  std::vector<E> r((size_t)log_n);
  for (E& x : r) x = sample_e(ch);
  std::vector<E> s = eq_table(r, E::one());
  s.resize(n);
  return s;
}

// SumcheckSubclaim (sumcheck/src/lib.rs:18-48).
struct Subclaim {
  E value;
  std::vector<E> r_rev;
  std::vector<E> r() const { return std::vector<E>(r_rev.rbegin(), r_rev.rend()); }
  void reduce(const E* rp, size_t n, const E& x) {
    value = horner(rp, n, x);
    r_rev.push_back(x);
  }
};

// The constants of EvalProver over EvalImprProver with HalfEq (sumcheck/src/
// function/eval.rs:27-116, eval_impr.rs:13-207) that the device transcript
// needs: the point's coordinates, their inverses and the correcting factors.
struct EvalScalars {
  std::vector<E> r, r_inv, one_minus_r_inv;
  // false when a coordinate is 0, or 1 below the last (their inverses are taken)
  bool init(const std::vector<E>& point) {
    r = point;
    std::vector<E> v = r, inv;  // r_k for every k, then 1 - r_k for k < n - 1
    for (size_t k = 0; k + 1 < r.size(); ++k) v.push_back(esub(E::one(), r[k]));
    if (!batch_einv(v, inv)) return false;
    r_inv.assign(inv.begin(), inv.begin() + r.size());
    one_minus_r_inv.assign(inv.begin() + r.size(), inv.end());
    return true;
  }
  // correcting factor of every round (eval_impr.rs:83-90): round k's is the
  // product of (1 - r_j)^-1 over j >= k, so one backward pass of suffix
  // products gives them all (1 past the last factor)
  std::vector<E> correcting_factors() const {
    std::vector<E> cf(r.size(), E::one());
    for (size_t k = one_minus_r_inv.size(); k-- > 0;) cf[k] = emul(one_minus_r_inv[k], cf[k + 1]);
    return cf;
  }
};

}  // namespace bbh
