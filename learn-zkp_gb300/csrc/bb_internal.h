// Internal interface between the prime-field host code (api_bb.cu) and its
// kernels (kernels_bb.cu).  Not part of the public C ABI.
//
// Arrays: evaluations as the caller gave them (canonical BabyBears,
// row-major, `w` per row); the codeword in Montgomery form, same layout,
// natural (DFT output) order; extension arrays as five Montgomery words per
// element.  Merkle trees use the reversed level storage of the binary path
// (leaf j of a 2^h-leaf tree at bitrev_h(j)), so launch_tree builds them.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "bb.cuh"

namespace bf {

constexpr int kBbMaxRounds = 27;  // num_vars + log2_c <= 27 (the two-adicity of BabyBear)

// g^k * scale for k < n (Montgomery in, Montgomery out).
cudaError_t bb_launch_pow_table(uint32_t* out, size_t n, uint32_t g_mont, uint32_t scale_mont, cudaStream_t st);
// Butterfly factors as Shoup pairs (w canonical, floor(w 2^32 / p)): g^k for
// k < n (g in Montgomery form), or the n canonical words at `in` (*bad set for
// a word >= p).
cudaError_t bb_launch_pow_shoup(uint2* out, size_t n, uint32_t g_mont, cudaStream_t st);
cudaError_t bb_launch_shoup_from(const uint32_t* in, uint2* out, size_t n, uint32_t* bad, cudaStream_t st);
// encode_batch of a 2^(d + log2_k0) x w matrix into its 2^(d + log2_k0 +
// log2_c) x w codeword (Montgomery).  `tw` holds the butterfly factors of
// layer s at tw[2^s - 1 + k] as Shoup pairs: g_s^k for the Reed–Solomon code
// (log2_k0 = 0), ts[s - log2_n0][k] for the generic code (`generic`), whose
// stage 0 is the dense G_0.  A data word >= p sets *bad.
// With `slices` > 1, input slice k (data rows [k R / slices, (k+1) R / slices))
// is ready when slice_ready[k] completes: the first stage waits for each slice
// just before the part of its grid that reads it.
cudaError_t bb_launch_encode(const uint32_t* m, uint32_t* cw, int d, int log2_c, int log2_k0, int generic, size_t w,
                             const uint2* tw, uint32_t* bad, cudaStream_t st,
                             const cudaEvent_t* slice_ready = nullptr, int slices = 0);
// out[k] = in[k] in canonical form (Montgomery in).
cudaError_t bb_launch_from_mont(const uint32_t* in, uint32_t* out, size_t n, cudaStream_t st);
// tinv[k] = (2 ts[k])^-1 (Montgomery); *bad set for a t that is 0 or >= p.
cudaError_t bb_launch_tinv(const uint32_t* ts, uint32_t* tinv, size_t n, uint32_t* bad, cudaStream_t st);
// Leaf of codeword row q (keccak256 of its w canonical words) at bitrev_bits(q).
cudaError_t bb_launch_leaves_rows(const uint32_t* cw, uint4* leaves, size_t rows, size_t w, int bits,
                                  cudaStream_t st);
// Leaf j = keccak256(pi[j] || pi[j + half]) as extension elements (pi is
// base-field Montgomery when `base`), at bitrev_bits(j).
cudaError_t bb_launch_leaves_pairs(const uint32_t* pi, int base, uint4* leaves, size_t half, int bits,
                                   cudaStream_t st);
// out[r] = sum_c mul(scalars[c], src[r w + c]) (extension out, Montgomery):
// pass s R for a Montgomery source (the codeword), s R^2 for canonical
// evaluations.
cudaError_t bb_launch_combine(const uint32_t* src, size_t rows, size_t w, const uint32_t* scalars, uint32_t* out,
                              cudaStream_t st);
// acc[5 c + k] += coefficient k of sum_r eq[r] * data[r w + c] (canonical data,
// canonical sums, reduced by the caller).
cudaError_t bb_launch_eval_cols(const uint32_t* eq, const uint32_t* data, size_t rows, size_t w,
                                unsigned long long* acc, cudaStream_t st);
// The eq table of the n coordinates x (Montgomery, n <= kBbMaxRounds): entry b
// is the product of x_i (bit i of b set) or 1 - x_i, as MultiPoly::eq builds
// it (p3/src/poly/multilinear.rs:41-64, 216-222).
cudaError_t bb_launch_eq_table(uint32_t* ev, const bb::E5* x, int n, cudaStream_t st);
// acc[k] += coefficient k of sum_{b < n} heq[b] * poly[b]; poly is canonical
// base-field data when `base` (canonical sums), else extension (Montgomery sums).
cudaError_t bb_launch_dot(const uint32_t* heq, const uint32_t* poly, int base, size_t n, unsigned long long* acc,
                          cudaStream_t st);
// out[b] = in[b] + x (in[b + half] - in[b]); `base`: in is canonical data.
// x is *xp (Montgomery, device memory) when xp is set.
cudaError_t bb_launch_fix(const uint32_t* in, int base, uint32_t* out, size_t half, const bb::E5& x,
                          cudaStream_t st, const uint32_t* xp = nullptr);

// Fold of round i (code.rs:66-84): out[j] = interpolate(tinv[j], w[j],
// w[j + n], x), j < n = n_i, with the next round's leaves when `leaves` is set.
struct BbFold {
  const uint32_t* w;  // 2n entries: extension, or base-field Montgomery when `base`
  int base;
  uint32_t* out;          // n extension entries
  const uint32_t* tinv;   // n entries (2 t_i^j)^-1, Montgomery
  size_t n;
  uint4* leaves;          // n/2 leaves of the next round, or null
  int leaf_bits;          // log2(n/2)
  const uint32_t* xp;     // the challenge in device memory (Montgomery), or null: the x argument
};
cudaError_t bb_launch_fold(const BbFold& p, const bb::E5& x, cudaStream_t st);

// The open's Fiat–Shamir transcript on the device: HashChallenger<u8,
// Keccak256Hash, 32> (p3/src/challenger.rs) as a sponge — the lanes of the
// input blocks absorbed so far plus the pending input bytes — and its output
// buffer, with the EvalProver subclaims of the folding sumcheck.  Field
// elements are Montgomery form.
struct BbTranscript {
  uint2 A[25];          // lanes (low word, high word) of the absorbed input blocks
  uint8_t pend[256];    // input bytes not yet absorbed (fewer than 136 between rounds)
  uint32_t pend_len;
  uint8_t out[32];      // output buffer: bytes out[0 .. out_len), popped from the end
  uint32_t out_len;
  bb::E5 outer;         // the open's subclaim (sumcheck/src/lib.rs:18-48)
  bb::E5 inner;         // EvalImprProver's inner subclaim value
  bb::E5 xs[kBbMaxRounds];  // challenges in sampling order
  uint32_t rounds;
};
// Per sumcheck round ri (< num_vars): the point coordinate, its inverse and
// the correcting factor prod_{k >= ri} (1 - r_k)^-1 (eval_impr.rs:83-90).
struct BbRoundConsts {
  bb::E5 r[kBbMaxRounds], r_inv[kBbMaxRounds], cf[kBbMaxRounds];
};
// One folding-sumcheck round's transcript (k rounds done before it): observe
// the round's folded-codeword root (interleaved digest at root_dev), compute
// the round polynomial from the GPU sum (Montgomery sums, or canonical ones
// when `canonical`), observe its compressed form, sample the challenge into
// x_out (Montgomery) and record the root and the compressed polynomial (72
// canonical bytes) at rec.
cudaError_t bb_launch_transcript_round(BbTranscript* t, const BbRoundConsts* c, int k, int ri, int num_vars,
                                       const uint4* root_dev, const unsigned long long* sums, int canonical,
                                       uint32_t* x_out, uint8_t* rec, cudaStream_t st);

// Query openings in the proof's bincode layout, one record per query:
// u64 w, w canonical words, u64 L, L digests, u64 d, then per round k:
// the sibling (five canonical words), u64 log2 n_i, the path.
struct BbGather {
  const uint32_t* cw;      // codeword (Montgomery), rows of w
  const uint4* cw_tree;
  const uint32_t* pi[kBbMaxRounds];  // the matrix committed in round k (extension; base codeword when k = 0 and pi0_base)
  const uint4* trees[kBbMaxRounds];
  int pi0_base;
  const uint64_t* idx;
  uint8_t* out;
  size_t w;
  size_t rec_bytes;
  int L, d, log2_n0, nq;  // round i's tree has n_0 << i leaves
};
cudaError_t bb_launch_gather(const BbGather& p, cudaStream_t st);

}  // namespace bf
