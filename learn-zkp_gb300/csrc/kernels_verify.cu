// Basefold::verify (poly-commit/src/basefold.rs:234-324) for many proofs at
// once: the per-query work on the GPU.
//
// The host replays each proof's transcript (a short serial chain), checks the
// final polynomial and samples the query positions; what is left is, for every
// query of every proof, one codeword Merkle path and d folded-codeword paths
// plus the fold chain that links them (basefold.rs:284-320).  The paths are
// independent once the chain's values are known, and the chain needs no
// hashes, so:
//  * verify_fold_kernel (one thread per query) runs the chain — the leaf row's
//    scalar combination, then per round the pair [folded, sibling] placed by
//    the index bit and the interpolation of binary_reed_solomon.rs:98-109 —
//    writes each round's pair and compares the last value with the final
//    polynomial (encode0 repeats it, binary_reed_solomon.rs:63-65);
//  * verify_path_kernel (one thread per path) hashes a leaf and walks its
//    sibling path to the root (MerkleTreeMmcs::verify_batch: leaf =
//    keccak256(row bytes), node = keccak256(left || right), the index bit of
//    each level choosing the side).  Paths are ordered level-major, so the 32
//    threads of a warp walk paths of the same length.
// Proof bytes are read where bincode put them: every field sits at a multiple
// of 8 bytes, so elements and digests load as 8-byte words.
#include <cuda_runtime.h>

#include <cstdint>

#include "bf_internal.h"
#include "gf128.cuh"
#include "keccak.cuh"

namespace bf {

namespace {

__device__ __forceinline__ uint4 load_elem8(const uint8_t* blob, uint64_t off) {
  const uint2* p = reinterpret_cast<const uint2*>(blob + off);
  const uint2 a = p[0], b = p[1];
  return make_uint4(a.x, a.y, b.x, b.y);
}

// A digest stored as bytes, in the interleaved lane form the tree hashes use.
__device__ __forceinline__ Digest load_digest_bytes(const uint8_t* blob, uint64_t off) {
  const uint2* p = reinterpret_cast<const uint2*>(blob + off);
  Digest d;
  const uint2 l0 = p[0], l1 = p[1], l2 = p[2], l3 = p[3];
  d.lo = make_uint4(l0.x, l0.y, l1.x, l1.y);
  d.hi = make_uint4(l2.x, l2.y, l3.x, l3.y);
  return digest_interleaved(d);
}

__device__ __forceinline__ bool digest_eq(const Digest& a, const Digest& b) {
  return a.lo.x == b.lo.x && a.lo.y == b.lo.y && a.lo.z == b.lo.z && a.lo.w == b.lo.w && a.hi.x == b.hi.x &&
         a.hi.y == b.hi.y && a.hi.z == b.hi.z && a.hi.w == b.hi.w;
}

__device__ __forceinline__ bool elem_eq(uint4 a, uint4 b) { return a.x == b.x && a.y == b.y && a.z == b.z && a.w == b.w; }

// Leaf of a row of `width` > 1 elements: keccak256 of its 16*width bytes,
// any number of 136-byte (17-lane) blocks; lanes are indexed statically so
// the state stays in registers.
__device__ __forceinline__ Digest hash_row(const uint8_t* blob, uint64_t off, uint32_t width) {
  uint2 s[25];
#pragma unroll
  for (int k = 0; k < 25; ++k) s[k] = make_uint2(0, 0);
  const uint2* row = reinterpret_cast<const uint2*>(blob + off);
  const uint64_t lanes = 2ull * width;
  for (uint64_t k = 0;; k += 17) {
    const uint64_t left = lanes - k;  // message lanes from this block on
#pragma unroll
    for (int r = 0; r < 17; ++r) {
      if ((uint64_t)r < left) s[r] = kx2(s[r], row[k + r]);
      if ((uint64_t)r == left) s[r].x ^= 0x01u;  // pad10*1 starts in this block
    }
    if (left < 17) {
      s[16].y ^= 0x80000000u;
      keccak_f1600(s);
      break;
    }
    keccak_f1600(s);
  }
  return digest_interleaved(digest_from_state(s));
}

__global__ void __launch_bounds__(128) verify_fold_kernel(VerifyParams P) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P.nq) return;
  const VerifyQuery Q = P.queries[q];
  if (Q.job == kVerifyInactive) {
    P.final_bad[q] = 0;
    return;
  }
  const VerifyJob J = P.jobs[Q.job];
  const uint8_t* blob = P.blob;
  uint4 folded;
  if (J.width == 1) {
    folded = load_elem8(blob, Q.leaves);  // scalars = [ONE] (basefold.rs:253-254)
  } else {
    folded = make_uint4(0, 0, 0, 0);
    for (uint32_t w = 0; w < J.width; ++w)
      folded = gf_add(folded, gf_mul(load_elem8(blob, J.scalars + 16ull * w), load_elem8(blob, Q.leaves + 16ull * w)));
  }
  const int d = P.d;
  for (int k = 0; k < d; ++k) {
    const int i = d - 1 - k;
    const int bits = P.log2_c + i;  // log2 n_i
    const uint64_t ii = Q.idx & ((1ull << bits) - 1);
    const bool sib_left = ((Q.idx >> bits) & 1) != 0;  // the sibling is values[0]
    const VerifyRound R = P.rounds[(size_t)q * d + k];
    const uint4 s = load_elem8(blob, R.sibling);
    uint4 v0 = sib_left ? s : folded, v1 = sib_left ? folded : s;
    P.pairs[2 * ((size_t)q * d + k)] = v0;
    P.pairs[2 * ((size_t)q * d + k) + 1] = v1;
    // interpolate: twiddle of stage k at bitrev(ii) (binary_reed_solomon.rs:29-35)
    const uint32_t K = bits ? (uint32_t)(__brevll(ii) >> (64 - bits)) : 0u;
    const uint4 t = gf_add(P.tw->lo[k][K & ((1u << kTwLoBits) - 1)], P.tw->hi[k][K >> kTwLoBits]);
    v1 = gf_add(v1, v0);
    v0 = gf_add(v0, gf_mul(v1, t));
    folded = gf_add(v0, gf_mul(gf_add(v1, v0), load_elem8(blob, J.challenges + 16ull * k)));
  }
  P.final_bad[q] = elem_eq(folded, load_elem8(blob, J.final_poly)) ? 0 : 1;
}

__global__ void __launch_bounds__(128) verify_path_kernel(VerifyParams P) {
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t total = (uint64_t)P.nq * (P.d + 1);
  if (t >= total) return;
  const uint32_t level = (uint32_t)(t / P.nq), q = (uint32_t)(t % P.nq);
  const VerifyQuery Q = P.queries[q];
  if (Q.job == kVerifyInactive) {
    P.path_bad[t] = 0;
    return;
  }
  const VerifyJob J = P.jobs[Q.job];
  const uint8_t* blob = P.blob;
  Digest cur, root;
  int log_h;
  uint64_t index, path;
  if (level == 0) {  // the codeword tree: leaf = keccak256 of the row's 16*width bytes
    log_h = P.d + P.log2_c;
    index = Q.idx;
    path = Q.path;
    root = load_digest_bytes(blob, J.root);
    cur = J.width == 1 ? hash_elem(load_elem8(blob, Q.leaves)) : hash_row(blob, Q.leaves, J.width);
  } else {  // folded codeword of round k: leaf = keccak256(values[0] || values[1])
    const int k = (int)level - 1;
    log_h = P.log2_c + P.d - 1 - k;
    index = Q.idx & ((1ull << log_h) - 1);
    path = P.rounds[(size_t)q * P.d + k].path;
    root = load_digest_bytes(blob, J.pi_comms + 32ull * k);
    const size_t pr = 2 * ((size_t)q * P.d + k);
    cur = hash_pair(P.pairs[pr], P.pairs[pr + 1]);
  }
  for (int b = 0; b < log_h; ++b) {
    const Digest sib = load_digest_bytes(blob, path + 32ull * b);
    // the side is picked by selects, not a branch: threads of a warp differ in it
    const bool right = ((index >> b) & 1) != 0;
    Digest l, r;
    l.lo = right ? sib.lo : cur.lo;
    l.hi = right ? sib.hi : cur.hi;
    r.lo = right ? cur.lo : sib.lo;
    r.hi = right ? cur.hi : sib.hi;
    cur = hash_node(l, r);
  }
  P.path_bad[t] = digest_eq(cur, root) ? 0 : 1;
}

}  // namespace

cudaError_t launch_verify(const VerifyParams& p, cudaStream_t st) {
  if (p.nq == 0) return cudaSuccess;
  verify_fold_kernel<<<(p.nq + 127) / 128, 128, 0, st>>>(p);
  count_launch();
  const uint64_t total = (uint64_t)p.nq * (p.d + 1);
  verify_path_kernel<<<(unsigned)((total + 127) / 128), 128, 0, st>>>(p);
  count_launch();
  return cudaGetLastError();
}

}  // namespace bf
