// The last rounds of Basefold::open in one single-block kernel, with the
// Fiat–Shamir transcript on the device.
//
// Once the folded codeword has at most a few thousand entries, a round is a
// chain of tiny steps (fold + leaf hashes, a handful of Merkle levels, the
// sumcheck fix and reduction) separated by one transcript step.  Driving them
// from the host costs a launch-and-synchronise round trip per round.  Here
// one block runs every remaining round: thread 0 keeps the transcript
// (GenericChallenger over Keccak-256, p3/src/challenger.rs) and the
// round-polynomial scalars (eval.rs:89-111, eval_impr.rs:45-58,116-127), the
// whole block does the data-parallel work, __syncthreads separates the steps.
// The bytes produced are the same as the host-driven rounds.
#include <cuda_runtime.h>

#include <cstdint>

#include "bf_internal.h"
#include "gf128.cuh"
#include "keccak.cuh"

namespace bf {

namespace {

__device__ __forceinline__ uint4 one_dev() { return make_uint4(1u, 0u, 0u, 0xc2000000u); }

// Byte-level HashChallenger<u8, Keccak256Hash, 32> held in shared memory.
struct DevTranscript {
  uint8_t in[kTailTranscriptMax];
  uint8_t out[32];
  int in_len, out_len;
};

__device__ void keccak256_bytes(const uint8_t* msg, int len, uint8_t digest[32]) {
  uint2 s[25];
#pragma unroll
  for (int k = 0; k < 25; ++k) s[k] = make_uint2(0, 0);
  int off = 0;
  while (true) {
    const int take = len - off < 136 ? len - off : 136;
    uint8_t block[136];
    for (int b = 0; b < 136; ++b) block[b] = 0;
    for (int b = 0; b < take; ++b) block[b] = msg[off + b];
    const bool last = take < 136;
    if (last) {
      block[take] ^= 0x01;  // pad10*1 (original Keccak)
      block[135] ^= 0x80;
    }
    for (int q = 0; q < 17; ++q) {
      uint32_t lo = 0, hi = 0;
      for (int b = 0; b < 4; ++b) {
        lo |= (uint32_t)block[8 * q + b] << (8 * b);
        hi |= (uint32_t)block[8 * q + 4 + b] << (8 * b);
      }
      s[q] = kx2(s[q], make_uint2(lo, hi));
    }
    keccak_f1600(s);
    off += take;
    if (last) break;
  }
  for (int q = 0; q < 4; ++q)
    for (int b = 0; b < 4; ++b) {
      digest[8 * q + b] = (uint8_t)(s[q].x >> (8 * b));
      digest[8 * q + 4 + b] = (uint8_t)(s[q].y >> (8 * b));
    }
}

__device__ void tr_observe(DevTranscript& t, const uint8_t* p, int n) {
  t.out_len = 0;
  for (int k = 0; k < n; ++k) t.in[t.in_len++] = p[k];
}

__device__ uint8_t tr_sample_byte(DevTranscript& t) {
  if (t.out_len == 0) {
    uint8_t d[32];
    keccak256_bytes(t.in, t.in_len, d);
    for (int k = 0; k < 32; ++k) {
      t.out[k] = d[k];
      t.in[k] = d[k];
    }
    t.out_len = 32;
    t.in_len = 32;
  }
  return t.out[--t.out_len];
}

__device__ uint4 tr_sample_elem(DevTranscript& t) {
  uint8_t b[16];
  for (int k = 0; k < 16; ++k) b[k] = tr_sample_byte(t);
  uint4 v;
  v.x = b[0] | (b[1] << 8) | (b[2] << 16) | ((uint32_t)b[3] << 24);
  v.y = b[4] | (b[5] << 8) | (b[6] << 16) | ((uint32_t)b[7] << 24);
  v.z = b[8] | (b[9] << 8) | (b[10] << 16) | ((uint32_t)b[11] << 24);
  v.w = b[12] | (b[13] << 8) | (b[14] << 16) | ((uint32_t)b[15] << 24);
  return v;
}

__device__ void put4(uint8_t* p, uint4 v) {
  const uint32_t w[4] = {v.x, v.y, v.z, v.w};
  for (int k = 0; k < 4; ++k)
    for (int b = 0; b < 4; ++b) p[4 * k + b] = (uint8_t)(w[k] >> (8 * b));
}

}  // namespace

__global__ void __launch_bounds__(kTailThreads, 1) open_tail_kernel(TailParams P) {
  __shared__ DevTranscript tr;
  __shared__ uint4 sh_x, sh_S, sh_root_lo, sh_root_hi;
  __shared__ uint4 scratch[32];
  const uint4 ONE = one_dev();
  const int d = P.d;
  const size_t c = (size_t)1 << P.log2_c;
  if (threadIdx.x == 0) {
    tr.in_len = P.tr_in_len;
    tr.out_len = P.tr_out_len;
    for (int k = 0; k < P.tr_in_len; ++k) tr.in[k] = P.tr_in[k];
    for (int k = 0; k < P.tr_out_len; ++k) tr.out[k] = P.tr_out[k];
    const uint4* st0 = reinterpret_cast<const uint4*>(P.stage_i0);
    sh_root_lo = P.root_in_params ? P.root_lo : st0[0];
    sh_root_hi = P.root_in_params ? P.root_hi : st0[1];
    sh_S = st0[2];
  }
  uint4 outer = P.outer, inner = P.inner, delta = P.delta;  // used by thread 0
  __syncthreads();
  int k = 0;
  for (int i = P.i0; i >= 0; --i, ++k) {
    // ---- transcript step (thread 0) ----
    if (threadIdx.x == 0) {
      const uint4 r = P.scal[3 * i], r_inv = P.scal[3 * i + 1], corr = P.scal[3 * i + 2];
      const uint4 sc_val = (i == d - 1) ? outer : inner;
      const uint4 c0 = gf_mul(corr, sh_S);
      const uint4 one_r = gf_add(ONE, r);
      const uint4 c1 = gf_add(gf_mul(gf_add(sc_val, gf_mul(one_r, c0)), r_inv), c0);
      const uint4 scalar = (i == d - 1) ? ONE : delta;
      const uint4 d0 = gf_mul(scalar, one_r);
      const uint4 d1 = gf_mul(scalar, gf_add(r, one_r));
      const uint4 rp0 = gf_mul(c0, d0);
      const uint4 rp1 = gf_add(gf_mul(c0, d1), gf_mul(c1, d0));
      const uint4 rp2 = gf_mul(c1, d1);
      uint8_t* rec = P.result + 64 * (size_t)k;
      put4(rec, sh_root_lo);
      put4(rec + 16, sh_root_hi);
      put4(rec + 32, rp0);
      put4(rec + 48, rp2);
      tr_observe(tr, rec, 64);  // root (basefold.rs:356), then [c0, c2] (sumcheck/src/lib.rs:97)
      const uint4 x = tr_sample_elem(tr);
      inner = gf_add(gf_mul(c1, x), c0);                              // horner([c0, c1], x)
      outer = gf_add(gf_mul(gf_add(gf_mul(rp2, x), rp1), x), rp0);    // horner(rp, x)
      delta = gf_mul(delta, gf_add(one_r, x));
      sh_x = x;
    }
    __syncthreads();
    const uint4 x = sh_x;
    // ---- fold (+ next leaves) and fix (+ next reduction), whole block ----
    const size_t ni = c << i;
    const uint4* pi_in = (i == d - 1) ? P.pi_first : P.pi_fold + c * (((size_t)1 << d) - ((size_t)1 << (i + 2)));
    uint4* pi_out = P.pi_fold + c * (((size_t)1 << d) - ((size_t)1 << (i + 1)));
    const uint4* tlo = P.tw->lo[d - 1 - i];
    const uint4* thi = P.tw->hi[d - 1 - i];
    uint4* leaves = nullptr;
    if (i > 0)
      leaves = P.pi_trees + 2 * ((c << 1) * (((size_t)1 << (d - 1)) - ((size_t)1 << i)) - (size_t)(d - 1 - i));
    if (i > 0) {
      for (size_t s = threadIdx.x; s < ni / 2; s += blockDim.x) {
        uint4 f[2];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const size_t t = 2 * s + q;
          const uint4 tw = gf_add(tlo[t & 4095], thi[t >> 12]);
          uint4 lo = pi_in[2 * t], hi = pi_in[2 * t + 1];
          hi = gf_add(hi, lo);
          lo = gf_add(lo, gf_mul(hi, tw));
          f[q] = gf_add(lo, gf_mul(gf_add(hi, lo), x));
          pi_out[t] = f[q];
        }
        store_digest(leaves, s, hash_pair(f[0], f[1]));
      }
    } else {
      for (size_t t = threadIdx.x; t < ni; t += blockDim.x) {
        const uint4 tw = gf_add(tlo[t & 4095], thi[t >> 12]);
        uint4 lo = pi_in[2 * t], hi = pi_in[2 * t + 1];
        hi = gf_add(hi, lo);
        lo = gf_add(lo, gf_mul(hi, tw));
        pi_out[t] = gf_add(lo, gf_mul(gf_add(hi, lo), x));
      }
    }
    const uint4* poly_in = (i == d - 1) ? P.poly_first : P.poly;
    const size_t half = (size_t)1 << i, next_half = i > 0 ? half / 2 : 0;
    uint4 part = make_uint4(0, 0, 0, 0);
    for (size_t b = threadIdx.x; b < half; b += blockDim.x) {
      const uint4 lo = poly_in[b], hi = poly_in[b + half];
      const uint4 v = gf_add(lo, gf_mul(x, gf_add(hi, lo)));
      P.poly[b] = v;
      if (b < next_half) part = gf_add(part, gf_mul(P.heq[b], v));
    }
    part = block_xor(part, scratch);
    if (threadIdx.x == 0) sh_S = part;
    __syncthreads();
    // ---- the next round's Merkle tree, level by level ----
    if (i > 0) {
      uint4* cur = leaves;
      size_t n = ni / 2;
      while (n > 1) {
        const size_t h = n >> 1;
        uint4* nxt = cur + 2 * n;
        for (size_t s = threadIdx.x; s < h; s += blockDim.x)
          store_digest(nxt, s, hash_node(load_digest(cur, s), load_digest(cur, s + h)));
        __syncthreads();
        cur = nxt;
        n = h;
      }
      if (threadIdx.x == 0) {
        sh_root_lo = cur[0];
        sh_root_hi = cur[1];
      }
      __syncthreads();
    }
  }
  // ---- final polynomial and the transcript state handed back ----
  if (threadIdx.x == 0) {
    uint8_t* fin = P.result + 64 * (size_t)k;
    put4(fin, P.poly[0]);
    uint8_t* st = fin + 16;
    st[0] = (uint8_t)tr.in_len;
    st[1] = (uint8_t)(tr.in_len >> 8);
    st[2] = (uint8_t)tr.out_len;
    st[3] = 0;
    for (int q = 0; q < tr.in_len; ++q) st[4 + q] = tr.in[q];
    for (int q = 0; q < tr.out_len; ++q) st[4 + tr.in_len + q] = tr.out[q];
  }
}

cudaError_t launch_open_tail(const TailParams& p, cudaStream_t st) {
  open_tail_kernel<<<1, kTailThreads, 0, st>>>(p);
  count_launch();
  return cudaGetLastError();
}

}  // namespace bf
