// Basefold::open with the Fiat–Shamir transcript on the device.
//
// The transcript (GenericChallenger over Keccak-256, p3/src/challenger.rs)
// and the round-polynomial scalars (eval.rs:89-111, eval_impr.rs:45-58,
// 116-127) live in an OpenState in device memory, so a whole open is one
// stream of kernels with no host round trip:
//  * open_observe_kernel observes the commitment root and the evaluation, as
//    the caller of open does (poly-commit/src/lib.rs:80-100);
//  * open_round_kernel is the transcript step of one large round; the fold,
//    fix and tree kernels of that round read the sampled challenge from the
//    state;
//  * open_tail_kernel runs every remaining round once the folded codeword has
//    at most a few thousand entries — fold + leaf hashes, Merkle levels, fix +
//    reduction and the transcript step, in one block separated by
//    __syncthreads — then observes the final polynomial (basefold.rs:196).
// The query positions (basefold.rs:200-203) are a serial chain of about 80
// Keccak digests, which the host computes far faster than one GPU thread, so
// they are sampled on the host from the returned transcript.
// The bytes produced are the same as the host-driven rounds'.
#include <cuda_runtime.h>

#include <cstdint>

#include "bf_internal.h"
#include "gf128.cuh"
#include "keccak.cuh"

namespace bf {

namespace {

__device__ __forceinline__ uint4 one_dev() { return make_uint4(1u, 0u, 0u, 0xc2000000u); }

// Keccak-256 (original padding) of `len` bytes.
__device__ void keccak256_bytes(const uint8_t* msg, int len, uint8_t digest[32]) {
  uint2 s[25];
#pragma unroll
  for (int k = 0; k < 25; ++k) s[k] = make_uint2(0, 0);
  int off = 0;
  while (true) {
    const int take = len - off < 136 ? len - off : 136;
    const bool last = take < 136;
#pragma unroll
    for (int q = 0; q < 17; ++q) {
      uint32_t w0 = 0, w1 = 0;
#pragma unroll
      for (int b = 0; b < 8; ++b) {
        const int pos = 8 * q + b;
        uint32_t v = pos < take ? msg[off + pos] : 0u;
        if (last && pos == take) v ^= 0x01u;  // pad10*1
        if (last && pos == 135) v ^= 0x80u;
        if (b < 4)
          w0 |= v << (8 * b);
        else
          w1 |= v << (8 * (b - 4));
      }
      s[q] = kx2(s[q], make_uint2(w0, w1));
    }
    keccak_f1600(s);
    off += take;
    if (last) break;
  }
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      digest[8 * q + b] = (uint8_t)(s[q].x >> (8 * b));
      digest[8 * q + 4 + b] = (uint8_t)(s[q].y >> (8 * b));
    }
}

// CanObserve<u8>: append to the input, drop unread output.
__device__ void tr_observe(OpenState& o, const uint8_t* p, int n) {
  DevTranscript& t = o.tr;
  t.out_len = 0;
  if (t.in_len + n > kTrMax) {
    o.status = 1;
    return;
  }
  for (int k = 0; k < n; ++k) t.in[t.in_len++] = p[k];
}

// CanSample<u8>: when the output is empty, hash the input; the digest becomes
// both the new input and the output, which is read from its end.
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

// A field element from 16 sampled bytes, little-endian (from_uniform_bytes.rs:20-26).
__device__ uint4 tr_sample_elem(DevTranscript& t) {
  uint32_t w[4] = {0, 0, 0, 0};
  for (int k = 0; k < 16; ++k) w[k >> 2] |= (uint32_t)tr_sample_byte(t) << (8 * (k & 3));
  return make_uint4(w[0], w[1], w[2], w[3]);
}

__device__ void put4(uint8_t* p, uint4 v) {
  const uint32_t w[4] = {v.x, v.y, v.z, v.w};
  for (int k = 0; k < 4; ++k)
    for (int b = 0; b < 4; ++b) p[4 * k + b] = (uint8_t)(w[k] >> (8 * b));
}

// Transcript step of round i (one thread).  S = sum_b half_eq[b] poly_lo[b].
__device__ void round_step(OpenState& o, int i, int d, const uint4* scal, uint4 root_lo, uint4 root_hi, uint4 S,
                           uint8_t* rec) {
  const uint4 ONE = one_dev();
  const uint4 r = scal[3 * i], r_inv = scal[3 * i + 1], corr = scal[3 * i + 2];
  const uint4 sc_val = (i == d - 1) ? o.outer : o.inner;
  const uint4 c0 = gf_mul(corr, S);
  const uint4 one_r = gf_add(ONE, r);
  const uint4 c1 = gf_add(gf_mul(gf_add(sc_val, gf_mul(one_r, c0)), r_inv), c0);
  const uint4 scalar = (i == d - 1) ? ONE : o.delta;
  const uint4 d0 = gf_mul(scalar, one_r);
  const uint4 d1 = gf_mul(scalar, gf_add(r, one_r));
  const uint4 rp0 = gf_mul(c0, d0);
  const uint4 rp1 = gf_add(gf_mul(c0, d1), gf_mul(c1, d0));
  const uint4 rp2 = gf_mul(c1, d1);
  put4(rec, root_lo);
  put4(rec + 16, root_hi);
  put4(rec + 32, rp0);
  put4(rec + 48, rp2);
  tr_observe(o, rec, 64);  // root (basefold.rs:356), then [c0, c2] (sumcheck/src/lib.rs:97)
  const uint4 x = tr_sample_elem(o.tr);
  o.inner = gf_add(gf_mul(c1, x), c0);                            // EvalProver::fix_last_var (eval.rs:108-111)
  o.outer = gf_add(gf_mul(gf_add(gf_mul(rp2, x), rp1), x), rp0);  // SumcheckSubclaim::reduce
  o.delta = gf_mul(o.delta, gf_add(one_r, x));
  o.x = x;
}

constexpr int kStateVecs = (int)(sizeof(OpenState) / sizeof(uint4));

__device__ __forceinline__ void state_load(OpenState& sh, const OpenState* g) {
  const uint4* src = reinterpret_cast<const uint4*>(g);
  uint4* dst = reinterpret_cast<uint4*>(&sh);
  for (int k = threadIdx.x; k < kStateVecs; k += blockDim.x) dst[k] = src[k];
}
__device__ __forceinline__ void state_store(OpenState* g, const OpenState& sh) {
  const uint4* src = reinterpret_cast<const uint4*>(&sh);
  uint4* dst = reinterpret_cast<uint4*>(g);
  for (int k = threadIdx.x; k < kStateVecs; k += blockDim.x) dst[k] = src[k];
}

}  // namespace

__global__ void __launch_bounds__(32) open_observe_kernel(OpenState* S, const uint4* root, const uint4* value) {
  __shared__ OpenState sh;
  state_load(sh, S);
  __syncthreads();
  if (threadIdx.x == 0) {
    uint8_t b[32];
    if (root) {
      put4(b, root[0]);
      put4(b + 16, root[1]);
      tr_observe(sh, b, 32);
    }
    if (value) {
      const uint4 v = value[0];
      put4(b, v);
      tr_observe(sh, b, 16);
      sh.outer = v;
    }
  }
  __syncthreads();
  state_store(S, sh);
}

__global__ void __launch_bounds__(32) open_round_kernel(OpenState* S, int i, int d, const uint4* scal,
                                                        const uint4* root, const uint4* Sred, uint8_t* rec) {
  __shared__ OpenState sh;
  state_load(sh, S);
  __syncthreads();
  if (threadIdx.x == 0) round_step(sh, i, d, scal, root[0], root[1], Sred[0], rec);
  __syncthreads();
  state_store(S, sh);
}

__global__ void __launch_bounds__(kTailThreads, 1) open_tail_kernel(TailParams P) {
  __shared__ OpenState sh;
  __shared__ uint4 sh_S, sh_root_lo, sh_root_hi;
  __shared__ uint4 scratch[32];
  const int d = P.d;
  const size_t c = (size_t)1 << P.log2_c;
  state_load(sh, P.state);
  if (threadIdx.x == 0 && P.i0 >= 0) {
    sh_root_lo = P.root_i0[0];
    sh_root_hi = P.root_i0[1];
    sh_S = P.S_i0[0];
  }
  __syncthreads();
  int k = 0;
  for (int i = P.i0; i >= 0; --i, ++k) {
    // ---- transcript step (thread 0) ----
    if (threadIdx.x == 0) round_step(sh, i, d, P.scal, sh_root_lo, sh_root_hi, sh_S, P.result + 64 * (size_t)k);
    __syncthreads();
    const uint4 x = sh.x;
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
  // ---- final polynomial (basefold.rs:196) ----
  if (threadIdx.x == 0) {
    const uint4 fin = (k == 0) ? P.poly_first[0] : P.poly[0];
    uint8_t* rec = P.result + 64 * (size_t)k;
    put4(rec, fin);
    tr_observe(sh, rec, 16);
  }
  __syncthreads();
  state_store(P.state, sh);
}

cudaError_t launch_open_observe(OpenState* s, const uint4* root, const uint4* value, cudaStream_t st) {
  open_observe_kernel<<<1, 32, 0, st>>>(s, root, value);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_open_round(OpenState* s, int i, int d, const uint4* scal, const uint4* root, const uint4* S,
                              uint8_t* rec, cudaStream_t st) {
  open_round_kernel<<<1, 32, 0, st>>>(s, i, d, scal, root, S, rec);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_open_tail(const TailParams& p, cudaStream_t st) {
  open_tail_kernel<<<1, kTailThreads, 0, st>>>(p);
  count_launch();
  return cudaGetLastError();
}

}  // namespace bf
