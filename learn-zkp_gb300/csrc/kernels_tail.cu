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

// The transcript is kept in shared memory and driven by one warp: the
// Keccak permutations run on all 32 lanes (WarpKeccak), the byte bookkeeping
// and the field arithmetic on lane 0, with __syncwarp between them.

// HashChallenger::flush: digest = keccak256(input); input = output = digest.
__device__ void warp_flush(const WarpKeccak& wk, DevTranscript& t) {
  __syncwarp();
  const int len = t.in_len;
  uint2 a = make_uint2(0, 0);
  for (int off = 0;; off += 136) {
    const int take = len - off < 136 ? len - off : 136;
    const bool last = take < 136;
    if (wk.lane < 17) {
      const int pos0 = 8 * wk.lane;
      uint2 w;
      if (pos0 + 8 <= take) {  // a whole message word (off and pos0 are multiples of 8)
        w = *reinterpret_cast<const uint2*>(t.in + off + pos0);
      } else {
        uint32_t h[2] = {0, 0};
        for (int b = 0; b < 8; ++b) {
          const int pos = pos0 + b;
          uint32_t v = pos < take ? t.in[off + pos] : 0u;
          if (last && pos == take) v ^= 0x01u;  // pad10*1 (original Keccak)
          h[b >> 2] |= v << (8 * (b & 3));
        }
        w = make_uint2(h[0], h[1]);
      }
      if (last && wk.lane == 16) w.y ^= 0x80000000u;  // last byte of the rate
      a = kx2(a, w);
    }
    a = wk.permute<false>(a);
    if (last) break;
  }
  __syncwarp();
  if (wk.lane < 4) {
    reinterpret_cast<uint2*>(t.out)[wk.lane] = a;
    reinterpret_cast<uint2*>(t.in)[wk.lane] = a;
  }
  if (wk.lane == 0) {
    t.out_len = 32;
    t.in_len = 32;
  }
  __syncwarp();
}

// CanObserve<u8> of the 16*N bytes of v (lane 0): append to the input, drop
// unread output.
template <int N>
__device__ void tr_observe(OpenState& o, const uint4 (&v)[N]) {
  DevTranscript& t = o.tr;
  t.out_len = 0;
  const int len = t.in_len;
  if (len + 16 * N > kTrMax) {
    o.status = 1;
    return;
  }
  if ((len & 15) == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) reinterpret_cast<uint4*>(t.in + len)[k] = v[k];
  } else {
#pragma unroll
    for (int k = 0; k < N; ++k) {
      const uint32_t w[4] = {v[k].x, v[k].y, v[k].z, v[k].w};
#pragma unroll
      for (int b = 0; b < 16; ++b) t.in[len + 16 * k + b] = (uint8_t)(w[b >> 2] >> (8 * (b & 3)));
    }
  }
  t.in_len = len + 16 * N;
}

// A field element from 16 sampled bytes, each popped from the end of the
// output, little-endian (challenger.rs sample, from_uniform_bytes.rs:20-26).
// Warp-collective; the element is returned on lane 0.
__device__ uint4 warp_sample_elem(const WarpKeccak& wk, OpenState& o) {
  __syncwarp();
  if (o.tr.out_len == 0) warp_flush(wk, o.tr);
  uint32_t w[4] = {0, 0, 0, 0};
  if (o.tr.out_len >= 16) {
    if (wk.lane == 0) {
      const int top = o.tr.out_len - 1;
#pragma unroll
      for (int k = 0; k < 16; ++k) w[k >> 2] |= (uint32_t)o.tr.out[top - k] << (8 * (k & 3));
      o.tr.out_len = top + 1 - 16;
    }
  } else {
    for (int k = 0; k < 16; ++k) {
      __syncwarp();
      if (o.tr.out_len == 0) warp_flush(wk, o.tr);
      if (wk.lane == 0) {
        const uint32_t byte = o.tr.out[--o.tr.out_len];
        w[k >> 2] |= byte << (8 * (k & 3));
      }
    }
  }
  __syncwarp();
  return make_uint4(w[0], w[1], w[2], w[3]);
}

// Transcript step of round i, warp-collective.  S = sum_b half_eq[b] poly_lo[b].
// `rec` (global, 16-byte aligned) receives root, c0, c2.
//
// EvalImprProver::compute_round_poly gives [c0, c1] (eval_impr.rs:116-127);
// EvalProver lifts it by delta = d * [1 - r, r - (1 - r)] = d * [1 + r, 1]
// in characteristic 2 (eval.rs:89-106), so the round polynomial is
// (c0 + c1 X)(d (1 + r) + d X): c0' = c0 d (1 + r), c2' = c1 d.  After the
// challenge x the EvalProver claim is c0 + c1 x and d becomes d (1 + r + x);
// the sumcheck claim (the round polynomial at x) is only read in the first
// round, so it is not carried.
__device__ void round_step(const WarpKeccak& wk, OpenState& o, int i, int d, const uint4* scal, uint4 root_lo_bi,
                           uint4 root_hi_bi, uint4 S, uint4* rec) {
  Digest rt;  // the round's root is a tree digest (interleaved): its bytes
  rt.lo = root_lo_bi;
  rt.hi = root_hi_bi;
  rt = digest_bytes(rt);
  const uint4 root_lo = rt.lo, root_hi = rt.hi;
  // Every lane computes the same scalars; the products are spread over the
  // warp (gf_mul_warp2), two independent ones at a time.
  const uint4 ONE = one_dev();
  const uint4 r = scal[3 * i], r_inv = scal[3 * i + 1], corr = scal[3 * i + 2];
  const uint4 claim = (i == d - 1) ? o.outer : o.inner;
  const uint4 delta = o.delta;
  const uint4 one_r = gf_add(ONE, r);
  uint4 c0, d0, t, rp0, c1, rp2;
  gf_mul_warp2(corr, S, delta, one_r, c0, d0);  // c0 = corr * S; d0 = delta (1 + r)
  gf_mul_warp2(one_r, c0, c0, d0, t, rp0);      // rp0 = c0 d0
  c1 = gf_add(gf_mul_warp(gf_add(claim, t), r_inv), c0);
  rp2 = gf_mul_warp(c1, delta);
  __syncwarp();
  if (wk.lane == 0) {
    rec[0] = root_lo;
    rec[1] = root_hi;
    rec[2] = rp0;
    rec[3] = rp2;
    const uint4 m[4] = {root_lo, root_hi, rp0, rp2};
    tr_observe(o, m);  // root (basefold.rs:356), then [c0, c2] (sumcheck/src/lib.rs:97)
  }
  uint4 x = warp_sample_elem(wk, o);  // valid on lane 0
  x.x = __shfl_sync(0xffffffffu, x.x, 0);
  x.y = __shfl_sync(0xffffffffu, x.y, 0);
  x.z = __shfl_sync(0xffffffffu, x.z, 0);
  x.w = __shfl_sync(0xffffffffu, x.w, 0);
  uint4 c1x, delta_next;
  gf_mul_warp2(c1, x, delta, gf_add(one_r, x), c1x, delta_next);
  if (wk.lane == 0) {
    o.inner = gf_add(c1x, c0);  // EvalProver::fix_last_var (eval.rs:108-111)
    o.delta = delta_next;
    o.x = x;
  }
  __syncwarp();
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
    if (root) {  // a tree root, stored interleaved
      const Digest rb = digest_bytes(load_digest(root, 0));
      const uint4 m[2] = {rb.lo, rb.hi};
      tr_observe(sh, m);
    }
    if (value) {
      const uint4 m[1] = {value[0]};
      tr_observe(sh, m);
      sh.outer = m[0];
    }
  }
  __syncthreads();
  state_store(S, sh);
}

__global__ void __launch_bounds__(32) open_round_kernel(OpenState* S, int i, int d, const uint4* scal,
                                                        const uint4* root, const uint4* Sred, uint8_t* rec) {
  __shared__ OpenState sh;
  const WarpKeccak wk;
  state_load(sh, S);
  __syncthreads();
  round_step(wk, sh, i, d, scal, root[0], root[1], Sred[0], reinterpret_cast<uint4*>(rec));
  __syncthreads();
  state_store(S, sh);
}

__global__ void __launch_bounds__(kTailThreads, 1) open_tail_kernel(TailParams P) {
  __shared__ OpenState sh;
  __shared__ uint4 sh_S, sh_root_lo, sh_root_hi;
  __shared__ uint4 scratch[32];
  const int d = P.d;
  const size_t c = (size_t)1 << P.log2_c;
  const WarpKeccak wk;
  const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  state_load(sh, P.state);
  if (threadIdx.x == 0 && P.i0 >= 0) {
    sh_root_lo = P.root_i0[0];
    sh_root_hi = P.root_i0[1];
    sh_S = P.S_i0[0];
  }
  __syncthreads();
  int k = 0;
  for (int i = P.i0; i >= 0; --i, ++k) {
    // ---- transcript step (warp 0) ----
    if (warp == 0)
      round_step(wk, sh, i, d, P.scal, sh_root_lo, sh_root_hi, sh_S, reinterpret_cast<uint4*>(P.result + 64 * (size_t)k));
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
        if (h <= (size_t)nwarps) {  // latency-bound: one warp per node
          for (size_t s = warp; s < h; s += nwarps) warp_hash_node(wk, cur, s, h, nxt);
        } else {
          for (size_t s = threadIdx.x; s < h; s += blockDim.x)
            store_digest(nxt, s, hash_node(load_digest(cur, s), load_digest(cur, s + h)));
        }
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
    reinterpret_cast<uint4*>(P.result + 64 * (size_t)k)[0] = fin;
    const uint4 m[1] = {fin};
    tr_observe(sh, m);
    // the reference's debug self-check encode0(final_poly) == pi (basefold.rs:198):
    // every entry of the last folded codeword is the final polynomial
    if (P.i0 >= 0) {
      const uint4* pi0 = P.pi_fold + c * (((size_t)1 << d) - 2);
      for (size_t t = 0; t < c; ++t) {
        const uint4 e = pi0[t];
        if (e.x != fin.x || e.y != fin.y || e.z != fin.z || e.w != fin.w) sh.status |= 2;
      }
    }
  }
  __syncthreads();
  state_store(P.state, sh);
}

// Product sumcheck round (warp): c = [c0, c2, c3] from the device sums.
__global__ void __launch_bounds__(32) sumcheck_round_kernel(OpenState* S, int k, const uint32_t* acc, uint8_t* rec) {
  __shared__ OpenState sh;
  const WarpKeccak wk;
  state_load(sh, S);
  __syncthreads();
  const uint4* a = reinterpret_cast<const uint4*>(acc);
  const uint4 c0 = a[0], c2 = a[1], c3 = a[2];
  const uint4 sc = sh.outer;
  // k = 2: compressed [c0, c2] (the pair scalar is ONE, quadratic.rs:118),
  // round polynomial [c0, sc - 2 c0 - c2 = sc + c2, c2]; k = 3: compressed
  // [c0, c2, c3], round polynomial [c0, sc + c2 + c3, c2, c3]
  if (wk.lane == 0) {
    uint4* r = reinterpret_cast<uint4*>(rec);
    r[0] = c0;
    r[1] = c2;
    if (k == 3) {
      r[2] = c3;
      const uint4 m[3] = {c0, c2, c3};
      tr_observe(sh, m);
    } else {
      const uint4 m[2] = {c0, c2};
      tr_observe(sh, m);
    }
  }
  uint4 x = warp_sample_elem(wk, sh);  // valid on lane 0
  x.x = __shfl_sync(0xffffffffu, x.x, 0);
  x.y = __shfl_sync(0xffffffffu, x.y, 0);
  x.z = __shfl_sync(0xffffffffu, x.z, 0);
  x.w = __shfl_sync(0xffffffffu, x.w, 0);
  // horner over the round polynomial at x
  const uint4 c1 = (k == 3) ? gf_add(sc, gf_add(c2, c3)) : gf_add(sc, c2);
  uint4 acc_h = (k == 3) ? c3 : c2;
  if (k == 3) acc_h = gf_add(gf_mul_warp(acc_h, x), c2);
  acc_h = gf_add(gf_mul_warp(acc_h, x), c1);
  acc_h = gf_add(gf_mul_warp(acc_h, x), c0);
  if (wk.lane == 0) {
    reinterpret_cast<uint4*>(rec)[k] = x;
    sh.outer = acc_h;
    sh.x = x;
  }
  __syncthreads();
  state_store(S, sh);
}

cudaError_t launch_sumcheck_round(OpenState* s, int k, const uint32_t* acc, uint8_t* rec, cudaStream_t st) {
  if (k != 2 && k != 3) return cudaErrorInvalidValue;
  sumcheck_round_kernel<<<1, 32, 0, st>>>(s, k, acc, rec);
  count_launch();
  return cudaGetLastError();
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
