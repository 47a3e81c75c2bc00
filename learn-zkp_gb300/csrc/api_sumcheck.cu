// libbasefold_gpu.so: the standalone product sumcheck prover.
#include <algorithm>
#include <cstring>
#include <vector>

#include "api_common.h"

using bfh::u128;
using namespace bfapi;

// ===========================================================================
// Standalone product sumcheck (sumcheck/src/lib.rs:56-103).
// ===========================================================================
namespace {

int sumcheck_run(cudaStream_t st, DevBuf& scratch, PinnedBuf& pinned, int k, int n, const uint4* polys,
                 const uint8_t* claim_b, bfh::Challenger& ch, uint8_t* out) {
  const size_t N = (size_t)1 << n;
  const u128 ONE = bfh::one();
  u128 sc = bfh::load(claim_b);
  size_t off_r = 16 * (size_t)k * n, off_f = off_r + 16 * (size_t)n, off_c = off_f + 16 * (size_t)k;
  if (n == 0) {  // lib.rs:63-65: no rounds, nothing observed
    CU(cudaMemcpyAsync(pinned.b(), polys, 16, cudaMemcpyDeviceToHost, st));
    for (int j = 1; j < k; ++j)
      CU(cudaMemcpyAsync(pinned.b() + 16 * j, polys + j * N, 16, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    std::memcpy(out + off_f, pinned.b(), 16 * (size_t)k);
    bfh::store(out + off_c, sc);
    return BF_OK;
  }
  const size_t half0 = N / 2;
  // scratch: k folded polynomials, the round sums (256 B), the transcript
  // state and the per-round records (compressed polynomial + challenge)
  const size_t rec_sz = 16 * (size_t)(k + 1);
  const size_t o_acc = 16 * (size_t)k * half0, o_state = o_acc + 256, o_rec = o_state + sizeof(bf::OpenState);
  const size_t need = o_rec + rec_sz * (size_t)n + 16 * (size_t)k;
  if (scratch.bytes < need) CU(scratch.alloc(need));
  uint32_t* acc = reinterpret_cast<uint32_t*>(scratch.as<uint8_t>() + o_acc);
  uint4* work[3];
  const uint4* in[3];
  for (int j = 0; j < k; ++j) {
    work[j] = scratch.as<uint4>() + j * half0;
    in[j] = polys + j * N;
  }
  ch.observe_elem(sc);  // lib.rs:67
  const size_t pin_need = std::max(sizeof(bf::OpenState), rec_sz * (size_t)n + 16 * (size_t)k) + 64;
  if (ch.in.size() + 16 * (size_t)k <= (size_t)bf::kTrMax && ch.out.size() <= 32 && pinned.ensure(pin_need) == cudaSuccess) {
    // every round with the transcript on the device: sums, transcript step,
    // fix + next sums; one copy back at the end
    bf::OpenState img;
    std::memset(&img, 0, sizeof(img));
    if (!ch.in.empty()) std::memcpy(img.tr.in, ch.in.data(), ch.in.size());
    if (!ch.out.empty()) std::memcpy(img.tr.out, ch.out.data(), ch.out.size());
    img.tr.in_len = (int)ch.in.size();
    img.tr.out_len = (int)ch.out.size();
    img.outer = to_uint4(sc);
    std::memcpy(pinned.b(), &img, sizeof(img));
    bf::OpenState* S = reinterpret_cast<bf::OpenState*>(scratch.as<uint8_t>() + o_state);
    uint8_t* rec = scratch.as<uint8_t>() + o_rec;
    CU(cudaMemcpyAsync(S, pinned.b(), sizeof(img), cudaMemcpyHostToDevice, st));
    CU(cudaMemsetAsync(acc, 0, 48, st));
    CU(bf::launch_prod_round_sums(in, k, half0, acc, st));
    int ri = 0;
    for (int round = n - 1; round >= 0; --round, ++ri) {
      CU(bf::launch_sumcheck_round(S, k, acc, rec + rec_sz * (size_t)ri, st));
      const size_t half = (size_t)1 << round;
      if (round > 0) CU(cudaMemsetAsync(acc, 0, 48, st));
      const uint4* const* src = (round == n - 1) ? in : const_cast<const uint4* const*>(work);
      CU(bf::launch_prod_fix(work, src, k, half, uint4{}, half / 2, acc, st, &S->x));
    }
    uint8_t* fin = rec + rec_sz * (size_t)n;
    for (int j = 0; j < k; ++j) CU(cudaMemcpyAsync(fin + 16 * j, work[j], 16, cudaMemcpyDeviceToDevice, st));
    // pinned: records and final evaluations, then the state
    const size_t rec_bytes = rec_sz * (size_t)n + 16 * (size_t)k;
    CU(cudaMemcpyAsync(pinned.b(), rec, rec_bytes, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    const uint8_t* r = pinned.b();
    for (int i = 0; i < n; ++i) {
      std::memcpy(out + 16 * (size_t)i * k, r + rec_sz * (size_t)i, 16 * (size_t)k);
      std::memcpy(out + off_r + 16 * (size_t)i, r + rec_sz * (size_t)i + 16 * (size_t)k, 16);
    }
    std::memcpy(out + off_f, r + rec_sz * (size_t)n, 16 * (size_t)k);
    CU(cudaMemcpyAsync(pinned.b(), S, sizeof(img), cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    std::memcpy(&img, pinned.b(), sizeof(img));
    if (img.status != 0) return fail(BF_ERR_ARG, "transcript input outgrew the device buffer");
    ch.in.assign(img.tr.in, img.tr.in + img.tr.in_len);
    ch.out.assign(img.tr.out, img.tr.out + img.tr.out_len);
    std::memcpy(out + off_c, &img.outer, 16);
    return BF_OK;
  }
  // a long pending transcript: the rounds' transcript on the host
  CU(cudaMemsetAsync(acc, 0, 48, st));
  CU(bf::launch_prod_round_sums(in, k, half0, acc, st));
  CU(cudaMemcpyAsync(pinned.b(), acc, 48, cudaMemcpyDeviceToHost, st));
  CU(cudaStreamSynchronize(st));
  int ri = 0;
  for (int round = n - 1; round >= 0; --round, ++ri) {
    u128 c0 = bfh::load(pinned.b()), c2 = bfh::load(pinned.b() + 16), c3 = bfh::load(pinned.b() + 32);
    std::vector<u128> comp, rp;
    if (k == 2) {
      c0 = bfh::mul(c0, ONE);  // pair scalar ONE (quadratic.rs:118)
      c2 = bfh::mul(c2, ONE);
      comp = {c0, c2};
      rp = {c0, sc ^ c2, c2};  // Quadratic::decompress (quadratic.rs:68-79)
    } else {
      comp = {c0, c2, c3};
      rp = {c0, sc ^ c2 ^ c3, c2, c3};
    }
    for (size_t t = 0; t < comp.size(); ++t) {
      ch.observe_elem(comp[t]);
      bfh::store(out + 16 * ((size_t)ri * k + t), comp[t]);
    }
    const u128 x = ch.sample_elem();
    bfh::store(out + off_r + 16 * (size_t)ri, x);
    sc = horner(rp.data(), (int)rp.size(), x);
    const size_t half = (size_t)1 << round;
    if (round > 0) CU(cudaMemsetAsync(acc, 0, 48, st));
    const uint4* const* src = (round == n - 1) ? in : const_cast<const uint4* const*>(work);
    CU(bf::launch_prod_fix(work, src, k, half, to_uint4(x), half / 2, acc, st));
    if (round > 0) {
      CU(cudaMemcpyAsync(pinned.b(), acc, 48, cudaMemcpyDeviceToHost, st));
    } else {
      for (int j = 0; j < k; ++j) CU(cudaMemcpyAsync(pinned.b() + 16 * j, work[j], 16, cudaMemcpyDeviceToHost, st));
    }
    CU(cudaStreamSynchronize(st));
  }
  std::memcpy(out + off_f, pinned.b(), 16 * (size_t)k);
  bfh::store(out + off_c, sc);
  return BF_OK;
}

}  // namespace

extern "C" int bf_sumcheck_prove_device(bf_pcs* p, int k, int n, const void* d_polys, const uint8_t* claim,
                                        bf_challenger* ch, uint8_t* out) {
  if (!p || !d_polys || !claim || !ch || !out) return fail(BF_ERR_ARG, "null argument");
  if (p->device < 0) return fail(BF_ERR_ARG, "verifier-only pcs (device < 0)");
  if ((k != 2 && k != 3) || n < 0 || n > 30) return fail(BF_ERR_ARG, "k must be 2 or 3, 0 <= num_vars <= 30");
  DeviceGuard g(p->device);
  return sumcheck_run(p->stream, p->sc_ws, p->pinned, k, n, reinterpret_cast<const uint4*>(d_polys), claim, ch->c, out);
}

extern "C" int bf_sumcheck_prove(int device, int k, int n, const uint8_t* polys, const uint8_t* claim,
                                 bf_challenger* ch, uint8_t* out) {
  if (!polys || !claim || !ch || !out) return fail(BF_ERR_ARG, "null argument");
  if ((k != 2 && k != 3) || n < 0 || n > 30) return fail(BF_ERR_ARG, "k must be 2 or 3, 0 <= num_vars <= 30");
  CU(cudaSetDevice(device));
  DevBuf dp, scratch;
  PinnedBuf pinned;
  CU(pinned.ensure(4096));
  const size_t bytes = 16 * (size_t)k * ((size_t)1 << n);
  CU(dp.alloc(bytes));
  cudaStream_t st;
  CU(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() { cudaStreamDestroy(s); }
  } sg{st};
  CU(cudaMemcpyAsync(dp.p, polys, bytes, cudaMemcpyHostToDevice, st));
  return sumcheck_run(st, scratch, pinned, k, n, dp.as<uint4>(), claim, ch->c, out);
}
