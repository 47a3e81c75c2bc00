"""The headline sizes, checked bit for bit against the oracle:

* a 2^24-evaluation proof identical to the oracle's and accepted by both
  verifiers;
* the encode + Merkle commit sweep (2^18 .. 2^26 evaluations, blowup 2 and
  4): every root equal to the oracle's (the 2^26 roots through the oracle's
  bounded-memory root, which hashes the codeword in subtrees);
* the product sumcheck of 2 and 3 polynomials at 2^20 and 2^24 points: every
  compressed round polynomial, every challenge, the final evaluations and the
  final claim equal to the oracle's, plus the verifier identity and the final
  evaluations against direct multilinear evaluation at the challenges.
* the prime-field scheme at the reference's largest prime bench shape (2^19
  rows x 256 BabyBear columns, blowup 2), both prime codes: root, column values
  and proof bytes equal to the oracle's.

Tolerance: bit-exact (exact GF(2^128) and Keccak arithmetic)."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from basefold_gpu import rand

pytestmark = pytest.mark.gpu
ONE = 0xC2000000000000000000000000000001


def test_proof_2_24_matches_oracle_and_verifies(built_lib):
    bg = built_lib
    n, log2_c = 24, 1
    data = rand.random_elems((1 << n) + n, 24)
    evals, point = data[: 1 << n], data[1 << n:]
    pcs = bg.Basefold.setup(bg.BasefoldConfig(bg.BinaryReedSolomonCode(128, log2_c, n)))
    comm = pcs.commit(evals)
    ch = bg.GenericChallenger.keccak256()
    ch.observe(comm.root)
    values = pcs.eval(pcs.data(comm), point)
    ch.observe_ext_slice(values)
    blob = ch.state()
    proof = pcs.open(comm, [bg.PolyEvals(values, point)], ch.clone())
    root_o, values_o, blob_o = O.harness_prepare(n, log2_c, evals, point)
    assert comm.root == root_o and np.array_equal(values, values_o) and blob == blob_o
    assert proof == O.open_proof(n, log2_c, evals, point, values_o, blob_o)
    pcs.verify(comm.root, [bg.PolyEvals(values, point)], proof, ch.clone())
    assert O.verify(n, log2_c, comm.root, point, values, blob, proof) == 0


def _host_mem_available_gb():
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) / 2**20
    except OSError:
        pass
    return None


# (num_vars, log2 blowup): every point of the encode + Merkle commit sweep
SWEEP = [(n, c) for c in (1, 2) for n in (18, 20, 22, 24, 26)]


@pytest.mark.parametrize("n,log2_c", SWEEP, ids=[f"2^{n}-c{1 << c}" for n, c in SWEEP])
def test_commit_sweep_root_matches_oracle(built_lib, n, log2_c):
    bg = built_lib
    if n + log2_c >= 27:
        # the oracle's bounded-memory root holds the codeword (16 B x 2^(n+c))
        # and its twiddle tables (same size) on the host
        need = 3 * (16 << (n + log2_c)) / 2**30
        avail = _host_mem_available_gb()
        if avail is not None and avail < need + 8:
            pytest.skip(f"host memory: {avail:.0f} GB available, {need + 8:.0f} GB needed")
    evals = rand.random_elems(1 << n, 1800 + 10 * n + log2_c)
    pcs = bg.Basefold.setup(bg.BasefoldConfig(bg.BinaryReedSolomonCode(128, log2_c, n)))
    comm = pcs.commit(evals)
    root = comm.root
    comm.free()
    del pcs
    O.set_threads(os.cpu_count() or 1)
    assert root == O.commit_root(n, log2_c, evals)


@pytest.mark.parametrize("k,n", [(2, 20), (3, 20), (2, 24), (3, 24)])
def test_product_sumcheck_full_size(built_lib, k, n):
    bg = built_lib
    polys = rand.random_elems(k << n, 7700 + 10 * k + n)
    P = polys.reshape(k, 1 << n, 16)
    prod = P[0]
    for j in range(1, k):
        prod = O.gf_mul(prod, P[j])
    claim = np.bitwise_xor.reduce(prod, axis=0)[None]
    init = b"full size"
    rp, r, fe, fc = bg.prove_sumcheck(k, polys, claim, bg.GenericChallenger(init))
    O.set_threads(os.cpu_count() or 1)
    rp_o, r_o, fe_o, fc_o = O.sumcheck_prove(k, n, polys, claim, O.challenger_blob(init))
    assert np.array_equal(rp, rp_o), "round polynomials differ from the oracle"
    assert np.array_equal(r, r_o), "challenges differ from the oracle"
    assert np.array_equal(fe, fe_o) and np.array_equal(fc, fc_o), "final evaluations / claim differ"
    assert O.sumcheck_verify(k, n, claim, rp, fe, O.challenger_blob(init)) == 0
    # fix_last_var takes the top variable first: the point is the challenges reversed
    point = r[::-1].copy()
    for j in range(k):
        assert np.array_equal(fe[j], O.eval_poly(n, P[j].copy(), point)[0]), j


def test_proof_2_26_blowup_4_verifies(built_lib):
    """The largest commit of the encode/commit sweep (2^26 evaluations,
    blowup 4: a 2^28-entry codeword): same root twice, and a full proof whose
    189 query paths through every tree the host verifier accepts."""
    bg = built_lib
    torch = pytest.importorskip("torch")
    n, log2_c = 26, 2
    data = rand.random_elems((1 << n) + n, 2626)
    evals, point = data[: 1 << n], data[1 << n:]
    dev = torch.from_numpy(evals).cuda()
    pcs = bg.Basefold.setup(bg.BasefoldConfig(bg.BinaryReedSolomonCode(128, log2_c, n)))
    first = pcs.commit_device(dev.data_ptr(), keep=dev)
    root0 = first.root
    first.free()
    comm = pcs.commit_device(dev.data_ptr(), keep=dev)
    assert comm.root == root0
    ch = bg.GenericChallenger.keccak256()
    ch.observe(comm.root)
    values = pcs.eval(pcs.data(comm), point)
    ch.observe_ext_slice(values)
    proof = pcs.open(comm, [bg.PolyEvals(values, point)], ch.clone())
    pcs.verify(comm.root, [bg.PolyEvals(values, point)], proof, ch.clone())
    bad = bytearray(proof)
    bad[-5] ^= 1
    with pytest.raises(bg.BasefoldError):
        pcs.verify(comm.root, [bg.PolyEvals(values, point)], bytes(bad), ch.clone())
    comm.free()


@pytest.mark.parametrize("generic", [0, 1])
def test_prime_bench_shape_2_19_x_256_matches_oracle(built_lib, generic):
    """The reference's largest prime bench shape (poly-commit/benches/poly-commit.rs:83-178:
    log_n 19, 2^8 columns, C = 1): Reed–Solomon and the generic code with log2_k_0 = 3.
    Root, the 256 column values and the whole proof byte-for-byte against the oracle (on all
    host threads), and the proof accepted by the library's verifier."""
    import torch
    from basefold_gpu import BasefoldConfig, GenericChallenger, prime

    n, log2_c, w = 19, 1, 256
    O.set_threads(os.cpu_count() or 1)
    rng = np.random.default_rng(1900 + generic)
    data = rng.integers(0, O.BB_P, size=(1 << n, w), dtype=np.uint64).astype(np.uint32)
    point = rng.integers(0, O.BB_P, size=(n, 5), dtype=np.uint64).astype(np.uint32)
    kw = {}
    if generic:
        lk = 3
        ts = O.bb_random_ts(n, log2_c, lk, 77)
        kw = dict(log2_k0=lk, ts=ts)
        code = prime.GenericRandomFoldableCode(128, log2_c, lk, n - lk, ts)
    else:
        code = prime.ReedSolomonCode(128, log2_c, n)
    pcs = prime.BabyBearBasefold.setup(BasefoldConfig(code), device=0)
    dev = torch.from_numpy(data.view(np.int32)).cuda()
    comm = pcs.commit_device(dev.data_ptr(), w, keep=dev)
    root, values, blob = O.bb_harness_prepare(n, log2_c, data, point, **kw)
    assert comm.root == root
    # from host memory: copied in slices, the stages inside a slice run per slice
    host_comm = pcs.commit(data)
    assert host_comm.root == root
    host_comm.free()
    got = pcs.eval(comm, point)
    assert np.array_equal(got, values)
    ev = [prime.PrimePolyEvals(got, point)]
    proof = pcs.open(comm, ev, GenericChallenger.from_state(blob))
    assert proof == O.bb_open(n, log2_c, data, point, values, blob, **kw)
    pcs.verify(root, ev, proof, GenericChallenger.from_state(blob))
