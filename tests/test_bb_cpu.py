"""Prime-field C ABI without a GPU: the library's host verifier and its
BabyBear transcript sampling against the oracle (proofs made by the oracle,
checked by a verifier-only pcs), with the same rejection code for every
tampered byte tried."""
import numpy as np
import pytest

from oracle import oracle as O

P = O.BB_P


def rnd(shape, seed):
    return np.random.default_rng(seed).integers(0, P, size=shape, dtype=np.uint64).astype(np.uint32)


def _verifier(prime, n, log2_c):
    from basefold_gpu import BasefoldConfig

    return prime.BabyBearBasefold.setup(BasefoldConfig(prime.ReedSolomonCode(128, log2_c, n)), device=-1)


@pytest.mark.parametrize("n,log2_c,w", [(0, 1, 1), (1, 0, 1), (3, 1, 1), (6, 2, 1), (4, 1, 3), (5, 1, 34),
                                        (2, 2, 35), (7, 1, 2)])
def test_host_verifier_agrees_with_oracle(built_lib, n, log2_c, w):
    from basefold_gpu import prime

    bg = built_lib
    data = rnd((1 << n, w) if w > 1 else 1 << n, 11 + n + 7 * w)
    point = rnd((n, 5), 50 + n)
    root, values, blob = O.bb_harness_prepare(n, log2_c, data, point)
    proof = O.bb_open(n, log2_c, data, point, values, blob)
    pcs = _verifier(prime, n, log2_c)
    assert pcs.num_queries() == O.bb_num_queries(log2_c)
    assert pcs.proof_size(w, 1) == len(proof)
    ev = [prime.PrimePolyEvals(values, point)]
    pcs.verify(root, ev, proof, bg.GenericChallenger.from_state(blob))
    positions = [len(proof) - 3, len(proof) - 40, len(proof) // 2, 20, 9, len(proof) - 100]
    for pos in positions:
        if pos < 0 or pos >= len(proof):
            continue
        bad = bytearray(proof)
        bad[pos] ^= 0x40
        want = O.bb_verify(n, log2_c, root, point, values, blob, bytes(bad))
        if want == 0:  # a flip the oracle accepts (none expected); the library must agree
            pcs.verify(root, ev, bytes(bad), bg.GenericChallenger.from_state(blob))
            continue
        with pytest.raises(bg.BasefoldError) as e:
            pcs.verify(root, ev, bytes(bad), bg.GenericChallenger.from_state(blob))
        assert e.value.code == want, (pos, e.value.kind, want)
    wrong = np.array(values).reshape(-1, 5).copy()
    wrong[-1, 0] = (int(wrong[-1, 0]) + 1) % P
    want = O.bb_verify(n, log2_c, root, point, wrong, blob, proof)
    assert want != 0
    with pytest.raises(bg.BasefoldError) as e:
        pcs.verify(root, [prime.PrimePolyEvals(wrong, point)], proof, bg.GenericChallenger.from_state(blob))
    assert e.value.code == want


def test_empty_evals_default_proof(built_lib):
    from basefold_gpu import prime

    bg = built_lib
    pcs = _verifier(prime, 3, 1)
    assert pcs.proof_size(1, 0) == 32
    pcs.verify(b"\0" * 32, [], b"", bg.GenericChallenger.keccak256())  # basefold.rs:241-243


def test_sample_ext_element_matches_byte_rule(built_lib):
    """Sampling E from the byte transcript (challenger.rs:62-74 with
    from_uniform_bytes.rs:37-45): 4 popped bytes little-endian, shifted right
    by one, rejected while >= p, five times.  Restated here over the state
    blob: pop the last output byte; when the output is empty, hash the input
    with keccak256 and make the digest both input and output."""
    from basefold_gpu import prime

    bg = built_lib
    ch = bg.GenericChallenger.keccak256()
    ch.observe(b"prime-field transcript")
    blob = ch.state()
    li = int.from_bytes(blob[:8], "little")
    inp = blob[8:8 + li]
    lo = int.from_bytes(blob[8 + li:16 + li], "little")
    out = list(blob[16 + li:16 + li + lo])

    def byte():
        nonlocal inp, out
        if not out:
            dg = O.keccak256(bytes(inp))
            inp, out = dg, list(dg)
        return out.pop()

    for _ in range(60):
        exp = []
        while len(exp) < 5:
            v = int.from_bytes(bytes(byte() for _ in range(4)), "little") >> 1
            if v < P:
                exp.append(v)
        assert prime.sample_ext_element(ch).tolist() == exp


def test_prime_entry_points_refuse_verifier_only_object(built_lib):
    from basefold_gpu import prime

    bg = built_lib
    pcs = _verifier(prime, 4, 1)
    with pytest.raises(bg.BasefoldGpuError) as e:
        pcs.commit(rnd(16, 1))
    assert e.value.code == -1
    with pytest.raises(bg.BasefoldGpuError):
        prime.BabyBearBasefold.setup(bg.BasefoldConfig(prime.ReedSolomonCode(128, 2, 26)), device=-1)


@pytest.mark.parametrize("n,log2_c,log2_k0,w", [(0, 1, 0, 1), (1, 1, 1, 1), (3, 0, 1, 1), (4, 2, 2, 1), (6, 1, 2, 3),
                                                (7, 2, 1, 9), (9, 1, 0, 1), (5, 1, 3, 2)])
def test_host_verifier_generic_code_agrees_with_oracle(built_lib, n, log2_c, log2_k0, w):
    """GenericRandomFoldableCode (generic.rs) with the reference test's
    ranges (log2_c 0..3, log2_k_0 0..3 capped at num_vars, basefold.rs:
    453-468): the library's query count and verifier against the oracle."""
    from basefold_gpu import BasefoldConfig, prime

    bg = built_lib
    ts = O.bb_random_ts(n, log2_c, log2_k0, 31 + n)
    kw = dict(log2_k0=log2_k0, ts=ts)
    data = rnd((1 << n, w) if w > 1 else 1 << n, 41 + n + w)
    point = rnd((n, 5), 51 + n)
    root, values, blob = O.bb_harness_prepare(n, log2_c, data, point, **kw)
    proof = O.bb_open(n, log2_c, data, point, values, blob, **kw)
    code = prime.GenericRandomFoldableCode(128, log2_c, log2_k0, n - log2_k0, ts)
    pcs = prime.BabyBearBasefold.setup(BasefoldConfig(code), device=-1)
    assert pcs.num_queries() == O.bb_num_queries(log2_c, n=n, log2_k0=log2_k0, generic=True)
    assert pcs.proof_size(w, 1) == len(proof)
    ev = [prime.PrimePolyEvals(values, point)]
    pcs.verify(root, ev, proof, bg.GenericChallenger.from_state(blob))
    for pos in (len(proof) - 3, len(proof) // 2, 20, len(proof) - 30):
        if not 0 <= pos < len(proof):
            continue
        bad = bytearray(proof)
        bad[pos] ^= 0x10
        want = O.bb_verify(n, log2_c, root, point, values, blob, bytes(bad), **kw)
        if want == 0:
            pcs.verify(root, ev, bytes(bad), bg.GenericChallenger.from_state(blob))
            continue
        with pytest.raises(bg.BasefoldError) as e:
            pcs.verify(root, ev, bytes(bad), bg.GenericChallenger.from_state(blob))
        assert e.value.code == want, (pos, e.value.kind, want)


def test_generic_setup_validates_ts(built_lib):
    from basefold_gpu import BasefoldConfig, prime

    bg = built_lib
    ts = O.bb_random_ts(4, 1, 1, 3)
    bad = ts.copy()
    bad[5] = 0
    with pytest.raises(bg.BasefoldGpuError):
        prime.BabyBearBasefold.setup(BasefoldConfig(prime.GenericRandomFoldableCode(128, 1, 1, 3, bad)), device=-1)
    with pytest.raises(bg.BasefoldGpuError):
        prime.BabyBearBasefold.setup(BasefoldConfig(prime.GenericRandomFoldableCode(128, 1, 1, 3, ts[:-1])), device=-1)
