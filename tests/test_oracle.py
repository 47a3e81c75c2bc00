"""The oracle against everything that pins it (CPU only).

The reference keeps no golden vectors, so the oracle is pinned by
  * constants read out of the reference's sources (tests/golden/reference_polyval.json);
  * the RFC 8452 POLYVAL known-answer vector and the Keccak-256("") KAT;
  * SHA3-256 from Python's hashlib (same Keccak-f[1600], different padding);
  * the reference's own definitional NTT test (p3/src/field/binary.rs:194-217)
    and field-axiom test (p3/src/polyval.rs:265-295), and the brute-force
    multilinear evaluation of its multilinear tests (multilinear.rs:312-379);
  * the reference's prove->verify harness (poly-commit/src/lib.rs:64-105,
    sumcheck/src/lib.rs:160-182);
and the committed oracle vectors guard it against regressions.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from basefold_gpu import rand

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
ONE = 0xC2000000000000000000000000000001


def ints(a):
    return [O.to_int(x) for x in a]


def test_montgomery_constants_match_reference_source():
    ref = json.load(open(os.path.join(GOLDEN, "reference_polyval.json")))
    one, r2 = O.field_consts()
    assert one == ONE  # Polyval::ONE = from_canonical(1) (polyval.rs:85)
    assert r2 == int(ref["r2"], 16)  # portable.rs:12


def test_nibble_table_matches_reference_source():
    """value[i][k][j] = from_canonical(j << 4k) ^ (2^(2<<i)) (portable.rs:169-376)."""
    ref = json.load(open(os.path.join(GOLDEN, "reference_polyval.json")))
    for i_str, rows in ref["table_rows"].items():
        i = int(i_str)
        inputs = [j << (4 * k) for k in range(32) for j in range(16)]
        v = O.from_canonical(O.from_ints(inputs))
        for _ in range(2 << i):  # exp_power_of_2(2 << i): square 2<<i times
            v = O.gf_mul(v, v)
        got = ints(v)
        want = [int(rows[k][j], 16) for k in range(32) for j in range(16)]
        assert got == want, f"row i={i}"


def test_rfc8452_polyval_vector():
    # RFC 8452 Appendix A: POLYVAL(H, X_1, X_2)
    h = bytes.fromhex("25629347589242761d31f826ba4b757b")
    xs = bytes.fromhex("4f4f95668c83dfb6401762bb2d01a262d1a24ddd2721d006bbe45f20d3c9f362")
    assert O.polyval_rfc(h, xs).hex() == "f7a3b47b846119fae5b7866cf5e5b77e"


def test_keccak256_kat_and_sha3_permutation():
    assert O.keccak256(b"").hex() == "c5d2460186f7233c927e7db2dcc703c0e500b653ca82273b7bfad8045d85a470"
    for m in [b"", b"abc", bytes(range(135)), bytes(136), bytes(range(256)) * 3]:
        assert O.sha3_256(m) == hashlib.sha3_256(m).digest()


def test_keccak_constants_from_spec():
    rc, rho = O.keccak_consts()
    assert int(rc[0]) == 1 and int(rc[23]) == 0x8000000080008008
    assert list(map(int, rho))[:5] == [0, 1, 62, 28, 27]


def test_field_axioms_and_inverse():
    """polyval.rs:265-295 plus inverse/div."""
    a, b, c = (rand.random_elems(500, s) for s in (1, 2, 3))
    mul = O.gf_mul
    assert np.array_equal(mul(a, b), mul(b, a))
    assert np.array_equal(mul(a, mul(b, c)), mul(mul(a, b), c))
    assert np.array_equal(mul(a, b ^ c), mul(a, b) ^ mul(a, c))
    one = O.from_ints([ONE] * 500)
    assert np.array_equal(mul(a, one), a)
    assert not mul(a, np.zeros_like(a)).any()
    assert np.array_equal(mul(a, b), O.gf_mul(a, b, definition=True))
    inv = O.gf_inv(a[:50])
    assert ints(mul(a[:50], inv)) == [ONE] * 50
    assert not O.gf_inv(np.zeros((1, 16), np.uint8)).any()  # invert_or_zero


@pytest.mark.parametrize("log_n", range(0, 10))
def test_ntt_matches_definition(log_n):
    """binary.rs:194-203"""
    d = rand.random_elems(1 << log_n, 100 + log_n)
    assert np.array_equal(O.ntt_forward(log_n, d), O.ntt_forward_definition(log_n, d))


def test_ntt_round_trip():
    """binary.rs:205-217"""
    for log_n in range(0, 10):
        for width in (1, 3, 9):
            a = rand.random_elems(width << log_n, 7 * log_n + width)
            assert np.array_equal(O.ntt_backward(log_n, O.ntt_forward(log_n, a, width), width), a)


@pytest.mark.parametrize("n", [0, 1, 3, 7])
def test_evaluate_matches_definition(n):
    """MultiPoly::evaluate (p3/src/poly/multilinear.rs:124-141) against the
    definition of the multilinear extension, as the reference's brute-force
    tests do (multilinear.rs:312-379): f(p) = sum_b f(b) prod_i w_i(b) with
    w_i = p_i when bit i of b is set, else 1 + p_i (characteristic 2)."""
    data = rand.random_elems((1 << n) + n, 900 + n)
    f, point = data[: 1 << n], data[1 << n:]
    one = O.from_ints([ONE])[0]
    w = np.tile(one, (1 << n, 1))
    for i in range(n):
        bit = ((np.arange(1 << n) >> i) & 1).astype(bool)
        factor = np.where(bit[:, None], point[i], point[i] ^ one)
        w = O.gf_mul(w, factor)
    terms = O.gf_mul(w, f)
    want = np.bitwise_xor.reduce(terms, axis=0) if n else f[0]
    assert np.array_equal(O.eval_poly(n, f, point)[0], want)


def test_num_queries():
    """binary_reed_solomon.rs:56-59; c = 1 degenerates to zero queries."""
    assert [O.num_queries(c) for c in range(4)] == [0, 309, 189, 155]


@pytest.mark.parametrize("log2_c", [0, 1, 2])
def test_basefold_round_trip(log2_c):
    """basefold.rs:480-490 through the harness of poly-commit/src/lib.rs:64-105."""
    for n in range(0, 10):
        for width in (1, 2, 5):
            data = rand.random_elems((width << n) + n, 1000 * log2_c + 10 * n + width)
            evals, point = data[: width << n], data[width << n:]
            root, values, blob = O.harness_prepare(n, log2_c, evals, point, width)
            proof = O.open_proof(n, log2_c, evals, point, values, blob, width)
            assert O.verify(n, log2_c, root, point, values, blob, proof, width) == 0
            if O.num_queries(log2_c):
                bad = bytearray(proof)
                bad[-5] ^= 0x10
                assert O.verify(n, log2_c, root, point, values, blob, bytes(bad), width) != 0


def test_basefold_empty_evals():
    d = rand.random_elems(16, 5)
    proof = O.open_proof(4, 1, d, None, None, O.challenger_blob(), n_evals=0)
    assert proof == bytes(32)


@pytest.mark.parametrize("k", [2, 3])
def test_sumcheck_identity(k):
    """sumcheck/src/lib.rs:160-182: verifier accepts, final subclaim = prod f_j(r)."""
    for n in range(0, 9):
        polys = rand.random_elems(k << n, 50 * k + n)
        P = polys.reshape(k, 1 << n, 16)
        prod = P[0]
        for j in range(1, k):
            prod = O.gf_mul(prod, P[j])
        claim = np.bitwise_xor.reduce(prod, axis=0)
        blob = O.challenger_blob(bytes(range(32)))
        rp, r, fe, fc = O.sumcheck_prove(k, n, polys, claim, blob)
        assert O.sumcheck_verify(k, n, claim, rp, fe, blob) == 0


def test_oracle_regression_vectors():
    vec = json.load(open(os.path.join(GOLDEN, "oracle_vectors.json")))
    for case in vec["basefold"]:
        n, log2_c, w, seed = case["n"], case["log2_c"], case["width"], case["seed"]
        if n > 12:
            continue
        data = rand.random_elems((w << n) + n, seed)
        evals, point = data[: w << n], data[w << n:]
        root, values, blob = O.harness_prepare(n, log2_c, evals, point, w)
        assert root.hex() == case["root"]
        proof = O.open_proof(n, log2_c, evals, point, values, blob, w)
        assert hashlib.sha256(proof).hexdigest() == case["proof_sha256"]
    for case in vec["sumcheck"]:
        k, n, seed = case["k"], case["n"], case["seed"]
        rp, r, fe, fc = O.sumcheck_prove(k, n, rand.random_elems(k << n, seed), rand.random_elems(1, seed + 1000),
                                         O.challenger_blob(bytes.fromhex(case["initial_state"])))
        assert hashlib.sha256(rp.tobytes()).hexdigest() == case["round_polys_sha256"]
        assert [bytes(v).hex() for v in fe] == case["final_evals"]
