"""The prime-field oracle (BabyBear, quintic extension, Reed–Solomon code)
against definitions: field axioms and inverses, the DFT against its
definition, the code's folding identity, and prove -> verify over the
reference's harness with tampered proofs rejected (the reference's own tests
for this path are prove/verify round trips, poly-commit/src/basefold.rs:
470-478)."""
import numpy as np
import pytest

from oracle import oracle as O

P = O.BB_P


def rnd(shape, seed):
    return np.random.default_rng(seed).integers(0, P, size=shape, dtype=np.uint64).astype(np.uint32)


def test_field_constants():
    assert pow(31, 15, P) == 0x1A427A41  # the two-adic generator
    g = 0x1A427A41
    assert pow(g, 1 << 26, P) == P - 1 and pow(g, 1 << 27, P) == 1
    assert pow(2, (P - 1) // 5, P) != 1  # X^5 - 2 is irreducible


def test_extension_inverse_and_product():
    a, b, c = rnd((200, 5), 1), rnd((200, 5), 2), rnd((200, 5), 3)
    one = np.zeros((200, 5), np.uint32)
    one[:, 0] = 1
    assert np.array_equal(O.bb_emul(a, O.bb_einv(a)), one)
    assert np.array_equal(O.bb_emul(O.bb_emul(a, b), c), O.bb_emul(a, O.bb_emul(b, c)))
    assert np.array_equal(O.bb_emul(a, b), O.bb_emul(b, a))
    # X^5 = 2
    x = np.zeros((1, 5), np.uint32)
    x[0, 1] = 1
    x5 = O.bb_emul(O.bb_emul(O.bb_emul(O.bb_emul(x, x), x), x), x)
    assert x5.tolist() == [[2, 0, 0, 0, 0]]


@pytest.mark.parametrize("log_n", [0, 1, 3, 6, 9])
def test_dft_matches_definition(log_n):
    a = rnd(1 << log_n, 10 + log_n)
    assert np.array_equal(O.bb_dft(log_n, a), O.bb_dft(log_n, a, definition=True))


def test_num_queries():
    # delta = 1 - (1 - 1/c) / 3 (reed_solomon.rs:58-64)
    import math
    for log2_c in (1, 2, 3):
        c = 1 << log2_c
        assert O.bb_num_queries(log2_c) == math.ceil(128 / -math.log2(1 - (1 - 1 / c) / 3))


@pytest.mark.parametrize("n,log2_c", [(0, 1), (1, 1), (4, 1), (6, 2), (8, 1), (9, 3)])
def test_prove_verify_round_trip(n, log2_c):
    data = rnd(1 << n, 100 + n)
    point = rnd((n, 5), 200 + n)
    root, value, blob = O.bb_harness_prepare(n, log2_c, data, point)
    assert root == O.bb_commit(n, log2_c, data)
    assert np.array_equal(value, O.bb_eval(n, data, point))
    proof = O.bb_open(n, log2_c, data, point, value, blob)
    assert O.bb_verify(n, log2_c, root, point, value, blob, proof) == 0
    if n == 0:
        return
    bad_value = value.copy()
    bad_value[0] = (int(bad_value[0]) + 1) % P
    assert O.bb_verify(n, log2_c, root, point, bad_value, blob, proof) != 0
    for pos in (30, len(proof) // 2, len(proof) - 3):
        b = bytearray(proof)
        b[pos] ^= 1
        assert O.bb_verify(n, log2_c, root, point, value, blob, bytes(b)) != 0, pos


def test_encode_is_columnwise_and_folds():
    """encode_batch codes each column; folding the codeword of m with r gives
    the codeword of the half-size message m_lo + r (m_hi - m_lo) (code.rs:
    66-84 against reed_solomon.rs:71-75), shown here on the base field."""
    n, log2_c, w = 5, 1, 3
    data = rnd((1 << n, w), 7)
    cw = O.bb_encode(n, log2_c, data)
    for c in range(w):
        assert np.array_equal(cw[:, c], O.bb_encode(n, log2_c, data[:, c]))


@pytest.mark.parametrize("n,log2_c,w", [(0, 1, 3), (3, 1, 2), (5, 1, 4), (6, 2, 5), (4, 1, 16)])
def test_prove_verify_round_trip_width(n, log2_c, w):
    data = rnd((1 << n, w), 300 + n + w)
    point = rnd((n, 5), 400 + n)
    root, values, blob = O.bb_harness_prepare(n, log2_c, data, point)
    assert root == O.bb_commit(n, log2_c, data)
    assert values.shape == (w, 5)
    for c in range(w):
        assert np.array_equal(values[c], O.bb_eval(n, data[:, c], point))
    proof = O.bb_open(n, log2_c, data, point, values, blob)
    assert O.bb_verify(n, log2_c, root, point, values, blob, proof) == 0
    bad = values.copy()
    bad[w - 1, 2] = (int(bad[w - 1, 2]) + 1) % P
    assert O.bb_verify(n, log2_c, root, point, bad, blob, proof) != 0
    b = bytearray(proof)
    b[len(proof) - 40] ^= 4
    assert O.bb_verify(n, log2_c, root, point, values, blob, bytes(b)) != 0


# ---- GenericRandomFoldableCode (generic.rs) ---------------------------------

def _z_c(lam, log2_f, c, i, log2_n_i):
    if i == 0:
        return 1.0 / c
    return (_z_c(lam, log2_f, c, i - 1, log2_n_i - 1) * (log2_f / (log2_f - 1.001))
            + 1.0 / (log2_f - 1.001) * ((2.0 * (log2_n_i - 1) + lam) / float(1 << log2_n_i) + 0.6))


def _generic_queries(lam, n, log2_c, log2_k0):
    import math
    d = n - log2_k0
    rel = 1.0 - _z_c(float(lam), 31.0, 1 << log2_c, d, log2_c + log2_k0 + d)
    delta = 1.0 - rel / 3.0
    try:
        q = math.ceil(lam / -math.log2(delta))
    except (ValueError, ZeroDivisionError, OverflowError):
        return 0
    return max(q, 0)


def test_generic_num_queries():
    """generic.rs:24-39 and :99-103 with F::bits() = 31."""
    for n in range(0, 12):
        for log2_c in range(0, 4):
            for log2_k0 in range(0, min(n, 3) + 1):
                got = O.bb_num_queries(log2_c, n=n, log2_k0=log2_k0, generic=True)
                assert got == _generic_queries(128, n, log2_c, log2_k0), (n, log2_c, log2_k0)


def test_generic_encode_definition():
    """generic.rs:112-141 on one column: G_0 rows are powers of the row index,
    then the butterflies (l + t r, l - t r) of ts[i-1], i = 1..d."""
    n, log2_c, log2_k0 = 4, 1, 2
    d, k0, n0 = n - log2_k0, 1 << log2_k0, (1 << log2_c) << log2_k0
    m = [int(v) for v in rnd(1 << n, 3)]
    ts = O.bb_random_ts(n, log2_c, log2_k0, 4)
    w = []
    for b in range(1 << d):
        for i in range(n0):
            w.append(sum(pow(i, j, P) * m[b * k0 + j] for j in range(k0)) % P)
    off = 0
    for i in range(1, d + 1):
        ni, t = n0 << i, [int(v) for v in ts[off:off + (n0 << (i - 1))]]
        off += n0 << (i - 1)
        for base in range(0, len(w), ni):
            for k in range(ni // 2):
                l, r = w[base + k], w[base + ni // 2 + k] * t[k] % P
                w[base + k], w[base + ni // 2 + k] = (l + r) % P, (l - r) % P
    assert O.bb_encode(n, log2_c, np.array(m, np.uint32), log2_k0=log2_k0, ts=ts).tolist() == w


@pytest.mark.parametrize("n,log2_c,log2_k0,w", [(0, 0, 0, 1), (1, 1, 1, 1), (3, 1, 0, 1), (4, 2, 2, 1), (5, 0, 1, 2),
                                                (6, 1, 2, 3), (7, 2, 1, 9), (9, 1, 2, 1), (2, 2, 2, 5), (8, 1, 0, 34)])
def test_generic_prove_verify_round_trip(n, log2_c, log2_k0, w):
    ts = O.bb_random_ts(n, log2_c, log2_k0, 500 + n)
    data = rnd((1 << n, w) if w > 1 else 1 << n, 600 + n + w)
    point = rnd((n, 5), 700 + n)
    kw = dict(log2_k0=log2_k0, ts=ts)
    root, values, blob = O.bb_harness_prepare(n, log2_c, data, point, **kw)
    assert root == O.bb_commit(n, log2_c, data, **kw)
    proof = O.bb_open(n, log2_c, data, point, values, blob, **kw)
    assert O.bb_verify(n, log2_c, root, point, values, blob, proof, **kw) == 0
    bad = np.asarray(values).reshape(-1, 5).copy()
    bad[0, 1] = (int(bad[0, 1]) + 1) % P
    assert O.bb_verify(n, log2_c, root, point, bad, blob, proof, **kw) != 0
    if O.bb_num_queries(log2_c, n=n, log2_k0=log2_k0, generic=True):
        b = bytearray(proof)
        b[len(proof) - 50] ^= 2
        assert O.bb_verify(n, log2_c, root, point, values, blob, bytes(b), **kw) != 0
    # another draw of the t's is another code: the proof does not carry over
    if n > log2_k0:
        ts2 = O.bb_random_ts(n, log2_c, log2_k0, 900 + n)
        assert O.bb_commit(n, log2_c, data, log2_k0=log2_k0, ts=ts2) != root
