"""Batched verify on the GPU (bf_verify_batch) against the oracle's verifier
and the host verifier: the same result code for every proof, valid or
tampered, and the same transcript state afterwards (codes are integers, so
the comparison is exact)."""
import numpy as np
import pytest

from oracle import oracle as O
from basefold_gpu import rand

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bg(built_lib):
    return built_lib


def setup_pcs(bg, n, log2_c):
    return bg.Basefold.setup(bg.BasefoldConfig(bg.BinaryReedSolomonCode(128, log2_c, n)), device=0)


def make_proofs(bg, pcs, n, count, width, seed):
    """The reference harness (poly-commit/src/lib.rs:64-105) `count` times:
    commit, observe the root, evaluate, observe the values, open."""
    out = []
    for j in range(count):
        data = rand.random_elems((width << n) + n, seed + j)
        evals, point = data[: width << n], data[width << n:]
        comm = pcs.commit(evals, width=width)
        ch = bg.GenericChallenger.keccak256()
        ch.observe(comm.root)
        values = pcs.eval(pcs.data(comm), point)
        ch.observe_ext_slice(values)
        proof = pcs.open(comm, [bg.PolyEvals(values, point)], ch.clone())
        out.append((comm.root, values, point, ch.state(), proof))
        comm.free()
    return out


def host_code(bg, pcs, root, values, point, blob, proof):
    ch = bg.GenericChallenger.from_state(blob)
    try:
        pcs.verify(root, [bg.PolyEvals(values, point)], proof, ch)
        return 0, ch.state()
    except bg.BasefoldError as e:
        return e.code, ch.state()


@pytest.mark.parametrize("log2_c", [0, 1, 2])
def test_valid_proofs_verify_with_host_transcript(bg, log2_c):
    for n in (0, 1, 2, 5, 9):
        pcs = setup_pcs(bg, n, log2_c)
        items = make_proofs(bg, pcs, n, 5, 1, 7000 + 31 * n + log2_c)
        chs = [bg.GenericChallenger.from_state(it[3]) for it in items]
        res = pcs.verify_batch([(r, [bg.PolyEvals(v, p)], pf, c) for (r, v, p, _, pf), c in zip(items, chs)])
        assert res == [0] * len(items), (n, log2_c, res)
        for (r, v, p, blob, pf), c in zip(items, chs):
            code, state = host_code(bg, pcs, r, v, p, blob, pf)
            assert code == 0 and c.state() == state


@pytest.mark.parametrize("log2_c", [1, 2])
def test_tampered_proofs_match_oracle(bg, log2_c):
    """Single-bit flips across every field of the proof (lengths, round
    polynomials, final polynomial, folded-codeword roots, opened rows, sibling
    elements and every kind of path digest), truncations and extensions, one
    batch: each code is the oracle's."""
    n = 6
    pcs = setup_pcs(bg, n, log2_c)
    root, values, point, blob, proof = make_proofs(bg, pcs, n, 1, 1, 8100 + log2_c)[0]
    step = max(1, len(proof) // 600)
    positions = sorted(set(list(range(0, 600, 5)) + list(range(600, len(proof), step)) + [len(proof) - 1]))
    variants = []
    for pos in positions:
        bad = bytearray(proof)
        bad[pos] ^= 1 << (pos % 8)
        variants.append(bytes(bad))
    variants += [proof[:-1], proof + b"\0", proof[: len(proof) // 2], b"", proof]
    chs = [bg.GenericChallenger.from_state(blob) for _ in variants]
    res = pcs.verify_batch([(root, [bg.PolyEvals(values, point)], v, c) for v, c in zip(variants, chs)])
    seen = set()
    for v, r, c in zip(variants, res, chs):
        want = O.verify(n, log2_c, root, point, values, blob, v)
        assert r == want, (log2_c, len(v), r, want)
        code, state = host_code(bg, pcs, root, values, point, blob, v)
        assert code == want and c.state() == state
        seen.add(r)
    # ok, InvalidFinalPoly, Mmcs and malformed all occur; InvalidQuery needs
    # Merkle paths that all verify around a broken fold chain, which no bit
    # flip of an honest proof gives (valid proofs check the chain: any error
    # in it would turn them into InvalidQuery)
    assert {0, 1, 3, 4} <= seen, seen


def test_wrong_claims_and_roots(bg):
    n, log2_c = 8, 1
    pcs = setup_pcs(bg, n, log2_c)
    items = make_proofs(bg, pcs, n, 4, 1, 8300)
    jobs, wants = [], []
    for j, (root, values, point, blob, proof) in enumerate(items):
        v2 = values.copy()
        r2 = bytearray(root)
        if j % 2:
            v2[0, 3] ^= 0x10
        else:
            r2[5] ^= 1
        jobs.append((bytes(r2), [bg.PolyEvals(v2, point)], proof, bg.GenericChallenger.from_state(blob)))
        wants.append(O.verify(n, log2_c, bytes(r2), point, v2, blob, proof))
        jobs.append((root, [bg.PolyEvals(values, point)], proof, bg.GenericChallenger.from_state(blob)))
        wants.append(0)
    res = pcs.verify_batch(jobs)
    assert res == wants and all(w != 0 for w in wants[::2])


@pytest.mark.parametrize("width", [2, 3, 9, 20])
def test_multi_column_rows(bg, width):
    """Rows of several columns: the eq-scalar combination of the opened row
    (basefold.rs:166-183, 283) and leaves longer than one Keccak block
    (20 columns = 320 bytes)."""
    n, log2_c = 5, 1
    pcs = setup_pcs(bg, n, log2_c)
    items = make_proofs(bg, pcs, n, 3, width, 8500 + width)
    jobs, wants = [], []
    for root, values, point, blob, proof in items:
        for pos in (None, 30, len(proof) // 3, len(proof) - 50):
            pf = proof
            if pos is not None:
                bad = bytearray(proof)
                bad[pos] ^= 4
                pf = bytes(bad)
            jobs.append((root, [bg.PolyEvals(values, point)], pf, bg.GenericChallenger.from_state(blob)))
            wants.append(O.verify(n, log2_c, root, point, values, blob, pf, width))
    assert pcs.verify_batch(jobs) == wants
    assert wants[0] == 0


def test_large_batch(bg):
    """Sixteen 2^16 proofs and four 2^20 proofs, one of each tampered in a deep path digest."""
    for n, count in ((16, 16), (20, 4)):
        pcs = setup_pcs(bg, n, 1)
        items = make_proofs(bg, pcs, n, count, 1, 9000 + n)
        jobs, wants = [], []
        for j, (root, values, point, blob, proof) in enumerate(items):
            pf = proof
            if j == 1:
                bad = bytearray(proof)
                bad[len(proof) - 40] ^= 0x80  # inside the last query's last path
                pf = bytes(bad)
            jobs.append((root, [bg.PolyEvals(values, point)], pf, bg.GenericChallenger.from_state(blob)))
            wants.append(0 if j != 1 else host_code(bg, pcs, root, values, point, blob, pf)[0])
        res = pcs.verify_batch(jobs)
        assert res == wants and wants[1] != 0, (n, res)


def test_empty_batch(bg):
    pcs = setup_pcs(bg, 4, 1)
    assert pcs.verify_batch([]) == []


def test_invalid_query_from_a_non_codeword(bg):
    """A proof whose Merkle paths all verify but whose opened values are not a
    codeword: num_vars 0, blowup 2, committed leaves [a, b] with a != b and the
    claim a.  Queries at position 1 open b, which folds to b != a = final
    polynomial: InvalidQuery (basefold.rs:318-320), as the oracle says."""
    import struct

    log2_c = 1
    pcs = setup_pcs(bg, 0, log2_c)
    a, b = rand.random_elems(2, 8800)
    a, b = a.tobytes(), b.tobytes()
    ha, hb = O.keccak256(a), O.keccak256(b)
    root = O.keccak256(ha + hb)
    value = np.frombuffer(a, dtype=np.uint8).reshape(1, 16)
    no_point = np.zeros((0, 16), np.uint8)
    ch = bg.GenericChallenger.keccak256()
    ch.observe(root)
    ch.observe_ext_slice(value)
    blob = ch.state()
    probe = bg.GenericChallenger.from_state(blob)
    probe.observe_ext_slice(value)  # the final polynomial [a]
    Q = O.num_queries(log2_c)
    idx = [probe.sample_bits(1) for _ in range(Q)]
    assert 0 in idx and 1 in idx
    pf = struct.pack("<Q", 0) + struct.pack("<Q", 1) + a + struct.pack("<Q", 0) + struct.pack("<Q", Q)
    for i in idx:
        pf += struct.pack("<Q", 1) + (b if i else a) + struct.pack("<Q", 1) + (ha if i else hb) + struct.pack("<Q", 0)
    assert O.verify(0, log2_c, root, no_point, value, blob, pf) == 2
    assert host_code(bg, pcs, root, value, no_point, blob, pf)[0] == 2
    honest = make_proofs(bg, pcs, 0, 1, 1, 8801)[0]
    jobs = [(root, [bg.PolyEvals(value, no_point)], pf, bg.GenericChallenger.from_state(blob)),
            (honest[0], [bg.PolyEvals(honest[1], honest[2])], honest[4], bg.GenericChallenger.from_state(honest[3]))]
    assert pcs.verify_batch(jobs) == [2, 0]
