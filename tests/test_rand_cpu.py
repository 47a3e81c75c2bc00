"""The seeded input generators, on the CPU: StdRng (ChaCha12, as the
reference's tests draw their polynomials and points) pinned by the RFC 7539
ChaCha block vectors and by rand's own StdRng value-stability vector, and
the seeded harness fixture regenerated by the oracle."""
import hashlib
import json
import os
import sys

import numpy as np

from basefold_gpu import rand
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
sys.path.insert(0, GOLDEN)


def test_chacha_block_rfc7539():
    # RFC 7539 section 2.3.2 (20 rounds; key 00..1f, counter 1, nonce 0:0x09000000:0x4a000000)
    key = np.frombuffer(bytes(range(32)), dtype="<u4")
    b = rand.chacha_blocks(key, 1 | (0x09000000 << 32), 1, rounds=20, stream=0x4A000000)[0]
    assert [int(v) for v in b] == [0xE4E7F110, 0x15593BD1, 0x1FDD0F50, 0xC47120A3, 0xC7F4D1C7, 0x0368C033,
                                   0x9AAA2204, 0x4E6CD4C3, 0x466482D2, 0x09AA9F07, 0x05D7C214, 0xA2028BD9,
                                   0xD19C12B5, 0xB94E16DE, 0xE883D0CB, 0x4E3C50A2]
    # all-zero key and nonce, counter 0: the first keystream block
    z = rand.chacha_blocks(np.zeros(8, np.uint32), 0, 1, rounds=20)[0]
    assert bytes(z.astype("<u4").tobytes()).hex().startswith("76b8e0ada0f13d90405d6ae55386bd28")


def test_stdrng_value_stability():
    """rand 0.8's own StdRng check: from_seed, next_u64, then from_rng of it."""
    seed = bytes([1, 0, 0, 0, 23, 0, 0, 0, 200, 1, 0, 0, 210, 30, 0, 0] + [0] * 16)
    r0 = rand.StdRng.from_seed(seed)
    x0 = r0.next_u64()
    r1 = rand.StdRng.from_seed(r0.fill_bytes(32))
    assert [x0, r1.next_u64()] == [10719222850664546238, 14064965282130556830]


def test_stdrng_reads_across_buffers():
    """Mixed reads (u32, u64 across a 64-word buffer edge, byte fills of odd
    length) take the keystream's words in order, whole words per fill."""
    r = rand.StdRng.seed_from_u64(7)
    key = rand.StdRng.seed_from_u64(7)._key
    flat = rand.chacha_blocks(key, 0, 8).reshape(-1)
    got = [r.next_u32() for _ in range(63)]
    assert got == [int(v) for v in flat[:63]]
    assert r.next_u64() == int(flat[63]) | (int(flat[64]) << 32)
    assert r.fill_bytes(5) == flat[65:67].astype("<u4").tobytes()[:5]
    e = r.random_elems(3)
    assert e.tobytes() == flat[67:79].astype("<u4").tobytes()


def test_seeded_harness_fixture():
    """The committed fixture equals what the oracle gives for the seeded
    inputs (first cases of each blowup)."""
    import make_seeded_harness as M

    doc = json.load(open(os.path.join(GOLDEN, "seeded_harness.json")))
    by_key = {(c["log2_c"], c["num_vars"], c["num_polys"]): c for c in doc["cases"]}
    assert len(by_key) == 270
    for log2_c in (0, 1, 2):
        for k, (n, w, evals, point) in enumerate(M.harness_inputs(doc["seed"])):
            if k >= 14:
                break
            c = by_key[(log2_c, n, w)]
            root, values, blob = O.harness_prepare(n, log2_c, evals, point, w)
            proof = O.open_proof(n, log2_c, evals, point, values, blob, w)
            assert root.hex() == c["root"] and values.tobytes().hex() == c["values"]
            assert hashlib.sha256(proof).hexdigest() == c["proof_sha256"]


def _bb_fixture_rows(step):
    import hashlib

    sys.path.insert(0, GOLDEN)
    import make_seeded_harness_bb as M

    doc = json.load(open(os.path.join(GOLDEN, "seeded_harness_bb.json")))
    rows = doc["cases"]
    assert doc["cols"] == M.COLS and len(rows) == 3 * 90 + 9 * 90
    k = 0
    for log2_c in range(3):
        for inp in M.harness_inputs(doc["seed"], log2_c):
            yield rows[k], ("reed_solomon", log2_c, None), inp, k % step == 0
            k += 1
    for log2_c in range(3):
        for log2_k0 in range(3):
            for inp in M.harness_inputs(doc["seed"], log2_c, log2_k0):
                yield rows[k], ("generic", log2_c, log2_k0), inp, k % step == 0
                k += 1


def test_seeded_harness_bb_fixture():
    """The prime fixture's draws follow the harness (every case's shape and
    order), and a sample of its cases is reproduced by the oracle."""
    import hashlib

    from oracle import oracle as O

    checked = 0
    for row, (code, log2_c, log2_k0), (n, w, lk, ts, evals, point), check in _bb_fixture_rows(11):
        assert row[:5] == [code, log2_c, log2_k0, n, w]
        if not check:
            continue
        kw = {} if ts is None else {"log2_k0": lk, "ts": ts}
        root, values, blob = O.bb_harness_prepare(n, log2_c, evals, point, **kw)
        proof = O.bb_open(n, log2_c, evals, point, values, blob, **kw)
        assert root.hex() == row[5]
        assert hashlib.sha256(values.tobytes()).hexdigest()[:16] == row[6]
        assert [len(proof), hashlib.sha256(proof).hexdigest()[:32]] == row[7:]
        checked += 1
    assert checked >= 90


def test_babybear_draws():
    """BabyBear::random takes one word >> 1 and redraws while >= p; the
    extension takes five words and redraws all five while any is >= p."""
    rng = rand.StdRng.seed_from_u64(3)
    words = rand.StdRng.seed_from_u64(3)._words(4000)
    got = rng.random_babybear(200)
    exp, i = [], 0
    while len(exp) < 200:
        v = int(words[i]) >> 1
        i += 1
        if v < 2013265921:
            exp.append(v)
    assert got.tolist() == exp
    rng = rand.StdRng.seed_from_u64(4)
    words = rand.StdRng.seed_from_u64(4)._words(4000)
    got = rng.random_babybear_ext(100)
    exp, i = [], 0
    while len(exp) < 100:
        v = [int(x) >> 1 for x in words[i:i + 5]]
        i += 5
        if all(x < 2013265921 for x in v):
            exp.append(v)
    assert got.tolist() == exp
