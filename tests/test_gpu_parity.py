"""GPU path against the oracle, byte for byte (bit-exact: all arithmetic is
exact GF(2^128) and Keccak, so the tolerance is zero).  Everything goes
through the C ABI of libbasefold_gpu.so."""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from basefold_gpu import rand

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
ONE = 0xC2000000000000000000000000000001


@pytest.fixture(scope="module")
def bg(built_lib):
    return built_lib


def setup_pcs(bg, n, log2_c):
    return bg.Basefold.setup(bg.BasefoldConfig(bg.BinaryReedSolomonCode(128, log2_c, n)), device=0)


def test_device_is_blackwell(bg):
    info = bg.device_info(0)
    assert info["cc"][0] >= 10 and info["num_sms"] > 0


def test_gf_mul_matches_oracle(bg):
    n = 1 << 17
    a, b = rand.random_elems(n, 1), rand.random_elems(n, 2)
    edge = O.from_ints([0, 1, ONE, (1 << 128) - 1, 1 << 127, 1 << 64, (1 << 64) - 1, 0x1E563DF92EA7081B4563DF92EA7081B5]
                       + [1 << i for i in range(0, 128, 7)])
    ea = np.repeat(edge, len(edge), axis=0)
    eb = np.tile(edge, (len(edge), 1))
    a, b = np.concatenate([a, ea]), np.concatenate([b, eb])
    assert np.array_equal(bg.test_gf_mul(a, b), O.gf_mul(a, b))


def test_gf_mul_ten_million_products(bg):
    """~10^7 random products (10 x 2^20) against the oracle, bit-exact."""
    for k in range(10):
        n = 1 << 20
        a, b = rand.random_elems(n, 100 + k), rand.random_elems(n, 200 + k)
        assert np.array_equal(bg.test_gf_mul(a, b), O.gf_mul(a, b)), k


def test_keccak_f_matches_oracle(bg):
    st = rand.splitmix64(25 * 1000, seed=9).reshape(1000, 25)
    got = bg.test_keccak_f(st)
    for i in range(1000):
        assert np.array_equal(got[i], O.keccak_f(st[i])), i


@pytest.mark.parametrize("log2_c", [0, 1, 2])
def test_commit_root_matches_oracle(bg, log2_c):
    for n in list(range(0, 15)) + [17]:
        evals = rand.random_elems(1 << n, 300 + n + 31 * log2_c)
        pcs = setup_pcs(bg, n, log2_c)
        comm = pcs.commit(evals)
        assert comm.root == O.commit(n, log2_c, evals), (n, log2_c)
        assert np.array_equal(pcs.data(comm).to_host(), evals)


def test_commit_root_large(bg):
    """2^20 evaluations at blowup 2 and 4: root identical to the oracle's."""
    for n, log2_c in ((20, 1), (19, 2)):
        evals = rand.random_elems(1 << n, 4000 + n)
        pcs = setup_pcs(bg, n, log2_c)
        assert pcs.commit(evals).root == O.commit(n, log2_c, evals)


def harness(bg, n, log2_c, seed):
    data = rand.random_elems((1 << n) + n, seed)
    evals, point = data[: 1 << n], data[1 << n:]
    pcs = setup_pcs(bg, n, log2_c)
    comm = pcs.commit(evals)
    ch = bg.GenericChallenger.keccak256()
    ch.observe(comm.root)
    values = pcs.eval(pcs.data(comm), point)
    ch.observe_ext_slice(values)
    proof = pcs.open(comm, [bg.PolyEvals(values, point)], ch.clone())
    return pcs, comm, evals, point, values, ch, proof


@pytest.mark.parametrize("log2_c", [0, 1, 2])
def test_open_proof_matches_oracle(bg, log2_c):
    for n in list(range(0, 12)) + [13]:
        pcs, comm, evals, point, values, ch, proof = harness(bg, n, log2_c, 500 + n + 17 * log2_c)
        root_o, values_o, blob = O.harness_prepare(n, log2_c, evals, point)
        assert comm.root == root_o
        assert np.array_equal(values, values_o), ("eval", n, log2_c)
        assert ch.state() == blob
        proof_o = O.open_proof(n, log2_c, evals, point, values_o, blob)
        assert len(proof) == len(proof_o), (n, log2_c)
        assert proof == proof_o, ("proof", n, log2_c)
        pcs.verify(comm.root, [bg.PolyEvals(values, point)], proof, ch.clone())


def test_open_matches_committed_vectors(bg):
    vec = json.load(open(os.path.join(GOLDEN, "oracle_vectors.json")))
    for case in vec["basefold"]:
        n, log2_c, w, seed = case["n"], case["log2_c"], case["width"], case["seed"]
        data = rand.random_elems((w << n) + n, seed)
        evals, point = data[: w << n], data[w << n:]
        pcs = setup_pcs(bg, n, log2_c)
        comm = pcs.commit(evals, width=w)
        assert comm.root.hex() == case["root"]
        values = pcs.eval(pcs.data(comm), point)
        assert [bytes(v).hex() for v in values] == case["values"]
        ch = bg.GenericChallenger.keccak256()
        ch.observe(comm.root)
        ch.observe_ext_slice(values)
        proof = pcs.open(comm, [bg.PolyEvals(values, point)], ch)
        assert len(proof) == case["proof_len"]
        assert hashlib.sha256(proof).hexdigest() == case["proof_sha256"]


def test_open_large_matches_oracle(bg):
    n, log2_c = 18, 1
    pcs, comm, evals, point, values, ch, proof = harness(bg, n, log2_c, 77)
    root_o, values_o, blob = O.harness_prepare(n, log2_c, evals, point)
    assert comm.root == root_o and np.array_equal(values, values_o)
    assert proof == O.open_proof(n, log2_c, evals, point, values_o, blob)


def test_open_empty_evals(bg):
    pcs = setup_pcs(bg, 4, 1)
    comm = pcs.commit(rand.random_elems(16, 3))
    assert pcs.open(comm, [], bg.GenericChallenger.keccak256()) == bytes(32)


def test_repeated_opens_are_identical(bg):
    """Workspace reuse across calls leaves no state behind."""
    pcs, comm, evals, point, values, ch, proof = harness(bg, 9, 1, 21)
    for _ in range(3):
        again = pcs.open(comm, [bg.PolyEvals(values, point)], ch.clone())
        assert again == proof


@pytest.mark.parametrize("k", [2, 3])
def test_sumcheck_matches_oracle(bg, k):
    for n in list(range(0, 11)) + [14]:
        polys = rand.random_elems(k << n, 900 + 10 * k + n)
        claim = rand.random_elems(1, 1900 + n)
        init = bytes(range(32))
        got = bg.prove_sumcheck(k, polys, claim, bg.GenericChallenger(init))
        want = O.sumcheck_prove(k, n, polys, claim, O.challenger_blob(init))
        for g, w in zip(got, want):
            assert np.array_equal(g, w), (k, n)


@pytest.mark.parametrize("k", [2, 3])
def test_sumcheck_prover_verifies(bg, k):
    n = 12
    polys = rand.random_elems(k << n, 41 + k)
    P = polys.reshape(k, 1 << n, 16)
    prod = P[0]
    for j in range(1, k):
        prod = O.gf_mul(prod, P[j])
    claim = np.bitwise_xor.reduce(prod, axis=0)[None]
    if k == 2:
        claim = O.gf_mul(claim, O.from_ints([ONE]))
    rp, r, fe, fc = bg.prove_sumcheck(k, polys, claim, bg.GenericChallenger(b"x"))
    assert O.sumcheck_verify(k, n, claim, rp, fe, O.challenger_blob(b"x")) == 0


def harness_w(bg, n, log2_c, width, seed):
    data = rand.random_elems((width << n) + n, seed)
    evals, point = data[: width << n], data[width << n:]
    pcs = setup_pcs(bg, n, log2_c)
    comm = pcs.commit(evals, width=width)
    ch = bg.GenericChallenger.keccak256()
    ch.observe(comm.root)
    values = pcs.eval(pcs.data(comm), point)
    ch.observe_ext_slice(values)
    proof = pcs.open(comm, [bg.PolyEvals(values, point)], ch.clone())
    return pcs, comm, evals, point, values, ch, proof


@pytest.mark.parametrize("log2_c", [0, 1, 2])
def test_reference_harness_matrix_matches_oracle(bg, log2_c):
    """The reference's own test matrix for the binary code (basefold.rs:480-490
    over poly-commit/src/lib.rs:64-105): num_vars 0..9, num_polys 1..9."""
    for n in range(0, 10):
        for width in range(1, 10):
            pcs, comm, evals, point, values, ch, proof = harness_w(bg, n, log2_c, width, 10000 + 100 * n + width)
            root_o, values_o, blob = O.harness_prepare(n, log2_c, evals, point, width)
            assert comm.root == root_o, (n, width, log2_c)
            assert np.array_equal(values, values_o), (n, width, log2_c)
            assert ch.state() == blob
            assert proof == O.open_proof(n, log2_c, evals, point, values_o, blob, width), (n, width, log2_c)
            pcs.verify(comm.root, [bg.PolyEvals(values, point)], proof, ch.clone())


def test_wide_commit_large(bg):
    n, log2_c, width = 15, 1, 3
    pcs, comm, evals, point, values, ch, proof = harness_w(bg, n, log2_c, width, 77)
    root_o, values_o, blob = O.harness_prepare(n, log2_c, evals, point, width)
    assert comm.root == root_o and np.array_equal(values, values_o)
    assert proof == O.open_proof(n, log2_c, evals, point, values_o, blob, width)


@pytest.mark.parametrize("n,log2_c,width", [(16, 1, 1), (17, 2, 2), (18, 1, 3)])
def test_commit_from_host_in_slices(bg, n, log2_c, width):
    """From 2^16 rows up bf_commit copies host rows in 8 slices on a second
    stream and the first NTT pass starts on each slice as it lands: same
    root, values and proof as the oracle, wide rows included."""
    pcs, comm, evals, point, values, ch, proof = harness_w(bg, n, log2_c, width, 91 + n)
    root_o, values_o, blob = O.harness_prepare(n, log2_c, evals, point, width)
    assert comm.root == root_o and np.array_equal(values, values_o)
    assert proof == O.open_proof(n, log2_c, evals, point, values_o, blob, width)


@pytest.mark.parametrize("pending", [0, 100, 400, 401, 600, 5000])
def test_open_with_long_pending_transcript(bg, pending):
    """Whatever the caller observed before open (here `pending` extra bytes,
    across the device transcript buffer's limit) the proof is the oracle's."""
    n, log2_c = 9, 1
    data = rand.random_elems((1 << n) + n, 4242 + pending)
    evals, point = data[: 1 << n], data[1 << n:]
    pcs = setup_pcs(bg, n, log2_c)
    comm = pcs.commit(evals)
    extra = bytes((7 * k + pending) & 0xFF for k in range(pending))
    ch = bg.GenericChallenger.keccak256()
    ch.observe(extra)
    ch.observe(comm.root)
    values = pcs.eval(pcs.data(comm), point)
    ch.observe_ext_slice(values)
    blob = ch.state()
    proof = pcs.open(comm, [bg.PolyEvals(values, point)], ch.clone())
    assert proof == O.open_proof(n, log2_c, evals, point, values, blob)


@pytest.mark.parametrize("init_len", [0, 400, 470, 3000])
def test_sumcheck_any_initial_transcript(bg, init_len):
    """The product sumcheck runs its rounds' transcript on the device when the
    initial state fits the device buffer and on the host otherwise; both give
    the oracle's rounds and leave the challenger in the oracle's state."""
    for k in (2, 3):
        n = 9
        polys = rand.random_elems(k << n, 300 + init_len + k)
        claim = rand.random_elems(1, 31 + k)
        init = bytes((5 * i + k) & 0xFF for i in range(init_len))
        ch = bg.GenericChallenger(init)
        got = bg.prove_sumcheck(k, polys, claim, ch)
        want = O.sumcheck_prove(k, n, polys, claim, O.challenger_blob(init))
        for g, w in zip(got, want):
            assert np.array_equal(g, w), (k, init_len)
        # the challenger continues like the oracle's after the proof
        ref = bg.GenericChallenger(init)
        ref.observe_ext_slice(claim)
        for i in range(n):
            ref.observe_ext_slice(want[0][i])
            ref.sample_ext_element()
        assert ch.sample_ext_element().tobytes() == ref.sample_ext_element().tobytes()


def test_open_zero_coordinate_then_valid_open(bg):
    """open at a point with a zero coordinate is refused (the reference would
    divide by zero in EvalImpr::new, eval_impr.rs:24) and leaves the pcs and
    the commitment usable for a valid open."""
    n, log2_c = 8, 1
    pcs, comm, evals, point, values, ch, proof = harness(bg, n, log2_c, 99)
    bad = point.copy()
    bad[2] = 0
    try:
        pcs.open(comm, [bg.PolyEvals(values, bad)], ch.clone())
        raise AssertionError("zero coordinate accepted")
    except bg.BasefoldGpuError as e:
        assert e.code == -6
    assert pcs.open(comm, [bg.PolyEvals(values, point)], ch.clone()) == proof


def test_seeded_reference_harness(bg):
    """The reference's test matrix (num_vars 0..9, num_polys 1..9, blowup
    1/2/4) with inputs drawn from StdRng::seed_from_u64(0) in the harness's
    order: every root, claim and proof equals the committed oracle fixture."""
    import hashlib
    import sys

    sys.path.insert(0, GOLDEN)
    import make_seeded_harness as M

    doc = json.load(open(os.path.join(GOLDEN, "seeded_harness.json")))
    by_key = {(c["log2_c"], c["num_vars"], c["num_polys"]): c for c in doc["cases"]}
    for log2_c in (0, 1, 2):
        for n, w, evals, point in M.harness_inputs(doc["seed"]):
            pcs = setup_pcs(bg, n, log2_c)
            comm = pcs.commit(evals, width=w)
            ch = bg.GenericChallenger.keccak256()
            ch.observe(comm.root)
            values = pcs.eval(pcs.data(comm), point)
            ch.observe_ext_slice(values)
            proof = pcs.open(comm, [bg.PolyEvals(values, point)], ch.clone())
            c = by_key[(log2_c, n, w)]
            assert comm.root.hex() == c["root"] and values.tobytes().hex() == c["values"], (log2_c, n, w)
            assert hashlib.sha256(proof).hexdigest() == c["proof_sha256"], (log2_c, n, w)


def test_data_changed_after_commit_is_caught(bg):
    """commit_device keeps a reference to the caller's buffer: if the caller
    changes it after committing, the sumcheck and the committed codeword no
    longer describe one polynomial.  The prover's self-check (the reference's
    debug assert encode0(final_poly) == pi, basefold.rs:198) turns that into
    an error instead of a proof that would not verify."""
    torch = pytest.importorskip("torch")
    n = 12
    data = rand.random_elems((1 << n) + n, 4242)
    ev = torch.from_numpy(data[: 1 << n].copy()).cuda()
    point = data[1 << n:]
    pcs = setup_pcs(bg, n, 1)
    comm = pcs.commit_device(ev.data_ptr(), keep=ev)
    ev[5, 0] ^= 1  # the committed data changes under the commitment
    torch.cuda.synchronize()
    ch = bg.GenericChallenger.keccak256()
    ch.observe(comm.root)
    values = pcs.eval(pcs.data(comm), point)
    ch.observe_ext_slice(values)
    with pytest.raises(bg.BasefoldGpuError) as e:
        pcs.open(comm, [bg.PolyEvals(values, point)], ch)
    assert e.value.code == -7
    # the same pcs proves the unchanged data afterwards
    ev[5, 0] ^= 1
    torch.cuda.synchronize()
    comm2 = pcs.commit_device(ev.data_ptr(), keep=ev)
    ch = bg.GenericChallenger.keccak256()
    ch.observe(comm2.root)
    values = pcs.eval(pcs.data(comm2), point)
    ch.observe_ext_slice(values)
    proof = pcs.open(comm2, [bg.PolyEvals(values, point)], ch.clone())
    pcs.verify(comm2.root, [bg.PolyEvals(values, point)], proof, ch.clone())


def test_free_order_does_not_matter(bg):
    """A pcs freed before its commitments and open sessions stays alive until
    the last of them is freed (the order a garbage collector may pick)."""
    from basefold_gpu import _native

    n = 10
    data = rand.random_elems((1 << n) + n, 515)
    pcs = setup_pcs(bg, n, 1)
    comm = pcs.commit(data[: 1 << n])
    root = comm.root
    point = data[1 << n:]
    sess = pcs.open_session(comm, bg.PolyEvals(pcs.eval(pcs.data(comm), point), point))
    _native.lib().bf_pcs_free(pcs._h)  # the caller's reference goes first
    pcs._h = None
    r = np.zeros(32, dtype=np.uint8)
    _native.check(_native.lib().bf_commitment_root(comm._h, r.ctypes.data))
    assert r.tobytes() == root
    del sess
    comm.free()


def test_concurrent_provers_on_threads(bg):
    """Four host threads, each with its own pcs (and stream), prove at once:
    every proof equals the one made alone.  Covers the library's shared state
    under concurrency (launch counting, kernel attributes, error text,
    pinned staging)."""
    from concurrent.futures import ThreadPoolExecutor

    cases = [(n, 1 + (k % 2), 7700 + k) for k, n in enumerate((9, 12, 14, 16, 11, 13, 15, 10))]

    def prove(case):
        n, log2_c, seed = case
        pcs, comm, evals, point, values, ch, proof = harness(bg, n, log2_c, seed)
        comm.free()
        return proof

    alone = [prove(c) for c in cases]
    for _ in range(2):
        with ThreadPoolExecutor(4) as ex:
            assert list(ex.map(prove, cases)) == alone


@pytest.mark.parametrize("log2_c", [3, 4])
def test_large_blowups_match_oracle(bg, log2_c):
    """Blowup 8 and 16 (more cosets per NTT pass, other tail thresholds):
    roots, claims and proofs equal the oracle's; the proofs verify on the
    host and in the batched GPU verifier."""
    for n, width in ((0, 1), (1, 2), (2, 1), (5, 3), (8, 1), (11, 2), (16, 1)):
        pcs, comm, evals, point, values, ch, proof = harness_w(bg, n, log2_c, width, 600 + 10 * n + log2_c)
        root_o, values_o, blob = O.harness_prepare(n, log2_c, evals, point, width)
        assert comm.root == root_o and np.array_equal(values, values_o), (n, log2_c, width)
        assert proof == O.open_proof(n, log2_c, evals, point, values_o, blob, width), (n, log2_c, width)
        pcs.verify(comm.root, [bg.PolyEvals(values, point)], proof, ch.clone())
        assert pcs.verify_batch([(comm.root, [bg.PolyEvals(values, point)], proof, ch.clone())]) == [0]


def test_random_configurations_match_oracle(bg):
    """Sixty configurations drawn with a fixed seed (num_vars 0..13, blowup
    1..16, 1..17 columns): every root, claim and proof equals the oracle's."""
    rng = np.random.default_rng(20261203)
    for k in range(60):
        log2_c = int(rng.integers(0, 5))
        n = int(rng.integers(0, 14 - (log2_c > 2) * 3))
        width = int(rng.choice([1, 1, 1, 2, 3, 5, 9, 17]))
        pcs, comm, evals, point, values, ch, proof = harness_w(bg, n, log2_c, width, 30000 + k)
        root_o, values_o, blob = O.harness_prepare(n, log2_c, evals, point, width)
        assert comm.root == root_o and np.array_equal(values, values_o), (k, n, log2_c, width)
        assert proof == O.open_proof(n, log2_c, evals, point, values_o, blob, width), (k, n, log2_c, width)


@pytest.mark.parametrize("width", list(range(1, 10)))
def test_eval_of_uncommitted_data_matches_oracle(bg, width):
    """PolyCommitScheme::eval(&Data, point) for data with no commitment
    (bf_eval_data): host rows and device rows give the oracle's
    MultiPoly::evaluate of every column, at widths 1..9 and sizes that take
    the single-block tail only (n = 0, 5) and the per-level launches (n = 15)."""
    torch = pytest.importorskip("torch")
    for n in (0, 5, 15):
        data = rand.random_elems((width << n) + n, 900 + 10 * width + n)
        evals, point = data[: width << n], data[width << n:]
        pcs = setup_pcs(bg, n, 1)
        want = O.eval_poly(n, evals, point, width)
        assert np.array_equal(pcs.eval(evals, point, width=width), want), (n, width)
        dev = torch.from_numpy(evals).cuda()
        assert np.array_equal(pcs.eval_device(dev.data_ptr(), point, width=width), want), (n, width)
        if width == 1:  # the same value through a commitment
            comm = pcs.commit(evals)
            assert np.array_equal(pcs.eval(pcs.data(comm), point), want)
