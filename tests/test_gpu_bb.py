"""Prime-field Basefold on the GPU (BabyBear, quintic extension, Reed–Solomon
code) against the oracle: commitment roots, column evaluations and whole
proofs byte-for-byte, over the reference test's grid of blowups and widths
(poly-commit/src/basefold.rs:470-478 runs log2_c 0..3, num_vars 0..10,
num_polys 1..10) plus widths around the 34-word Keccak rate and the
benchmark's 256 columns; proofs are also accepted by the library's own
verifier.  Edge cases: no variables, blowup 1 (no queries), non-canonical
evaluations, a zero coordinate."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

P = O.BB_P


def rnd(shape, seed):
    return np.random.default_rng(seed).integers(0, P, size=shape, dtype=np.uint64).astype(np.uint32)


def _pcs(n, log2_c):
    from basefold_gpu import BasefoldConfig, prime

    return prime.BabyBearBasefold.setup(BasefoldConfig(prime.ReedSolomonCode(128, log2_c, n)), device=0)


def _check(n, log2_c, w, seed):
    from basefold_gpu import GenericChallenger, prime

    data = rnd((1 << n, w) if w > 1 else 1 << n, seed)
    point = rnd((n, 5), seed + 1)
    pcs = _pcs(n, log2_c)
    comm = pcs.commit(data)
    root, values, blob = O.bb_harness_prepare(n, log2_c, data, point)
    assert comm.root == root
    got = pcs.eval(comm, point)
    assert np.array_equal(got, np.asarray(values).reshape(-1, 5))
    ev = [prime.PrimePolyEvals(got, point)]
    proof = pcs.open(comm, ev, GenericChallenger.from_state(blob))
    assert len(proof) == pcs.proof_size(w, 1)
    want = O.bb_open(n, log2_c, data, point, values, blob)
    assert proof == want
    pcs.verify(root, ev, proof, GenericChallenger.from_state(blob))


# (num_vars, log2_c, width)
SMALL = [(0, 0, 1), (0, 1, 1), (0, 2, 3), (1, 0, 1), (1, 1, 1), (2, 2, 1), (3, 1, 1), (5, 0, 2), (6, 2, 1),
         (9, 1, 1), (9, 2, 9), (4, 1, 3), (5, 1, 33), (5, 1, 34), (2, 2, 35), (7, 1, 2), (3, 3, 68), (8, 1, 32)]


@pytest.mark.parametrize("n,log2_c,w", SMALL)
def test_commit_eval_open_match_oracle(built_lib, n, log2_c, w):
    _check(n, log2_c, w, 1000 + 31 * n + 7 * log2_c + w)


@pytest.mark.parametrize("n,log2_c,w", [(14, 1, 1), (16, 2, 1), (20, 1, 1), (12, 1, 256), (14, 1, 256), (13, 2, 100),
                                        (16, 1, 100)])
def test_larger_sizes_match_oracle(built_lib, n, log2_c, w):
    """Sizes where the DFT runs several passes (tiles of up to 2^12 rows for
    one column, 2^8 rows x 32 columns otherwise) and the trees several
    launch kinds; from 2^16 rows the host commit copies in slices and runs
    the passes inside a slice per slice (width 100: four 32-column chunks,
    the last one partial)."""
    _check(n, log2_c, w, 77 + n + w)


def test_commit_device_matches_host_commit(built_lib):
    import torch

    n, log2_c, w = 10, 1, 5
    data = rnd((1 << n, w), 5)
    pcs = _pcs(n, log2_c)
    dev = torch.from_numpy(data.view(np.int32)).cuda()
    c1 = pcs.commit(data)
    c2 = pcs.commit_device(dev.data_ptr(), w, keep=dev)
    assert c1.root == c2.root == O.bb_commit(n, log2_c, data)
    point = rnd((n, 5), 6)
    assert np.array_equal(pcs.eval(c2, point), O.bb_eval(n, data, point))


def test_rejects_non_canonical_and_zero_coordinate(built_lib):
    from basefold_gpu import BasefoldGpuError, GenericChallenger, prime

    n = 6
    pcs = _pcs(n, 1)
    data = rnd(1 << n, 9)
    data[17] = P  # not a canonical BabyBear
    with pytest.raises(BasefoldGpuError) as e:
        pcs.commit(data)
    assert e.value.code == -1
    data[17] = P - 1
    comm = pcs.commit(data)
    point = rnd((n, 5), 10)
    point[2] = 0
    values = pcs.eval(comm, point)
    with pytest.raises(BasefoldGpuError) as e:
        pcs.open(comm, [prime.PrimePolyEvals(values, point)], GenericChallenger.keccak256())
    assert e.value.code == -6
    assert pcs.open(comm, [], GenericChallenger.keccak256()) == bytes(32)  # basefold.rs:139-141


def _check_generic(n, log2_c, log2_k0, w, seed):
    from basefold_gpu import BasefoldConfig, GenericChallenger, prime

    ts = O.bb_random_ts(n, log2_c, log2_k0, seed)
    kw = dict(log2_k0=log2_k0, ts=ts)
    data = rnd((1 << n, w) if w > 1 else 1 << n, seed + 1)
    point = rnd((n, 5), seed + 2)
    code = prime.GenericRandomFoldableCode(128, log2_c, log2_k0, n - log2_k0, ts)
    pcs = prime.BabyBearBasefold.setup(BasefoldConfig(code), device=0)
    comm = pcs.commit(data)
    root, values, blob = O.bb_harness_prepare(n, log2_c, data, point, **kw)
    assert comm.root == root
    got = pcs.eval(comm, point)
    assert np.array_equal(got, np.asarray(values).reshape(-1, 5))
    ev = [prime.PrimePolyEvals(got, point)]
    proof = pcs.open(comm, ev, GenericChallenger.from_state(blob))
    assert proof == O.bb_open(n, log2_c, data, point, values, blob, **kw)
    pcs.verify(root, ev, proof, GenericChallenger.from_state(blob))


# (num_vars, log2_c, log2_k0, width): the reference test's log2_c 0..3 and
# log2_k_0 0..3 (capped at num_vars), generic.rs via basefold.rs:453-468
GENERIC = [(0, 0, 0, 1), (0, 2, 0, 2), (1, 1, 1, 1), (2, 0, 2, 1), (3, 1, 0, 1), (4, 2, 2, 1), (5, 1, 1, 3),
           (6, 1, 2, 9), (7, 2, 0, 34), (8, 1, 2, 1), (9, 0, 1, 2), (12, 1, 2, 1), (16, 1, 1, 1), (11, 1, 1, 64)]


@pytest.mark.parametrize("n,log2_c,log2_k0,w", GENERIC)
def test_generic_code_matches_oracle(built_lib, n, log2_c, log2_k0, w):
    _check_generic(n, log2_c, log2_k0, w, 3000 + 17 * n + 5 * log2_c + log2_k0 + w)


# Stage-0 shapes past the reference test's range: k_0 = 16 with n_0 = 32, 64
# and 128 (rows past k_0 from backward differences), k_0 = 32 with n_0 = 32 and
# 128 (the general kernel), and a 2^17-row host commit whose stage 0 runs per
# input slice.
@pytest.mark.parametrize("n,log2_c,log2_k0,w", [(6, 1, 4, 3), (7, 2, 4, 2), (8, 3, 4, 1), (6, 0, 5, 2),
                                                (9, 2, 5, 1), (17, 1, 3, 4), (16, 1, 3, 100)])
def test_generic_code_stage0_shapes(built_lib, n, log2_c, log2_k0, w):
    _check_generic(n, log2_c, log2_k0, w, 3500 + 17 * n + 5 * log2_c + log2_k0 + w)


def test_caller_stream_and_two_threads(built_lib):
    """Two pcs objects, each on its own caller-made CUDA stream, driven from
    two host threads at once: the same bytes as one at a time."""
    import threading

    import torch
    from basefold_gpu import BasefoldConfig, GenericChallenger, prime

    cases = [(9, 1, 3, 31), (10, 2, 1, 32)]
    want = {}
    for n, log2_c, w, seed in cases:
        data = rnd((1 << n, w) if w > 1 else 1 << n, seed)
        point = rnd((n, 5), seed + 1)
        root, values, blob = O.bb_harness_prepare(n, log2_c, data, point)
        want[seed] = (data, point, root, values, blob, O.bb_open(n, log2_c, data, point, values, blob))
    got, errors = {}, []

    def run(n, log2_c, w, seed):
        try:
            stream = torch.cuda.Stream()
            pcs = prime.BabyBearBasefold.setup(BasefoldConfig(prime.ReedSolomonCode(128, log2_c, n)), device=0,
                                               stream=stream.cuda_stream)
            data, point, root, values, blob, _ = want[seed]
            for _ in range(3):
                comm = pcs.commit(data)
                vals = pcs.eval(comm, point)
                proof = pcs.open(comm, [prime.PrimePolyEvals(vals, point)], GenericChallenger.from_state(blob))
                got[seed] = (comm.root, vals, proof)
                comm.free()
        except Exception as e:  # reported by the main thread
            errors.append(e)

    ts = [threading.Thread(target=run, args=c) for c in cases]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errors, errors
    for n, log2_c, w, seed in cases:
        root, vals, proof = got[seed]
        assert root == want[seed][2]
        assert np.array_equal(vals, np.asarray(want[seed][3]).reshape(-1, 5))
        assert proof == want[seed][5]


def test_open_buffer_too_small_reports_size(built_lib):
    import ctypes as C

    from basefold_gpu import GenericChallenger, prime
    from basefold_gpu._native import lib

    n = 5
    pcs = _pcs(n, 1)
    data = rnd(1 << n, 41)
    point = rnd((n, 5), 42)
    comm = pcs.commit(data)
    vals = pcs.eval(comm, point)
    need = pcs.proof_size(1, 1)
    small = np.zeros(16, np.uint8)
    ln = C.c_size_t()
    rc = lib().bf_bb_open(pcs._h, comm._h, C.c_void_p(point.ctypes.data), C.c_void_p(vals.ctypes.data), 1,
                          GenericChallenger.keccak256()._h, C.c_void_p(small.ctypes.data), small.size, C.byref(ln))
    assert rc == -4 and ln.value == need
    # the full-size call still works and matches the oracle
    _, values, blob = O.bb_harness_prepare(n, 1, data, point)
    proof = pcs.open(comm, [prime.PrimePolyEvals(vals, point)], GenericChallenger.from_state(blob))
    assert proof == O.bb_open(n, 1, data, point, values, blob)


@pytest.mark.parametrize("n,w", [(0, 1), (1, 3), (7, 1), (9, 40), (12, 2)])
def test_eval_of_uncommitted_data(built_lib, n, w):
    """The trait's eval(&Data, point) for rows that have no commitment
    (bf_bb_eval_data), from host and from device memory, against the oracle."""
    import torch

    pcs = _pcs(n, 1)
    data = rnd((1 << n, w) if w > 1 else 1 << n, 500 + n + w)
    point = rnd((n, 5), 600 + n)
    want = np.asarray(O.bb_eval(n, data, point)).reshape(-1, 5)
    assert np.array_equal(pcs.eval(data, point), want)
    dev = torch.from_numpy(data.view(np.int32)).cuda()
    assert np.array_equal(pcs.eval_device(dev.data_ptr(), point, w), want)


def test_seeded_harness_fixture_on_gpu(built_lib):
    """All 1080 cases of the reference's prime-field tests with StdRng-seeded
    inputs (tests/golden/seeded_harness_bb.json): the library's roots,
    evaluation claims and proofs equal the fixture's."""
    import hashlib
    import json
    import os
    import sys

    from basefold_gpu import BasefoldConfig, GenericChallenger, prime

    golden = os.path.join(os.path.dirname(__file__), "golden")
    sys.path.insert(0, golden)
    import make_seeded_harness_bb as M

    doc = json.load(open(os.path.join(golden, "seeded_harness_bb.json")))
    rows = doc["cases"]
    k = 0
    configs = [(lc, None) for lc in range(3)] + [(lc, lk) for lc in range(3) for lk in range(3)]
    pcs_rs = {}
    for log2_c, log2_k0 in configs:
        for n, w, lk, ts, evals, point in M.harness_inputs(doc["seed"], log2_c, log2_k0):
            row = rows[k]
            k += 1
            if ts is None:
                if (n, log2_c) not in pcs_rs:
                    pcs_rs[(n, log2_c)] = _pcs(n, log2_c)
                pcs = pcs_rs[(n, log2_c)]
            else:
                code = prime.GenericRandomFoldableCode(128, log2_c, lk, n - lk, ts)
                pcs = prime.BabyBearBasefold.setup(BasefoldConfig(code), device=0)
            comm = pcs.commit(evals)
            ch = GenericChallenger.keccak256()
            ch.observe(comm.root)
            values = pcs.eval(comm, point)
            prime.observe_ext_slice(ch, values)
            proof = pcs.open(comm, [prime.PrimePolyEvals(values, point)], ch)
            got = [comm.root.hex(), hashlib.sha256(values.tobytes()).hexdigest()[:16], len(proof),
                   hashlib.sha256(proof).hexdigest()[:32]]
            assert got == row[5:], (row[:5], got, row[5:])
            comm.free()
    assert k == len(rows)
