"""Launch shapes (NTT tile and block size, Merkle top and open-tail
thresholds) change how the work is launched, never the proof: every shape,
and the autotuner's pick, gives the oracle's bytes."""
import numpy as np
import pytest

from oracle import oracle as O
from basefold_gpu import rand

pytestmark = pytest.mark.gpu

SHAPES = [
    dict(ntt_threads=128, ntt_max_T=6, top_nodes=64, tail_log=1),
    dict(ntt_threads=512, ntt_max_T=12, top_nodes=4096, tail_log=11),
    dict(ntt_threads=256, ntt_max_T=7, top_nodes=128, tail_log=3),
    dict(ntt_threads=128, ntt_max_T=10, top_nodes=2048, tail_log=6),
]


def prove(bg, pcs, evals, point):
    comm = pcs.commit(evals)
    ch = bg.GenericChallenger.keccak256()
    ch.observe(comm.root)
    values = pcs.eval(pcs.data(comm), point)
    ch.observe_ext_slice(values)
    return comm.root, values, pcs.open(comm, [bg.PolyEvals(values, point)], ch)


@pytest.mark.parametrize("n,log2_c", [(1, 1), (5, 0), (9, 1), (13, 2), (15, 1)])
def test_every_shape_gives_the_oracle_proof(built_lib, n, log2_c):
    bg = built_lib
    data = rand.random_elems((1 << n) + n, 7000 + n)
    evals, point = data[: 1 << n], data[1 << n:]
    root_o, values_o, blob = O.harness_prepare(n, log2_c, evals, point)
    want = O.open_proof(n, log2_c, evals, point, values_o, blob)
    pcs = bg.Basefold.setup(bg.BasefoldConfig(bg.BinaryReedSolomonCode(128, log2_c, n)))
    for shape in SHAPES:
        pcs.tune = shape
        assert pcs.tune == shape
        root, values, proof = prove(bg, pcs, evals, point)
        assert root == root_o and np.array_equal(values, values_o), shape
        assert proof == want, shape


def test_autotune_keeps_the_proof(built_lib):
    bg = built_lib
    n, log2_c = 11, 1
    data = rand.random_elems((1 << n) + n, 77)
    evals, point = data[: 1 << n], data[1 << n:]
    pcs = bg.Basefold.setup(bg.BasefoldConfig(bg.BinaryReedSolomonCode(128, log2_c, n)))
    before = prove(bg, pcs, evals, point)
    rep = pcs.autotune(1)
    assert rep["tune"] == pcs.tune
    assert set(rep["axes"]) == {"ntt_max_T", "ntt_threads", "top_nodes", "tail_log"}
    assert rep["best_ms"] <= rep["start_ms"]
    after = prove(bg, pcs, evals, point)
    assert after[0] == before[0] and np.array_equal(after[1], before[1]) and after[2] == before[2]


def test_engine_autotune(built_lib):
    bg = built_lib
    jobs, want = [], []
    for n in (6, 10):
        data = rand.random_elems((1 << n) + n, 500 + n)
        evals, point = data[: 1 << n], data[1 << n:]
        jobs.append((n, evals, point))
        root_o, values_o, blob = O.harness_prepare(n, 1, evals, point)
        want.append(O.open_proof(n, 1, evals, point, values_o, blob))
    eng = bg.Engine(max_inflight=4, autotune_reps=1)
    res = eng.prove(jobs)
    assert [r["proof"] for r in res] == want
