"""Launch shapes (NTT tile and block size, Merkle top and open-tail
thresholds) change how the work is launched, never the proof: every shape,
and the autotuner's pick, gives the oracle's bytes."""
import numpy as np
import pytest

from oracle import oracle as O
from basefold_gpu import rand

pytestmark = pytest.mark.gpu

# every NTT pass kind (0 shared-memory layers, 1 register-blocked tiles,
# 2 warp-specialized last pass), tile sizes that make the kinds apply to one
# or several passes, and the Merkle levels per launch at both ends
SHAPES = [
    dict(ntt_threads=128, ntt_max_T=6, top_nodes=64, tail_log=1, subtree_log=10, ntt_kind=0),
    dict(ntt_threads=512, ntt_max_T=12, top_nodes=4096, tail_log=11, subtree_log=20, ntt_kind=2),
    dict(ntt_threads=256, ntt_max_T=7, top_nodes=128, tail_log=3, subtree_log=12, ntt_kind=1),
    dict(ntt_threads=128, ntt_max_T=10, top_nodes=2048, tail_log=6, subtree_log=14, ntt_kind=2),
    dict(ntt_threads=256, ntt_max_T=9, top_nodes=512, tail_log=8, subtree_log=16, ntt_kind=1),
    dict(ntt_threads=256, ntt_max_T=6, top_nodes=256, tail_log=5, subtree_log=18, ntt_kind=2),
    dict(ntt_threads=256, ntt_max_T=12, top_nodes=512, tail_log=8, subtree_log=16, ntt_kind=3),
    dict(ntt_threads=128, ntt_max_T=8, top_nodes=1024, tail_log=4, subtree_log=16, ntt_kind=3),
    # the field products of the passes without hashing with 1..4 of their nine
    # 32 x 32 products from 16-bit pieces, and other splits of the
    # warp-specialized pass
    dict(ntt_threads=256, ntt_max_T=7, top_nodes=512, tail_log=8, subtree_log=16, ntt_kind=2, gf_mix=1,
         ntt_ws_warps=4),
    dict(ntt_threads=256, ntt_max_T=8, top_nodes=512, tail_log=8, subtree_log=16, ntt_kind=0, gf_mix=2,
         ntt_ws_warps=12),
    dict(ntt_threads=512, ntt_max_T=9, top_nodes=512, tail_log=8, subtree_log=16, ntt_kind=2, gf_mix=3,
         ntt_ws_warps=2),
    dict(ntt_threads=128, ntt_max_T=6, top_nodes=512, tail_log=8, subtree_log=16, ntt_kind=3, gf_mix=4,
         ntt_ws_warps=14),
]


def prove(bg, pcs, evals, point):
    comm = pcs.commit(evals)
    ch = bg.GenericChallenger.keccak256()
    ch.observe(comm.root)
    values = pcs.eval(pcs.data(comm), point)
    ch.observe_ext_slice(values)
    return comm.root, values, pcs.open(comm, [bg.PolyEvals(values, point)], ch)


@pytest.mark.parametrize("n,log2_c", [(1, 1), (5, 0), (9, 1), (13, 2), (15, 1), (18, 1)])
def test_every_shape_gives_the_oracle_proof(built_lib, n, log2_c):
    bg = built_lib
    data = rand.random_elems((1 << n) + n, 7000 + n)
    evals, point = data[: 1 << n], data[1 << n:]
    root_o, values_o, blob = O.harness_prepare(n, log2_c, evals, point)
    want = O.open_proof(n, log2_c, evals, point, values_o, blob)
    pcs = bg.Basefold.setup(bg.BasefoldConfig(bg.BinaryReedSolomonCode(128, log2_c, n)))
    for shape in SHAPES:
        pcs.tune = shape
        assert {k: pcs.tune[k] for k in shape} == shape
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
    assert set(rep["axes"]) == {"ntt_kind", "ntt_max_T", "ntt_threads", "top_nodes", "subtree_log", "tail_log", "gf_mix",
                                "ntt_ws_warps"}
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


def test_tune_cache_applies_to_later_pcs_and_engine(built_lib, tmp_path):
    """bf_pcs_autotune's pick lands in the tune cache: a later pcs of the same
    device and size starts from it, it survives a save / clear / load round
    trip through the JSON file, and proofs made with it (alone and by the
    engine, which sets up its own pcs per size) are the oracle's."""
    bg = built_lib
    bg.tune_cache_clear()
    n, log2_c = 12, 1
    cfg = bg.BasefoldConfig(bg.BinaryReedSolomonCode(128, log2_c, n))
    default = bg.Basefold.setup(cfg).tune
    pcs = bg.Basefold.setup(cfg)
    pcs.autotune(1)
    tuned = pcs.tune
    assert bg.Basefold.setup(cfg).tune == tuned
    f = tmp_path / "tune.json"
    bg.tune_cache_save(str(f))
    bg.tune_cache_clear()
    assert bg.Basefold.setup(cfg).tune == default
    assert bg.tune_cache_load(str(f)) == 1
    later = bg.Basefold.setup(cfg)
    assert later.tune == tuned
    data = rand.random_elems((1 << n) + n, 4242)
    evals, point = data[: 1 << n], data[1 << n:]
    root_o, values_o, blob = O.harness_prepare(n, log2_c, evals, point)
    want = O.open_proof(n, log2_c, evals, point, values_o, blob)
    assert prove(bg, later, evals, point)[2] == want
    eng = bg.Engine(max_inflight=2, log2_c=log2_c)
    assert eng.prove([(n, evals, point)])[0]["proof"] == want
    bg.tune_cache_clear()
