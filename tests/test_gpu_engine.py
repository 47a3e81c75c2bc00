"""The prover engine (batched and served forms): every proof is identical to
the one produced by commit/eval/open one at a time (tolerance: bit-exact),
alone or in the mix."""
import time

import numpy as np
import pytest

from oracle import oracle as O
from basefold_gpu import rand

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bg(built_lib):
    return built_lib


def alone(bg, n, evals, point, log2_c=1):
    pcs = bg.Basefold.setup(bg.BasefoldConfig(bg.BinaryReedSolomonCode(128, log2_c, n)), device=0)
    comm = pcs.commit(evals)
    ch = bg.GenericChallenger.keccak256()
    ch.observe(comm.root)
    values = pcs.eval(pcs.data(comm), point)
    ch.observe_ext_slice(values)
    return comm.root, values, pcs.open(comm, [bg.PolyEvals(values, point)], ch)


def make_jobs(sizes, seed0):
    jobs = []
    for k, n in enumerate(sizes):
        data = rand.random_elems((1 << n) + n, seed0 + k)
        jobs.append((n, data[: 1 << n], data[1 << n:]))
    return jobs


def test_engine_batch_matches_alone(bg):
    sizes = [0, 1, 3, 12, 7, 10, 5, 14, 9, 11, 6, 13, 8, 2, 4, 10]
    jobs = make_jobs(sizes, 8000)
    eng = bg.Engine(max_inflight=6)
    res = eng.prove(jobs)
    for (n, ev, pt), r in zip(jobs, res):
        root, values, proof = alone(bg, n, ev, pt)
        assert r["status"] == 0
        assert r["root"] == root and np.array_equal(r["value"], values) and r["proof"] == proof, n
    n, ev, pt = jobs[3]
    root_o, values_o, blob = O.harness_prepare(n, 1, ev, pt)
    assert res[3]["proof"] == O.open_proof(n, 1, ev, pt, values_o, blob)


def test_engine_device_input(bg):
    torch = pytest.importorskip("torch")
    jobs = make_jobs([9, 11, 6], 8100)
    devs = [torch.from_numpy(ev).cuda() for _, ev, _ in jobs]
    eng = bg.Engine(max_inflight=3)
    res = eng.prove([(n, d.data_ptr(), pt) for (n, _, pt), d in zip(jobs, devs)], device_input=True)
    for (n, ev, pt), r in zip(jobs, res):
        assert r["proof"] == alone(bg, n, ev, pt)[2]


def test_engine_serving_continuous_batching(bg):
    """Requests submitted while others run are admitted between rounds; each
    result equals the alone result."""
    sizes = [13, 8, 11, 6, 12, 9, 10, 7, 14, 5]
    jobs = make_jobs(sizes, 8200)
    eng = bg.Engine(max_inflight=4)
    eng.start()
    got = {}
    for k, (n, ev, pt) in enumerate(jobs):
        eng.submit(n, ev, pt, tag=k)
        time.sleep(0.002)
        for tag, r in eng.poll():
            got[tag] = r
    deadline = time.time() + 60
    while len(got) < len(jobs) and time.time() < deadline:
        for tag, r in eng.poll():
            got[tag] = r
        time.sleep(0.001)
    eng.stop()
    assert len(got) == len(jobs)
    for k, (n, ev, pt) in enumerate(jobs):
        assert got[k]["status"] == 0 and got[k]["latency_ms"] > 0
        assert got[k]["proof"] == alone(bg, n, ev, pt)[2], k


def test_engine_admission_by_memory_budget(bg):
    """A budget smaller than one job still completes (one job at a time)."""
    jobs = make_jobs([10, 11, 9], 8300)
    eng = bg.Engine(max_inflight=4, mem_budget=1 << 20)
    res = eng.prove(jobs)
    for (n, ev, pt), r in zip(jobs, res):
        assert r["proof"] == alone(bg, n, ev, pt)[2]


def test_engine_graph_replay_matches_direct(bg):
    """Captured-graph jobs (one plan per slot and size, replayed) give the
    same bytes as the direct path and as proofs made one at a time, with
    sizes repeating so plans are reused and other sizes evict them."""
    sizes = [8, 8, 11, 8, 11, 5, 8, 13, 5, 11, 8, 0, 1, 8]
    jobs = make_jobs(sizes, 8400)
    direct = bg.Engine(max_inflight=3, graphs=False).prove(jobs)
    for max_inflight in (1, 3):
        replay = bg.Engine(max_inflight=max_inflight, graphs=True).prove(jobs)
        for d, r in zip(direct, replay):
            assert r["status"] == 0 and r["proof"] == d["proof"] and r["root"] == d["root"]
    for k in (0, 2, 7):
        n, ev, pt = jobs[k]
        assert direct[k]["proof"] == alone(bg, n, ev, pt)[2]


def test_engine_graph_eviction_under_budget(bg):
    """A budget below one plan: every new size evicts the idle plans first,
    jobs then run one at a time, results unchanged."""
    jobs = make_jobs([9, 6, 9, 10, 6], 8500)
    res = bg.Engine(max_inflight=4, mem_budget=1, graphs=True).prove(jobs)
    for (n, ev, pt), r in zip(jobs, res):
        assert r["status"] == 0 and r["proof"] == alone(bg, n, ev, pt)[2]


@pytest.mark.parametrize("graphs", [False, True])
def test_engine_bad_job_fails_alone(bg, graphs):
    """A job whose point has a zero coordinate (EvalImpr::new would divide by
    zero, eval_impr.rs:24) fails with BF_ERR_NOT_INVERTIBLE; the jobs around
    it, before and after, and later batches are unaffected."""
    jobs = make_jobs([9, 9, 7, 9], 8600)
    n, ev, pt = jobs[1]
    bad_pt = pt.copy()
    bad_pt[3] = 0
    jobs[1] = (n, ev, bad_pt)
    eng = bg.Engine(max_inflight=2, graphs=graphs)
    res = eng.prove(jobs, raise_on_error=False)
    assert res[1]["status"] == -6  # BF_ERR_NOT_INVERTIBLE
    for k in (0, 2, 3):
        n, ev, pt = jobs[k]
        assert res[k]["status"] == 0 and res[k]["proof"] == alone(bg, n, ev, pt)[2]
    again = eng.prove([jobs[0], jobs[3]])
    assert again[0]["proof"] == res[0]["proof"] and again[1]["proof"] == res[3]["proof"]


def test_engine_proofs_verify_in_one_batch(bg):
    """Served flow: proofs made by the engine, checked by bf_verify_batch per
    size, all accepted; one altered claim per size rejected as the host
    verifier rejects it."""
    sizes = [6, 9, 12, 9, 6, 12, 16, 16]
    jobs = make_jobs(sizes, 8600)
    res = bg.Engine(max_inflight=4).prove(jobs)
    for n in sorted(set(sizes)):
        pcs = bg.Basefold.setup(bg.BasefoldConfig(bg.BinaryReedSolomonCode(128, 1, n)), device=0)
        items, wants = [], []
        for (m, ev, pt), r in zip(jobs, res):
            if m != n:
                continue
            for bad in (False, True):
                vals = r["value"].copy()
                if bad:
                    vals[0, 0] ^= 2
                ch = bg.GenericChallenger.keccak256()
                ch.observe(r["root"])
                ch.observe_ext_slice(vals)
                items.append((r["root"], [bg.PolyEvals(vals, pt)], r["proof"], ch))
                host = ch.clone()
                try:
                    pcs.verify(r["root"], [bg.PolyEvals(vals, pt)], r["proof"], host)
                    wants.append(0)
                except bg.BasefoldError as e:
                    wants.append(e.code)
        got = pcs.verify_batch(items)
        assert got == wants and got[0::2] == [0] * (len(got) // 2) and all(w != 0 for w in wants[1::2]), n


def test_engine_set_tune_keeps_proofs(bg):
    """Engine-wide launch shapes change no proof byte; invalid shapes are refused."""
    jobs = make_jobs([11, 13, 9], 8700)
    base = bg.Engine(max_inflight=3).prove(jobs)
    eng = bg.Engine(max_inflight=3)
    eng.set_tune({"ntt_threads": 128, "ntt_max_T": 7, "top_nodes": 128, "tail_log": 11})
    for r0, r1 in zip(base, eng.prove(jobs)):
        assert r0["proof"] == r1["proof"] and r0["root"] == r1["root"]
    with pytest.raises(bg.BasefoldGpuError):
        eng.set_tune({"ntt_threads": 96, "ntt_max_T": 12, "top_nodes": 512, "tail_log": 8})


def test_engine_cancel_queued_job(bg):
    """A served request still waiting for a slot can be cancelled: it comes
    back from poll with BF_ERR_CANCELLED; the others complete unchanged."""
    jobs = make_jobs([21, 10, 11, 12, 9], 8800)
    eng = bg.Engine(max_inflight=1)  # the 2^21 job holds the only slot for milliseconds
    eng.start()
    keys = [eng.submit(n, ev, pt, tag=i) for i, (n, ev, pt) in enumerate(jobs)]
    assert eng.cancel(keys[2])
    res, t0 = {}, time.time()
    while len(res) < len(jobs) and time.time() - t0 < 120:
        for tag, r in eng.poll():
            res[tag] = r
        time.sleep(0.001)
    eng.stop()
    assert res[2]["status"] == -8 and res[2]["proof"] == b""
    for i in (0, 1, 3, 4):
        assert res[i]["status"] == 0 and res[i]["proof"] == alone(bg, *jobs[i])[2], i
    assert not eng.cancel(keys[0])  # finished: nothing to cancel


@pytest.mark.parametrize("log2_c", [0, 2])
def test_engine_other_blowups(bg, log2_c):
    """Blowup 1 (no queries, binary_reed_solomon.rs:56-59) and 4 in the engine:
    the same proofs as one at a time."""
    jobs = make_jobs([0, 3, 9, 12, 6, 14], 8900 + log2_c)
    res = bg.Engine(max_inflight=4, log2_c=log2_c).prove(jobs)
    for (n, ev, pt), r in zip(jobs, res):
        root, values, proof = alone(bg, n, ev, pt, log2_c)
        assert r["status"] == 0 and r["root"] == root and np.array_equal(r["value"], values), (n, log2_c)
        assert r["proof"] == proof, (n, log2_c)


def test_engine_serving_policy_keeps_proofs(bg):
    """Smallest-first admission and high-priority streams for small jobs change
    the order of work, never a proof byte; bad policy values are refused."""
    jobs = make_jobs([14, 3, 12, 9, 16, 6, 11], 9100)
    eng = bg.Engine(max_inflight=2, smallest_first=True, priority_max_vars=11)
    eng.start()
    keys = {eng.submit(n, ev, pt, tag=i): i for i, (n, ev, pt) in enumerate(jobs)}
    res, t0 = {}, time.time()
    while len(res) < len(jobs) and time.time() - t0 < 120:
        for tag, r in eng.poll():
            res[tag] = r
        time.sleep(0.001)
    eng.stop()
    assert len(keys) == len(jobs)
    for i, (n, ev, pt) in enumerate(jobs):
        assert res[i]["status"] == 0 and res[i]["proof"] == alone(bg, n, ev, pt)[2], i
    with pytest.raises(bg.BasefoldGpuError):
        bg.Engine(max_inflight=1, priority_max_vars=31)
