"""Round-level open sessions: driven by the caller's transcript they give the
same proof bytes as the one-shot open and the oracle, alone or with several
sessions interleaved on different CUDA streams (tolerance: bit-exact)."""
import numpy as np
import pytest

from oracle import oracle as O
from basefold_gpu import rand

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bg(built_lib):
    return built_lib


def prepare(bg, n, log2_c, seed):
    data = rand.random_elems((1 << n) + n, seed)
    evals, point = data[: 1 << n], data[1 << n:]
    pcs = bg.Basefold.setup(bg.BasefoldConfig(bg.BinaryReedSolomonCode(128, log2_c, n)), device=0)
    comm = pcs.commit(evals)
    ch = bg.GenericChallenger.keccak256()
    ch.observe(comm.root)
    values = pcs.eval(pcs.data(comm), point)
    ch.observe_ext_slice(values)
    return pcs, comm, evals, point, values, ch


@pytest.mark.parametrize("n,log2_c", [(0, 1), (1, 1), (5, 0), (9, 1), (12, 2)])
def test_session_matches_one_shot_and_oracle(bg, n, log2_c):
    pcs, comm, evals, point, values, ch = prepare(bg, n, log2_c, 60 + n)
    one_shot = pcs.open(comm, [bg.PolyEvals(values, point)], ch.clone())
    sess = pcs.open_session(comm, bg.PolyEvals(values, point))
    assert sess.prove(ch.clone()) == one_shot
    root_o, values_o, blob = O.harness_prepare(n, log2_c, evals, point)
    assert one_shot == O.open_proof(n, log2_c, evals, point, values_o, blob)


def test_session_rejects_misuse(bg):
    pcs, comm, evals, point, values, ch = prepare(bg, 4, 1, 5)
    sess = pcs.open_session(comm, bg.PolyEvals(values, point))
    with pytest.raises(bg.BasefoldGpuError):
        sess.finish([0] * pcs.num_queries())  # rounds remain
    with pytest.raises(bg.BasefoldGpuError):
        sess.final_poly()


def test_interleaved_sessions_on_streams_match_alone(bg):
    torch = pytest.importorskip("torch")
    jobs = [prepare(bg, n, 1, 700 + n) for n in (6, 9, 11, 8, 12, 10)]
    alone = [pcs.open(comm, [bg.PolyEvals(v, p)], ch.clone()) for pcs, comm, e, p, v, ch in jobs]
    streams = [torch.cuda.Stream() for _ in jobs]
    sessions = [pcs.open_session(comm, bg.PolyEvals(v, p), stream=s.cuda_stream)
                for (pcs, comm, e, p, v, ch), s in zip(jobs, streams)]
    chs = [ch.clone() for (*_, ch) in jobs]
    proofs = [None] * len(jobs)
    active = set(range(len(jobs)))
    while active:
        for j in sorted(active):
            s, c = sessions[j], chs[j]
            i, root, poly = s.round()
            if i >= 0:
                c.observe(root)
                c.observe_ext_slice(poly)
                s.challenge(c.sample_ext_element())  # returns before the GPU finishes
                continue
            c.observe_ext_slice(s.final_poly())
            pcs = jobs[j][0]
            L = pcs.config.code.log2_c + pcs.config.code.d
            proofs[j] = s.finish([c.sample_bits(L) for _ in range(pcs.num_queries())])
            active.discard(j)
    assert proofs == alone
