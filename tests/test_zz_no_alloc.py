"""bf_eval_noalloc: the evaluation entry point that allocates nothing, for
callers whose device memory is already fully reserved (fixed per-request
slots) or that cannot afford a synchronising cudaMalloc at this point.  Its
output must equal bf_eval's (bit-exact) on consecutive calls, which share the
library's fixed scratch array.  This file runs last so that a failure here
leaves every other test already run."""
import ctypes as C

import numpy as np
import pytest

from basefold_gpu import rand

pytestmark = pytest.mark.gpu


def test_eval_noalloc_matches_eval_on_consecutive_calls(built_lib):
    torch = pytest.importorskip("torch")
    bg = built_lib
    from basefold_gpu import _native

    L = _native.lib()
    out = torch.zeros(16, dtype=torch.uint8, device="cuda:0")
    side = torch.cuda.Stream()
    # consecutive calls of different sizes share the scratch: n = 0 (a copy),
    # 1 (one fix), the single-block tail (9, 13) and the per-level launches
    # (14, 17); the last runs on a caller-created stream
    cases = [(14, 31), (9, 32), (0, 35), (17, 33), (1, 36), (13, 37), (14, 34)]
    for call, (n, seed) in enumerate(cases):
        data = rand.random_elems((1 << n) + n, seed)
        evals, point = data[: 1 << n], data[1 << n:]
        pcs = bg.Basefold.setup(bg.BasefoldConfig(bg.BinaryReedSolomonCode(128, 1, n)), device=0)
        want = pcs.eval(pcs.data(pcs.commit(evals)), point)
        dev = torch.from_numpy(evals).cuda()
        pt = np.ascontiguousarray(point) if n else np.zeros((1, 16), np.uint8)
        on_side = call == len(cases) - 1
        if on_side:
            side.wait_stream(torch.cuda.current_stream())
        st = C.c_void_p(side.cuda_stream) if on_side else None
        _native.check(L.bf_eval_noalloc(C.c_void_p(dev.data_ptr()), n, C.c_void_p(pt.ctypes.data),
                                        C.c_void_p(out.data_ptr()), st))
        torch.cuda.synchronize()
        got = out.cpu().numpy().reshape(1, 16)
        assert np.array_equal(got, want), (call, n)


def test_eval_noalloc_rejects_oversized(built_lib):
    torch = pytest.importorskip("torch")
    from basefold_gpu import _native

    L = _native.lib()
    dev = torch.zeros(16, dtype=torch.uint8, device="cuda:0")
    pt = np.zeros((18, 16), np.uint8)
    rc = L.bf_eval_noalloc(C.c_void_p(dev.data_ptr()), 18, C.c_void_p(pt.ctypes.data), C.c_void_p(dev.data_ptr()),
                           None)
    assert rc == _native.BF_ERR_ARG
    assert "exceeds the fixed scratch" in _native.last_error()
