"""The C ABI without a GPU: the library loads, exports every declared symbol,
and its host-side logic (transcript, verifier) matches the oracle."""
import os
import re

import numpy as np

from oracle import oracle as O
from basefold_gpu import rand

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "basefold_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(bf_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(built_lib):
    from basefold_gpu import _native

    L = _native.lib()
    decl = declared_symbols()
    assert len(decl) >= 25
    for name in decl:
        assert hasattr(L, name), name
    assert sorted(_native.EXPORTS) == decl


def test_status_codes_match_header(built_lib):
    """Every BF_* status code of the header has the same value in the binding,
    and the verifier codes are BasefoldError's (basefold.rs:79-84) plus 4."""
    from basefold_gpu import _native

    bg = built_lib
    text = open(os.path.join(ROOT, "include", "basefold_gpu.h")).read()
    codes = {k: int(v) for k, v in re.findall(r"#define (BF_[A-Z_]+) \(?(-?\d+)\)?", text)}
    assert len(codes) >= 14
    for name, value in codes.items():
        if name.startswith("BF_VERIFY_"):
            continue
        assert getattr(_native, name) == value, name
    verify = {v: k for k, v in codes.items() if k.startswith("BF_VERIFY_") and v}
    assert {v: bg.BasefoldError.KINDS[v] for v in verify} == {
        1: "InvalidFinalPoly", 2: "InvalidQuery", 3: "Mmcs", 4: "Malformed"}


def test_challenger_matches_oracle(built_lib):
    bg = built_lib
    ch = bg.GenericChallenger(b"init")
    blob = O.challenger_blob(b"init")
    ch.observe(b"\x01" * 32)
    blob = O.challenger_blob(b"init" + b"\x01" * 32)
    got = [ch.sample_ext_element() for _ in range(3)]
    want, blob2 = O.challenger_sample(blob, 3)
    assert all(np.array_equal(g, w) for g, w in zip(got, want))
    assert ch.state() == blob2
    bits = [ch.sample_bits(21) for _ in range(9)]
    wb, _ = O.challenger_sample(blob2, 9, bits=21)
    assert bits == [int(x) for x in wb]
    c2 = bg.GenericChallenger.from_state(ch.state())
    assert np.array_equal(c2.sample_ext_element(), ch.clone().sample_ext_element())


def _setup_verifier(bg, n, log2_c):
    import ctypes as C

    from basefold_gpu import _native

    h = C.c_void_p()
    _native.check(_native.lib().bf_pcs_setup(-1, 128, log2_c, n, None, C.byref(h)))
    return bg.Basefold(h, bg.BasefoldConfig(bg.BinaryReedSolomonCode(128, log2_c, n)), -1)


def test_host_verifier_agrees_with_oracle(built_lib):
    bg = built_lib
    for log2_c in (0, 1, 2):
        for n in (0, 1, 3, 7):
            data = rand.random_elems((1 << n) + n, 77 + n + 13 * log2_c)
            evals, point = data[: 1 << n], data[1 << n:]
            root, values, blob = O.harness_prepare(n, log2_c, evals, point)
            proof = O.open_proof(n, log2_c, evals, point, values, blob)
            pcs = _setup_verifier(bg, n, log2_c)
            assert pcs.num_queries() == O.num_queries(log2_c)
            assert pcs.proof_size(1, 1) == len(proof)
            pcs.verify(root, [bg.PolyEvals(values, point)], proof, bg.GenericChallenger.from_state(blob))
            if O.num_queries(log2_c) == 0:
                continue
            for pos in (-3, -40, len(proof) // 2, 20):
                bad = bytearray(proof)
                bad[pos] ^= 1
                want = O.verify(n, log2_c, root, point, values, blob, bytes(bad))
                assert want != 0
                try:
                    pcs.verify(root, [bg.PolyEvals(values, point)], bytes(bad), bg.GenericChallenger.from_state(blob))
                    raise AssertionError("tampered proof accepted")
                except bg.BasefoldError as e:
                    assert e.code == want, (n, log2_c, pos, e.kind, want)
            wrong = values.copy()
            wrong[0, 0] ^= 1
            try:
                pcs.verify(root, [bg.PolyEvals(wrong, point)], proof, bg.GenericChallenger.from_state(blob))
                raise AssertionError("wrong claim accepted")
            except bg.BasefoldError as e:
                assert e.kind in ("InvalidFinalPoly", "Mmcs", "InvalidQuery")


def test_gpu_entry_points_refuse_verifier_only_object(built_lib):
    bg = built_lib
    pcs = _setup_verifier(bg, 4, 1)
    try:
        pcs.verify_batch([])
        raise AssertionError("batched verify ran without a device")
    except bg.BasefoldGpuError as e:
        assert e.code == -1
    try:
        pcs.commit(rand.random_elems(16, 1))
        raise AssertionError("commit ran without a device")
    except bg.BasefoldGpuError as e:
        assert e.code == -1


def test_launch_shape_validation(built_lib):
    """bf_pcs_set_tune accepts only the documented ranges; the autotuner
    needs a device."""
    bg = built_lib
    pcs = _setup_verifier(bg, 4, 1)
    default = dict(ntt_threads=256, ntt_max_T=12, top_nodes=512, tail_log=8, subtree_log=16, ntt_kind=2, gf_mix=0,
                   ntt_ws_warps=8)
    assert pcs.tune == default
    pcs.tune = dict(ntt_threads=512, tail_log=3, subtree_log=12, ntt_kind=0)
    assert pcs.tune == dict(default, ntt_threads=512, tail_log=3, subtree_log=12, ntt_kind=0)
    for bad in (dict(ntt_threads=96), dict(ntt_max_T=13), dict(ntt_max_T=5), dict(top_nodes=100),
                dict(top_nodes=8192), dict(tail_log=0), dict(tail_log=12), dict(subtree_log=9),
                dict(subtree_log=21), dict(ntt_kind=4), dict(ntt_kind=-1), dict(gf_mix=5),
                dict(ntt_ws_warps=1), dict(ntt_ws_warps=15)):
        try:
            pcs.tune = bad
            raise AssertionError(f"accepted {bad}")
        except bg.BasefoldGpuError as e:
            assert e.code == -1
    assert pcs.tune["ntt_threads"] == 512
    try:
        pcs.autotune(1)
        raise AssertionError("autotune ran without a device")
    except bg.BasefoldGpuError as e:
        assert e.code == -1


def test_engine_rejects_bad_parameters(built_lib):
    """Engine parameters are checked before any device is touched."""
    import ctypes as C
    bg = built_lib
    h = C.c_void_p()
    for args in ((0, 128, 1, 0, 0), (0, 128, 1, 300, 0), (0, 128, -1, 4, 0), (0, 128, 5, 4, 0)):
        assert bg.lib().bf_engine_create(*args, C.byref(h)) == -1


def test_tune_cache_file_round_trip(built_lib, tmp_path):
    """The tune cache file: entries load (count returned), save back with the
    same shapes, a verifier-only pcs (no device) keeps its defaults, and a
    malformed or invalid entry is refused."""
    bg = built_lib
    bg.tune_cache_clear()
    f = tmp_path / "tune.json"
    f.write_text('{"version": 1, "entries": [\n'
                 ' {"device": "NVIDIA GB300", "num_vars": 20, "log2_c": 1, "tune": [256, 10, 1024, 9, 14, 2, 3, 6], '
                 '"ms": 4.25},\n'
                 ' {"device": "NVIDIA GB300", "num_vars": 22, "log2_c": 2, "tune": [128, 11, 512, 8], "ms": 12.5}\n'
                 ']}\n')
    assert bg.tune_cache_load(str(f)) == 2
    out = tmp_path / "out.json"
    bg.tune_cache_save(str(out))
    text = out.read_text()
    assert '"num_vars": 20, "log2_c": 1, "tune": [256, 10, 1024, 9, 14, 2, 3, 6]' in text
    assert '"num_vars": 22, "log2_c": 2, "tune": [128, 11, 512, 8, 16, 2, 0, 8]' in text  # defaults fill the rest
    bg.tune_cache_clear()
    assert bg.tune_cache_load(str(out)) == 2
    assert _setup_verifier(bg, 20, 1).tune["ntt_max_T"] == 12  # no device: nothing applied
    bad = tmp_path / "bad.json"
    bad.write_text(' {"device": "X", "num_vars": 20, "log2_c": 1, "tune": [96, 10, 1024, 9], "ms": 1}\n')
    try:
        bg.tune_cache_load(str(bad))
        raise AssertionError("accepted an invalid entry")
    except bg.BasefoldGpuError as e:
        assert e.code == -1
    bg.tune_cache_clear()
