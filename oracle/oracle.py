"""ctypes front end of the oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
import this module.  Field elements are numpy uint8 arrays of shape (n, 16):
the raw little-endian Montgomery-form u128 of Polyval.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        u8p = C.POINTER(C.c_uint8)
        sz = C.c_size_t
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_set_threads.restype = C.c_int
        for name in ("orc_gf_mul", "orc_gf_mul_definition"):
            getattr(L, name).argtypes = [u8p, u8p, u8p, sz]
            getattr(L, name).restype = None
        for name in ("orc_gf_inv", "orc_from_canonical", "orc_to_canonical"):
            getattr(L, name).argtypes = [u8p, u8p, sz]
            getattr(L, name).restype = None
        L.orc_field_consts.argtypes = [u8p]
        L.orc_polyval_rfc.argtypes = [u8p, u8p, sz, u8p]
        L.orc_keccak_f.argtypes = [C.POINTER(C.c_uint64)]
        L.orc_keccak_consts.argtypes = [C.POINTER(C.c_uint64), C.POINTER(C.c_int)]
        L.orc_keccak256.argtypes = [u8p, sz, u8p]
        L.orc_sha3_256.argtypes = [u8p, sz, u8p]
        L.orc_ntt_twiddles.argtypes = [C.c_int, u8p]
        L.orc_ntt_forward.argtypes = [C.c_int, sz, u8p]
        L.orc_ntt_backward.argtypes = [C.c_int, sz, u8p]
        L.orc_ntt_forward_definition.argtypes = [C.c_int, u8p]
        L.orc_num_queries.argtypes = [C.c_int, C.c_int]
        L.orc_num_queries.restype = sz
        L.orc_encode.argtypes = [C.c_int, C.c_int, sz, u8p, u8p]
        L.orc_merkle_commit.argtypes = [u8p, sz, sz, u8p, u8p]
        L.orc_commit.argtypes = [C.c_int, C.c_int, sz, u8p, u8p]
        L.orc_commit_root.argtypes = [C.c_int, C.c_int, sz, u8p, u8p]
        L.orc_eval.argtypes = [C.c_int, sz, u8p, u8p, u8p]
        L.orc_challenger_sample.argtypes = [u8p, sz, C.c_int, sz, C.c_int, u8p, u8p, C.POINTER(sz)]
        L.orc_harness_prepare.argtypes = [C.c_int, C.c_int, sz, u8p, u8p, u8p, u8p, u8p, C.POINTER(sz)]
        L.orc_open.argtypes = [C.c_int, C.c_int, sz, u8p, u8p, u8p, C.c_int, u8p, sz, u8p, sz, C.POINTER(sz)]
        L.orc_verify.argtypes = [C.c_int, C.c_int, sz, u8p, u8p, u8p, C.c_int, u8p, sz, u8p, sz]
        L.orc_commit_eval_open.argtypes = [C.c_int, C.c_int, u8p, u8p, u8p, u8p, sz, C.POINTER(sz)]
        L.orc_sumcheck_prove.argtypes = [C.c_int, C.c_int, u8p, u8p, u8p, sz, u8p]
        L.orc_sumcheck_verify.argtypes = [C.c_int, C.c_int, u8p, u8p, u8p, u8p, sz, u8p]
        # prime field (BabyBear, quintic extension; oracle_bb.cpp)
        L.orc_bb_emul.argtypes = [u8p, u8p, u8p, sz]
        L.orc_bb_einv.argtypes = [u8p, u8p, sz]
        L.orc_bb_dft.argtypes = [C.c_int, C.POINTER(C.c_uint32), C.c_int]
        L.orc_bb_num_queries.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        L.orc_bb_num_queries.restype = sz
        u32p = C.POINTER(C.c_uint32)
        L.orc_bb_encode.argtypes = [C.c_int, C.c_int, C.c_int, u32p, sz, u8p, u8p]
        L.orc_bb_commit.argtypes = [C.c_int, C.c_int, C.c_int, u32p, sz, u8p, u8p]
        L.orc_bb_eval.argtypes = [C.c_int, sz, u8p, u8p, u8p]
        L.orc_bb_harness_prepare.argtypes = [C.c_int, C.c_int, C.c_int, u32p, sz, u8p, u8p, u8p, u8p, u8p,
                                             C.POINTER(sz)]
        L.orc_bb_open.argtypes = [C.c_int, C.c_int, C.c_int, u32p, sz, u8p, u8p, u8p, u8p, sz, u8p, sz,
                                  C.POINTER(sz)]
        L.orc_bb_verify.argtypes = [C.c_int, C.c_int, C.c_int, u32p, sz, u8p, u8p, u8p, u8p, sz, u8p, sz]
        _lib = L
    return _lib


def _p(a):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(C.c_uint8))


def _buf(x):
    """bytes / bytearray / numpy -> contiguous uint8 numpy array."""
    if isinstance(x, np.ndarray):
        return np.ascontiguousarray(x, dtype=np.uint8).reshape(-1)
    return np.frombuffer(bytes(x), dtype=np.uint8).copy()


def _elems(x):
    a = _buf(x)
    assert a.size % 16 == 0
    return a.reshape(-1, 16)


def set_threads(n: int) -> int:
    return lib().orc_set_threads(n)


def to_int(e) -> int:
    return int.from_bytes(bytes(np.asarray(e, dtype=np.uint8).reshape(16)), "little")


def from_ints(vals):
    out = np.zeros((len(vals), 16), dtype=np.uint8)
    for i, v in enumerate(vals):
        out[i] = np.frombuffer(int(v).to_bytes(16, "little"), dtype=np.uint8)
    return out


def gf_mul(a, b, definition=False):
    a, b = _elems(a), _elems(b)
    out = np.zeros_like(a)
    f = lib().orc_gf_mul_definition if definition else lib().orc_gf_mul
    f(_p(a), _p(b), _p(out), a.shape[0])
    return out


def gf_inv(a):
    a = _elems(a)
    out = np.zeros_like(a)
    lib().orc_gf_inv(_p(a), _p(out), a.shape[0])
    return out


def from_canonical(a):
    a = _elems(a)
    out = np.zeros_like(a)
    lib().orc_from_canonical(_p(a), _p(out), a.shape[0])
    return out


def to_canonical(a):
    a = _elems(a)
    out = np.zeros_like(a)
    lib().orc_to_canonical(_p(a), _p(out), a.shape[0])
    return out


def field_consts():
    out = np.zeros((2, 16), dtype=np.uint8)
    lib().orc_field_consts(_p(out))
    return to_int(out[0]), to_int(out[1])


def polyval_rfc(h: bytes, xs: bytes) -> bytes:
    hh, xx = _buf(h), _buf(xs)
    out = np.zeros(16, dtype=np.uint8)
    lib().orc_polyval_rfc(_p(hh), _p(xx), xx.size // 16, _p(out))
    return out.tobytes()


def keccak_f(state):
    st = np.ascontiguousarray(state, dtype=np.uint64).copy()
    lib().orc_keccak_f(st.ctypes.data_as(C.POINTER(C.c_uint64)))
    return st


def keccak_consts():
    rc = np.zeros(24, dtype=np.uint64)
    rho = np.zeros(25, dtype=np.int32)
    lib().orc_keccak_consts(rc.ctypes.data_as(C.POINTER(C.c_uint64)), rho.ctypes.data_as(C.POINTER(C.c_int)))
    return rc, rho


def keccak256(msg: bytes) -> bytes:
    m = _buf(msg)
    out = np.zeros(32, dtype=np.uint8)
    lib().orc_keccak256(_p(m) if m.size else None, m.size, _p(out))
    return out.tobytes()


def sha3_256(msg: bytes) -> bytes:
    m = _buf(msg)
    out = np.zeros(32, dtype=np.uint8)
    lib().orc_sha3_256(_p(m) if m.size else None, m.size, _p(out))
    return out.tobytes()


def ntt_twiddles(log_n: int):
    out = np.zeros(((1 << log_n) - 1, 16), dtype=np.uint8)
    assert lib().orc_ntt_twiddles(log_n, _p(out) if out.size else None) == 0
    return out


def ntt_forward(log_n: int, data, width: int = 1):
    d = _elems(data).copy()
    assert lib().orc_ntt_forward(log_n, width, _p(d)) == 0
    return d


def ntt_backward(log_n: int, data, width: int = 1):
    d = _elems(data).copy()
    assert lib().orc_ntt_backward(log_n, width, _p(d)) == 0
    return d


def ntt_forward_definition(log_n: int, data):
    d = _elems(data).copy()
    assert lib().orc_ntt_forward_definition(log_n, _p(d)) == 0
    return d


def num_queries(log2_c: int, lam: int = 128) -> int:
    return int(lib().orc_num_queries(lam, log2_c))


def encode(n: int, log2_c: int, data, width: int = 1):
    d = _elems(data)
    out = np.zeros(((width << n) << log2_c, 16), dtype=np.uint8)
    assert lib().orc_encode(n, log2_c, width, _p(d), _p(out)) == 0
    return out


def merkle_commit(rows, height: int, width: int, layers: bool = False):
    r = _elems(rows)
    root = np.zeros(32, dtype=np.uint8)
    lay = np.zeros(((2 * height - 1), 32), dtype=np.uint8) if layers else None
    assert lib().orc_merkle_commit(_p(r), height, width, _p(root), _p(lay)) == 0
    return (root.tobytes(), lay) if layers else root.tobytes()


def commit(n: int, log2_c: int, data, width: int = 1) -> bytes:
    d = _elems(data)
    root = np.zeros(32, dtype=np.uint8)
    assert lib().orc_commit(n, log2_c, width, _p(d), _p(root)) == 0
    return root.tobytes()


def commit_root(n: int, log2_c: int, data, width: int = 1) -> bytes:
    """commit()'s root in bounded host memory (subtrees of 2^14 leaves)."""
    d = _elems(data)
    root = np.zeros(32, dtype=np.uint8)
    assert lib().orc_commit_root(n, log2_c, width, _p(d), _p(root)) == 0
    return root.tobytes()


def eval_poly(n: int, data, point, width: int = 1):
    d, p = _elems(data), _elems(point) if n else np.zeros((0, 16), np.uint8)
    out = np.zeros((width, 16), dtype=np.uint8)
    assert lib().orc_eval(n, width, _p(d), _p(p) if n else None, _p(out)) == 0
    return out


def challenger_blob(inp: bytes = b"", out: bytes = b"") -> bytes:
    return (len(inp).to_bytes(8, "little") + bytes(inp) + len(out).to_bytes(8, "little") + bytes(out))


def challenger_sample(blob: bytes, count: int, bits: int = -1):
    """bits < 0: `count` field elements; else `count` sample_bits(bits)."""
    b = _buf(blob)
    kind = 0 if bits < 0 else 1
    out = np.zeros(count * (16 if kind == 0 else 8), dtype=np.uint8)
    nb = np.zeros(len(blob) + 64, dtype=np.uint8)
    nl = C.c_size_t(nb.size)
    rc = lib().orc_challenger_sample(_p(b), b.size, kind, count, max(bits, 0), _p(out), _p(nb), C.byref(nl))
    assert rc == 0
    vals = out.reshape(-1, 16) if kind == 0 else out.view(np.uint64)
    return vals, nb[: nl.value].tobytes()


def harness_prepare(n: int, log2_c: int, data, point, width: int = 1):
    """commit, observe root, eval at point, observe values (poly-commit/src/lib.rs:80-98)."""
    d = _elems(data)
    p = _elems(point) if n else np.zeros((1, 16), np.uint8)
    root = np.zeros(32, dtype=np.uint8)
    vals = np.zeros((width, 16), dtype=np.uint8)
    blob = np.zeros(64 + 16 * width, dtype=np.uint8)
    bl = C.c_size_t(blob.size)
    assert lib().orc_harness_prepare(n, log2_c, width, _p(d), _p(p), _p(root), _p(vals), _p(blob), C.byref(bl)) == 0
    return root.tobytes(), vals, blob[: bl.value].tobytes()


def open_proof(n: int, log2_c: int, data, point, values, blob: bytes, width: int = 1, n_evals: int = 1) -> bytes:
    d = _elems(data)
    p = _elems(point) if (n and n_evals) else np.zeros((1, 16), np.uint8)
    v = _elems(values) if n_evals else np.zeros((1, 16), np.uint8)
    b = _buf(blob)
    cap = 1 << 16
    while True:
        out = np.zeros(cap, dtype=np.uint8)
        ln = C.c_size_t(0)
        rc = lib().orc_open(n, log2_c, width, _p(d), _p(p), _p(v), n_evals, _p(b), b.size, _p(out), cap, C.byref(ln))
        if rc == -2:
            cap = ln.value
            continue
        assert rc == 0, rc
        return out[: ln.value].tobytes()


def commit_eval_open(n: int, log2_c: int, data, point):
    """One full prover step (commit, eval, open with the harness transcript); returns (root, proof)."""
    d = _elems(data)
    p = _elems(point) if n else np.zeros((1, 16), np.uint8)
    root = np.zeros(32, dtype=np.uint8)
    cap = 1 << 23
    out = np.zeros(cap, dtype=np.uint8)
    ln = C.c_size_t(0)
    rc = lib().orc_commit_eval_open(n, log2_c, _p(d), _p(p), _p(root), _p(out), cap, C.byref(ln))
    assert rc == 0, rc
    return root.tobytes(), out[: ln.value].tobytes()


def verify(n: int, log2_c: int, root: bytes, point, values, blob: bytes, proof: bytes, width: int = 1,
           n_evals: int = 1) -> int:
    p = _elems(point) if n else np.zeros((1, 16), np.uint8)
    v = _elems(values) if n_evals else np.zeros((1, 16), np.uint8)
    r, b, pf = _buf(root), _buf(blob), _buf(proof)
    return lib().orc_verify(n, log2_c, width, _p(r), _p(p), _p(v), n_evals, _p(b), b.size,
                            _p(pf) if pf.size else _p(np.zeros(1, np.uint8)), pf.size)


def sumcheck_prove(k: int, n: int, polys, claim, blob: bytes):
    """Returns (compressed round polys [n, k], challenges [n], final evals [k], final claim)."""
    ps = _elems(polys)
    c = _elems(claim)
    b = _buf(blob)
    out = np.zeros((n * k + n + k + 1, 16), dtype=np.uint8)
    assert lib().orc_sumcheck_prove(k, n, _p(ps), _p(c), _p(b), b.size, _p(out)) == 0
    rp = out[: n * k].reshape(n, k, 16)
    r = out[n * k: n * k + n]
    fe = out[n * k + n: n * k + n + k]
    return rp, r, fe, out[-1]


def sumcheck_verify(k: int, n: int, claim, round_polys, final_evals, blob: bytes) -> int:
    c = _elems(claim)
    rp = _elems(round_polys) if n else np.zeros((1, 16), np.uint8)
    fe = _elems(final_evals)
    b = _buf(blob)
    return lib().orc_sumcheck_verify(k, n, _p(c), _p(rp), _p(fe), _p(b), b.size, None)


# ---------------------------------------------------------------------------
# Prime field: BabyBear elements are uint32 (canonical), extension elements
# uint32 arrays of shape (n, 5) (coefficients of 1, X, .., X^4).
# ---------------------------------------------------------------------------
BB_P = 2013265921


def _u32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.uint32))


def _pu(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint8))


def bb_emul(a, b):
    a, b = _u32(a).reshape(-1, 5), _u32(b).reshape(-1, 5)
    out = np.zeros_like(a)
    lib().orc_bb_emul(_pu(a), _pu(b), _pu(out), a.shape[0])
    return out


def bb_einv(a):
    a = _u32(a).reshape(-1, 5)
    out = np.zeros_like(a)
    lib().orc_bb_einv(_pu(a), _pu(out), a.shape[0])
    return out


def bb_dft(log_n: int, data, definition: bool = False):
    d = _u32(data).copy()
    assert lib().orc_bb_dft(log_n, d.ctypes.data_as(C.POINTER(C.c_uint32)), 1 if definition else 0) == 0
    return d


def bb_num_queries(log2_c: int, lam: int = 128, n: int = 0, log2_k0: int = 0, generic: bool = False) -> int:
    """Queries of the Reed–Solomon code, or (generic) of the random foldable
    code with num_vars n and log2_k0 (its distance bound depends on both)."""
    return int(lib().orc_bb_num_queries(lam, n, log2_c, log2_k0, 1 if generic else 0))


def bb_random_ts(n: int, log2_c: int, log2_k0: int, seed: int):
    """t's of the generic code for rounds 0..d-1 back to back (n_0 << i each),
    uniform nonzero BabyBears from a seeded generator (the reference draws
    them from its caller's RNG)."""
    d = n - log2_k0
    total = (1 << (log2_c + log2_k0)) * ((1 << d) - 1)
    rng = np.random.default_rng(seed)
    return rng.integers(1, BB_P, size=max(total, 1), dtype=np.uint64).astype(np.uint32)[:total]


def _code(ts):
    """(pointer, keep-alive) of the generic code's t's, or a null pointer for Reed–Solomon."""
    if ts is None:
        return None, None
    t = _u32(ts).reshape(-1)
    if t.size == 0:
        t = np.zeros(1, np.uint32)
    return t.ctypes.data_as(C.POINTER(C.c_uint32)), t


def _mat(data, n: int):
    """Row-major 2^n x width data (a 1-D array is width 1) and its width."""
    d = _u32(data).reshape(-1)
    assert d.size % (1 << n) == 0 and d.size > 0
    return d, d.size >> n


def _pt(point, n: int):
    return _u32(point).reshape(-1, 5) if n else np.zeros((1, 5), np.uint32)


def bb_encode(n: int, log2_c: int, data, log2_k0: int = 0, ts=None):
    """Codeword of each column; returns n_d x width (1-D for width 1)."""
    d, w = _mat(data, n)
    out = np.zeros(w << (n + log2_c), dtype=np.uint32)
    tp, _keep = _code(ts)
    assert lib().orc_bb_encode(n, log2_c, log2_k0, tp, w, _pu(d), _pu(out)) == 0
    return out if w == 1 else out.reshape(-1, w)


def bb_commit(n: int, log2_c: int, data, log2_k0: int = 0, ts=None) -> bytes:
    d, w = _mat(data, n)
    root = np.zeros(32, dtype=np.uint8)
    tp, _keep = _code(ts)
    assert lib().orc_bb_commit(n, log2_c, log2_k0, tp, w, _pu(d), _p(root)) == 0
    return root.tobytes()


def bb_eval(n: int, data, point):
    """Values of the columns at the point: shape (5,) for width 1, else (width, 5)."""
    d, w = _mat(data, n)
    out = np.zeros((w, 5), dtype=np.uint32)
    assert lib().orc_bb_eval(n, w, _pu(d), _pu(_pt(point, n)), _pu(out)) == 0
    return out[0] if w == 1 else out


def bb_harness_prepare(n: int, log2_c: int, data, point, log2_k0: int = 0, ts=None):
    d, w = _mat(data, n)
    root = np.zeros(32, dtype=np.uint8)
    val = np.zeros((w, 5), dtype=np.uint32)
    blob = np.zeros(128 + 20 * w, dtype=np.uint8)
    bl = C.c_size_t(blob.size)
    tp, _keep = _code(ts)
    assert lib().orc_bb_harness_prepare(n, log2_c, log2_k0, tp, w, _pu(d), _pu(_pt(point, n)), _p(root), _pu(val),
                                        _p(blob), C.byref(bl)) == 0
    return root.tobytes(), (val[0] if w == 1 else val), blob[: bl.value].tobytes()


def bb_open(n: int, log2_c: int, data, point, value, blob: bytes, log2_k0: int = 0, ts=None) -> bytes:
    d, w = _mat(data, n)
    v, b = _u32(value).reshape(w, 5), _buf(blob)
    tp, _keep = _code(ts)
    cap = 1 << 16
    while True:
        out = np.zeros(cap, dtype=np.uint8)
        ln = C.c_size_t(0)
        rc = lib().orc_bb_open(n, log2_c, log2_k0, tp, w, _pu(d), _pu(_pt(point, n)), _pu(v), _p(b), b.size,
                               _p(out), cap, C.byref(ln))
        if rc == -2:
            cap = ln.value
            continue
        assert rc == 0, rc
        return out[: ln.value].tobytes()


def bb_verify(n: int, log2_c: int, root: bytes, point, value, blob: bytes, proof: bytes, log2_k0: int = 0,
              ts=None) -> int:
    """0 accepted; 1 final poly, 2 query, 3 Merkle path, 4 malformed."""
    v = _u32(value).reshape(-1, 5)
    r, b, pf = _buf(root), _buf(blob), _buf(proof)
    tp, _keep = _code(ts)
    return lib().orc_bb_verify(n, log2_c, log2_k0, tp, v.shape[0], _p(r), _pu(_pt(point, n)), _pu(v), _p(b),
                               b.size, _p(pf) if pf.size else _p(np.zeros(1, np.uint8)), pf.size)
