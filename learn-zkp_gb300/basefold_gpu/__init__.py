"""GB300-native Basefold prover (POLYVAL field, binary Reed–Solomon code,
Keccak-256 Merkle trees) behind the reference's PolyCommitScheme interface.

Mirrors han0110/learn-zkp:
  * `Basefold` with setup / commit / data / eval / open / verify
    (poly-commit/src/lib.rs:20-51, poly-commit/src/basefold.rs:86-325);
  * `BinaryReedSolomonCode` (poly-commit/src/basefold/code/binary_reed_solomon.rs);
  * `GenericChallenger.keccak256()` (p3/src/challenger.rs);
  * `prove_sumcheck` for products of 2 (Quadratic) and 3 multilinear
    polynomials (sumcheck/src/lib.rs:56-79).
All computation runs in libbasefold_gpu.so on the GPU; field elements are
numpy uint8 arrays of shape (n, 16) holding Polyval's raw little-endian value.
"""
import ctypes as C
import os

import numpy as np

from ._native import BasefoldGpuError, BfJob, check, lib  # noqa: F401
from . import rand  # noqa: F401

__all__ = [
    "Basefold", "BasefoldConfig", "BinaryReedSolomonCode", "BasefoldError", "BasefoldGpuError", "CommitmentData",
    "Engine", "GenericChallenger", "PolyEvals", "prove_sumcheck", "rand",
]

_u8p = C.c_void_p


def _elems(x, n=None) -> np.ndarray:
    if isinstance(x, (bytes, bytearray)):
        a = np.frombuffer(bytes(x), dtype=np.uint8)
    else:
        a = np.ascontiguousarray(np.asarray(x, dtype=np.uint8))
    a = a.reshape(-1, 16)
    if n is not None and a.shape[0] != n:
        raise ValueError(f"expected {n} field elements, got {a.shape[0]}")
    return np.ascontiguousarray(a)


def _p(a: np.ndarray):
    return C.c_void_p(a.ctypes.data)


class GenericChallenger:
    """GenericChallenger<Polyval, Keccak256Hash> (p3/src/challenger.rs:24-83)."""

    def __init__(self, initial_state: bytes = b"", _handle=None):
        if _handle is not None:
            self._h = _handle
            return
        h = C.c_void_p()
        buf = (C.c_uint8 * max(1, len(initial_state))).from_buffer_copy(bytes(initial_state) or b"\0")
        check(lib().bf_challenger_new(C.cast(buf, C.c_void_p) if initial_state else None, len(initial_state),
                                      C.byref(h)))
        self._h = h

    @classmethod
    def keccak256(cls) -> "GenericChallenger":
        return cls(b"")

    @classmethod
    def from_state(cls, blob: bytes) -> "GenericChallenger":
        h = C.c_void_p()
        b = np.frombuffer(bytes(blob), dtype=np.uint8).copy()
        check(lib().bf_challenger_from_state(_p(b), b.size, C.byref(h)))
        return cls(_handle=h)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and lib is not None:
            try:
                lib().bf_challenger_free(h)
            except Exception:
                pass
            self._h = None

    def clone(self) -> "GenericChallenger":
        h = C.c_void_p()
        check(lib().bf_challenger_clone(self._h, C.byref(h)))
        return GenericChallenger(_handle=h)

    def observe(self, data: bytes) -> None:
        """CanObserve::observe of already-bincoded bytes (a commitment is its 32 bytes)."""
        b = np.frombuffer(bytes(data), dtype=np.uint8).copy()
        check(lib().bf_challenger_observe(self._h, _p(b) if b.size else None, b.size))

    def observe_ext_slice(self, elems) -> None:
        self.observe(_elems(elems).tobytes())

    def sample_ext_element(self) -> np.ndarray:
        out = np.zeros(16, dtype=np.uint8)
        check(lib().bf_challenger_sample_ext(self._h, _p(out)))
        return out

    def sample_bits(self, bits: int) -> int:
        v = C.c_uint64()
        check(lib().bf_challenger_sample_bits(self._h, bits, C.byref(v)))
        return v.value

    def state(self) -> bytes:
        n = C.c_size_t()
        lib().bf_challenger_state(self._h, None, 0, C.byref(n))
        out = np.zeros(n.value, dtype=np.uint8)
        check(lib().bf_challenger_state(self._h, _p(out), out.size, C.byref(n)))
        return out.tobytes()


class BinaryReedSolomonCode:
    """BinaryReedSolomonCode::new(lambda, log2_c, d) (binary_reed_solomon.rs:20-27)."""

    def __init__(self, lambda_: int, log2_c: int, d: int):
        self.lambda_, self.log2_c, self.d = lambda_, log2_c, d

    def c(self) -> int:
        return 1 << self.log2_c

    def k_d(self) -> int:
        return 1 << self.d

    def n_d(self) -> int:
        return self.c() << self.d


class BasefoldConfig:
    """BasefoldConfig { code, mmcs = keccak256_merkle_tree() } (basefold.rs:31-35)."""

    def __init__(self, code: BinaryReedSolomonCode):
        self.code = code


class PolyEvals:
    """PolyEvals { values, point } (poly-commit/src/lib.rs:14-18)."""

    def __init__(self, values, point):
        self.values = _elems(values)
        self.point = _elems(point) if len(point) else np.zeros((0, 16), np.uint8)


class BasefoldError(Exception):
    """BasefoldError::{InvalidFinalPoly, InvalidQuery, Mmcs} (basefold.rs:79-84), plus Malformed."""

    KINDS = {1: "InvalidFinalPoly", 2: "InvalidQuery", 3: "Mmcs", 4: "Malformed"}

    def __init__(self, code: int):
        self.code = code
        self.kind = self.KINDS.get(code, str(code))
        super().__init__(self.kind)


class CommitmentData:
    """BasefoldCommitmentData: device-resident data, codeword and tree."""

    def __init__(self, pcs, handle, root: bytes, width: int, keep=None):
        self._pcs, self._h, self.root, self.width, self._keep = pcs, handle, root, width, keep

    def as_ref(self) -> bytes:
        return self.root

    def free(self):
        if self._h:
            lib().bf_commitment_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class _DeviceData:
    """What `Basefold.data` returns: the commitment's device-resident evaluations."""

    def __init__(self, comm: CommitmentData):
        self.comm = comm

    def to_host(self) -> np.ndarray:
        pcs = self.comm._pcs
        out = np.zeros(((self.comm.width << pcs.config.code.d), 16), dtype=np.uint8)
        check(lib().bf_commitment_data(self.comm._h, _p(out), out.nbytes))
        return out


class Basefold:
    """PolyCommitScheme<Polyval, Polyval> for
    Basefold<Polyval, Polyval, BinaryReedSolomonCode<Polyval>, Keccak256MerkleTreeMmcs<Polyval>>."""

    def __init__(self, handle, config: BasefoldConfig, device: int):
        self._h, self.config, self.device = handle, config, device

    @classmethod
    def setup(cls, config: BasefoldConfig, device: int = 0, stream=None) -> "Basefold":
        h = C.c_void_p()
        code = config.code
        check(lib().bf_pcs_setup(device, code.lambda_, code.log2_c, code.d,
                                 C.c_void_p(stream) if stream else None, C.byref(h)))
        return cls(h, config, device)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                lib().bf_pcs_free(h)
            except Exception:
                pass
            self._h = None

    def num_queries(self) -> int:
        return int(lib().bf_pcs_num_queries(self._h))

    def proof_size(self, width: int = 1, n_evals: int = 1) -> int:
        return int(lib().bf_pcs_proof_size(self._h, width, n_evals))

    def commit(self, data, width: int = 1) -> CommitmentData:
        """commit (basefold.rs:112-120) of host evaluations (2^d * width elements, row-major)."""
        d = _elems(data, (width << self.config.code.d))
        h = C.c_void_p()
        root = np.zeros(32, dtype=np.uint8)
        check(lib().bf_commit(self._h, _p(d), width, C.byref(h), _p(root)))
        return CommitmentData(self, h, root.tobytes(), width)

    def commit_device(self, dev_ptr: int, width: int = 1, keep=None) -> CommitmentData:
        """commit of evaluations already in device memory (kept by reference, not copied)."""
        h = C.c_void_p()
        root = np.zeros(32, dtype=np.uint8)
        check(lib().bf_commit_device(self._h, C.c_void_p(dev_ptr), width, C.byref(h), _p(root)))
        return CommitmentData(self, h, root.tobytes(), width, keep=keep)

    def data(self, comm: CommitmentData) -> _DeviceData:
        return _DeviceData(comm)

    def eval(self, data, point, width: int = 1) -> np.ndarray:
        """eval (basefold.rs:126-131) on the GPU: of `data(comm)` (or the
        commitment itself) through its device-resident evaluations, or of
        host evaluations that have no commitment (row-major, `width`
        columns), which are copied in."""
        p = _elems(point, self.config.code.d) if self.config.code.d else np.zeros((1, 16), np.uint8)
        comm = data.comm if isinstance(data, _DeviceData) else data
        if isinstance(comm, CommitmentData):
            out = np.zeros((comm.width, 16), dtype=np.uint8)
            check(lib().bf_eval(self._h, comm._h, _p(p), _p(out)))
            return out
        ev = _elems(data, width << self.config.code.d)
        out = np.zeros((width, 16), dtype=np.uint8)
        check(lib().bf_eval_data(self._h, _p(ev), 0, width, _p(p), _p(out)))
        return out

    def eval_device(self, dev_ptr: int, point, width: int = 1) -> np.ndarray:
        """eval of device-resident evaluations (2^num_vars rows of `width`
        columns at dev_ptr) that have no commitment."""
        p = _elems(point, self.config.code.d) if self.config.code.d else np.zeros((1, 16), np.uint8)
        out = np.zeros((width, 16), dtype=np.uint8)
        check(lib().bf_eval_data(self._h, C.c_void_p(dev_ptr), 1, width, _p(p), _p(out)))
        return out

    def open(self, comm: CommitmentData, evals, challenger: GenericChallenger) -> bytes:
        """open (basefold.rs:133-232); `challenger` is advanced in place (pass a clone)."""
        if len(evals) > 1:
            raise ValueError("one evaluation point only (basefold.rs:143-144)")
        n_evals = len(evals)
        size = max(self.proof_size(comm.width, n_evals), 1)
        # one output buffer per object, reused: its pages are already mapped
        # (a fresh multi-MB array faults every page in while the proof is
        # written); the proof is returned as a copy
        out = getattr(self, "_proof_buf", None)
        if out is None or out.size < size:
            out = self._proof_buf = np.empty(size, dtype=np.uint8)
        ln = C.c_size_t()
        if n_evals:
            pt = evals[0].point if self.config.code.d else np.zeros((1, 16), np.uint8)
            pt, vals = _elems(pt), _elems(evals[0].values, comm.width)
            check(lib().bf_open(self._h, comm._h, _p(pt), _p(vals), 1, challenger._h, _p(out), out.size,
                                C.byref(ln)))
        else:
            check(lib().bf_open(self._h, comm._h, None, None, 0, challenger._h, _p(out), out.size, C.byref(ln)))
        return out[: ln.value].tobytes()

    def open_session(self, comm: CommitmentData, evals: "PolyEvals", stream=None, scalars=None) -> "OpenSession":
        """Round-level open driven by the caller's transcript (see OpenSession);
        width > 1 needs the caller's eq scalars (basefold.rs:398-408)."""
        return OpenSession(self, comm, evals, stream, scalars)

    def verify(self, comm: bytes, evals, proof: bytes, challenger: GenericChallenger) -> None:
        """verify (basefold.rs:234-324); raises BasefoldError on rejection."""
        root = np.frombuffer(bytes(comm), dtype=np.uint8).copy()
        pf = np.frombuffer(bytes(proof), dtype=np.uint8).copy() if proof else np.zeros(1, np.uint8)
        if evals:
            pt = evals[0].point if self.config.code.d else np.zeros((1, 16), np.uint8)
            pt, vals = _elems(pt), _elems(evals[0].values)
            rc = lib().bf_verify(self._h, _p(root), _p(pt), _p(vals), vals.shape[0], 1, challenger._h, _p(pf),
                                 len(proof))
        else:
            rc = lib().bf_verify(self._h, _p(root), None, None, 1, 0, challenger._h, _p(pf), len(proof))
        check(rc)
        if rc != 0:
            raise BasefoldError(rc)

    def verify_batch(self, items) -> list:
        """verify (basefold.rs:234-324) of many proofs at once on the GPU.

        `items` holds (comm, evals, proof, challenger) tuples as verify takes
        them, one evaluation point each.  Returns one code per item: 0 when it
        verifies, else the BasefoldError code verify would raise.  Every
        challenger is advanced as verify advances it."""
        from ._native import BfVerifyJob
        items = list(items)
        jobs = (BfVerifyJob * max(1, len(items)))()
        keep = []
        for j, (comm, evals, proof, challenger) in enumerate(items):
            if len(evals) != 1:
                raise ValueError("verify_batch takes exactly one PolyEvals per proof")
            root = np.frombuffer(bytes(comm), dtype=np.uint8).copy()
            pf = bytes(proof)  # read in place: no copy when it already is bytes
            pt = evals[0].point if self.config.code.d else np.zeros((1, 16), np.uint8)
            pt, vals = _elems(pt), _elems(evals[0].values)
            keep += [root, pf, pt, vals]
            jobs[j].root, jobs[j].point, jobs[j].values = root.ctypes.data, pt.ctypes.data, vals.ctypes.data
            jobs[j].width, jobs[j].challenger = vals.shape[0], C.cast(challenger._h, C.c_void_p).value
            jobs[j].proof = C.cast(C.c_char_p(pf), C.c_void_p).value if pf else None
            jobs[j].proof_len = len(pf)
        check(lib().bf_verify_batch(self._h, jobs, len(items)))
        return [int(jobs[j].result) for j in range(len(items))]

    # -- standalone sumcheck on device-resident polynomials -------------------
    def prove_sumcheck_device(self, k: int, num_vars: int, dev_ptr: int, claim, challenger: GenericChallenger):
        out = np.zeros((num_vars * k + num_vars + k + 1, 16), dtype=np.uint8)
        c = _elems(claim, 1)
        check(lib().bf_sumcheck_prove_device(self._h, k, num_vars, C.c_void_p(dev_ptr), _p(c), challenger._h,
                                             _p(out)))
        return _split_sumcheck(out, k, num_vars)

    # -- timing of kernel classes -----------------------------------------------
    PROFILE_CLASSES = ["encode", "leaves", "tree", "pi_leaves", "fold", "fix", "eq", "gather", "open_tail",
                       "transcript", "encode_last"]

    # -- launch shapes -----------------------------------------------------------
    TUNE_KEYS = ["ntt_threads", "ntt_max_T", "top_nodes", "tail_log", "subtree_log", "ntt_kind", "gf_mix",
                 "ntt_ws_warps"]

    def autotune(self, reps: int = 3) -> dict:
        """Times whole proofs per candidate launch shape and keeps the fastest
        in this pcs (bf_pcs_autotune); returns the report."""
        buf = C.create_string_buffer(8192)
        check(lib().bf_pcs_autotune(self._h, reps, buf, len(buf)))
        import json
        return json.loads(buf.value.decode())

    @property
    def tune(self) -> dict:
        n = len(self.TUNE_KEYS)
        v = (C.c_int * n)()
        check(lib().bf_pcs_get_tune(self._h, v, n))
        return dict(zip(self.TUNE_KEYS, list(v)))

    @tune.setter
    def tune(self, t: dict) -> None:
        cur = self.tune
        cur.update(t)
        v = (C.c_int * len(self.TUNE_KEYS))(*[int(cur[k]) for k in self.TUNE_KEYS])
        check(lib().bf_pcs_set_tune(self._h, v, len(self.TUNE_KEYS)))

    def profile(self, on: bool = True) -> None:
        check(lib().bf_profile_enable(self._h, 1 if on else 0))

    def profile_read(self) -> dict:
        n = len(self.PROFILE_CLASSES)
        ms = (C.c_double * n)()
        cnt = (C.c_uint64 * n)()
        check(lib().bf_profile_read(self._h, ms, cnt, n))
        return {name: (ms[i], cnt[i]) for i, name in enumerate(self.PROFILE_CLASSES)}


class OpenSession:
    """Basefold::open (basefold.rs:133-232) one round at a time.

    Loop: `round()` gives (i, pi_root, compressed round poly) for rounds
    i = d-1 .. 0; the caller observes the root and the poly, samples r and calls
    `challenge(r)`.  When `round()` returns i = -1, `final_poly()` is observed,
    `num_queries` indices are sampled and `finish(indices)` returns the proof."""

    def __init__(self, pcs: "Basefold", comm: CommitmentData, evals: "PolyEvals", stream=None, scalars=None):
        self._pcs, self._comm = pcs, comm
        d = pcs.config.code.d
        pt = _elems(evals.point) if d else np.zeros((1, 16), np.uint8)
        vals = _elems(evals.values, comm.width)
        sc = _elems(scalars, comm.width) if scalars is not None else None
        h = C.c_void_p()
        check(lib().bf_open_start(pcs._h, comm._h, _p(pt), _p(vals), _p(sc) if sc is not None else None,
                                  C.c_void_p(stream) if stream else None, C.byref(h)))
        self._h = h

    def round(self):
        rnd = C.c_int()
        root = np.zeros(32, dtype=np.uint8)
        poly = np.zeros((2, 16), dtype=np.uint8)
        check(lib().bf_open_round(self._h, C.byref(rnd), _p(root), _p(poly)))
        return rnd.value, root.tobytes(), poly

    def challenge(self, r) -> None:
        check(lib().bf_open_challenge(self._h, _p(_elems(r, 1))))

    def poll(self) -> bool:
        return check(lib().bf_open_poll(self._h)) == 1

    def final_poly(self) -> np.ndarray:
        out = np.zeros((1, 16), dtype=np.uint8)
        check(lib().bf_open_final(self._h, _p(out)))
        return out

    def finish(self, indices) -> bytes:
        idx = np.ascontiguousarray(np.asarray(indices, dtype=np.uint64))
        size = self._pcs.proof_size(self._comm.width, 1)
        out = np.zeros(size, dtype=np.uint8)
        ln = C.c_size_t()
        check(lib().bf_open_finish(self._h, idx.ctypes.data_as(C.POINTER(C.c_uint64)), idx.size, _p(out), out.size,
                                   C.byref(ln)))
        return out[: ln.value].tobytes()

    def free(self):
        if getattr(self, "_h", None):
            lib().bf_open_session_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def prove(self, challenger: GenericChallenger) -> bytes:
        """Drive every round with `challenger` (the same transcript as Basefold.open)."""
        while True:
            i, root, poly = self.round()
            if i < 0:
                break
            challenger.observe(root)
            challenger.observe_ext_slice(poly)
            self.challenge(challenger.sample_ext_element())
        challenger.observe_ext_slice(self.final_poly())
        L = self._pcs.config.code.log2_c + self._pcs.config.code.d
        idx = [challenger.sample_bits(L) for _ in range(self._pcs.num_queries())]
        return self.finish(idx)


class Engine:
    """Many commit+eval+open jobs of different sizes in flight on one GPU.

    Each job is the reference's harness (commit, observe root, eval at the
    point, observe the value, open with GenericChallenger::keccak256());
    results are identical to Basefold.commit/eval/open one at a time.
    `prove` runs a batch to completion; `start`/`submit`/`poll`/`stop` serve
    requests from a background thread (continuous batching)."""

    def __init__(self, device: int = 0, lambda_: int = 128, log2_c: int = 1, max_inflight: int = 16,
                 mem_budget: int = 0, autotune_reps: int = 0, graphs: bool = False,
                 smallest_first: bool = False, priority_max_vars: int = -1):
        """smallest_first / priority_max_vars: the serving policy (bf_engine_schedule)."""
        h = C.c_void_p()
        check(lib().bf_engine_create(device, lambda_, log2_c, max_inflight, mem_budget, C.byref(h)))
        self._h, self.log2_c = h, log2_c
        self._keep = {}
        if autotune_reps:
            check(lib().bf_engine_autotune(h, autotune_reps))
        check(lib().bf_engine_graphs(h, 1 if graphs else 0))
        check(lib().bf_engine_schedule(h, 1 if smallest_first else 0, priority_max_vars))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                lib().bf_engine_free(h)
            except Exception:
                pass
            self._h = None

    def proof_size(self, num_vars: int) -> int:
        return int(lib().bf_engine_proof_size(self._h, num_vars))

    def set_tune(self, tune: dict) -> None:
        """Launch shapes (Basefold.TUNE_KEYS) for every size (bf_engine_set_tune)."""
        keys = [k for k in Basefold.TUNE_KEYS if k in tune]
        if keys != Basefold.TUNE_KEYS[: len(keys)] or len(keys) < 4:
            raise ValueError(f"tune needs the leading keys of {Basefold.TUNE_KEYS} (at least 4)")
        vals = (C.c_int * len(keys))(*[int(tune[k]) for k in keys])
        check(lib().bf_engine_set_tune(self._h, vals, len(keys)))

    def stats(self) -> dict:
        """Host-side accounting (bf_engine_stats)."""
        v = (C.c_double * 6)()
        check(lib().bf_engine_stats(self._h, v, 6))
        keys = ["host_ms_enqueue", "host_ms_graph_launch", "host_ms_complete", "plans_built", "plans_dropped",
                "jobs_done"]
        return dict(zip(keys, list(v)))

    def _job(self, num_vars, evals, point, device_input):
        job = BfJob()
        job.num_vars = num_vars
        if device_input:
            job.evals = int(evals)
            ev = None
        else:
            ev = _elems(evals, 1 << num_vars)
            job.evals = ev.ctypes.data
        pt = _elems(point, num_vars) if num_vars else np.zeros((1, 16), np.uint8)
        job.point = pt.ctypes.data
        buf = np.zeros(self.proof_size(num_vars), dtype=np.uint8)
        job.proof = buf.ctypes.data
        job.proof_cap = buf.size
        return job, (ev, pt, buf)

    @staticmethod
    def _result(job, keep):
        buf = keep[2]
        return {"status": job.status, "root": bytes(job.root), "value": np.frombuffer(bytes(job.value), np.uint8)
                .reshape(1, 16), "proof": buf[: job.proof_len].tobytes(), "latency_ms": job.latency_ms}

    def prove(self, jobs, device_input: bool = False, raise_on_error: bool = True):
        """jobs: list of (num_vars, evals, point); evals are host arrays or device pointers.
        With raise_on_error False, failed jobs come back with a negative `status`."""
        arr = (BfJob * len(jobs))()
        keeps = []
        for i, (n, ev, pt) in enumerate(jobs):
            job, keep = self._job(n, ev, pt, device_input)
            arr[i] = job
            keeps.append(keep)
        rc = lib().bf_engine_prove(self._h, arr, len(jobs), 1 if device_input else 0)
        if raise_on_error:
            check(rc)
        return [self._result(arr[i], keeps[i]) for i in range(len(jobs))]

    def start(self) -> None:
        check(lib().bf_engine_start(self._h))

    def stop(self) -> None:
        check(lib().bf_engine_stop(self._h))

    def submit(self, num_vars: int, evals, point, device_input: bool = False, tag=None) -> int:
        job, keep = self._job(num_vars, evals, point, device_input)
        key = C.addressof(job)
        self._keep[key] = (job, keep, tag)
        check(lib().bf_engine_submit(self._h, C.byref(job), 1 if device_input else 0))
        return key

    def cancel(self, key) -> bool:
        """Cancel a submitted job (the key `submit` returned) that has not
        started: True if it left the queue (poll then returns it with status
        BF_ERR_CANCELLED), False if it is already running or done."""
        if key not in self._keep:
            return False
        return lib().bf_engine_cancel(self._h, C.c_void_p(key)) == 0

    def poll(self):
        """Finished jobs since the last poll: list of (tag, result)."""
        out = (C.POINTER(BfJob) * 64)()
        n = C.c_size_t()
        res = []
        while True:
            check(lib().bf_engine_poll(self._h, out, 64, C.byref(n)))
            for i in range(n.value):
                key = C.addressof(out[i].contents)
                job, keep, tag = self._keep.pop(key)
                res.append((tag, self._result(job, keep)))
            if n.value < 64:
                return res


def _split_sumcheck(out, k, n):
    rp = out[: n * k].reshape(n, k, 16)
    r = out[n * k: n * k + n]
    fe = out[n * k + n: n * k + n + k]
    return rp, r, fe, out[-1]


def prove_sumcheck(k: int, polys, claim, challenger: GenericChallenger, device: int = 0):
    """prove_sumcheck (sumcheck/src/lib.rs:56-79) of sum_b prod_{j<k} f_j(b), host input.

    Returns (compressed round polys [n, k, 16], challenges [n, 16],
    final evaluations [k, 16], final subclaim [16])."""
    ps = _elems(polys)
    n = int(ps.shape[0] // k).bit_length() - 1
    if (k << n) != ps.shape[0]:
        raise ValueError("polys must hold k arrays of 2^n elements")
    out = np.zeros((n * k + n + k + 1, 16), dtype=np.uint8)
    c = _elems(claim, 1)
    check(lib().bf_sumcheck_prove(device, k, n, _p(ps), _p(c), challenger._h, _p(out)))
    return _split_sumcheck(out, k, n)


def tune_cache_load(path: str) -> int:
    """Merges the tuned launch shapes of a JSON tune file (bf_tune_cache_load);
    every later setup of a matching (device, num_vars, blowup) starts from them."""
    rc = lib().bf_tune_cache_load(os.fsencode(path))
    check(rc)
    return rc


def tune_cache_save(path: str) -> None:
    """Writes every cached (device, num_vars, blowup) -> launch shapes entry."""
    check(lib().bf_tune_cache_save(os.fsencode(path)))


def tune_cache_clear() -> None:
    check(lib().bf_tune_cache_clear())


def device_info(device: int = 0):
    sms, ma, mi = C.c_int(), C.c_int(), C.c_int()
    check(lib().bf_device_info(device, C.byref(sms), C.byref(ma), C.byref(mi)))
    return {"num_sms": sms.value, "cc": (ma.value, mi.value)}


def kernel_launches() -> int:
    """Kernels launched by libbasefold_gpu.so since it was loaded."""
    v = C.c_uint64()
    check(lib().bf_kernel_launches(C.byref(v)))
    return v.value


def test_gf_mul(a, b, device: int = 0) -> np.ndarray:
    a, b = _elems(a), _elems(b)
    out = np.zeros_like(a)
    check(lib().bf_test_gf_mul(device, _p(a), _p(b), _p(out), a.shape[0]))
    return out


def test_keccak_f(states, device: int = 0) -> np.ndarray:
    st = np.ascontiguousarray(states, dtype=np.uint64).copy()
    check(lib().bf_test_keccak_f(device, st.ctypes.data_as(C.POINTER(C.c_uint64)), st.size // 25))
    return st
