"""Prime-field Basefold on the GPU: the reference's PolyCommitScheme
instantiated as

    Basefold<BabyBear, BinomialExtensionField<BabyBear, 5>,
             ReedSolomonCode<BabyBear>, Keccak256MerkleTreeMmcs<BabyBear>>

(poly-commit/src/basefold.rs, poly-commit/src/basefold/code/reed_solomon.rs,
poly-commit/benches/poly-commit.rs:44-58).

Values: a BabyBear is its canonical value (< p = 15 * 2^27 + 1) as uint32;
an extension element is five uint32 coefficients (of 1, X, .., X^4 with
X^5 = 2), so points are (num_vars, 5) arrays and values (width, 5).
Evaluations are 2^num_vars rows of `width` columns, row-major (1-D for
width 1).  The transcript is the package's GenericChallenger: its byte
buffer is the same for both fields; observe_ext_slice / sample_ext_element
below handle BabyBear elements as GenericChallenger<BabyBear, _> does.
All computation runs in libbasefold_gpu.so; there is no CPU fallback.
"""
import ctypes as C

import numpy as np

from ._native import check, lib
from . import BasefoldConfig, BasefoldError, GenericChallenger

P = 2013265921

__all__ = [
    "P", "ReedSolomonCode", "GenericRandomFoldableCode", "BasefoldConfig", "PrimePolyEvals", "PrimeCommitmentData", "BabyBearBasefold",
    "observe_ext_slice", "sample_ext_element",
]


def _p(a: np.ndarray):
    return C.c_void_p(a.ctypes.data)


def _ext(x, n=None) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(x, dtype=np.uint32)).reshape(-1, 5)
    if n is not None and a.shape[0] != n:
        raise ValueError(f"expected {n} extension elements, got {a.shape[0]}")
    return a


def observe_ext_slice(ch: GenericChallenger, elems) -> None:
    """FieldChallengerExt::observe_ext_slice (p3/src/challenger.rs:11-14):
    each coefficient's 4 canonical bytes."""
    ch.observe(_ext(elems).tobytes())


def sample_ext_element(ch: GenericChallenger) -> np.ndarray:
    """CanSample<BinomialExtensionField<BabyBear, 5>> (challenger.rs:62-74)."""
    out = np.zeros(5, dtype=np.uint32)
    check(lib().bf_challenger_sample_bb_ext(ch._h, _p(out)))
    return out


class ReedSolomonCode:
    """ReedSolomonCode::new(lambda, log2_c, d) (reed_solomon.rs:19-39)."""

    def __init__(self, lambda_: int, log2_c: int, d: int):
        self.lambda_, self.log2_c, self.d = lambda_, log2_c, d

    def c(self) -> int:
        return 1 << self.log2_c

    def n_d(self) -> int:
        return self.c() << self.d


class GenericRandomFoldableCode:
    """GenericRandomFoldableCode::reed_solomon_g_0_with_random_ts(lambda,
    log2_c, log2_k_0, d, rng) (generic.rs:43-71) with the random vectors
    given: `ts` holds ts[0], .., ts[d-1] back to back (n_0 << i nonzero
    canonical BabyBears each, n_0 = 2^(log2_c + log2_k_0))."""

    def __init__(self, lambda_: int, log2_c: int, log2_k_0: int, d: int, ts):
        self.lambda_, self.log2_c, self.log2_k_0, self.d = lambda_, log2_c, log2_k_0, d
        self.ts = np.ascontiguousarray(np.asarray(ts, dtype=np.uint32)).reshape(-1)

    @property
    def num_vars(self) -> int:
        return self.log2_k_0 + self.d

    def n_0(self) -> int:
        return 1 << (self.log2_c + self.log2_k_0)


class PrimePolyEvals:
    """PolyEvals { values, point } (poly-commit/src/lib.rs:14-18) over E."""

    def __init__(self, values, point):
        self.values = _ext(values)
        self.point = _ext(point) if len(point) else np.zeros((0, 5), np.uint32)


class PrimeCommitmentData:
    """BasefoldCommitmentData: device-resident evaluations, codeword and tree."""

    def __init__(self, pcs, handle, root: bytes, width: int, keep=None):
        self._pcs, self._h, self.root, self.width, self._keep = pcs, handle, root, width, keep

    def as_ref(self) -> bytes:
        return self.root

    def free(self):
        if self._h:
            lib().bf_bb_commitment_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class BabyBearBasefold:
    """PolyCommitScheme<BabyBear, BinomialExtensionField<BabyBear, 5>> with the Reed–Solomon code."""

    def __init__(self, handle, config: BasefoldConfig, device: int):
        self._h, self.config, self.device = handle, config, device

    @classmethod
    def setup(cls, config: BasefoldConfig, device: int = 0, stream=None) -> "BabyBearBasefold":
        h = C.c_void_p()
        code = config.code
        st = C.c_void_p(stream) if stream else None
        if isinstance(code, GenericRandomFoldableCode):
            ts = code.ts if code.ts.size else np.zeros(1, np.uint32)
            check(lib().bf_bb_pcs_setup_generic(device, code.lambda_, code.log2_c, code.log2_k_0, code.num_vars,
                                                _p(ts), code.ts.size, st, C.byref(h)))
        else:
            check(lib().bf_bb_pcs_setup(device, code.lambda_, code.log2_c, code.d, st, C.byref(h)))
        return cls(h, config, device)

    @property
    def num_vars(self) -> int:
        code = self.config.code
        return code.num_vars if isinstance(code, GenericRandomFoldableCode) else code.d

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                lib().bf_bb_pcs_free(h)
            except Exception:
                pass
            self._h = None

    def num_queries(self) -> int:
        return int(lib().bf_bb_pcs_num_queries(self._h))

    def proof_size(self, width: int = 1, n_evals: int = 1) -> int:
        return int(lib().bf_bb_pcs_proof_size(self._h, width, n_evals))

    def _rows(self) -> int:
        return 1 << self.num_vars

    def commit(self, data) -> PrimeCommitmentData:
        """commit (basefold.rs:112-120) of host evaluations: 2^d rows x width.
        A 4-byte integer array is passed as it lies (no copy), so pinned
        buffers keep their fast copy path."""
        d = np.asarray(data)
        d = d.view(np.uint32) if d.dtype in (np.int32, np.uint32) else d.astype(np.uint32)
        d = np.ascontiguousarray(d)
        width = d.size // self._rows()
        if width == 0 or width * self._rows() != d.size:
            raise ValueError(f"{d.size} evaluations is not a multiple of 2^{self.num_vars} rows")
        h = C.c_void_p()
        root = np.zeros(32, dtype=np.uint8)
        check(lib().bf_bb_commit(self._h, _p(d), width, C.byref(h), _p(root)))
        return PrimeCommitmentData(self, h, root.tobytes(), width)

    def commit_device(self, dev_ptr: int, width: int = 1, keep=None) -> PrimeCommitmentData:
        """commit of evaluations in device memory (kept by reference, not copied)."""
        h = C.c_void_p()
        root = np.zeros(32, dtype=np.uint8)
        check(lib().bf_bb_commit_device(self._h, C.c_void_p(dev_ptr), width, C.byref(h), _p(root)))
        return PrimeCommitmentData(self, h, root.tobytes(), width, keep=keep)

    def _point(self, point) -> np.ndarray:
        d = self.num_vars
        return _ext(point, d) if d else np.zeros((1, 5), np.uint32)

    def eval(self, data, point) -> np.ndarray:
        """eval (basefold.rs:126-131): the (width, 5) column values at the
        point, of a commitment's device-resident evaluations or of host rows
        that have no commitment (copied in, evaluated on the GPU)."""
        if isinstance(data, PrimeCommitmentData):
            out = np.zeros((data.width, 5), dtype=np.uint32)
            check(lib().bf_bb_eval(self._h, data._h, _p(self._point(point)), _p(out)))
            return out
        d = np.asarray(data)
        d = np.ascontiguousarray(d.view(np.uint32) if d.dtype in (np.int32, np.uint32) else d.astype(np.uint32))
        width = d.size // self._rows()
        if width == 0 or width * self._rows() != d.size:
            raise ValueError(f"{d.size} evaluations is not a multiple of 2^{self.num_vars} rows")
        out = np.zeros((width, 5), dtype=np.uint32)
        check(lib().bf_bb_eval_data(self._h, _p(d), 0, width, _p(self._point(point)), _p(out)))
        return out

    def eval_device(self, dev_ptr: int, point, width: int = 1) -> np.ndarray:
        """eval of device-resident rows (2^num_vars x width canonical words) with no commitment."""
        out = np.zeros((width, 5), dtype=np.uint32)
        check(lib().bf_bb_eval_data(self._h, C.c_void_p(dev_ptr), 1, width, _p(self._point(point)), _p(out)))
        return out

    def open(self, comm: PrimeCommitmentData, evals, challenger: GenericChallenger) -> bytes:
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
            pt, vals = self._point(evals[0].point), _ext(evals[0].values, comm.width)
            check(lib().bf_bb_open(self._h, comm._h, _p(pt), _p(vals), 1, challenger._h, _p(out), out.size,
                                   C.byref(ln)))
        else:
            check(lib().bf_bb_open(self._h, comm._h, None, None, 0, challenger._h, _p(out), out.size, C.byref(ln)))
        return out[: ln.value].tobytes()

    def verify(self, comm: bytes, evals, proof: bytes, challenger: GenericChallenger) -> None:
        """verify (basefold.rs:234-324) on the host; raises BasefoldError on rejection."""
        root = np.frombuffer(bytes(comm), dtype=np.uint8).copy()
        pf = np.frombuffer(bytes(proof), dtype=np.uint8).copy() if proof else np.zeros(1, np.uint8)
        if len(evals):
            pt, vals = self._point(evals[0].point), _ext(evals[0].values)
            rc = lib().bf_bb_verify(self._h, _p(root), _p(pt), _p(vals), vals.shape[0], 1, challenger._h, _p(pf),
                                    len(proof))
        else:
            rc = lib().bf_bb_verify(self._h, _p(root), None, None, 1, 0, challenger._h, _p(pf), len(proof))
        check(rc)
        if rc != 0:
            raise BasefoldError(rc)
