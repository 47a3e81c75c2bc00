"""Generate tests/golden/seeded_harness_bb.json: the reference's prime-field
Basefold tests (poly-commit/src/basefold.rs:453-478 over
poly-commit/src/lib.rs:64-105) with their inputs drawn as the harness draws
them, but from StdRng::seed_from_u64(SEED) instead of from_entropy, one rng
per run_basefold call:
  * reed_solomon_code: log2_c in 0..3; for num_vars in 0..10, num_polys in
    1..10: the polys (BabyBear::random_vec(num_polys << num_vars), row-major
    with num_polys columns), then the point
    (BinomialExtensionField<BabyBear, 5>::random_vec(num_vars));
  * generic_random_foldable_code: (log2_c, log2_k_0) in (0..3) x (0..3),
    log2_k_0 capped at num_vars; per case first the code's t's
    (BabyBear::random_vec(n_0 << i) for i in 0..d, drawn by
    reed_solomon_g_0_with_random_ts), then the polys, then the point.
Roots, evaluation claims and SHA-256 of the proofs come from the oracle; a
Rust run of those tests seeded the same way must reproduce them byte for
byte.

Usage:  python tests/golden/make_seeded_harness_bb.py
"""
import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "learn-zkp_gb300"))

from oracle import oracle as O  # noqa: E402
from basefold_gpu import rand  # noqa: E402

SEED = 0
# one row per case; the values' and the proof's SHA-256 are truncated to 64 and 128 bits
COLS = ["code", "log2_c", "log2_k0", "num_vars", "num_polys", "root", "values_sha256_64", "proof_len",
        "proof_sha256_128"]


def harness_inputs(seed, log2_c, log2_k0=None):
    """(num_vars, num_polys, log2_k0, ts, evals, point) in the harness's loop
    order; ts is None for the Reed-Solomon code."""
    rng = rand.StdRng.seed_from_u64(seed)
    for num_vars in range(10):
        for num_polys in range(1, 10):
            ts = None
            lk = 0
            if log2_k0 is not None:
                lk = min(log2_k0, num_vars)
                d = num_vars - lk
                n0 = 1 << (log2_c + lk)
                ts = [rng.random_babybear(n0 << i) for i in range(d)]
                ts = __import__("numpy").concatenate(ts) if ts else __import__("numpy").zeros(0, "uint32")
            evals = rng.random_babybear(num_polys << num_vars).reshape(-1, num_polys)
            point = rng.random_babybear_ext(num_vars)
            yield num_vars, num_polys, lk, ts, evals, point


def case(code, log2_c, log2_k0_cfg, n, w, lk, ts, evals, point):
    kw = {} if ts is None else {"log2_k0": lk, "ts": ts}
    root, values, blob = O.bb_harness_prepare(n, log2_c, evals, point, **kw)
    proof = O.bb_open(n, log2_c, evals, point, values, blob, **kw)
    assert O.bb_verify(n, log2_c, root, point, values, blob, proof, **kw) == 0
    return [code, log2_c, log2_k0_cfg, n, w, root.hex(), hashlib.sha256(values.tobytes()).hexdigest()[:16],
            len(proof), hashlib.sha256(proof).hexdigest()[:32]]


def cases():
    out = []
    for log2_c in range(3):
        for n, w, lk, ts, evals, point in harness_inputs(SEED, log2_c):
            out.append(case("reed_solomon", log2_c, None, n, w, lk, ts, evals, point))
    for log2_c in range(3):
        for log2_k0 in range(3):
            for n, w, lk, ts, evals, point in harness_inputs(SEED, log2_c, log2_k0):
                out.append(case("generic", log2_c, log2_k0, n, w, lk, ts, evals, point))
    return out


if __name__ == "__main__":
    doc = {"seed": SEED, "rng": "StdRng::seed_from_u64 (rand 0.8.5: ChaCha12 of rand_chacha 0.3.1, "
                                "seed expansion of rand_core 0.6.4)",
           "order": "per run_basefold call: for num_vars in 0..10, num_polys in 1..10: [ts], polys, point",
           "cols": COLS, "cases": cases()}
    with open(os.path.join(HERE, "seeded_harness_bb.json"), "w") as f:
        f.write(json.dumps({k: v for k, v in doc.items() if k != "cases"})[:-1] + ', "cases": [\n')
        f.write(",\n".join(json.dumps(c, separators=(",", ":")) for c in doc["cases"]))
        f.write("\n]}\n")
    print(len(doc["cases"]), "cases")
