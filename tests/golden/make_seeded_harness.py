"""Generate tests/golden/seeded_harness.json: the reference's own Basefold
test matrix for the binary code (basefold.rs:480-490 over
poly-commit/src/lib.rs:64-105: num_vars 0..9, num_polys 1..9, one point,
blowup 1/2/4) with its inputs drawn as the harness draws them, but from
StdRng::seed_from_u64(SEED) instead of from_entropy: for each case in loop
order, the polynomials (F::random_vec(num_polys << num_vars), row-major with
num_polys columns) and then the point (E::random_vec(num_vars)), one rng for
the whole matrix of one blowup.  Roots, evaluation claims and SHA-256 of the
proofs come from the oracle.  A Rust run of the harness seeded the same way
must reproduce them byte for byte.

Usage:  python tests/golden/make_seeded_harness.py
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


def harness_inputs(seed):
    """(num_vars, num_polys, evals (rows of num_polys), point) in the
    harness's loop order (lib.rs:74-91)."""
    rng = rand.StdRng.seed_from_u64(seed)
    for num_vars in range(10):
        for num_polys in range(1, 10):
            evals = rng.random_elems(num_polys << num_vars)
            point = rng.random_elems(num_vars)
            yield num_vars, num_polys, evals, point


def cases():
    out = []
    for log2_c in (0, 1, 2):
        for n, w, evals, point in harness_inputs(SEED):
            root, values, blob = O.harness_prepare(n, log2_c, evals, point, w)
            proof = O.open_proof(n, log2_c, evals, point, values, blob, w)
            assert O.verify(n, log2_c, root, point, values, blob, proof, w) == 0
            out.append({"log2_c": log2_c, "num_vars": n, "num_polys": w, "root": root.hex(),
                        "values": values.tobytes().hex(), "proof_len": len(proof),
                        "proof_sha256": hashlib.sha256(proof).hexdigest()})
    return out


if __name__ == "__main__":
    doc = {"seed": SEED, "rng": "StdRng::seed_from_u64 (rand 0.8.5: ChaCha12 of rand_chacha 0.3.1, "
                                "seed expansion of rand_core 0.6.4)",
           "order": "per blowup: for num_vars in 0..10, num_polys in 1..10: polys then point",
           "cases": cases()}
    with open(os.path.join(HERE, "seeded_harness.json"), "w") as f:
        json.dump(doc, f, indent=0)
    print(len(doc["cases"]), "cases")
