"""Generate the committed golden fixtures under tests/golden/.

1. reference_polyval.json — constants read as text out of the reference's own
   sources (needs the reference checkout; run in the build container):
     * the x^256 mod P constant of p3/src/polyval/portable.rs:12
       (from_canonical multiplies by it);
     * POLYVAL_NIBBLE_POW_2_N_TABLE (portable.rs:169-376), where
       value[i][k][j] = from_canonical(j << 4k) ^ (2^(2<<i)); rows i = 0 and
       i = 5 are kept (1024 entries).
2. oracle_vectors.json — seeded regression vectors produced by the oracle:
   commitment roots, evaluation claims and SHA-256 of the serialized proofs
   for small Basefold configurations, plus product-sumcheck outputs.  Inputs
   come from the SplitMix64 generator of basefold_gpu.rand with the seed
   listed beside each case.

Usage:  python tests/golden/make_golden.py [--reference /path/to/learn-zkp]
        (or LEARN_ZKP_REFERENCE=/path/to/learn-zkp); without a reference
        checkout only oracle_vectors.json is regenerated.
"""
import argparse
import hashlib
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "learn-zkp_gb300"))

from oracle import oracle as O  # noqa: E402
from basefold_gpu import rand  # noqa: E402


def reference_constants(ref_root):
    src = open(os.path.join(ref_root, "p3/src/polyval/portable.rs")).read()
    m = re.search(r"montgomery_multiply\(a, (0x[0-9a-f]+)\)", src)
    r2 = m.group(1)
    body = src[src.index("POLYVAL_NIBBLE_POW_2_N_TABLE: [[[u128; 16]; 32]; 6] = ["):]
    nums = re.findall(r"0x[0-9a-f]+", body)
    assert len(nums) >= 6 * 32 * 16
    table = [[[nums[(i * 32 + k) * 16 + j] for j in range(16)] for k in range(32)] for i in range(6)]
    return {
        "source": "p3/src/polyval/portable.rs",
        "r2_line": 12,
        "r2": r2,
        "table_lines": "169-376",
        "table_definition": "value[i][k][j] = from_canonical(j << 4k).exp_power_of_2(2 << i)",
        "table_rows": {"0": table[0], "5": table[5]},
    }


def basefold_cases():
    cases = []
    for (n, log2_c, width, seed) in [(0, 1, 1, 11), (1, 1, 1, 12), (4, 1, 1, 13), (8, 1, 1, 14), (10, 1, 1, 15),
                                     (6, 0, 1, 16), (6, 2, 1, 17), (5, 1, 3, 18), (12, 1, 1, 19), (16, 1, 1, 0)]:
        data = rand.random_elems((width << n) + n, seed)
        evals, point = data[: width << n], data[width << n:]
        root, values, blob = O.harness_prepare(n, log2_c, evals, point, width)
        proof = O.open_proof(n, log2_c, evals, point, values, blob, width)
        assert O.verify(n, log2_c, root, point, values, blob, proof, width) == 0
        cases.append({
            "n": n, "log2_c": log2_c, "width": width, "seed": seed,
            "inputs": "random_elems(width*2^n + n, seed): evaluations first, then the point",
            "root": root.hex(),
            "values": [bytes(v).hex() for v in values],
            "proof_len": len(proof),
            "proof_sha256": hashlib.sha256(proof).hexdigest(),
        })
    return cases


def sumcheck_cases():
    cases = []
    for (k, n, seed) in [(2, 0, 30), (2, 1, 31), (2, 8, 32), (3, 1, 33), (3, 8, 34), (2, 12, 35), (3, 12, 36)]:
        polys = rand.random_elems(k << n, seed)
        claim = rand.random_elems(1, seed + 1000)  # the prover does not check the claim
        blob = O.challenger_blob(bytes(range(32)))
        rp, r, fe, fc = O.sumcheck_prove(k, n, polys, claim, blob)
        cases.append({
            "k": k, "n": n, "seed": seed, "claim_seed": seed + 1000,
            "initial_state": bytes(range(32)).hex(),
            "round_polys_sha256": hashlib.sha256(rp.tobytes()).hexdigest(),
            "challenges_sha256": hashlib.sha256(r.tobytes()).hexdigest(),
            "final_evals": [bytes(v).hex() for v in fe],
            "final_claim": bytes(fc).hex(),
        })
    return cases


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("LEARN_ZKP_REFERENCE"),
                    help="learn-zkp checkout to read constants from (default: $LEARN_ZKP_REFERENCE)")
    args = ap.parse_args()
    if args.reference and os.path.isdir(args.reference):
        with open(os.path.join(HERE, "reference_polyval.json"), "w") as f:
            json.dump(reference_constants(args.reference), f, indent=1)
    vec = {"basefold": basefold_cases(), "sumcheck": sumcheck_cases()}
    with open(os.path.join(HERE, "oracle_vectors.json"), "w") as f:
        json.dump(vec, f, indent=1)


if __name__ == "__main__":
    main()
