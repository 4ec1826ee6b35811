"""Writes oracle_proofs.json: SHA-256 of the oracle's NARG string and hints for a few small WHIR
configurations, a regression pin of the transcript bytes (which the GPU prover must reproduce)."""

import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))

import oracle as orc  # noqa: E402
from test_oracle_pins import make_statement  # noqa: E402

CASES = [
    {"field": "Goldilocks2", "nv": 10, "points": 1, "seed": 1, "session": "fixture a",
     "params": {"unique_decoding": True, "security_level": 60, "pow_bits": 8, "initial_folding_factor": 4,
                "folding_factor": 4}, "hash": "ENGINE_BLAKE3"},
    {"field": "Goldilocks3", "nv": 9, "points": 2, "seed": 2, "session": "fixture b",
     "params": {"unique_decoding": False, "security_level": 40, "pow_bits": 5, "initial_folding_factor": 3,
                "folding_factor": 2}, "hash": "ENGINE_SHA3"},
    {"field": "Goldilocks1", "nv": 8, "points": 0, "seed": 3, "session": "fixture c",
     "params": {"unique_decoding": True, "security_level": 32, "pow_bits": 0, "initial_folding_factor": 2,
                "folding_factor": 2}, "hash": "ENGINE_SHA2"},
]


def main():
    out = {"cases": []}
    for c in CASES:
        hid = getattr(orc, c["hash"])
        p = orc.make_params(**c["params"], hash_id=hid)
        f, vecs, pts, covs, evals = make_statement(orc, c["field"], c["nv"], c["points"], 1, 1, False, seed=c["seed"])
        pr = orc.whir_prove(f, p, c["nv"], c["session"], vecs, pts, covs, evals)
        e = dict(c)
        e.pop("hash")
        e["hash_id"] = hid.hex()
        e["narg_sha256"] = hashlib.sha256(pr.narg).hexdigest()
        e["hints_sha256"] = hashlib.sha256(pr.hints).hexdigest()
        out["cases"].append(e)
    with open(os.path.join(HERE, "oracle_proofs.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
