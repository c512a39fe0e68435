"""Generate tests/golden/exhaustive36_golden.json: the full answer of the
n = 36 exhaustive-search workload (dense QUBO, integer coefficients U{-8..8},
2^36 states) for seeds 0, 1 and 2.

Each answer is the oracle's own scan of all 2^36 states on the host cores
(oracle.exhaustive_int_all: every state's energy evaluated on its own, exact
in int64), never the GPU library: the ground energy, the reference's answer
(the smallest minimising state, exhaustive.hpp:130-133,158-166), the number
of degenerate minimisers and all of them. It takes about fifteen minutes per
seed on eight cores.

Usage: python tests/golden/make_exhaustive36.py [seed ...]
"""
from __future__ import annotations

import json
import sys
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import oracle  # noqa: E402
from qubo_text import random_int_qubo  # noqa: E402

OUT = HERE / "exhaustive36_golden.json"


def main(seeds: list[int]) -> None:
    oracle.build()
    data = json.loads(OUT.read_text()) if OUT.exists() else {}
    for seed in seeds:
        f = random_int_qubo(36, seed)
        t0 = time.time()
        e, count, states = oracle.exhaustive_int_all(f, cap=1 << 16)
        entry = {
            "n": 36, "seed": seed, "lo": -8, "hi": 8,
            "energy": e, "state": int(states[0]), "count": count,
            "states": [int(s) for s in states],
            "scan_seconds": round(time.time() - t0, 1),
        }
        data[str(seed)] = entry
        OUT.write_text(json.dumps(data, indent=1, sort_keys=True) + "\n")
        print(f"seed {seed}: E = {e}, state {entry['state']}, count {count} ({entry['scan_seconds']} s)",
              flush=True)


if __name__ == "__main__":
    main([int(a) for a in sys.argv[1:]] or [0, 1, 2])
