"""Write tests/golden/known_answers.json from the restated reference tests.

    python tests/golden/make_golden.py

Expected rows come from cases.py's formula-level restatements of thinDB's
integration tests, never from the oracle or the engine.  Pages longer than
100 rows are stored as a row count plus a SHA-256 digest of the canonical
rows (rows_digest) to keep the fixture small.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

import cases  # noqa: E402

OUT = os.path.join(HERE, "known_answers.json")


def canon(v):
    if isinstance(v, float):
        return repr(v)
    return v


def rows_digest(rows) -> str:
    blob = json.dumps([[canon(x) for x in r] for r in rows], separators=(",", ":"))
    return hashlib.sha256(blob.encode()).hexdigest()


def main() -> None:
    out = {}
    for fn in cases.ALL_CASES:
        c = cases.build_case(fn)
        qs = {}
        for q in c.queries:
            e = {"ordered": q.ordered, "tol": q.tol}
            if q.expected is not None:
                e["rows"] = len(q.expected)
                if len(q.expected) <= 100:
                    e["expected"] = [[canon(x) for x in r] for r in q.expected]
                else:
                    e["digest"] = rows_digest(q.expected)
            if q.expected_count is not None:
                e["expected_count"] = q.expected_count
            qs[q.name] = e
        out[c.name] = qs
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
        f.write("\n")
    print("wrote", OUT)


if __name__ == "__main__":
    main()
