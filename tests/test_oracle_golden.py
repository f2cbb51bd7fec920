"""The oracle against the reference's known answers (CPU; pins the oracle)."""
import pytest

import cases
import oracle
from helpers import check_known_answer, load_known_answers

KNOWN = load_known_answers()


@pytest.mark.parametrize("case_fn", cases.ALL_CASES, ids=[f.__name__ for f in cases.ALL_CASES])
@pytest.mark.parametrize("threads", [1, 4])
def test_oracle_known_answers(case_fn, threads):
    c = case_fn()
    t = oracle.HostTable(c.columns, c.row_group_rows)
    for q in c.queries:
        res = oracle.run(t, q.request, threads=threads)
        check_known_answer(c, q, KNOWN[c.name][q.name], res)


def test_golden_fixture_is_current():
    """known_answers.json matches what make_golden.py derives from the formulas."""
    from helpers import rows_digest

    for fn in cases.ALL_CASES:
        c = cases.build_case(fn)
        for q in c.queries:
            e = KNOWN[c.name][q.name]
            if q.expected is not None:
                assert e["rows"] == len(q.expected)
                if "digest" in e:
                    assert e["digest"] == rows_digest(q.expected)
