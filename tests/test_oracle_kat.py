"""The CPU oracle against the known-answer cases of lala-pc's PIR tests
(tests/pir_test.cpp, transcribed in tests/golden/kat_cases.py)."""
import pytest

from golden import kat_cases as K
from kat_runner import OracleEngine, run_case


@pytest.mark.parametrize("case", K.CASES, ids=[c.name for c in K.CASES])
def test_kat_oracle(case, oracle):
    assert run_case(case, OracleEngine) == []


def test_kat_count():
    # every PIRTest of tests/pir_test.cpp except the three set/element
    # decompositions (ReifiedIn, ElementConstraint1, InConstraint1) and the
    # exhaustive ones (covered in test_oracle_props.py)
    assert len(K.CASES) >= 70


def test_kat_runner_detects_mismatch(oracle):
    import copy
    case = copy.deepcopy([c for c in K.CASES if c.name == "IntTDiv1"][0])
    case.steps[0].after = [(2, 10), (-20, 25), (-2, 3)]  # the EDIV answer; TDIV gives -21
    assert run_case(case, OracleEngine)
