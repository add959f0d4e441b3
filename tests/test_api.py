"""The Python mirrors accept the reference's calls: every public method of the
reference classes exists on the mirror, and its parameters start with the
reference's parameters in the same order (the mirrors' additions are
keyword-only or trail with defaults).  The reference side is recorded in
tests/golden/api_signatures.json by tests/golden/make_golden.py."""
import inspect
import json
import os

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _mirrors():
    from pyqed_gb300 import HEOMSolver, Lindblad_solver, LindbladSolver, RedfieldSolver
    return dict(LindbladSolver=LindbladSolver, RedfieldSolver=RedfieldSolver, HEOMSolver=HEOMSolver,
                Lindblad_solver=Lindblad_solver)


def _positional(f):
    return [p.name for p in inspect.signature(f).parameters.values()
            if p.kind in (p.POSITIONAL_ONLY, p.POSITIONAL_OR_KEYWORD)]


@pytest.mark.parametrize("cls", ["LindbladSolver", "RedfieldSolver", "HEOMSolver", "Lindblad_solver"])
def test_mirror_accepts_the_reference_calls(cls):
    with open(os.path.join(HERE, "golden", "api_signatures.json")) as f:
        ref = json.load(f)[cls]
    mine = _mirrors()[cls]
    for name, params in ref.items():
        assert hasattr(mine, name), "%s.%s is missing" % (cls, name)
        if name == "steady_state" and params == []:
            continue  # the reference's takes no self and cannot be called
        got = _positional(getattr(mine, name))
        assert got[:len(params)] == params, (cls, name, params, got)
        extra = [p for p in inspect.signature(getattr(mine, name)).parameters.values()
                 if p.kind in (p.POSITIONAL_ONLY, p.POSITIONAL_OR_KEYWORD)][len(params):]
        assert all(p.default is not p.empty for p in extra), (cls, name, [p.name for p in extra])
