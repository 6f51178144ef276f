"""CPU tests of the host-side literal helpers in quickfoil_gb300/engine.py.

join_key restates FoilLiteral::UpdateJoinKey (schema/FoilLiteral.hpp:133-140):
the join argument is the bound argument with the largest variable type id,
the first one on ties.  Literal.to_c fills the C ABI's qfg_literal exactly
as include/qfgpu.h describes it (unused argument slots -1).
"""
import pytest

from quickfoil_gb300 import _capi as C
from quickfoil_gb300.engine import Literal, join_key


def test_join_key_takes_the_first_bound_argument_without_types():
    assert join_key((-1, 3, 0)) == 1
    assert join_key((2, -1, 5)) == 0


def test_join_key_prefers_the_largest_type_and_the_first_on_ties():
    assert join_key((0, 1, 2), var_types=(1, 3, 2)) == 1
    assert join_key((0, 1, 2), var_types=(2, 2, 2)) == 0
    assert join_key((-1, 1, 2), var_types=(9, 1, 1)) == 1  # unbound arguments never join


def test_join_key_needs_a_bound_argument():
    with pytest.raises(ValueError):
        join_key((-1, -1))


def test_literal_to_c_fills_every_field():
    lit = Literal(7, (-1, 4, 2))
    assert lit.join_pos == 1
    s = lit.to_c()
    assert (s.relation_id, s.num_args, s.join_pos) == (7, 3, 1)
    assert list(s.vars)[:3] == [-1, 4, 2]
    assert all(v == -1 for v in list(s.vars)[3:])
    assert len(list(s.vars)) == C.MAX_ARITY
    assert lit.as_tuple() == (7, [-1, 4, 2], 1)


def test_literal_keeps_an_explicit_join_position():
    assert Literal(3, (0, 1), 1).join_pos == 1
