"""The reference learner's literal score, computed from the four counts.

Restates LiteralSelector::Insert's scoring (learner/LiteralSelector.cpp:
47-68) with ComputeMccScore and ComputeAreaUnderEntropyCurve
(learner/LiteralSelector.hpp:236-281) in double precision, so that scores of
GPU counts can be compared with the reference's choices.  The learner itself
stays on the reference side; this is for checking and reporting only.
"""
from __future__ import annotations

import math
from typing import Optional, Sequence


def area_under_entropy_curve(num_positive: int, num_negative: int) -> float:
    if num_positive == 0:
        return 0.0
    if num_negative == 0:
        return 1.0
    p = num_positive / (num_positive + num_negative)
    return ((1 - p) * (1 - p) * math.log2(1 - p) - p * p * math.log2(p)) * math.log(2) + p


def mcc_score(covered_pos: int, covered_neg: int, clause_pos: int, clause_neg: int) -> float:
    if covered_pos == 0:
        return -1.0  # deviates from the true MCC, as the reference does
    if covered_pos == clause_pos and covered_neg == clause_neg:
        return 0.0
    true_neg = clause_neg - covered_neg
    false_neg = clause_pos - covered_pos
    covered = covered_pos + covered_neg
    return (covered_pos * true_neg - covered_neg * false_neg) / math.sqrt(
        covered * ((clause_pos + clause_neg) - covered) * clause_neg * clause_pos)


def literal_score(counts: Sequence[int], clause_pos: int, clause_neg: int) -> Optional[float]:
    """Score of a literal with counts (covered+, covered-, binding+, binding-)
    on a clause with clause_pos / clause_neg bindings; None when the reference
    excludes it (an MCC or entropy term of 0)."""
    cp, cn, bp, bn = (int(c) for c in counts)
    mcc = 1 + mcc_score(cp, cn, clause_pos, clause_neg)
    auec = 1 + (area_under_entropy_curve(bp, bn) - area_under_entropy_curve(clause_pos, clause_neg))
    if mcc == 0 or auec == 0:
        return None
    return 5 * auec * mcc / (mcc + 4 * auec)
