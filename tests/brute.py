"""Brute-force counts straight from the definitions (test helper).

For a literal, a binding row b and a relation tuple r join when every bound
argument k has R[k][r] == B[vars[k]][b].  binding counts = joining pairs per
label; covered counts = binding rows per label with at least one pair.
Independent of the reference's algorithm; used for small cases only.
"""
import collections

import numpy as np


def brute_counts(relations, binding_columns, num_positive, literals):
    B = [np.asarray(c) for c in binding_columns]
    n = len(B[0]) if B else 0
    out = np.zeros((len(literals), 4), dtype=np.int64)
    for i, lit in enumerate(literals):
        rid, vars_, _ = lit.as_tuple() if hasattr(lit, "as_tuple") else lit
        R = relations[rid]
        bound = [k for k in range(len(vars_)) if vars_[k] >= 0]
        cnt = collections.Counter(zip(*[np.asarray(R[k]).tolist() for k in bound]))
        if n == 0:
            continue
        keys = list(zip(*[B[vars_[k]].tolist() for k in bound]))
        m = np.fromiter((cnt.get(t, 0) for t in keys), dtype=np.int64, count=n)
        pos = np.arange(n) < num_positive
        out[i, 0] = np.count_nonzero(m[pos])
        out[i, 1] = np.count_nonzero(m[~pos])
        out[i, 2] = m[pos].sum()
        out[i, 3] = m[~pos].sum()
    return out
