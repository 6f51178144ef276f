"""Readers of the golden fixtures (produced by make_golden.py from the
reference's own code)."""
from __future__ import annotations

import os

import numpy as np

from quickfoil_gb300.engine import Literal

HERE = os.path.dirname(os.path.abspath(__file__))


def unpack_relations(z, prefix):
    rels = []
    for i in range(int(z[f"{prefix}num"][0])):
        cols = []
        k = 0
        while f"{prefix}{i}_{k}" in z:
            cols.append(z[f"{prefix}{i}_{k}"])
            k += 1
        rels.append(cols)
    return rels


def unpack_literals(a):
    lits = []
    for row in a:
        vars_ = []
        for v in row[2:]:
            if v == -2:
                break
            vars_.append(int(v))
        lits.append(Literal(int(row[0]), tuple(vars_), int(row[1])))
    return lits


def eval_cases():
    """[(relations, binding_columns, num_positive, literals, reference counts)]"""
    z = np.load(os.path.join(HERE, "eval_cases.npz"))
    out = []
    for i in range(int(z["num_cases"][0])):
        nb, P = (int(v) for v in z[f"c{i}_meta"])
        out.append((unpack_relations(z, f"c{i}_r"), [z[f"c{i}_b{k}"] for k in range(nb)], P,
                    unpack_literals(z[f"c{i}_lits"]), z[f"c{i}_counts"]))
    return out


def kinship():
    return learn_trace("kinship")


def bongard():
    return learn_trace("bongard")


def learn_trace(name):
    """(relations, calls, clauses) of a learn-loop fixture; calls are
    ("evaluate", join_var, binding_columns, P, literals, counts) and
    ("extend", (npos, nneg), binding_columns, P, [literal], output_columns)."""
    z = np.load(os.path.join(HERE, f"{name}.npz"))
    rels = unpack_relations(z, "r")
    calls = []
    for j in range(int(z["num_calls"][0])):
        ncols, P = (int(v) for v in z[f"k{j}_meta"])
        cols = [z[f"k{j}_b{k}"] for k in range(ncols)]
        lits = unpack_literals(z[f"k{j}_lits"])
        if int(z[f"k{j}_kind"][0]) == 0:
            calls.append(("evaluate", int(z[f"k{j}_key"][0]), cols, P, lits, z[f"k{j}_counts"]))
        else:
            nout = int(z[f"k{j}_nout"][0])
            calls.append(("extend", tuple(int(v) for v in z[f"k{j}_key"]), cols, P, lits,
                          [z[f"k{j}_out{k}"] for k in range(nout)]))
    return rels, calls, [str(c) for c in z["clauses"]]


def input_checksum(w):
    """Order-sensitive checksums of a workload's binding columns and relations
    (one per column, below 2^61)."""
    def col_sum(c):
        c = np.asarray(c, dtype=np.int64)
        return int((c * (np.arange(len(c), dtype=np.int64) % 1000003 + 1)).sum() % (1 << 61))
    return [col_sum(c) for c in w.binding_columns] + [col_sum(c) for r in w.relations for c in r]


def batched_step_reference():
    """(distinct literals, reference counts, input checksums) of the full-size
    batched step (32M x 6 bindings, 32 relations, 256 literals)."""
    z = np.load(os.path.join(HERE, "batched_step_reference.npz"))
    return unpack_literals(z["lits"]), z["counts"], [int(v) for v in z["checksum"]]
