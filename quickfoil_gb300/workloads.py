"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No external dataset is involved; every array is generated from a fixed seed
so the GPU engine and the CPU oracle see identical int32 columns.

* ``single_literal``  -- one candidate literal over a 16M x 4 binding set
  (10% positive) and a 4M-tuple relation r(A, B) with A uniform over
  [0, 1M) (or Zipf s=1.1); the literal binds binding column 2 to A.
* ``batched_step``    -- one refinement step: a 32M x 6 binding set (10%
  positive, uniform over a 2M domain), 32 relations of arity 1-3 with
  log-uniform tuple counts in [1K, 8M] and Zipf s=1.1 keys over the 2M
  domain, and 256 candidate literals with random bound/unbound arguments.

Binding columns are uniform over the key domain, which keeps every count
below 2^31 (the reference counts in int32).  Zipf keys are drawn by inverse
CDF of P(k) ~ k^-s over k = 1..D followed by a seeded permutation of the
domain, so frequent keys are scattered over the value range.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List

import numpy as np

from .engine import Literal


class Zipf:
    """Finite-domain Zipf sampler: values in [0, domain)."""

    def __init__(self, domain: int, s: float, rng: np.random.Generator):
        k = np.arange(1, domain + 1, dtype=np.float64)
        w = k ** (-s)
        self.cdf = np.cumsum(w)
        self.cdf /= self.cdf[-1]
        self.perm = rng.permutation(domain).astype(np.int32)

    def sample(self, n: int, rng: np.random.Generator) -> np.ndarray:
        u = rng.random(n)
        idx = np.searchsorted(self.cdf, u, side="left")
        np.minimum(idx, len(self.cdf) - 1, out=idx)
        return self.perm[idx]


@dataclass
class Workload:
    name: str
    binding_columns: List[np.ndarray]
    num_positive: int
    relations: List[List[np.ndarray]]   # relation id = index
    literals: List[Literal]
    domain: int

    @property
    def num_bindings(self) -> int:
        return len(self.binding_columns[0])

    def relation_tuples(self) -> int:
        return sum(len(r[0]) for r in self.relations)


def uniform_bindings(n: int, ncols: int, domain: int, rng) -> List[np.ndarray]:
    return [rng.integers(0, domain, n, dtype=np.int32) for _ in range(ncols)]


def single_literal(n_bindings: int = 16_000_000, n_relation: int = 4_000_000,
                   domain: int = 1_000_000, zipf: bool = False, seed: int = 2) -> Workload:
    rng = np.random.default_rng(seed)
    B = uniform_bindings(n_bindings, 4, domain, rng)
    if zipf:
        A = Zipf(domain, 1.1, rng).sample(n_relation, rng)
    else:
        A = rng.integers(0, domain, n_relation, dtype=np.int32)
    Bcol = rng.integers(0, domain, n_relation, dtype=np.int32)
    lit = Literal(0, (2, -1), 0)
    return Workload("single_literal" + ("_zipf" if zipf else ""), B, n_bindings // 10, [[A, Bcol]],
                    [lit], domain)


def random_literals(num: int, relations, ncols: int, rng) -> List[Literal]:
    """Random relation, random bound/unbound arguments with at least one bound
    argument (learner/CandidateLiteralEnumerator.cpp:75,151 never emits an
    all-unbound literal); bound arguments get random clause variables.  All
    arguments share one type, so the join key is the first bound argument."""
    out = []
    for _ in range(num):
        rid = int(rng.integers(0, len(relations)))
        arity = len(relations[rid])
        while True:
            bound = rng.random(arity) < 0.5
            if bound.any():
                break
        vars_ = tuple(int(rng.integers(0, ncols)) if b else -1 for b in bound)
        out.append(Literal(rid, vars_))
    return out


def batched_step(n_bindings: int = 32_000_000, ncols: int = 6, num_relations: int = 32,
                 min_tuples: int = 1_000, max_tuples: int = 8_000_000, num_literals: int = 256,
                 domain: int = 2_000_000, seed: int = 3) -> Workload:
    rng = np.random.default_rng(seed)
    B = uniform_bindings(n_bindings, ncols, domain, rng)
    relations = []
    for _ in range(num_relations):
        arity = int(rng.integers(1, 4))
        n = int(np.exp(rng.uniform(np.log(min_tuples), np.log(max_tuples))))
        z = Zipf(domain, 1.1, rng)
        relations.append([z.sample(n, rng) for _ in range(arity)])
    lits = random_literals(num_literals, relations, ncols, rng)
    return Workload("batched_step", B, n_bindings // 10, relations, lits, domain)


def small_random(seed: int, n_bindings: int = 3000, ncols: int = 4, num_relations: int = 5,
                 max_tuples: int = 2000, num_literals: int = 40, domain: int = 300,
                 zipf: bool = True) -> Workload:
    """Small mixed case for parity tests (runs through the oracle in ms)."""
    rng = np.random.default_rng(seed)
    B = uniform_bindings(n_bindings, ncols, domain, rng)
    relations = []
    for _ in range(num_relations):
        arity = int(rng.integers(1, 4))
        n = int(rng.integers(1, max_tuples + 1))
        if zipf:
            z = Zipf(domain, 1.1, rng)
            relations.append([z.sample(n, rng) for _ in range(arity)])
        else:
            relations.append([rng.integers(0, domain, n, dtype=np.int32) for _ in range(arity)])
    lits = random_literals(num_literals, relations, ncols, rng)
    P = int(rng.integers(0, n_bindings + 1))
    return Workload(f"small_random_{seed}", B, P, relations, lits, domain)


@dataclass
class LearnTask:
    name: str
    relations: List[List[np.ndarray]]   # background relations, id = index
    relation_names: List[str]
    target_columns: List[np.ndarray]    # positives first
    num_positive: int
    max_clause_length: int


def kinship(seed: int = 1, persons: int = 200, generations: int = 4, max_positive: int = 60,
            num_negative: int = 600) -> LearnTask:
    """Kinship knowledge base: `persons` ids split evenly over `generations`
    generations and over male/female; every person outside the first
    generation has a father and a mother in the previous generation, so
    parent(person, person) forms a random forest of that depth.  sibling(X, Y)
    holds for X != Y sharing a parent.  The target uncle(X, Y) =
    male(X) & sibling(X, Z) & parent(Z, Y): up to `max_positive` positive
    pairs sampled from that rule and `num_negative` pairs drawn uniformly from
    the other ordered pairs."""
    rng = np.random.default_rng(seed)
    ids = rng.permutation(persons).astype(np.int32)
    per_gen = persons // generations
    gens = [ids[g * per_gen:(g + 1) * per_gen] for g in range(generations)]
    male, female, parent = [], [], []
    for g, people in enumerate(gens):
        half = len(people) // 2
        male.extend(people[:half].tolist())
        female.extend(people[half:].tolist())
        if g == 0:
            continue
        fathers = gens[g - 1][:len(gens[g - 1]) // 2]
        mothers = gens[g - 1][len(gens[g - 1]) // 2:]
        for child in people:
            parent.append((int(rng.choice(fathers)), int(child)))
            parent.append((int(rng.choice(mothers)), int(child)))
    parents_of = {}
    for p, c in parent:
        parents_of.setdefault(c, set()).add(p)
    children_of = {}
    for p, c in parent:
        children_of.setdefault(p, set()).add(c)
    sibling = sorted({(x, y) for p, cs in children_of.items() for x in cs for y in cs if x != y})
    male_set = set(male)
    uncle = sorted({(x, y) for (x, z) in sibling if x in male_set for y in children_of.get(z, ())})
    pos_idx = rng.permutation(len(uncle))[:max_positive]
    positives = [uncle[i] for i in sorted(pos_idx)]
    uncle_set = set(uncle)
    negatives = set()
    while len(negatives) < num_negative:
        x, y = (int(v) for v in rng.integers(0, persons, 2))
        if x != y and (x, y) not in uncle_set:
            negatives.add((x, y))
    negatives = sorted(negatives)
    cols = lambda pairs, k: np.array([p[k] for p in pairs], dtype=np.int32)
    relations = [[cols(parent, 0), cols(parent, 1)],
                 [np.array(sorted(male), dtype=np.int32)],
                 [np.array(sorted(female), dtype=np.int32)],
                 [cols(sibling, 0), cols(sibling, 1)]]
    target = positives + negatives
    return LearnTask("kinship", relations, ["parent", "male", "female", "sibling"],
                     [cols(target, 0), cols(target, 1)], len(positives), 3)


def bongard(seed: int = 1, pictures: int = 300, mean_objects: float = 10.0,
            inside_per_object: float = 2.0, max_positive: int = 100,
            max_clause_length: int = 4) -> LearnTask:
    """Bongard-like knowledge base (the planted-rule learn loop, scaled down):
    `pictures` picture ids and object ids in disjoint ranges (one argument
    type, as the learner sees them); element(picture, object) with
    Poisson(mean_objects) objects per picture; circle/triangle/square(object)
    unary, each object one shape uniformly; inside(object, object) random
    ordered pairs of distinct objects of the same picture, about
    `inside_per_object` per object.  The target pos(picture) holds for the
    pictures with a circle inside a triangle: up to `max_positive` of them
    are positives, every other picture is a negative."""
    rng = np.random.default_rng(seed)
    counts = rng.poisson(mean_objects, pictures)
    counts = np.maximum(counts, 1)
    obj_pic = np.repeat(np.arange(pictures), counts)
    nobj = len(obj_pic)
    obj_ids = (pictures + np.arange(nobj)).astype(np.int32)
    shape = rng.integers(0, 3, nobj)
    starts = np.concatenate([[0], np.cumsum(counts)[:-1]])
    inside = set()
    for p in range(pictures):
        c = int(counts[p])
        if c < 2:
            continue
        m = int(rng.poisson(inside_per_object * c))
        for _ in range(m):
            a, b = rng.integers(0, c, 2)
            if a != b:
                inside.add((int(obj_ids[starts[p] + a]), int(obj_ids[starts[p] + b])))
    inside = sorted(inside)
    shape_of = {int(o): int(s) for o, s in zip(obj_ids, shape)}
    pic_of = {int(o): int(p) for o, p in zip(obj_ids, obj_pic)}
    hit = sorted({pic_of[a] for a, b in inside if shape_of[a] == 0 and shape_of[b] == 1})
    pos = set(int(v) for v in rng.permutation(hit)[:max_positive])
    positives = sorted(pos)
    hit_set = set(hit)
    negatives = [p for p in range(pictures) if p not in hit_set]
    cols = lambda pairs, k: np.array([x[k] for x in pairs], dtype=np.int32)
    element = [(int(p), int(o)) for p, o in zip(obj_pic, obj_ids)]
    relations = [[cols(element, 0), cols(element, 1)],
                 [obj_ids[shape == 0].copy()],
                 [obj_ids[shape == 1].copy()],
                 [obj_ids[shape == 2].copy()],
                 [cols(inside, 0), cols(inside, 1)]]
    target = np.array(positives + negatives, dtype=np.int32)
    return LearnTask("bongard", relations, ["element", "circle", "triangle", "square", "inside"],
                     [target], len(positives), max_clause_length)


def bongard_kb(seed: int = 4, pictures: int = 1_000_000, mean_objects: float = 10.0,
               inside_per_object: float = 2.0, max_positive: int = 100_000,
               max_clause_length: int = 4) -> LearnTask:
    """The Bongard-like knowledge base of the full-scale learn loop, generated
    with array operations (seconds for a million pictures): the rules of
    `bongard` -- Poisson(mean_objects) objects per picture (at least one),
    one of three shapes per object uniformly, Poisson(inside_per_object x
    objects) ordered within-picture object pairs per picture with pairs of an
    object with itself dropped and repeats merged, positives = up to
    `max_positive` pictures with a circle inside a triangle, negatives =
    every picture without one -- drawn in a different order, so its knowledge
    base differs from `bongard`'s for the same seed.  At the defaults:
    element 10M, inside about 16M tuples, 100K positives."""
    rng = np.random.default_rng(seed)
    counts = np.maximum(rng.poisson(mean_objects, pictures), 1).astype(np.int64)
    obj_pic = np.repeat(np.arange(pictures, dtype=np.int64), counts)
    nobj = len(obj_pic)
    obj_ids = (pictures + np.arange(nobj)).astype(np.int32)
    shape = rng.integers(0, 3, nobj)
    starts = np.concatenate([[0], np.cumsum(counts)[:-1]])
    m = rng.poisson(inside_per_object * counts)
    m[counts < 2] = 0
    pair_pic = np.repeat(np.arange(pictures, dtype=np.int64), m)
    c = counts[pair_pic]
    a = (rng.random(len(pair_pic)) * c).astype(np.int64)
    b = (rng.random(len(pair_pic)) * c).astype(np.int64)
    keep = a != b
    ga = starts[pair_pic[keep]] + a[keep]
    gb = starts[pair_pic[keep]] + b[keep]
    code = np.unique(ga * nobj + gb)  # sorted by (a, b): object ids grow with the index
    ia, ib = code // nobj, code % nobj
    hit = np.unique(obj_pic[ia[(shape[ia] == 0) & (shape[ib] == 1)]])
    pos = np.sort(rng.permutation(hit)[:max_positive])
    is_hit = np.zeros(pictures, dtype=bool)
    is_hit[hit] = True
    neg = np.nonzero(~is_hit)[0]
    relations = [[obj_pic.astype(np.int32), obj_ids],
                 [obj_ids[shape == 0].copy()],
                 [obj_ids[shape == 1].copy()],
                 [obj_ids[shape == 2].copy()],
                 [obj_ids[ia], obj_ids[ib]]]
    target = np.concatenate([pos, neg]).astype(np.int32)
    return LearnTask("bongard_kb", relations, ["element", "circle", "triangle", "square", "inside"],
                     [target], len(pos), max_clause_length)


def facts_text(columns) -> bytes:
    """int32 columns as '|'-delimited lines, one fact a line (the fact-file
    format of the reference's loader), built with numpy: every value's
    decimal digits are written at offsets from a prefix sum of the field
    widths."""
    cols = [np.asarray(c, dtype=np.int64) for c in columns]
    n = len(cols[0]) if cols else 0
    if n == 0:
        return b""
    widths = []
    for c in cols:
        mag = np.abs(c)
        digits = np.ones(n, dtype=np.int64)
        t = mag // 10
        while t.any():
            digits += t > 0
            t //= 10
        widths.append(digits + (c < 0))
    line_len = sum(widths) + len(cols)  # separators and the newline
    start = np.concatenate([[0], np.cumsum(line_len)[:-1]])
    out = np.empty(int(line_len.sum()), dtype=np.uint8)
    pos = start.copy()
    for q, (c, w) in enumerate(zip(cols, widths)):
        neg = c < 0
        out[pos[neg]] = ord("-")
        mag = np.abs(c)
        end = pos + w  # one past the last digit
        k = 0
        while True:
            live = w - neg > k
            if not live.any():
                break
            out[end[live] - 1 - k] = (ord("0") + (mag[live] // 10 ** k) % 10).astype(np.uint8)
            k += 1
        out[end] = ord("|") if q + 1 < len(cols) else ord("\n")
        pos = end + 1
    return out.tobytes()
