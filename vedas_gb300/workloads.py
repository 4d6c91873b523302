"""Seeded synthetic RDF graphs and query workloads for VEDAS.

The reference's WatDiv/LUBM suites are not available, so seeded synthetic
graphs with the stated shapes stand in for them.  ID spaces follow the
reference's loader (src/loader.cu:15, src/vedas.h:31):

* entities (subjects and entity objects) use IDs 1..E,
* predicates use IDs 1..P where ID k is the predicate of frequency rank k,
* literals use IDs LITERAL_START_ID + k (LITERAL_START_ID = 5e7).

Duplicate triples are removed (the graph is an RDF set).  Every generator
uses numpy's PCG64 with an explicit seed, so a configuration always yields
the same bytes.
"""
from __future__ import annotations

import dataclasses
import os
import struct

import numpy as np

LITERAL_START_ID = 50_000_000  # src/vedas.h:31 (5E7)

GRAPH_MAGIC = b"VGRAPH1\0"


@dataclasses.dataclass
class Graph:
    s: np.ndarray  # uint32 subjects
    p: np.ndarray  # uint32 predicates
    o: np.ndarray  # uint32 objects
    name: str = ""

    @property
    def n(self) -> int:
        return int(self.s.shape[0])

    def save(self, path: str) -> None:
        with open(path, "wb") as f:
            f.write(GRAPH_MAGIC)
            f.write(struct.pack("<Q", self.n))
            for a in (self.s, self.p, self.o):
                f.write(np.ascontiguousarray(a, dtype=np.uint32).tobytes())

    @staticmethod
    def load(path: str) -> "Graph":
        with open(path, "rb") as f:
            if f.read(8) != GRAPH_MAGIC:
                raise ValueError(f"{path}: not a graph file")
            (n,) = struct.unpack("<Q", f.read(8))
            arr = np.frombuffer(f.read(12 * n), dtype=np.uint32)
        return Graph(arr[:n].copy(), arr[n:2 * n].copy(), arr[2 * n:].copy(),
                     os.path.basename(path))


def _zipf_probs(k: int, s: float) -> np.ndarray:
    w = 1.0 / np.arange(1, k + 1, dtype=np.float64) ** s
    return w / w.sum()


def _bits(x) -> int:
    m = int(x.max(initial=0))
    return max(1, m.bit_length())


def _dedup(s, p, o, n_target):
    """Remove duplicate triples keeping first occurrences, then cut to n_target."""
    bs, bp, bo = _bits(s), _bits(p), _bits(o)
    if bs + bp + bo <= 64:
        # (p, s, o) packed at their bit widths: injective
        key = (p.astype(np.uint64) << np.uint64(bs + bo)) | (s.astype(np.uint64) << np.uint64(bo)) \
            | o.astype(np.uint64)
        _, first = np.unique(key, return_index=True)
    else:
        rec = np.rec.fromarrays([s, p, o])
        _, first = np.unique(rec, return_index=True)
    first.sort()
    first = first[:n_target]
    return s[first], p[first], o[first]


def graph_small_star(n: int = 1_000_000, n_subjects: int = 50_000, n_predicates: int = 32,
                     zipf_s: float = 1.1, literal_range: int = 200_000, seed: int = 0) -> Graph:
    """The 1M-triple graph of the plain star workload (and scaled-down copies).

    Subjects uniform over [1, n_subjects]; predicates Zipf(zipf_s) over
    n_predicates ranks; objects 70% uniform entities [1, n_subjects] and 30%
    uniform literals [LITERAL_START_ID, LITERAL_START_ID + literal_range).
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    m = int(n * 1.02) + 1024
    s = rng.integers(1, n_subjects + 1, size=m, dtype=np.uint32)
    p = (rng.choice(n_predicates, size=m, p=_zipf_probs(n_predicates, zipf_s)) + 1).astype(np.uint32)
    is_lit = rng.random(m) < 0.30
    ent = rng.integers(1, n_subjects + 1, size=m, dtype=np.uint32)
    lit = rng.integers(LITERAL_START_ID, LITERAL_START_ID + literal_range, size=m, dtype=np.uint32)
    o = np.where(is_lit, lit, ent).astype(np.uint32)
    s, p, o = _dedup(s, p, o, n)
    return Graph(s, p, o, f"star_n{n}")


def graph_chain(n: int = 100_000_000, n_entities: int = 2_000_000, n_predicates: int = 86,
                zipf_s: float = 1.0, mean_degree: float = 3.0, literal_frac: float = 0.30,
                seed: int = 0) -> Graph:
    """The 100M-triple graph of the linear path / batching workloads.

    (subject, predicate) pairs are drawn with subjects uniform over
    [1, n_entities] and predicates Zipf(zipf_s); each pair gets a
    Geometric(1/mean_degree) out-degree, and pairs are taken until n triples
    exist.  Objects are uniform entities (1 - literal_frac) or uniform
    literals in [LITERAL_START_ID, LITERAL_START_ID + n_entities // 10).
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    pairs = int(n / mean_degree * 1.05) + 1024
    ps = rng.integers(1, n_entities + 1, size=pairs, dtype=np.uint32)
    pp = (rng.choice(n_predicates, size=pairs, p=_zipf_probs(n_predicates, zipf_s)) + 1).astype(np.uint32)
    deg = rng.geometric(1.0 / mean_degree, size=pairs).astype(np.int64)
    csum = np.cumsum(deg)
    take = int(np.searchsorted(csum, int(n * 1.01) + 1024)) + 1
    ps, pp, deg = ps[:take], pp[:take], deg[:take]
    s = np.repeat(ps, deg)
    p = np.repeat(pp, deg)
    m = s.shape[0]
    is_lit = rng.random(m) < literal_frac
    ent = rng.integers(1, n_entities + 1, size=m, dtype=np.uint32)
    lit = rng.integers(LITERAL_START_ID, LITERAL_START_ID + max(1, n_entities // 10), size=m,
                       dtype=np.uint32)
    o = np.where(is_lit, lit, ent).astype(np.uint32)
    s, p, o = _dedup(s, p, o, n)
    return Graph(s, p, o, f"chain_n{n}")


# ---------------------------------------------------------------------------
# Query templates: star (S), chain (C) and snowflake (F), 1-8 patterns.
# Placeholders: P<k> a predicate, O<k> an object and S<k> a subject constant.
# instantiate() fills them along a path that exists in the graph, so every
# query has at least one answer.  Variable-only patterns take predicates from
# the rarer half of the ranks to bound result sizes; the globally-last
# predicate is never used (the reference's own lookups read past its index
# there, so no workload sends it).
# ---------------------------------------------------------------------------
TEMPLATES = [
    ("S", "SELECT ?x WHERE { ?x P1 O1 . }"),
    ("S", "SELECT ?o WHERE { S1 P1 ?o . }"),
    ("S", "SELECT * WHERE { ?x P1 ?a . ?x P2 ?b . }"),
    ("S", "SELECT * WHERE { ?x P1 O1 . ?x P2 ?b . }"),
    ("S", "SELECT * WHERE { ?x P1 O1 . ?x P2 ?b . ?x P3 ?c . }"),
    ("S", "SELECT ?x ?c WHERE { ?x P1 ?a . ?x P2 O2 . ?x P3 ?c . }"),
    ("S", "SELECT * WHERE { ?x P1 O1 . ?x P2 ?b . ?x P3 ?c . ?x P4 ?d . }"),
    ("S", "SELECT ?x ?b WHERE { ?x P1 O1 . ?x P2 ?b . ?x P3 ?c . ?x P4 ?d . ?x P5 ?e . }"),
    ("C", "SELECT * WHERE { ?a P1 ?b . ?b P2 O2 . }"),
    ("C", "SELECT * WHERE { S1 P1 ?b . ?b P2 ?c . }"),
    ("C", "SELECT * WHERE { S1 P1 ?b . ?b P2 ?c . ?c P3 ?d . }"),
    ("C", "SELECT * WHERE { ?a P1 ?b . ?b P2 ?c . ?c P3 O3 . }"),
    ("C", "SELECT * WHERE { ?a P1 ?b . ?b P2 ?c . ?c P3 ?d . ?d P4 O4 . }"),
    ("C", "SELECT ?a ?e WHERE { ?a P1 ?b . ?b P2 ?c . ?c P3 ?d . ?d P4 ?e . ?e P5 O5 . }"),
    ("C", "SELECT ?b WHERE { S1 P1 ?b . ?b P2 ?c . ?c P3 ?d . }"),
    ("F", "SELECT * WHERE { ?x P1 O1 . ?x P2 ?y . ?y P3 ?c . ?y P4 ?d . }"),
    ("F", "SELECT * WHERE { ?x P1 O1 . ?x P2 ?a . ?x P3 ?y . ?y P4 ?c . ?y P5 ?d . }"),
    ("F", "SELECT ?x ?y ?d WHERE { ?x P1 O1 . ?x P2 ?a . ?x P3 ?y . ?y P4 ?c . ?y P5 ?d . ?y P6 ?e . }"),
    ("F", "SELECT * WHERE { ?x P1 O1 . ?x P2 ?a . ?x P3 ?b . ?x P4 ?y . ?y P5 ?c . ?y P6 ?d . ?y P7 O7 . }"),
    ("F", "SELECT ?x ?y WHERE { ?x P1 O1 . ?x P2 ?a . ?x P3 ?b . ?x P4 ?y . ?y P5 ?c . ?y P6 ?d . "
          "?y P7 O7 . ?d P8 ?f . }"),
]


def _packed_order(keys: np.ndarray):
    """(sorted keys, original positions) of a uint32 array: a stable sort done
    as one sort of (key << 32 | position) words, several times faster than a
    stable argsort."""
    n = keys.shape[0]
    if n >= (1 << 32):
        order = np.argsort(keys, kind="stable")
        return keys[order], order
    w = (keys.astype(np.uint64) << np.uint64(32)) | np.arange(n, dtype=np.uint64)
    w.sort()
    return (w >> np.uint64(32)).astype(np.uint32), (w & np.uint64(0xFFFFFFFF)).astype(np.uint32)


class ConstantSampler:
    """A graph's triples grouped by predicate, subject and object, for drawing
    query constants along paths that exist in the graph."""

    def __init__(self, g: Graph):
        self.g = g
        self.p_sorted, self.p_pos = _packed_order(g.p)
        self.preds = np.unique(self.p_sorted)
        self.start = np.searchsorted(self.p_sorted, self.preds, side="left")
        self.end = np.searchsorted(self.p_sorted, self.preds, side="right")
        self.count = {int(p): int(e - b) for p, b, e in zip(self.preds, self.start, self.end)}
        self.span = {int(p): (int(b), int(e)) for p, b, e in zip(self.preds, self.start, self.end)}
        self._by_s = None
        self._by_o = None

    def usable_predicates(self):
        return [int(p) for p in self.preds[:-1]]   # never the last predicate id

    def by_subject(self):
        if self._by_s is None:
            self._by_s = _packed_order(self.g.s)
        return self._by_s

    def by_object(self):
        if self._by_o is None:
            self._by_o = _packed_order(self.g.o)
        return self._by_o

    def out_edges(self, node: int):
        """Positions of the triples whose subject is `node`."""
        keys, pos = self.by_subject()
        k = np.uint32(node)      # a uint32 key: a Python int would convert the whole array
        return pos[keys.searchsorted(k, "left"):keys.searchsorted(k, "right")]

    def in_edges(self, node: int):
        """Positions of the triples whose object is `node`."""
        keys, pos = self.by_object()
        k = np.uint32(node)
        return pos[keys.searchsorted(k, "left"):keys.searchsorted(k, "right")]

    def has_out(self, node: int) -> bool:
        keys, _ = self.by_subject()
        i = keys.searchsorted(np.uint32(node), "left")
        return bool(i < keys.shape[0] and keys[i] == node)

    def has_in(self, node: int) -> bool:
        keys, _ = self.by_object()
        i = keys.searchsorted(np.uint32(node), "left")
        return bool(i < keys.shape[0] and keys[i] == node)

    def triple_of(self, rng, p: int) -> int:
        """Position of a uniformly drawn triple of predicate p."""
        b, e = self.span[p]
        return int(self.p_pos[rng.integers(b, e)])

    def obj(self, rng, p: int) -> int:
        return int(self.g.o[self.triple_of(rng, p)])

    def subj(self, rng, p: int) -> int:
        return int(self.g.s[self.triple_of(rng, p)])


def _patterns(template: str):
    body = template.split("{", 1)[1].rsplit("}", 1)[0]
    return [tuple(t.strip().rstrip(" .").split()) for t in body.split(" . ") if t.strip()]


def _walk_order(pats):
    """Pattern order for a walk: each pattern after the first shares a
    variable with one placed before it (the templates are trees)."""
    order, seen = [0], {v for v in (pats[0][0], pats[0][2]) if v.startswith("?")}
    while len(order) < len(pats):
        for i, (s, _, o) in enumerate(pats):
            if i not in order and (s in seen or o in seen):
                order.append(i)
                seen.update(v for v in (s, o) if v.startswith("?"))
                break
        else:
            raise ValueError("template patterns are not connected")
    return order


_TRIES_PER_EDGE = 64
_TRIES_PER_QUERY = 200


def _walk(pats, cs: ConstantSampler, rng, pools):
    """One embedding of the patterns in the graph: a triple for every
    pattern, consistent on shared variables, found by a random walk from a
    random triple of the first pattern.  pools[i] is the set of predicates
    pattern i may use.  Returns {pattern: triple position} or None."""
    g = cs.g
    order = _walk_order(pats)
    subj_of = {}
    obj_of = {}
    for i, (s, _, o) in enumerate(pats):
        if s.startswith("?"):
            subj_of.setdefault(s, []).append(i)
        if o.startswith("?"):
            obj_of.setdefault(o, []).append(i)

    def fits(i, t, assign):
        """Triple t for pattern i: its predicate is allowed and every variable
        it binds afresh can continue the walk (edges out of it where a later
        pattern has it as subject, edges into it where as object)."""
        if int(g.p[t]) not in pools[i]:
            return False
        s, _, o = pats[i]
        for v, node in ((s, int(g.s[t])), (o, int(g.o[t]))):
            if not v.startswith("?"):
                continue
            if v in assign:
                if assign[v] != node:
                    return False
                continue
            if any(j != i for j in subj_of.get(v, ())) and not cs.has_out(node):
                return False
            if any(j != i for j in obj_of.get(v, ())) and not cs.has_in(node):
                return False
        if s.startswith("?") and s == o and int(g.s[t]) != int(g.o[t]):
            return False
        return True

    def pick(i, cand, assign, taken):
        """A fitting triple among cand, preferring a predicate that no
        placed pattern at the same variable uses (stars then look like the
        benchmark suites' ones: one predicate per branch)."""
        m = cand.shape[0]
        if m == 0:
            return None
        idx = rng.permutation(m)[:_TRIES_PER_EDGE] if m <= 4 * _TRIES_PER_EDGE \
            else rng.integers(0, m, size=_TRIES_PER_EDGE)
        second = None
        for k in idx:
            t = int(cand[k])
            if fits(i, t, assign):
                if int(g.p[t]) not in taken:
                    return t
                if second is None:
                    second = t
        return second

    for _ in range(_TRIES_PER_QUERY):
        assign, chosen = {}, {}
        for i in order:
            s, _, o = pats[i]
            if s in assign:
                taken = {int(g.p[chosen[j]]) for j in chosen if pats[j][0] == s}
                t = pick(i, cs.out_edges(assign[s]), assign, taken)
            elif o in assign:
                taken = {int(g.p[chosen[j]]) for j in chosen if pats[j][2] == o}
                t = pick(i, cs.in_edges(assign[o]), assign, taken)
            else:
                pool = sorted(pools[i])
                t = None
                for _ in range(_TRIES_PER_EDGE):
                    p = pool[rng.integers(0, len(pool))]
                    c = cs.triple_of(rng, p)
                    if fits(i, c, assign):
                        t = c
                        break
            if t is None:
                break
            chosen[i] = t
            if s.startswith("?"):
                assign[s] = int(g.s[t])
            if o.startswith("?"):
                assign[o] = int(g.o[t])
        else:
            return chosen
    return None


def instantiate(template: str, cs: ConstantSampler, rng) -> str:
    """Fills a template's placeholders along a path of the graph: every
    pattern gets the predicate and constants of one triple, and the triples
    agree on every shared variable, so the query has at least that answer.
    Patterns whose ends are both variables take predicates from the rarer
    half of the ranks, which bounds result sizes; the globally-last predicate
    is never used (the reference's own lookups read past its index there, so
    no workload sends it)."""
    preds = cs.usable_predicates()
    rare = set(preds[len(preds) // 2:] or preds)
    every = set(preds)
    pats = _patterns(template)
    pools = [rare if (s.startswith("?") and o.startswith("?")) else every for s, _, o in pats]
    chosen = _walk(pats, cs, rng, pools)
    if chosen is None:
        # no embedding found: constants drawn per pattern (may have no answer)
        chosen = {i: cs.triple_of(rng, sorted(pools[i])[rng.integers(0, len(pools[i]))])
                  for i in range(len(pats))}
    out = template
    g = cs.g
    for i in sorted(chosen, key=lambda i: -int(pats[i][1][1:])):
        k = pats[i][1][1:]
        t = chosen[i]
        out = out.replace(f"O{k}", f"<{int(g.o[t])}>").replace(f"S{k}", f"<{int(g.s[t])}>")
        out = out.replace(f"P{k}", f"<{int(g.p[t])}>")
    return out


def query_mix(g: Graph, n_queries: int, seed: int = 0, cs: ConstantSampler | None = None,
              mix=None):
    """n_queries instantiated templates, round-robin over the 20 templates (or
    drawn with the given per-shape weights, e.g. {"S": .6, "C": .3, "F": .1})."""
    rng = np.random.Generator(np.random.PCG64(seed))
    cs = cs or ConstantSampler(g)
    out = []
    if mix is None:
        for i in range(n_queries):
            out.append(instantiate(TEMPLATES[i % len(TEMPLATES)][1], cs, rng))
        return out
    shapes = list(mix)
    w = np.array([mix[s] for s in shapes], dtype=np.float64)
    w /= w.sum()
    by_shape = {s: [t for sh, t in TEMPLATES if sh == s] for s in shapes}
    for _ in range(n_queries):
        sh = shapes[rng.choice(len(shapes), p=w)]
        ts = by_shape[sh]
        out.append(instantiate(ts[rng.integers(0, len(ts))], cs, rng))
    return out


def graph_hub(n: int = 500_000_000, n_entities: int = 10_000_000, n_predicates: int = 86,
              zipf_s: float = 1.0, mean_degree: float = 3.0, hub_frac: float = 0.01,
              hub_share: float = 0.3, alpha: float = 2.1, literal_frac: float = 0.2,
              seed: int = 0, dedup: bool = True) -> Graph:
    """The 500M-triple graph of the large-query and serving workloads.

    Like graph_chain, plus heavy-tailed in-degree: hub_frac of the entities
    are hubs that receive hub_share of all object slots, hub k of rank r with
    weight r^(-1/(alpha-1)) (a power law of in-degree with exponent alpha).
    Remaining objects are literal_frac literals and uniform entities.
    dedup=False keeps repeated triples, as the reference's loader does
    (src/loader.cu:19-53); it spares the 500M-element host sort.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    pairs = int(n / mean_degree * 1.03) + 1024
    ps = rng.integers(1, n_entities + 1, size=pairs, dtype=np.uint32)
    pp = (rng.choice(n_predicates, size=pairs, p=_zipf_probs(n_predicates, zipf_s)) + 1).astype(np.uint32)
    deg = rng.geometric(1.0 / mean_degree, size=pairs).astype(np.int64)
    csum = np.cumsum(deg)
    take = int(np.searchsorted(csum, int(n * 1.005) + 1024)) + 1
    s = np.repeat(ps[:take], deg[:take])
    p = np.repeat(pp[:take], deg[:take])
    del ps, pp, deg, csum
    m = s.shape[0]
    n_hubs = max(1, int(n_entities * hub_frac))
    hubs = (rng.choice(n_entities, size=n_hubs, replace=False) + 1).astype(np.uint32)
    w = np.arange(1, n_hubs + 1, dtype=np.float64) ** (-1.0 / (alpha - 1.0))
    w /= w.sum()
    u = rng.random(m, dtype=np.float32)
    o = rng.integers(1, n_entities + 1, size=m, dtype=np.uint32)
    lit = u >= 1.0 - literal_frac
    o[lit] = rng.integers(LITERAL_START_ID, LITERAL_START_ID + max(1, n_entities // 10),
                          size=int(lit.sum()), dtype=np.uint32)
    hub = u < hub_share
    o[hub] = hubs[rng.choice(n_hubs, size=int(hub.sum()), p=w)]
    del u, lit, hub
    if dedup:
        s, p, o = _dedup(s, p, o, n)
    else:
        s, p, o = s[:n], p[:n], o[:n]
    return Graph(s, p, o, f"hub_n{n}")


# Predicates of the large single query on the 500M-triple hub graph: stars
# (p4, p8, p11) at ?x and (p6, p9, p10) at ?y joined by ?x p1 ?y.  On that
# graph the reference's plan builds intermediate relations of up to about
# 1.6e8 rows and a result of about 4.6e8 rows x 8 columns (measured with the
# oracle on the same generator at 50M triples, where every size is a tenth).
C3_SNOWFLAKE = (4, 8, 11, 1, 6, 9, 10)


def snowflake_query(preds=(1, 2, 3, 4, 5, 6, 7)) -> str:
    """Seven-pattern snowflake: two three-pattern stars (?x, ?y) joined by one
    object-subject edge (?x p4 ?y), with preds = (a, b, c, d, e, f, g) giving
    ?x a/b/c, ?x d ?y and ?y e/f/g."""
    a, b, c, d, e, f, g = preds
    return (f"SELECT * WHERE {{ ?x <{a}> ?a . ?x <{b}> ?b . ?x <{c}> ?c . ?x <{d}> ?y . "
            f"?y <{e}> ?e . ?y <{f}> ?f . ?y <{g}> ?g . }}")


def star_query(pa: int = 3, pb: int = 7) -> str:
    """Two-pattern subject-subject star: (?x pa ?a . ?x pb ?b), SELECT *."""
    return f"SELECT * WHERE {{ ?x <{pa}> ?a . ?x <{pb}> ?b . }}"


def chain_query_open(preds=(1, 2, 5, 9)) -> str:
    """The same four-pattern chain with its end a variable too
    (?a p1 ?b . ?b p2 ?c . ?c p5 ?d . ?d p9 ?e): on the 100M-triple chain
    graph the reference's plan re-sorts relations of millions of rows twice
    (two index swaps) and returns about 7e7 rows."""
    a, b, c, d = preds
    return f"SELECT * WHERE {{ ?a <{a}> ?b . ?b <{b}> ?c . ?c <{c}> ?d . ?d <{d}> ?e . }}"


def chain_query(g: Graph, preds=(1, 2, 5, 9), seed: int = 0, cs: ConstantSampler | None = None) -> str:
    """Four-pattern chain (?a p1 ?b . ?b p2 ?c . ?c p5 ?d . ?d p9 c), where c
    is the end of a four-hop path p1, p2, p5, p9 that exists in the graph (so
    the query has at least one answer)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    cs = cs or ConstantSampler(g)
    a, b, cc, d = preds
    pats = [("?a", "P1", "?b"), ("?b", "P2", "?c"), ("?c", "P3", "?d"), ("?d", "P4", "O4")]
    chosen = _walk(pats, cs, rng, [{a}, {b}, {cc}, {d}])
    if chosen is None:
        c = cs.obj(rng, d)
    else:
        c = int(g.o[chosen[3]])
    return (f"SELECT * WHERE {{ ?a <{a}> ?b . ?b <{b}> ?c . ?c <{cc}> ?d . "
            f"?d <{d}> <{c}> . }}")


def to_ntriples(g: Graph, blank_every: int = 97, lang_every: int = 5) -> bytes:
    """The graph as N-Triples text, one statement per line in triple order.

    Entities are IRIs <http://example.org/eNNNNNNNNNN>, except ids with
    id % blank_every == 7, which are blank nodes _:bNNNNNNNNNN; predicates
    are <http://example.org/pNNNNNNNNNN>; objects with ids from
    LITERAL_START_ID are literals "vNNNNNNNNNN", every lang_every-th of them
    tagged @en.  Every line is 101 bytes (terms padded with spaces), so the
    text is built with array arithmetic."""
    n = g.n
    W = 101
    buf = np.full((n, W), ord(" "), dtype=np.uint8)
    s = g.s.astype(np.uint64)
    p = g.p.astype(np.uint64)
    o = g.o.astype(np.uint64)

    def put(rows, col, text: bytes):
        buf[rows, col:col + len(text)] = np.frombuffer(text, dtype=np.uint8)

    def digits(rows, col, vals):
        v = vals.copy()
        for k in range(9, -1, -1):
            buf[rows, col + k] = (48 + v % 10).astype(np.uint8)
            v //= 10

    def entity(col, ids):
        blank = (ids % blank_every) == 7
        iri = ~blank
        put(iri, col, b"<http://example.org/e")
        digits(iri, col + 21, ids[iri])
        buf[iri, col + 31] = ord(">")
        put(blank, col, b"_:b")
        digits(blank, col + 3, ids[blank])

    entity(0, s)
    put(slice(None), 33, b"<http://example.org/p")
    digits(slice(None), 54, p)
    buf[:, 64] = ord(">")
    lit = o >= LITERAL_START_ID
    ent_rows = np.nonzero(~lit)[0]
    if ent_rows.size:
        # entity objects at column 66
        ids = o[ent_rows]
        blank = (ids % blank_every) == 7
        iri_r, blank_r = ent_rows[~blank], ent_rows[blank]
        put(iri_r, 66, b"<http://example.org/e")
        digits(iri_r, 87, ids[~blank])
        buf[iri_r, 97] = ord(">")
        put(blank_r, 66, b"_:b")
        digits(blank_r, 69, ids[blank])
    lit_rows = np.nonzero(lit)[0]
    if lit_rows.size:
        put(lit_rows, 66, b'"v')
        digits(lit_rows, 68, o[lit_rows])
        buf[lit_rows, 78] = ord('"')
        tagged = lit_rows[(o[lit_rows] % lang_every) == 0]
        put(tagged, 79, b"@en")
    buf[:, 99] = ord(".")
    buf[:, 100] = ord("\n")
    return buf.tobytes()
