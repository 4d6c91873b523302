"""N-Triples ingest on the device equals the loader's rules (the oracle):
ids, columns and dictionaries, with and without a literal dictionary, when
hash collisions force the exact path, and end to end into a query."""
import numpy as np
import pytest

from oracle import oracle_py
from vedas_gb300 import workloads

pytestmark = pytest.mark.gpu


def _same(ing, ref):
    s, p, o, d = ref
    cols = ing.columns()
    np.testing.assert_array_equal(cols[0], s)
    np.testing.assert_array_equal(cols[1], p)
    np.testing.assert_array_equal(cols[2], o)
    assert ing.dict.terms("so") == d["so"]
    assert ing.dict.terms("p") == d["p"]
    assert ing.dict.terms("l") == d["l"]


@pytest.mark.parametrize("literal_dict", [False, True])
def test_ingest_matches_loader_rules(ctx, literal_dict):
    import vedas_gb300 as vg
    g = workloads.graph_chain(n=300_000, n_entities=40_000, seed=21)
    text = workloads.to_ntriples(g)
    # comments, blank lines and a CRLF line between statements
    text = b"# header\n\n" + text[:101 * 1000] + b"<x> <y> \"z\"@en .\r\n" + text[101 * 1000:]
    ing = vg.ingest_ntriples(ctx, text, literal_dict=literal_dict)
    assert ing.n == g.n + 1
    _same(ing, oracle_py.ingest_ntriples(text, literal_dict))
    ing.free()


def test_ingest_hash_collisions_resolved_exactly(ctx):
    import vedas_gb300 as vg
    g = workloads.graph_small_star(n=50_000, n_subjects=4_000, seed=22)
    text = workloads.to_ntriples(g)
    vg.set_ingest_hash_bits(6)          # 64 hash values: every dictionary collides
    try:
        ing = vg.ingest_ntriples(ctx, text, literal_dict=True)
    finally:
        vg.set_ingest_hash_bits(63)
    _same(ing, oracle_py.ingest_ntriples(text, True))
    ing.free()


def test_ingest_reports_malformed_line(ctx):
    import vedas_gb300 as vg
    g = workloads.graph_small_star(n=5_000, n_subjects=500, seed=23)
    lines = workloads.to_ntriples(g).split(b"\n")
    lines[56] = b"<a> <b> oops ."
    text = b"\n".join(lines)
    with pytest.raises(vg.VgError, match="line 57"):
        vg.ingest_ntriples(ctx, text)
    with pytest.raises(ValueError, match="line 57$"):
        oracle_py.ingest_ntriples(text)


def test_ingested_columns_build_the_index_and_answer_queries(ctx, tmp_path):
    import vedas_gb300 as vg
    g = workloads.graph_chain(n=200_000, n_entities=20_000, seed=24)
    text = workloads.to_ntriples(g)
    ing = vg.ingest_ntriples(ctx, text)
    s, p, o, d = oracle_py.ingest_ntriples(text)
    ix = ing.index()
    ref = oracle_py.OracleIndex(s, p, o)
    for name in ("pso_data", "pos_data", "p_idx_values", "ps_s_idx_values"):
        np.testing.assert_array_equal(ix.array(name), ref.array(name))
    # a star query written with IRIs, mapped through the dictionary
    p1, p2 = ing.dict.lookup("p", "<http://example.org/p0000000001>"), \
        ing.dict.lookup("p", "<http://example.org/p0000000002>")
    assert p1 and p2
    q = f"SELECT * WHERE {{ ?x <{p1}> ?a . ?x <{p2}> ?b . }}"
    r, rr = ix.query(q), ref.query(q)
    for a, b in zip(r.columns(), rr.columns):
        np.testing.assert_array_equal(a, b)
    # the dictionary survives a .vdd round trip
    path = str(tmp_path / "g.vdd")
    ing.dict.write(path)
    d2 = vg.Dict.open(path)
    assert d2.terms("so") == d["so"] and d2.terms("p") == d["p"]
    r.close()
    ix.close()
    ing.free()


def test_iri_queries_and_decoded_results(ctx):
    """Queries written with IRIs and literals go through the dictionary as the
    reference's TriplePattern maps them; results decode back to terms."""
    import vedas_gb300 as vg
    g = workloads.graph_chain(n=200_000, n_entities=20_000, seed=25)
    text = workloads.to_ntriples(g)
    ing = vg.ingest_ntriples(ctx, text, literal_dict=True)
    s, p, o, d = oracle_py.ingest_ntriples(text, True)
    ix = ing.index()
    ix.set_dict(ing.dict)
    ref = oracle_py.OracleIndex(s, p, o)
    so_id = {t: i + 1 for i, t in enumerate(d["so"])}
    p_id = {t: i + 1 for i, t in enumerate(d["p"])}
    l_id = {t: i + 50_000_000 for i, t in enumerate(d["l"])}
    P1, P2 = "<http://example.org/p0000000001>", "<http://example.org/p0000000002>"
    # an entity object and an untagged literal that occur with P1
    rows = np.nonzero(p == p_id[P1])[0]
    ent = next(d["so"][o[r] - 1] for r in rows if o[r] < 50_000_000)
    lit = next(d["l"][o[r] - 50_000_000] for r in rows if o[r] >= 50_000_000 and "@" not in d["l"][o[r] - 50_000_000])
    cases = [
        (f"SELECT * WHERE {{ ?x {P1} ?a . ?x {P2} ?b . }}",
         f"SELECT * WHERE {{ ?x <{p_id[P1]}> ?a . ?x <{p_id[P2]}> ?b . }}"),
        (f"SELECT ?x WHERE {{ ?x {P1} {ent} . }}", f"SELECT ?x WHERE {{ ?x <{p_id[P1]}> <{so_id[ent]}> . }}"),
        (f"SELECT ?x WHERE {{ ?x {P1} {lit} . }}", f"SELECT ?x WHERE {{ ?x <{p_id[P1]}> <{l_id[lit]}> . }}"),
        # Rasqal keeps only the literal's text: the tag is dropped before the lookup
        (f"SELECT ?x WHERE {{ ?x {P1} {lit}@en . }}", f"SELECT ?x WHERE {{ ?x <{p_id[P1]}> <{l_id[lit]}> . }}"),
        # an absent IRI is id 0, which matches nothing
        (f"SELECT ?x WHERE {{ ?x {P1} <http://example.org/nowhere> . }}", f"SELECT ?x WHERE {{ ?x <{p_id[P1]}> <0> . }}"),
    ]
    batch = vg.Batch(ix, [c[0] for c in cases], to_host=True)
    for qi, (iri_q, num_q) in enumerate(cases):
        r, rr = ix.query(iri_q), ref.query(num_q)
        assert rr.status == 0
        for a, b in zip(r.columns(), rr.columns):
            np.testing.assert_array_equal(a, b)
        want = [[(d["l"][v - 50_000_000] if v >= 50_000_000 else d["so"][v - 1]) for v in row]
                for row in zip(*rr.columns)] if rr.columns and len(rr.columns[0]) else []
        assert vg.decode_result(r, ing.dict) == want
        assert vg.decode_batch(batch, qi, ing.dict) == want
        r.close()
    batch.close()
    ix.close()
    ing.free()
