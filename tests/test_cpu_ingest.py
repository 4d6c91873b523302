"""The ingest oracle against the loader's rules written out by hand, and the
.vdd dictionary reader/writer (host code, no device)."""
import os

import numpy as np
import pytest

from oracle import oracle_py


TEXT = (b"# a comment\n"
        b"<a> <p> <b> .\n"
        b"  <b>\t<q> \"x y\"@en .   # trailing comment\n"
        b"\n"
        b"_:n1 <p> <a> .\r\n"
        b"<a> <p> \"y\\\" z\"^^<http://t> .\n"
        b"<b> <p> \"x y\"@en .")   # no final newline


def test_first_appearance_ids_shared_dictionary():
    s, p, o, d = oracle_py.ingest_ntriples(TEXT, literal_dict=False)
    # src/loader.cu:27-52: subject, then object, then predicate get the next id
    assert d["so"] == ["<a>", "<b>", '"x y"@en', "_:n1", '"y\\" z"^^<http://t>']
    assert d["p"] == ["<p>", "<q>"]
    assert d["l"] == []
    np.testing.assert_array_equal(s, [1, 2, 4, 1, 2])
    np.testing.assert_array_equal(p, [1, 2, 1, 1, 1])
    np.testing.assert_array_equal(o, [2, 3, 1, 5, 3])


def test_literal_dictionary_ids_start_at_50m():
    s, p, o, d = oracle_py.ingest_ntriples(TEXT, literal_dict=True)
    assert d["so"] == ["<a>", "<b>", "_:n1"]
    assert d["l"] == ['"x y"@en', '"y\\" z"^^<http://t>']
    np.testing.assert_array_equal(s, [1, 2, 3, 1, 2])
    np.testing.assert_array_equal(o, [2, 50000000, 1, 50000001, 50000000])


@pytest.mark.parametrize("bad,line", [(b"<a> <p> <b>\n", 1), (b"<a> <p> <b> .\n<a> \"p\" <b> .\n", 2),
                                      (b"<a> <p>\n", 1), (b"<a> <p> \"open .\n", 1)])
def test_malformed_statement_line_numbers(bad, line):
    with pytest.raises(ValueError, match=f"line {line}$"):
        oracle_py.ingest_ntriples(bad)


def test_vdd_reader_accepts_reference_order(built, tmp_path):
    """The reference writes .vdd sections in hash-map order
    (src/VedasBuild.cu:145-160); the reader sorts them by id."""
    import vedas_gb300 as vg
    path = tmp_path / "g.vdd"
    path.write_text("3\n2 <b>\n1 <a>\n3 _:n1\n1\n1 <p>\n2\n50000001 \"y\"\n50000000 \"x\"@en\n")
    d = vg.Dict.open(str(path))
    assert d.terms("so") == ["<a>", "<b>", "_:n1"]
    assert d.terms("p") == ["<p>"]
    assert d.terms("l") == ['"x"@en', '"y"']
    assert d.lookup("so", "<b>") == 2 and d.lookup("l", '"y"') == 50000001 and d.lookup("p", "<zz>") == 0
    out = tmp_path / "w.vdd"
    d.write(str(out))
    assert out.read_text() == "3\n1 <a>\n2 <b>\n3 _:n1\n1\n1 <p>\n2\n50000000 \"x\"@en\n50000001 \"y\"\n"
    d.close()
