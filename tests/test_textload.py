"""The '|'-delimited fact loader (LoadData) on the oracle: against the
reference's own LoadData (golden fixture: columns or their checksums), and
the lines the reference rejects (it aborts on them; the oracle names the
first one)."""
import numpy as np
import pytest

import oracle
from oracle import TextError
from tests import golden


def test_oracle_loader_matches_reference():
    cases = golden.text_cases()
    assert {c[0] for c in cases} >= {"plain", "tricky", "crlf", "skipped", "random_200k"}
    for name, text, nargs, skipped, want, rows, checksum in cases:
        got = oracle.parse_text(text, nargs, skipped)
        assert (len(got[0]) if got else 0) == rows, name
        assert golden.column_checksums(got) == checksum, name
        if want is not None:
            for g, w in zip(got, want):
                np.testing.assert_array_equal(g, w)


# (error code, first bad line) per golden.text_rejects() entry: field
# count, empty field, no digits, a sign then no digit, a space after the
# sign, a blank line (not empty), a lone CR, out of int32 (three), and the
# first bad line winning over a later one.
REJECTS = [(2, 2), (2, 1), (3, 2), (3, 1), (3, 1), (3, 1), (3, 1), (3, 2), (4, 1), (4, 2),
           (4, 1), (2, 2)]


def test_oracle_loader_rejects_what_the_reference_rejects():
    # the reference aborted on every one of these texts (child processes)
    assert not any(golden.text_rejects_accepted())
    for (text, nargs), (code, line) in zip(golden.text_rejects(), REJECTS):
        with pytest.raises(TextError) as e:
            oracle.parse_text(text, nargs)
        assert (e.value.code, e.value.line) == (code, line), text


def test_oracle_loader_does_not_convert_skipped_arguments():
    got = oracle.parse_text(b"1|junk|2\n3||4\n", 3, [0, 1, 0])
    assert [c.tolist() for c in got] == [[1, 3], [2, 4]]
