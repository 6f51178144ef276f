"""qfg_parse_text / qfg_relation_register_text (the device loader, the
drop-in for LoadData) against the reference's own LoadData (golden fixture)
and the oracle: columns bit-exact, the first bad line named, texts from
host memory and from device memory, lines across tile boundaries."""
import re

import numpy as np
import pytest

import oracle
from quickfoil_gb300 import QfgError, workloads
from quickfoil_gb300.engine import Literal
from tests import golden
from tests.test_textload import REJECTS

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _dev_text(text):
    return torch.from_numpy(np.frombuffer(text, dtype=np.uint8).copy()).cuda()


def test_loader_matches_reference(engine):
    for name, text, nargs, skipped, want, rows, checksum in golden.text_cases():
        for src in (text, _dev_text(text) if text else text):
            got = [c.cpu().numpy() for c in engine.parse_text(src, nargs, skipped)]
            assert (len(got[0]) if got else 0) == rows, name
            assert golden.column_checksums(got) == checksum, name
            if want is not None:
                for g, w in zip(got, want):
                    np.testing.assert_array_equal(g, w)


def test_loader_names_the_first_bad_line(engine):
    for (text, nargs), (_, line) in zip(golden.text_rejects(), REJECTS):
        with pytest.raises(QfgError) as e:
            engine.parse_text(text, nargs)
        assert re.search(r"line (\d+):", str(e.value)).group(1) == str(line), text


@pytest.mark.parametrize("seed", [0, 1])
def test_loader_on_a_large_text_with_long_and_odd_lines(engine, seed):
    rng = np.random.default_rng(seed)
    n = 400_000
    vals = rng.integers(-2 ** 31, 2 ** 31, (n, 2))
    pad = rng.integers(0, 4, n)
    lines = [b" " * int(p) + b"%d|%+d\r" % (a, b) for (a, b), p in zip(vals, pad)]  # CR LF
    lines[1234] = b"# " + b"x" * 9000          # a comment longer than two tiles
    lines[5000] = b" " * 5000 + b"7|8"          # a line across a tile boundary
    for i in range(17, n, 4099):
        lines[i] = b""                          # empty lines (no CR)
    text = b"\n".join(lines) + (b"" if seed else b"\n")
    want = oracle.parse_text(text, 2)
    for src in (text, _dev_text(text)):
        got = engine.parse_text(src, 2)
        for g, w in zip(got, want):
            np.testing.assert_array_equal(g.cpu().numpy(), w)


def test_relation_from_text_evaluates_like_the_parsed_columns(engine):
    w = workloads.small_random(5, n_bindings=20000, max_tuples=4000, num_literals=30)
    base = 1_500_000
    for i, r in enumerate(w.relations):
        text = b"\n".join(b"|".join(b"%d" % v for v in row) for row in zip(*r)) + b"\n"
        text = b"# facts\n" + text
        assert engine.register_relation_text(base + i, text, len(r)) == len(r[0])
    lits = [Literal(base + l.relation, l.vars, l.join_pos) for l in dict.fromkeys(w.literals)]
    b = engine.bindings(w.binding_columns, w.num_positive)
    got = engine.evaluate_step(b, lits)
    want = oracle.evaluate(w.relations, w.binding_columns, w.num_positive,
                           [(l.relation - base, l.vars, l.join_pos) for l in lits], bits=5)
    np.testing.assert_array_equal(got, want)
    b.close()


@pytest.mark.parametrize("offset", [1, 2, 3, 5])
def test_loader_on_device_text_at_any_byte_offset(engine, offset):
    """A device text that does not start on a 4- or 16-byte boundary (a view
    into a larger buffer): the byte-wise passes and the cursor's partial
    words give the same columns."""
    rng = np.random.default_rng(offset)
    vals = rng.integers(-2 ** 31, 2 ** 31, (50_001, 3))
    text = b"\n".join(b"%d|%d|%d" % tuple(r) for r in vals) + b"\n#end"
    buf = torch.from_numpy(np.frombuffer(b"\n" * offset + text, dtype=np.uint8).copy()).cuda()
    view = buf[offset:]
    assert view.data_ptr() % 4 != 0 or offset % 4 == 0
    got = engine.parse_text(view, 3)
    for g, w in zip(got, oracle.parse_text(text, 3)):
        np.testing.assert_array_equal(g.cpu().numpy(), w)


def test_relation_from_text_with_a_skipped_argument(engine):
    text = b"# name|id|parent\nann|1|7\nbob|2|7\n\ncid|3|1\n"
    rid = 1_600_000
    assert engine.register_relation_text(rid, text, 3, [1, 0, 0]) == 3
    b = engine.bindings([np.array([7, 1, 9, 2], np.int32), np.array([1, 3, 3, 2], np.int32)], 2)
    got = engine.evaluate_step(b, [Literal(rid, (-1, 0)), Literal(rid, (1, 0))])
    want = oracle.evaluate([[np.array([1, 2, 3], np.int32), np.array([7, 7, 1], np.int32)]],
                           [np.array([7, 1, 9, 2], np.int32), np.array([1, 3, 3, 2], np.int32)], 2,
                           [(0, (-1, 0), 1), (0, (1, 0), 0)], bits=5)
    np.testing.assert_array_equal(got, want)
    b.close()
