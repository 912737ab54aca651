"""The seeded document generators: pure functions of their seed (the same bytes on
every machine and call), sized as asked, and carrying the bytes each workload is
meant to exercise."""
import numpy as np
import pytest

from pars_gb300 import synth


@pytest.mark.parametrize("grammar,must", [
    ("toml", b"[]{}=#\"'\\\n"),
    ("clike", b"{};/*\n"),
    ("ini", b"[]=;\n"),
    ("xml", b"<>/=?!\"'"),
])
def test_config_doc(grammar, must):
    a = synth.config_doc(grammar, 3, 1 << 20)
    b = synth.config_doc(grammar, 3, 1 << 20)
    c = synth.config_doc(grammar, 4, 1 << 20)
    assert np.array_equal(a, b) and not np.array_equal(a[:4096], c[:4096])
    assert (1 << 20) <= a.size < (1 << 20) + 4096
    present = set(np.unique(a).tolist())
    assert set(must) <= present, bytes(sorted(set(must) - present))


def test_json_and_csv_docs_are_seeded():
    assert np.array_equal(synth.json_doc(9, 1 << 18), synth.json_doc(9, 1 << 18))
    assert np.array_equal(synth.csv_doc(9, 1 << 18), synth.csv_doc(9, 1 << 18))
    d = synth.csv_doc(9, 1 << 18)
    assert d[-1] == ord("\n") and d.size >= 1 << 18
