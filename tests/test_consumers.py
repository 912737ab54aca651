"""Stage-2 consumers over a structural index (CPU): the cursor and the replay see
every byte exactly once, in order, and partners point at each other."""
import numpy as np

from conftest import plan_bytes

from oracle import oracle
from pars_gb300.consumers import StructuralCursor, replay, trim


def index(doc: bytes):
    data = np.frombuffer(doc, np.uint8).copy()
    plan = plan_bytes("json")
    sr = oracle.scan(plan, data)
    pr = oracle.pair(plan, sr.bracket_char)
    return data, sr.positions.astype(np.int64), oracle.pair_struct_space(sr, pr)


def test_cursor_on_json():
    data, pos, pair = index(b'{"a": [1, 2, {"b": "x,y"}], "c": 3}')
    cur = StructuralCursor(data, pos, pair)
    assert cur.ch(0) == "{" and cur.match_index(0) == cur.n - 1
    assert "".join(cur.ch(i) for i in range(cur.n)) == '{:[,,{:}],:}'
    assert trim(cur.gap(1)) == b'"a"'
    for i in range(cur.n):
        j = cur.match_index(i)
        assert j == -1 or cur.match_index(j) == i
    assert not cur.valid(cur.n)


def test_replay_covers_every_byte_in_order():
    doc = b' [1, {"k": ["v\\"w", 2]}, "t"] '
    data, pos, pair = index(doc)
    seen = bytearray()
    events = []

    class V:
        def scalar(self, b, e):
            seen.extend(doc[b:e]); events.append(("s", b, e))

        def symbol(self, p, c, m):
            seen.append(ord(c)); events.append(("y", p, m))

    replay(data, len(doc), pos, pair, V())
    assert bytes(seen) == doc
    opens = [(p, m) for k, p, m in events if k == "y" and doc[p:p + 1] in (b"[", b"{")]
    assert all(doc[m:m + 1] in (b"]", b"}") for _, m in opens)
