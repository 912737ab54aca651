"""The repeated-record payloads of the reference's throughput benchmarks, and the
structural offsets they must produce.

bench/bench_boundary.cu:315-336 (and bench/bench_scan.cpp:40-53 for JSON and CSV)
build every benchmark input by repeating one fixed record per grammar:
  * JSON: ``[`` + records joined by ``,`` + ``]``, records appended while the text
    is shorter than the target;
  * the other grammars: whole records appended while the text is shorter than the
    target (``repeat_rec``, bench_boundary.cu:35-40), so the size is a multiple of
    the record length and at least the target.

paper/plots/data/pars.csv holds the reference's token counts (structural
offsets) and input sizes for these payloads at 8-512 MiB; the committed fixture
``published_tokens.json`` is that table (``make_golden.py published`` writes it).

Every record ends in the grammar's start state, so a payload's offsets are one
unit's offsets tiled at the unit's stride: ``tiled_positions`` builds them at any
size from the offsets of a single unit.
"""
from __future__ import annotations

import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PUBLISHED = os.path.join(HERE, "published_tokens.json")

RECORDS = {
    "json": b"{\"id\":123,\"name\":\"x \\\"y\\\"\",\"a\":[1,2,3],\"n\":{\"z\":null}}",
    "csv": b"alpha,beta,\"quoted, field\",\"has \"\"q\"\"\",42,true\n",
    "toml": (b"[server]\nhost = \"localhost\"\nport = 8080\nname = 'a # b'\n"
             b"# comment { } , = with \"quotes\"\narr = [1, 2, 3]\n"),
    "clike": b"int x; /* c { ; } */ y = 1; // { ; }\n",
    "ini": b"[section]\nkey = value\nnum = 123\n; comment\nother = x\n",
    "xml": b"<item id=\"1\" name=\"x &amp; y\">alpha</item>",
}


def unit(grammar: str) -> bytes:
    """The repeated unit: the record, followed by its separator for JSON."""
    return RECORDS[grammar] + (b"," if grammar == "json" else b"")


def units(grammar: str, target: int) -> int:
    """Records in the payload of `target` bytes."""
    return -(-target // len(unit(grammar)))


def payload_size(grammar: str, target: int) -> int:
    k, u = units(grammar, target), len(unit(grammar))
    return k * u + 1 if grammar == "json" else k * u


def payload(grammar: str, target: int) -> np.ndarray:
    """The benchmark input of (at least) `target` bytes, as uint8."""
    k = units(grammar, target)
    if grammar != "json":
        return np.frombuffer(RECORDS[grammar] * k, np.uint8).copy()
    body = np.frombuffer(unit(grammar) * k, np.uint8)
    out = np.empty(body.size + 1, np.uint8)
    out[0] = ord("[")
    out[1:] = body
    out[-1] = ord("]")  # the last separator closes the array
    return out


def tiled_positions(grammar: str, target: int, unit_pos: np.ndarray) -> np.ndarray:
    """Structural offsets of payload(grammar, target), given the offsets of one unit.

    For JSON the opening ``[`` is structural, the units start at byte 1, and the
    closing ``]`` takes the place of the last ``,`` (both structural)."""
    k, u = units(grammar, target), len(unit(grammar))
    start = 1 if grammar == "json" else 0
    tiles = np.add.outer(np.arange(k, dtype=np.int64) * u + start,
                         unit_pos.astype(np.int64)).ravel()
    if grammar == "json":
        tiles = np.concatenate([np.zeros(1, np.int64), tiles])
    return tiles


def published() -> list[dict]:
    """[{grammar, scale_mb, tokens, bytes}] from the reference's published table."""
    with open(PUBLISHED) as f:
        return json.load(f)
