"""Generate the golden fixtures under tests/golden/ from the UNMODIFIED reference CPU
backend (built by ``make -C oracle ref`` from the reference headers where they lie).

Run where the reference sources exist:

    make -C oracle ref && python tests/golden/make_golden.py
    python tests/golden/make_golden.py published <reference>/paper/plots/data/pars.csv

Writes tests/golden/<grammar>.npz: for every case, the input bytes and the reference
outputs (positions, chars, bracket_pos, bracket_char, pair [bracket-index space],
depth keys, per-byte mask words) plus scalars (unclosed, balanced, well_formed,
max_depth).  Plans were dumped by ``oracle/_ref/ref_driver plans tests/golden/plans``.

Case sources:
  * the reference's own known-answer tests (tests/test_model.cpp:154, 179, 205,
    220-228);
  * the repeated records of bench/bench_boundary.cu:317-337;
  * uniform random strings over the alphabets of bench/bench_boundary.cu:349-354
    with seeds 12345 and 999 (drawn with this repo's own seeded generator);
  * hand-written edge cases (empty, unbalanced, unclosed modes, escape runs at
    word and tile boundaries, deep nesting past the key window);
  * small seeded synthetic documents of the benchmark workloads.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from pars_gb300 import synth  # noqa: E402

sys.path.insert(0, HERE)
from bench_records import PUBLISHED, RECORDS  # noqa: E402

DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")

ALPHABETS = {
    "json": b"{}[]:,\"\\0123456789tfn.-eE \n",
    "csv": b",.\n\r\"abc0123 ",
    "toml": b"[]{}.,=\"'#\nabc0123 \n",
    "clike": b"{};/*\n abc123",
    "ini": b"[]=;\n abc0123",
    "xml": b"<>/=?!\"' ab0123",
}


def repeat(rec: bytes, n: int) -> bytes:
    return (rec * (n // len(rec) + 1))[:n]


def cases(g: str) -> dict[str, bytes]:
    c: dict[str, bytes] = {}
    c["empty"] = b""
    if g == "json":
        c["ref_known"] = b'{"name":"a\\"b","n":[1,2.5e-3,true,null],"x":{}}'
        c["ref_pair"] = b'{"a":[1,{"b":2}],"c":[]}'
        body = b",".join([RECORDS["json"]] * 200)
        c["bench_record"] = b"[" + body + b"]"
        for s in ["[", "]", "][", "]]][[[", "[[]", "[{]}", "{[}]", '"', '\\"', '"\\',
                  '["\\\\"]', '\\"[1]"', 'a\\"b["]"', '[\\\\\\"]', '"a\\\\\\\\"b"[',
                  '{"k":"v"}"', '[1,2]\\', '\\\\"x"', '"\\' + ']',
                  '}{' * 5, ']' * 40 + '[' * 40]:
            c[f"edge_{len(c)}"] = s.encode()
        c["deep_3000"] = b"[" * 3000 + b"]" * 3000
        c["deep_unbalanced"] = b"[" * 1500 + b"{" + b"]" * 2000
        # escape runs straddling a 32-byte word and a 16 KiB tile boundary
        for off in (29, 30, 31, 32, 33):
            pre = b"[\"" + b"a" * (off - 2)
            c[f"esc_word_{off}"] = pre + b"\\\\\\\"x\",1]"
        tile = 16384
        c["esc_tile"] = b"[\"" + b"b" * (tile - 5) + b"\\\\\\\\\\\"q\", [2]]"
        c["bs_run_tile"] = b"[\"" + b"\\" * (tile + 4) + b"\",{}]"
        c["synth_doc"] = bytes(synth.json_doc(7, 64 * 1024))
        c["synth_deep"] = bytes(synth.json_deep(8, 256 * 1024))
    elif g == "csv":
        c["ref_known"] = b'a,"b, c","d""e",f\n1,2,3,4\n'
        c["bench_record"] = repeat(RECORDS["csv"], 8192)
        for s in ['"', '""', '"a"', 'a"b', ',,,\n\n', '"""', '"a""', 'x,"\n"\n,', '""""""",',
                  '\n' * 33, '"' * 33 + ',']:
            c[f"edge_{len(c)}"] = s.encode()
        c["synth_doc"] = bytes(synth.csv_doc(9, 64 * 1024))
    elif g == "clike":
        for i, s in enumerate([
                "a;b/* { ; } */c;// x { } ;\nd;{e;f}", "/**/;", "/***/;", "/* * */x;",
                "/*/**/;", "a/*a**b*/;c", "// /* ; { */\n;"]):
            c[f"ref_known_{i}"] = s.encode()
        c["bench_record"] = repeat(RECORDS["clike"], 8192)
    else:
        c["bench_record"] = repeat(RECORDS[g], 8192)
    for seed in (12345, 999):
        c[f"random_{seed}"] = bytes(synth.alpha(seed, ALPHABETS[g], 16384))
    return c


def run_ref(g: str, data: bytes, tmp: str) -> dict[str, np.ndarray]:
    inp = os.path.join(tmp, "in.bin")
    with open(inp, "wb") as f:
        f.write(data)
    out = os.path.join(tmp, "out")
    subprocess.run([DRIVER, "run", g, inp, out], check=True)
    r = {
        "pos": np.fromfile(out + ".pos", np.uint32),
        "chars": np.fromfile(out + ".chars", np.uint8),
        "bpos": np.fromfile(out + ".bpos", np.uint32),
        "bchar": np.fromfile(out + ".bchar", np.uint8),
        "pair": np.fromfile(out + ".pair", np.int32),
        "depth": np.fromfile(out + ".depth", np.int32),
        "mask": np.fromfile(out + ".mask", np.uint32),
    }
    meta = {}
    for line in open(out + ".meta"):
        k, v = line.split()
        meta[k] = int(v)
    r["meta"] = np.array([meta["unclosed"], meta["balanced"], meta["well_formed"],
                          meta["max_depth"]], np.int64)
    return r


def published(csv_path: str) -> None:
    """Write published_tokens.json from the reference's table of benchmark runs
    (paper/plots/data/pars.csv: format, impl, variant, scale_mb, five GB/s columns,
    tokens, bytes_moved).  Every variant of a (format, scale) reports the same
    token count; the N2 variant moves exactly the payload to the device, so its
    bytes_moved is the payload size."""
    import csv
    import json
    rows: dict[tuple[str, int], dict] = {}
    with open(csv_path) as f:
        for r in csv.reader(line for line in f if not line.startswith("#")):
            if len(r) < 11 or r[1] != "pars":
                continue
            key = (r[0], int(r[3]))
            e = rows.setdefault(key, {"grammar": r[0], "scale_mb": int(r[3]),
                                      "tokens": int(r[9]), "bytes": None})
            if e["tokens"] != int(r[9]):
                sys.exit(f"token counts differ between variants of {key}")
            if r[2] == "N2":
                e["bytes"] = int(r[10])
    out = sorted(rows.values(), key=lambda e: (e["grammar"], e["scale_mb"]))
    with open(PUBLISHED, "w") as f:
        f.write("[\n" + ",\n".join(json.dumps(e) for e in out) + "\n]\n")
    print(len(out), "published (grammar, scale) entries")


def main() -> None:
    if len(sys.argv) == 3 and sys.argv[1] == "published":
        published(sys.argv[2])
        return
    if not os.path.exists(DRIVER):
        sys.exit("oracle/_ref/ref_driver missing: run `make -C oracle ref` first")
    with tempfile.TemporaryDirectory() as tmp:
        for g in ALPHABETS:
            arrays: dict[str, np.ndarray] = {}
            names = []
            for name, data in cases(g).items():
                r = run_ref(g, data, tmp)
                names.append(name)
                arrays[f"{name}.in"] = np.frombuffer(data, np.uint8)
                for k, v in r.items():
                    arrays[f"{name}.{k}"] = v
            arrays["_cases"] = np.array(names)
            np.savez_compressed(os.path.join(HERE, f"{g}.npz"), **arrays)
            print(g, len(names), "cases")


if __name__ == "__main__":
    main()
