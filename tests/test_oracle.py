"""The CPU oracle is pinned against the unmodified reference CPU backend.

Golden fixtures (tests/golden/*.npz) were produced by oracle/_ref/ref_driver, which
compiles include/pars/model/scan.hpp and nest.hpp unchanged; see
tests/golden/make_golden.py.  Where that driver is present (it needs the reference
sources) the oracle is additionally compared on fresh random inputs.
"""
import os
import subprocess
import sys
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN, GRAMMARS, ROOT, golden_cases, plan_bytes
from oracle import oracle
from pars_gb300 import synth

sys.path.insert(0, GOLDEN)
import bench_records  # noqa: E402

DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")


def check_case(plan, c, name):
    sr = oracle.scan(plan, c["in"])
    assert np.array_equal(sr.positions, c["pos"]), name
    assert np.array_equal(sr.chars, c["chars"]), name
    assert np.array_equal(sr.bracket_pos, c["bpos"]), name
    assert np.array_equal(sr.bracket_char, c["bchar"]), name
    assert np.array_equal(sr.mask, c["mask"]), name
    pr = oracle.pair(plan, sr.bracket_char)
    assert np.array_equal(pr.pair, c["pair"]), name
    assert np.array_equal(pr.depth, c["depth"]), name
    unclosed, balanced, wf, md = c["meta"].tolist()
    assert (sr.unclosed_mode, pr.balanced, pr.well_formed, pr.max_depth) == (
        bool(unclosed), bool(balanced), bool(wf), md), name


@pytest.mark.parametrize("grammar", GRAMMARS)
def test_oracle_matches_reference_goldens(grammar):
    plan = plan_bytes(grammar)
    n = 0
    for name, c in golden_cases(grammar):
        check_case(plan, c, name)
        n += 1
    assert n >= 4


def test_reference_known_answers():
    """tests/test_model.cpp:152-217 restated on the oracle."""
    pj = plan_bytes("json")
    r = oracle.scan(pj, b'{"name":"a\\"b","n":[1,2.5e-3,true,null],"x":{}}')
    assert bytes(r.chars) == b'{:,:[,,,],:{}}'
    pc = plan_bytes("csv")
    r = oracle.scan(pc, b'a,"b, c","d""e",f\n1,2,3,4\n')
    assert r.positions.tolist() == [1, 8, 15, 17, 19, 21, 23, 25]
    r = oracle.scan(pj, b'{"a":[1,{"b":2}],"c":[]}')
    p = oracle.pair(pj, r.bracket_char)
    assert p.balanced and p.well_formed and p.max_depth == 3
    assert all(p.pair[p.pair[i]] == i for i in range(p.pair.size))


def test_pair_struct_space_roundtrip():
    pj = plan_bytes("json")
    d = synth.json_doc(3, 4096)
    sr = oracle.scan(pj, d)
    pr = oracle.pair(pj, sr.bracket_char)
    ps = oracle.pair_struct_space(sr, pr)
    bsi = np.searchsorted(sr.positions, sr.bracket_pos)
    assert np.all(ps[bsi] >= 0)
    assert np.array_equal(ps[ps[bsi]], bsi)
    nb = np.ones(sr.positions.size, bool)
    nb[bsi] = False
    assert np.all(ps[nb] == -1)


def test_benchmark_payload_sizes():
    """The payload builder restates bench/bench_boundary.cu:315-336: its sizes are
    the input sizes the reference reports for all 42 published runs."""
    pub = bench_records.published()
    assert len(pub) == 42 and {e["grammar"] for e in pub} == set(GRAMMARS)
    for e in pub:
        target = e["scale_mb"] << 20
        assert bench_records.payload_size(e["grammar"], target) == e["bytes"], e
    for g in GRAMMARS:
        for target in (1, 100, 4096, 1 << 20):
            assert bench_records.payload(g, target).size == bench_records.payload_size(g, target)


@pytest.mark.parametrize("grammar", GRAMMARS)
def test_oracle_published_token_counts(grammar):
    """The oracle's structural count on the reference's benchmark payloads equals
    the token count the reference published (paper/plots/data/pars.csv) at every
    scale up to 64 MiB, and the offsets are one unit's offsets tiled, which is what
    lets the GPU test check the 128-512 MiB runs without the oracle."""
    plan = plan_bytes(grammar)
    unit_pos = oracle.scan(plan, np.frombuffer(bench_records.unit(grammar), np.uint8)).positions
    for e in bench_records.published():
        if e["grammar"] != grammar or e["scale_mb"] > 64:
            continue
        target = e["scale_mb"] << 20
        data = bench_records.payload(grammar, target)
        sr = oracle.scan(plan, data)
        assert sr.positions.size == e["tokens"], e
        tiled = bench_records.tiled_positions(grammar, target, unit_pos)
        assert np.array_equal(sr.positions.astype(np.int64), tiled), e


@pytest.mark.skipif(not os.path.exists(DRIVER), reason="reference sources not built here")
@pytest.mark.parametrize("grammar", GRAMMARS)
def test_oracle_vs_reference_random(grammar):
    """Fresh random inputs (not in the fixtures) through the unmodified reference."""
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "make_golden", os.path.join(ROOT, "tests", "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    plan = plan_bytes(grammar)
    with tempfile.TemporaryDirectory() as tmp:
        for seed in range(1, 6):
            data = bytes(synth.alpha(seed * 7919, mg.ALPHABETS[grammar], 3000 + seed * 517))
            r = mg.run_ref(grammar, data, tmp)
            r["in"] = np.frombuffer(data, np.uint8)
            check_case(plan, r, f"{grammar}-{seed}")
