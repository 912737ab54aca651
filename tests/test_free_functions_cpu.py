"""The free functions scan_device / scan_host / scan_chunk keep one Scanner per
(function, plan, device) and calling thread, as the reference's free functions keep
a static thread_local scanner<S> each (backend/cuda/pipeline.cuh:1260-1281).
Checked on the CPU with a stand-in Scanner: no device work."""
import threading

import pytest

import pars_gb300
from pars_gb300 import scanner as S
from pars_gb300 import _lib


class FakeScanner:
    made = []

    def __init__(self, plan, device=0, ctx=None):
        self.plan, self.device, self.calls = plan, device, []
        FakeScanner.made.append(self)

    def scan_device(self, d_ptr, n, stream=0, want_pairs=False):
        self.calls.append(("device", d_ptr, n, stream, want_pairs))
        return ("device", self)

    def scan_host(self, data, want_pairs=False):
        self.calls.append(("host", bytes(data), want_pairs))
        return ("host", self)

    def new_carry(self):
        return _lib.ChunkCarry()

    def scan_chunk(self, d_ptr, n, carry, stream=0):
        carry.byte_base += n
        self.calls.append(("chunk", d_ptr, n))


@pytest.fixture
def fake(monkeypatch):
    FakeScanner.made = []
    monkeypatch.setattr(S, "Scanner", FakeScanner)
    monkeypatch.setattr(S, "_tls", threading.local())
    return FakeScanner


def test_one_scanner_per_function_plan_and_device(fake):
    a, b = b"A" * 3177, b"B" * 3177
    r1 = pars_gb300.scan_device(a, 1000, 64, want_pairs=True)
    r2 = pars_gb300.scan_device(a, 2000, 64)
    assert r1[1] is r2[1] and len(fake.made) == 1            # same thread, function, plan
    pars_gb300.scan_device(b, 1000, 64)
    pars_gb300.scan_host(a, b"xy")
    pars_gb300.scan_device(a, 1000, 64, device=1)
    assert len(fake.made) == 4                               # other plan, function, device
    assert r1[1].calls == [("device", 1000, 64, 0, True), ("device", 2000, 64, 0, False)]
    assert pars_gb300.thread_scanner("scan_device", a) is r1[1]


def test_threads_do_not_share_scanners(fake):
    plan = b"P" * 3177
    got = {}

    def run(k):
        got[k] = pars_gb300.scan_device(plan, 1, 1)[1]
    ts = [threading.Thread(target=run, args=(k,)) for k in range(3)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    mine = pars_gb300.scan_device(plan, 1, 1)[1]
    assert len({id(x) for x in list(got.values()) + [mine]}) == 4


def test_scan_chunk_threads_the_carry(fake):
    plan = b"C" * 3177
    c = pars_gb300.scan_chunk(plan, 100, 10)
    assert isinstance(c, _lib.ChunkCarry) and c.byte_base == 10
    c2 = pars_gb300.scan_chunk(plan, 200, 5, c)
    assert c2 is c and c.byte_base == 15
    sc = pars_gb300.thread_scanner("scan_chunk", plan)
    assert sc.calls == [("chunk", 100, 10), ("chunk", 200, 5)]
