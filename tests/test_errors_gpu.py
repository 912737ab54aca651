"""Errors come back as codes and messages and leave the context usable; the process
is never ended (the reference's scanner calls std::exit,
backend/cuda/pipeline.cuh:520-555).  Every case here is rejected by the host-side
argument checks before any device work: no kernel runs on a bad argument."""
import ctypes

import numpy as np
import pytest

from conftest import plan_bytes

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import oracle  # noqa: E402
from pars_gb300 import Context, Scanner, _lib  # noqa: E402
from pars_gb300._lib import ParsError  # noqa: E402

EINVAL, EPLAN, ERANGE = -22, -71, -34
DESC0 = 48  # first lex_desc of the scan_plan POD: kind, n_states, n_classes, start, ...


def load(ctx, plan: bytes):
    buf = ctypes.create_string_buffer(plan, len(plan))
    pid = ctypes.c_int(-1)
    rc = _lib.lib().pars_plan_load(ctx.handle, buf, len(plan), ctypes.byref(pid))
    return rc, pid.value


def test_malformed_plans_are_rejected():
    ctx = Context(0)
    good = plan_bytes("json")
    assert load(ctx, good[:-1])[0] == EPLAN  # wrong size
    bad = bytearray(good)
    bad[DESC0 + 1] = 0  # descriptor 0 with no states
    assert load(ctx, bytes(bad))[0] == EPLAN
    assert b"malformed" in _lib.lib().pars_last_error(ctx.handle)
    bad = bytearray(good)
    bad[DESC0 + 263] = 9  # trans[0][0] names a state past n_states
    assert load(ctx, bytes(bad))[0] == EPLAN
    rc, pid = load(ctx, good)
    assert rc == 0 and pid >= 0


def test_scan_argument_errors_leave_the_context_usable():
    plan = plan_bytes("json")
    sc = Scanner(plan, ctx=Context(0))
    L, h = _lib.lib(), sc.ctx.handle
    data = np.frombuffer(b'{"a":[1,2,{"b":"x\\"y"}]}', np.uint8)
    t = torch.from_numpy(data.copy()).cuda()
    out = _lib.DeviceResult()
    p = ctypes.c_void_p(t.data_ptr())

    def scan(ptr, n, flags=_lib.PARS_RUN_PAIRS, pid=sc.plan_id):
        return L.pars_scan_device(h, pid, ptr, n, flags, None, ctypes.byref(out))

    assert scan(p, data.size, pid=99) == EINVAL                       # no such plan
    assert scan(None, data.size) == EINVAL                            # null input
    assert scan(p, 1 << 32) == ERANGE                                 # offsets are uint32
    assert b"2^32" in L.pars_last_error(h)
    assert scan(ctypes.c_void_p(t.data_ptr() + 1), data.size - 1,
                _lib.PARS_WANT_MASK) == EINVAL                        # mask wants 16-byte alignment
    hr = _lib.HostResult()
    host = np.zeros(64, np.uint8)
    assert L.pars_scan_host(h, sc.plan_id, host.ctypes.data_as(ctypes.c_void_p), 1 << 32,
                            _lib.PARS_RUN_PAIRS, None, ctypes.byref(hr)) == ERANGE
    assert L.pars_scan_host(h, sc.plan_id, None, 16, _lib.PARS_RUN_PAIRS, None,
                            ctypes.byref(hr)) == EINVAL
    with pytest.raises(ParsError) as e:
        sc.scan_device(t.data_ptr(), 1 << 32)
    assert e.value.code == ERANGE
    # the context still scans, bit-exact
    r = sc.scan_tensor(t, want_pairs=True)
    torch.cuda.synchronize()
    sr = oracle.scan(plan, data)
    assert np.array_equal(r.to_numpy()["pos"], sr.positions)


def test_batch_argument_errors():
    sc = Scanner(plan_bytes("csv"), ctx=Context(0))
    L, h = _lib.lib(), sc.ctx.handle
    t = torch.zeros(64, dtype=torch.uint8, device="cuda")
    out = _lib.BatchResult()

    def batch(offs, ndocs=None, flags=_lib.PARS_RUN_PAIRS):
        o = np.ascontiguousarray(offs, dtype=np.uint64)
        n = o.size - 1 if ndocs is None else ndocs
        return L.pars_scan_batch(h, sc.plan_id, ctypes.c_void_p(t.data_ptr()),
                                 o.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), n, flags,
                                 None, ctypes.byref(out))

    assert batch([0, 10, 5]) == ERANGE                 # offsets decrease
    assert batch([4, 10]) == EINVAL                    # offsets start past 0
    assert batch([0, 8], ndocs=(1 << 20) + 1) == ERANGE  # too many documents (checked first)
    assert batch([0, 8], flags=_lib.PARS_WANT_MASK) == EINVAL
    assert batch([0, 8, 16]) == 0                      # and a valid batch still runs
