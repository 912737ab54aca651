"""pars_autotune: the (tile shape, grid) pair it picks is one it timed, and the scan's
results are the same for every worker count and grid size."""
import numpy as np
import pytest

from conftest import plan_bytes

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import oracle  # noqa: E402
from pars_gb300 import Context, Scanner, synth  # noqa: E402
from pars_gb300._lib import ParsError  # noqa: E402


@pytest.mark.parametrize("grammar", ["csv", "json"])
def test_results_independent_of_shape_and_grid(grammar):
    ctx = Context(0)
    sc = Scanner(plan_bytes(grammar), ctx=ctx)
    data = synth.csv_doc(21, 6 << 20) if grammar == "csv" else synth.json_doc(21, 6 << 20)
    t = torch.from_numpy(data).cuda()
    rep = sc.autotune(t.data_ptr(), t.numel(), want_pairs=True)
    pairs = list(zip(rep["workers_tried"], rep["candidates"]))
    assert (rep["workers"], rep["grid"]) in pairs and len(pairs) == 8
    assert set(rep["workers_tried"]) == {16, 24}
    sr = oracle.scan(plan_bytes(grammar), data)
    pr = oracle.pair(plan_bytes(grammar), sr.bracket_char)
    for w, g in pairs + [(16, 1), (24, 1), (16, 7), (24, 7), (0, 0)]:
        sc.tune_set(t.numel(), g, w)
        r = sc.scan_tensor(t, want_pairs=True)
        torch.cuda.synchronize()
        got = r.to_numpy()
        assert np.array_equal(got["pos"], sr.positions), f"workers {w} grid {g}"
        assert np.array_equal(got["bpair"], pr.pair), f"workers {w} grid {g}"


def test_tune_set_rejects_other_worker_counts():
    sc = Scanner(plan_bytes("csv"), ctx=Context(0))
    with pytest.raises(ParsError):
        sc.tune_set(1 << 20, 0, 20)
