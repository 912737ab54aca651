"""pars_autotune: the grid (look-back depth) it picks is one it timed, and the scan's
results are the same for every grid size."""
import numpy as np
import pytest

from conftest import plan_bytes

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import oracle  # noqa: E402
from pars_gb300 import Context, Scanner, synth  # noqa: E402


@pytest.mark.parametrize("grammar", ["csv", "json"])
def test_results_independent_of_grid(grammar):
    ctx = Context(0)
    sc = Scanner(plan_bytes(grammar), ctx=ctx)
    data = synth.csv_doc(21, 6 << 20) if grammar == "csv" else synth.json_doc(21, 6 << 20)
    t = torch.from_numpy(data).cuda()
    rep = sc.autotune(t.data_ptr(), t.numel(), want_pairs=True)
    assert rep["grid"] in rep["candidates"] and len(rep["candidates"]) >= 2
    exp = oracle.scan(plan_bytes(grammar), data).positions
    for g in rep["candidates"] + [1, 7]:
        sc.tune_set(t.numel(), g)
        r = sc.scan_tensor(t, want_pairs=True)
        torch.cuda.synchronize()
        assert np.array_equal(r.to_numpy()["pos"], exp), f"grid {g}"
