"""The continuous-batching server: each request's result is the same alone (one
pars_scan_device on it) and in the mix (folded into launches with others), for mixed
grammars and sizes submitted while earlier launches are running."""
import numpy as np
import pytest

from conftest import plan_bytes

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from pars_gb300 import Scanner, synth  # noqa: E402
from pars_gb300.server import Server  # noqa: E402


def make_requests(seed, n):
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n):
        g = "json" if rng.random() < 0.7 else "csv"
        size = int(np.exp(rng.uniform(np.log(256), np.log(1 << 20))))
        d = synth.json_doc(seed * 100 + i, size) if g == "json" else synth.csv_doc(seed * 100 + i, size)
        reqs.append((g, torch.from_numpy(d).pin_memory()))
    return reqs


@pytest.mark.parametrize("max_batch_docs,result_mib", [(4096, 0), (1, 0), (4096, 1), (1, 1)])
def test_server_results_equal_single_scans(max_batch_docs, result_mib):
    """With the default pinned result pool every result lands in it; with a 1 MiB
    pool most do not fit and go through staging into the request's own buffers."""
    srv = Server(arena_bytes=1 << 30, workers=2, max_batch_docs=max_batch_docs, result_mib=result_mib)
    plans = {g: srv.load_plan(plan_bytes(g)) for g in ("json", "csv")}
    reqs = make_requests(11, 120)
    tickets = [srv.submit(plans[g], t.data_ptr(), t.numel(), want_pairs=True) for g, t in reqs]
    got = [srv.wait(tk) for tk in tickets]
    srv.close()
    scanners = {g: Scanner(plan_bytes(g)) for g in ("json", "csv")}
    folded = 0
    for (g, t), r in zip(reqs, got):
        assert r["status"] == 0
        d = t.cuda()
        e = scanners[g].scan_device(d.data_ptr(), d.numel(), want_pairs=True)
        torch.cuda.synchronize()
        en = e.to_numpy()
        assert np.array_equal(r["pos"], en["pos"])
        assert np.array_equal(r["pair"], en["pair"])
        assert (r["balanced"], r["well_formed"], r["max_depth"], r["unclosed_mode"]) == \
            (int(e.balanced), int(e.well_formed), e.max_depth, e.unclosed_mode)
        folded += r["batch_docs"] > 1
    if max_batch_docs > 1:
        assert folded > 0, "no request shared a launch"
    else:
        assert folded == 0
