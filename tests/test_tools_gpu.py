"""GPU: telemetry reads of the current device, and a result dump of a device
array."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_telemetry_reads_the_device(grus):
    t = grus.telemetry()
    assert t["valid"] & grus.TEL_HBM
    assert 0 < t["hbm_free_bytes"] <= t["hbm_total_bytes"]
    if t["valid"] & grus.TEL_CLOCKS:
        assert t["sm_clock_mhz"] > 0
    if t["valid"] & grus.TEL_POWER:
        assert t["power_mw"] > 0


def test_result_dump_from_device(grus, tmp_path):
    torch = pytest.importorskip("torch")
    g = grus.Graph.rmat(10, 8, 2, symmetric=True)
    out = torch.empty(g.n, dtype=torch.int32, device="cuda")
    grus.bfs(g, g.max_degree_vertex, out=out)
    torch.cuda.synchronize()
    grus.save_result(tmp_path / "bfs.res", out)
    assert np.array_equal(grus.load_result(tmp_path / "bfs.res"), out.cpu().numpy().view(np.uint32))
