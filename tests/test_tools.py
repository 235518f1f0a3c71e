"""CPU: the .gr converter, the binary result dump and telemetry without a
device.  The converted files are read back with the oracle's .gr reader (the
restatement pinned against the reference loader)."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def grus_lib():
    """The product package, built if needed; no device is initialised."""
    from grus_framework_gb300 import build as b
    b.build()
    import grus_framework_gb300 as g
    return g


def read(oracle_mod, path):
    return oracle_mod.read_gr(str(path))


def test_edgelist_to_gr(grus_lib, oracle_mod, tmp_path):
    src = tmp_path / "e.txt"
    src.write_text("# toy graph\n0 1 5\n0 2 3\n2 1 7\n\n3 0 1\n")
    out = tmp_path / "e.gr"
    grus_lib.convert_edgelist(src, out, weighted=True)
    g = read(oracle_mod, out)
    assert g.n == 4 and g.m == 4
    assert list(g.offs) == [0, 2, 2, 3, 4]
    assert list(g.cols) == [1, 2, 1, 0]
    assert list(g.wts) == [5, 3, 7, 1]


def test_edgelist_symmetric_dedup(grus_lib, oracle_mod, tmp_path):
    src = tmp_path / "s.txt"
    src.write_text("0 1 4\n1 0 2\n1 2\n2 2\n")
    out = tmp_path / "s.gr"
    grus_lib.convert_edgelist(src, out, symmetric=True, weighted=True)
    g = read(oracle_mod, out)
    # (0,1) listed both ways: one copy each direction, the lightest weight
    assert list(g.offs) == [0, 1, 3, 5]
    assert list(g.cols) == [1, 0, 2, 1, 2]
    assert list(g.wts) == [2, 2, 1, 1, 1]


def test_matrix_market_to_gr(grus_lib, oracle_mod, tmp_path):
    src = tmp_path / "m.mtx"
    src.write_text("%%MatrixMarket matrix coordinate integer symmetric\n% c\n3 3 2\n2 1 9\n3 2 4\n")
    out = tmp_path / "m.gr"
    grus_lib.convert_edgelist(src, out, weighted=True)
    g = read(oracle_mod, out)
    assert g.n == 3 and g.m == 4
    assert list(g.cols) == [1, 0, 2, 1] and list(g.wts) == [9, 9, 4, 4]
    pat = tmp_path / "p.mtx"
    pat.write_text("%%MatrixMarket matrix coordinate pattern general\n2 2 1\n1 2\n")
    grus_lib.convert_edgelist(pat, tmp_path / "p.gr", weighted=True)
    gp = read(oracle_mod, tmp_path / "p.gr")
    assert gp.m == 1
    assert np.fromfile(tmp_path / "p.gr", np.uint64, 4)[1] == 0  # no weights stored


@pytest.mark.parametrize("text", ["0 x\n", "%%MatrixMarket matrix coordinate real general\n2 2 1\n0 1\n",
                                  "%%MatrixMarket matrix array real general\n2 2\n"])
def test_converter_rejects_bad_input(grus_lib, tmp_path, text):
    src = tmp_path / "bad.txt"
    src.write_text(text)
    with pytest.raises(grus_lib.GrusError):
        grus_lib.convert_edgelist(src, tmp_path / "bad.gr")
    with pytest.raises(grus_lib.GrusError):
        grus_lib.convert_edgelist(tmp_path / "missing.txt", tmp_path / "x.gr")


def test_result_dump_round_trip(grus_lib, tmp_path):
    d = np.array([0, 3, 4294967294, 7], np.uint32)
    grus_lib.save_result(tmp_path / "d.res", d)
    assert np.array_equal(grus_lib.load_result(tmp_path / "d.res"), d)
    r = np.array([0.25, 1e-3, 3.5], np.float32)
    grus_lib.save_result(tmp_path / "r.res", r)
    back = grus_lib.load_result(tmp_path / "r.res")
    assert back.dtype == np.float32 and np.array_equal(back, r)


def test_telemetry_without_device(grus_lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a device is visible: covered by the GPU test")
    with pytest.raises(grus_lib.GrusError) as e:
        grus_lib.telemetry()
    assert e.value.status == grus_lib.ENODEV


def test_tuning_cache_mix_signature():
    """Batch/server tunings are keyed by graph set and query mix: the key
    changes when either changes and is stable otherwise."""
    from grus_framework_gb300 import tuning_cache as tc
    gs = ["0:100:400:3:7:12", "0:50:90:3:1:9"]
    q = [(0, 1, 5), (1, 0, 7)]
    k = tc.mix_signature("batch", gs, q)
    assert k == tc.mix_signature("batch", list(gs), [tuple(x) for x in q])
    assert k != tc.mix_signature("server", gs, q)
    assert k != tc.mix_signature("batch", gs[::-1], q)
    assert k != tc.mix_signature("batch", gs, [(0, 1, 6), (1, 0, 7)])


def test_tuning_cache_unwritable_location(tmp_path):
    """A cache that cannot be written only loses the reuse: the store reports
    it and nothing is raised; a writable one round-trips."""
    from grus_framework_gb300 import tuning_cache as tc
    blocked = tmp_path / "file"
    blocked.write_text("not a directory")
    assert tc._store(blocked / "sub" / "t.json", "k", {"x": 1}) is False
    ok = tmp_path / "cache" / "t.json"
    assert tc._store(ok, "k", {"x": 1}) is True
    assert tc.load(ok) == {"k": {"x": 1}}
