"""MLP endpoint and path files and image checkpoints (needs a GPU): a
reconstruction resumed from the files gives the same rows and, with the
reproducible tiled DROP form, the same image bit for bit."""
import numpy as np
import pytest

from pct_gb300 import phantoms, recon

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def first(tmp_path_factory):
    d = tmp_path_factory.mktemp("files")
    w = phantoms.tiny(num_histories=40000, seed=7, v_extent=0.3)
    over = dict(w.config)
    over["drop_form"] = 2
    cfg = phantoms.make_config(over)
    data, angles = phantoms.generate(w)
    r = recon.run_full(cfg, data, angles)
    r.collect_mlp_endpoints()
    r.write_mlp_endpoints(d / "endpoints.bin")
    hist = {k: r.array(k) for k in ("H_WEPL", "H_X_ENTRY", "H_XZ_EXIT_ANGLE", "H_BIN_NUM", "H_FIRST_VOXEL")}
    r.mlp_rows()
    r.write_mlp_paths(d / "paths.bin")
    rows = (r.array("ROW_OFFSETS"), r.array("ROWS"), r.array("CHORD"))
    x0 = r.array("X0")
    r.drop(cfg.iterations)
    x = r.array("X")
    r.write_image(d / "x.bin")
    r.close()
    return cfg, d, hist, rows, x0, x


def test_endpoint_file_layout(first):
    cfg, d, hist, rows, x0, x = first
    raw = (d / "endpoints.bin").read_bytes()
    n = int(np.frombuffer(raw[:4], dtype="<u4")[0])
    assert n == len(hist["H_WEPL"]) and len(raw) == 4 + 60 * n
    ints = np.frombuffer(raw[4:4 + 16 * n], dtype="<i4").reshape(4, n)
    floats = np.frombuffer(raw[4 + 16 * n:], dtype="<f4").reshape(11, n)
    C, R = cfg.columns, cfg.rows
    assert np.array_equal(ints[0] + C * ints[1] + C * R * ints[2], hist["H_FIRST_VOXEL"].astype(np.int64))
    assert np.array_equal(ints[3], hist["H_BIN_NUM"])
    assert floats[0].tobytes() == hist["H_WEPL"].tobytes()
    assert floats[1].tobytes() == hist["H_X_ENTRY"].tobytes()
    assert floats[10].tobytes() == hist["H_XZ_EXIT_ANGLE"].tobytes()
    text = (d / "paths.bin").read_bytes()
    assert text.split(b"\n", 1)[0] == str(n).encode()


def test_resume_from_endpoints(first):
    cfg, d, hist, rows, x0, x = first
    r = recon.Reconstruction(cfg)
    r.read_mlp_endpoints(d / "endpoints.bin")
    r.set_image(x0)
    r.mlp_rows()
    assert r.array("ROW_OFFSETS").tobytes() == rows[0].tobytes()
    assert r.array("ROWS").tobytes() == rows[1].tobytes()
    assert r.array("CHORD").tobytes() == rows[2].tobytes()
    r.drop(cfg.iterations)
    assert r.array("X").tobytes() == x.tobytes()
    r.close()


def test_resume_from_paths_and_image(first):
    cfg, d, hist, rows, x0, x = first
    r = recon.Reconstruction(cfg)
    r.read_mlp_endpoints(d / "endpoints.bin")
    r.set_image(x0)
    r.read_mlp_paths(d / "paths.bin")
    assert r.array("ROWS").tobytes() == rows[1].tobytes()
    assert r.array("CHORD").tobytes() == rows[2].tobytes()
    r.drop(cfg.iterations)
    assert r.array("X").tobytes() == x.tobytes()
    r.read_image(d / "x.bin")
    assert r.array("X").tobytes() == x.tobytes()
    r.close()
