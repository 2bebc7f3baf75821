"""CPU: the point-file readers and the BMP writer / reader of the library
against the reference's own outputs (golden fixtures), byte for byte.  Host
code only: no GPU."""
import numpy as np

import openol_gb300 as og


def _write(tmp_path, name, data):
    p = tmp_path / name
    p.write_bytes(np.asarray(data, np.uint8).tobytes())
    return p


def test_objread_3d_and_3df(golden, tmp_path):
    f3d = _write(tmp_path, "obj.3d", golden["obj_3d_bytes"])
    assert np.array_equal(og.objread(f3d), golden["obj_read"])
    f3df = _write(tmp_path, "obj.3df", golden["obj_3df_bytes"])
    assert np.array_equal(og.objread(f3df), golden["obj_read_3df"])


def test_objread_scaled(golden, tmp_path):
    f3d = _write(tmp_path, "obj.3d", golden["obj_3d_bytes"])
    out = og.objread(f3d, offset=(1e-3, -2e-3, 0.1), scale=1.7e-5)
    assert np.array_equal(out, golden["obj_read_scaled"])


def test_objwrite_3d_round_trip(tmp_path):
    pts = np.array([[1, -2, 3], [40, 50, -60]], np.int32)
    og.objwrite_3d(tmp_path / "p.3d", pts)
    assert np.array_equal(og.objread(tmp_path / "p.3d"), pts.astype(np.float32))


def test_bmpwrite_matches_reference_bytes(golden, tmp_path):
    for i in range(int(golden["n_bmp"])):
        img = golden[f"bmp{i}_img"]
        ny, nx = img.shape
        f = tmp_path / f"img{i}.bmp"
        og.bmpwrite(f, img, ny, nx)
        assert f.read_bytes() == golden[f"bmp{i}_bytes"].tobytes(), (ny, nx)
        assert np.array_equal(og.bmpread(f, ny, nx), img)


def test_bad_files_raise(tmp_path):
    import pytest
    with pytest.raises(og.OlgError):
        og.objread(tmp_path / "missing.3d")
    with pytest.raises(og.OlgError):
        og.objread(_write(tmp_path, "x.obj", [0, 0, 0, 0]))
    with pytest.raises(og.OlgError):  # count larger than the records present
        og.objread(_write(tmp_path, "short.3d", np.frombuffer(np.int32(5).tobytes() + b"\0" * 12, np.uint8)))
