"""The run configuration file (CConfiguration::ReadConfigurationFileWithDrag,
Configuration.cpp:21-452) and the drag file (IO::Load, IO.cpp:524-648): the library's
readers (include/mps_io.h) against the oracle restatement (oracle/config_oracle.py) on
the reference's own input decks and on synthetic files in the full dialect, with CRLF
line ends, missing trailing lines and fields, every drag mode and the reference's
quirks (any D/DE input token other than V or T reads both sets; only the last record of
a drag file followed by whitespace counts).  Host-only."""
import os
import struct
import sys
import zipfile

import numpy as np
import pytest

from simulation_project_gb300 import config
from simulation_project_gb300.types import CParameter, MpsError

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import config_oracle  # noqa: E402

REF_ROOT = os.environ.get("MPS_REFERENCE_ROOT", "/root/reference")
DECKS = [os.path.join(REF_ROOT, "solver", "TESTDATA", n) for n in
         ("velocity simulation in evaporator and heater.zip", "Temperature simulation in Evaporator and Heater.zip")]


def _compare(got: dict, want: dict):
    for k in ("input_path", "parameter_file", "particle_file", "output_path", "output_name", "bucket_count",
              "model_count", "drag_count", "output_interval", "has_compute_zone", "section", "start_step",
              "output_ascii"):
        assert got[k] == want[k], (k, got[k], want[k])
    if want["compute_zone"] is None:
        assert got["compute_zone"] is None
    else:
        assert np.array_equal(np.float32(got["compute_zone"]), np.float32(want["compute_zone"]))
    assert got["buckets"] == want["buckets"]
    assert len(got["models"]) == len(want["models"])
    for gm, wm in zip(got["models"], want["models"]):
        for k, v in wm.items():
            if k == "drag":
                for dk, dv in v.items():
                    g = gm["drag"][dk]
                    if isinstance(dv, str):
                        assert g == dv, (gm["file"], dk, g, dv)
                    else:
                        assert np.float32(g) == np.float32(dv), (gm["file"], dk, g, dv)
            elif isinstance(v, tuple):
                assert np.array_equal(np.float32(gm[k]), np.float32(v)), (gm["file"], k, gm[k], v)
            elif isinstance(v, float):
                assert np.float32(gm[k]) == np.float32(v), (gm["file"], k, gm[k], v)
            else:
                assert gm[k] == v, (gm["file"], k, gm[k], v)


def _roundtrip(tmp_path, text: str, name="config.txt"):
    p = tmp_path / name
    p.write_bytes(text.encode("latin-1"))
    return config.read_configuration(p), config_oracle.read_configuration(text)


@pytest.mark.parametrize("deck", DECKS, ids=["velocity", "temperature"])
def test_reference_decks(tmp_path, deck):
    if not os.path.exists(deck):
        pytest.skip("reference test deck not available")
    text = zipfile.ZipFile(deck).read("configurationDragTemp.txt").decode("latin-1")
    got, want = _roundtrip(tmp_path, text)
    _compare(got, want)
    # the decks' own values: 4 models (bounding box, two drag bodies, a plate), one bucket
    assert got["model_count"] == 4 and got["drag_count"] == 2 and got["bucket_count"] == 1
    assert got["buckets"][0]["file"] == "bucket.dat" and got["buckets"][0]["interval"] == 16
    assert got["models"][0]["temperature"] == 32.0 and got["models"][0]["drag_id"] == -1
    ev = got["models"][1]["drag"]
    assert ev["DragToken"] == "E" and ev["CoefficientofInflueneRegion"] == 1.0
    assert np.float32(ev["VelocityIndex"]) == np.float32(0.0007)
    assert got["output_interval"] == 32 and got["compute_zone"] is None and got["section"] == (1, 1, 1)
    assert got["output_ascii"] == 1 and got["models"][3]["file"] == "movingplate.Stl"


FULL = ("/data/run/IN/\r\nparameter.dat\r\nparticle.dat\r\nbucket1.dat 10 200\r\nbucket2.dat 7\r\n\r\n"
        # full-dialect wall line: rotating drum with every field
        "drum.stl 0 0 0 300 0.01 -0.02 0.5 0 0 1 30 0.25 1.5 0 0 0 1 0 0 0.8 1e-3 16.5 1 2.5 0 0 1 101325\r\n"
        # linear wall, short (older dialect) line
        "plate.stl 0.1 0 -0.2 290 0 0 0 1 40\r\n"
        "e.stl DE V V 1.5 0.0007 1.5061 -0.75\r\n"
        "t.stl de t t 2 0.5 0.6668 -55\r\n"
        "b.stl D VT VT 1 0.1 0.2 0.3 0.4 0.5 0.6\r\n"
        "q.stl DE X Y 1 0.1 0.2 0.3 0.4 0.5 0.6\r\n"     # any other token: both sets
        "c.stl DC V V 3 0.1 -0.2 0.3\r\n"
        "f.stl DF V V 2 0.75\r\n"
        "g.stl DF T T 2 0.75\r\n"                          # DF without V: factor unread
        "\r\n/data/run/OUT\r\nframe\r\n25\r\n-0.1 -0.2 -0.3 0.4 0.5 0.6\r\n2 1 3\r\n1200\r\nBiNaRy\r\n")


def test_full_dialect_every_drag_mode(tmp_path):
    got, want = _roundtrip(tmp_path, FULL)
    _compare(got, want)
    m = got["models"]
    assert [x["is_drag"] for x in m] == [0, 0, 1, 1, 1, 1, 1, 1, 1]
    assert [x["drag_id"] for x in m] == [-1, -1, 0, 1, 2, 3, 4, 5, 6]
    assert m[0]["rotating"] == 1 and m[0]["rpm"] == 30 and m[0]["pressure_gas"] == 101325.0
    assert m[1]["linear_movable"] == 1 and m[1]["reset_interval"] == 40 and m[1]["rotating"] == 0
    assert [x["drag"]["InputVelocityToken1"] for x in m[2:]] == ["V", "T", "B", "B", "V", "V", ""]
    assert [x["drag"]["DragToken"] for x in m[2:]] == ["E", "E", "E", "E", "C", "F", "F"]
    assert got["buckets"][1] == {"file": "bucket2.dat", "interval": 7, "total_steps": 0}
    assert got["output_ascii"] == 0 and got["start_step"] == 1200 and got["section"] == (2, 1, 3)
    assert got["compute_zone"] is not None
    # per-model triangle parameters (MultiGPUHandler.cpp:466-555)
    cfg, _, models = config.read_configuration_raw(tmp_path / "config.txt")
    p = CParameter()
    p.Dt = 5e-5
    tp = config.triangle_parameters(models, p)
    want_tp = config_oracle.model_parameters(want["models"], 5e-5)
    for t, w in zip(tp, want_tp):
        for k, v in w.items():
            assert np.float32(getattr(t, k)) == np.float32(v), k


def test_missing_tail_lines_and_lf_endings(tmp_path):
    text = "in\nparam.dat\nparticles.dat\n\nwall.stl 0 0 0 20\n\nout\nname\n"
    got, want = _roundtrip(tmp_path, text)
    _compare(got, want)
    assert got["output_interval"] == 0 and got["compute_zone"] is None and got["output_ascii"] == 1
    assert got["bucket_count"] == 0 and got["model_count"] == 1


def test_non_numeric_wall_token_is_an_error(tmp_path):
    p = tmp_path / "bad.txt"
    p.write_text("in\np\nq\n\nwall.stl X 0 0 1\n\n")
    with pytest.raises(MpsError):
        config.read_configuration(p)
    with pytest.raises(ValueError):
        config_oracle.read_configuration(p.read_text())


def test_configuration_path_join():
    for d, n in (("C:\\run\\IN", "p.dat"), ("/data/in/", "p.dat"), ("C:\\x\\", "y"), ("", "z.dat")):
        assert config.configuration_path(d, n) == config_oracle.join(d, n)


def _stl_ascii(tris, normals):
    out = ["solid model"]
    for t, n in zip(tris, normals):
        out.append(f"facet normal {n[0]:.6e} {n[1]:.6e} {n[2]:.6e}")
        out.append("outer loop")
        out += [f"vertex {v[0]:.6e} {v[1]:.6e} {v[2]:.6e}" for v in t]
        out.append("endloop")
        out.append("endfacet")
    out.append("endsolid model")
    return "\n".join(out) + "\n"


def _stl_binary(tris, normals):
    b = bytearray(80) + struct.pack("<I", len(tris))
    for t, n in zip(tris, normals):
        b += struct.pack("<12f", *n, *t.reshape(-1)) + b"\0\0"
    return bytes(b)


def test_drag_file(tmp_path):
    rng = np.random.default_rng(4)
    models = []
    for k, binary in ((0, False), (1, True), (2, False)):
        t = rng.normal(0, 0.01, (3 + k, 3, 3)).astype(np.float32)
        nrm = rng.normal(0, 1, (3 + k, 3)).astype(np.float32)   # file normals, kept as they are
        name = f"drag{k}.stl"
        (tmp_path / name).write_bytes(_stl_binary(t, nrm) if binary else _stl_ascii(t, nrm).encode())
        models.append((name, t, nrm))
    root = str(tmp_path) + "/"
    recs = ["drag0.stl 0.5 10 20 300 0 0 -9.81 0.1 0 0",
            "missing.stl 1 1 2 3 1 1 1 0 0 0",        # not on disk: skipped
            "drag1.stl 0.25 0 5 100 1 2 3 -1 -2 -3",
            "drag2.stl 0.125 7 8 9 0.5 0.5 0.5 0 0 1"]
    text = f"{root}\r\ninner.dat\r\n" + "\r\n".join(recs) + "\r\n"
    (tmp_path / "drag.txt").write_text(text)
    tris, inner = config.read_drag_file(tmp_path / "drag.txt")
    o_root, o_inner, o_recs = config_oracle.read_drag_records(text)
    assert inner == config_oracle.join(o_root, o_inner)
    assert len(o_recs) == 4
    # the loaded models take the records' values in loaded order (drag0: rec 0, drag1:
    # rec 1 (of the missing model), drag2: rec 2), as the reference's index does
    assert len(tris) == 3 + 4 + 5
    tid = 0
    for i, (name, t, nrm) in enumerate(models):
        r = o_recs[i]
        for j in range(len(t)):
            row = tris[tid]
            assert row["ID"] == tid
            assert np.allclose(row["Vertex"], t[j], rtol=1e-6, atol=1e-9)
            assert np.allclose(row["Normal"], nrm[j], rtol=1e-6, atol=1e-9)
            assert np.float32(row["DragLength"]) == np.float32(r[1])
            assert (row["StartStep01"], row["StartStep02"], row["EndStep"]) == r[2:5]
            assert np.array_equal(row["InitialAcc"], np.float32(r[5]))
            assert np.array_equal(row["GradAcc"], np.float32(r[6]))
            tid += 1


def test_drag_file_last_record_needs_trailing_whitespace(tmp_path):
    t = np.zeros((1, 3, 3), np.float32)
    t[0, 1, 0] = t[0, 2, 1] = 1
    (tmp_path / "a.stl").write_bytes(_stl_binary(t, np.float32([[0, 0, 1]])))
    (tmp_path / "b.stl").write_bytes(_stl_binary(t, np.float32([[0, 0, 1]])))
    text = f"{tmp_path}/ inner.dat a.stl 1 0 0 0 0 0 0 0 0 0 b.stl 2 0 0 0 0 0 0 0 0 0"
    (tmp_path / "d.txt").write_text(text)
    tris, _ = config.read_drag_file(tmp_path / "d.txt")
    assert len(config_oracle.read_drag_records(text)[2]) == 1
    assert len(tris) == 1 and tris[0]["DragLength"] == 1.0
    (tmp_path / "e.txt").write_text(f"{tmp_path}/ inner.dat nothing.stl 1 x")
    with pytest.raises(MpsError):   # no triangle at all
        config.read_drag_file(tmp_path / "e.txt")
