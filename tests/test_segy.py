"""SEG-Y output of receiver traces (segyUtils/src/segyUtils.cpp:11-217).

The writer is held to the reference converter's own bytes: the committed
golden file made by the reference's convert() (tests/golden/segy/), and,
where the reference driver has been built, fresh seeded cases of every
receiver quantity and both interval units. The date card is the only
run-dependent field; each comparison passes the reference file's date in.
"""
import os
import subprocess

import numpy as np
import pytest

from cudafemproject_gb300 import segy

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "segy")
DRIVER = os.path.join(os.path.dirname(HERE), "oracle", "_ref", "ref_driver")
DATE_AT = slice(410, 434)  # card 6, column 10 of the 80-byte card grid


def _nodes(path):
    with open(path) as f:
        n = int(f.readline())
        return np.array([[float(v) for v in f.readline().split()] for _ in range(n)], dtype=np.float32)


def test_ibm_known_values():
    enc = segy.ibm_from_float([1.0, -118.625, 0.15625, 0.0, -0.0, 16.0, 1.0 / 16, -1.0])
    words = np.frombuffer(enc, dtype=">u4")
    assert [hex(w) for w in words] == ["0x41100000", "0xc276a000", "0x40280000", "0x0", "0x0", "0x42100000",
                                       "0x40100000", "0xc1100000"]


def test_ibm_truncates_within_hex_digit():
    rng = np.random.default_rng(0)
    x = (rng.standard_normal(20000) * 10.0 ** rng.integers(-30, 30, 20000)).astype(np.float32)
    back = segy.float_from_ibm(segy.ibm_from_float(x))
    xd = x.astype(np.float64)
    assert np.all(np.abs(back) <= np.abs(xd))           # truncation toward zero
    assert np.all(np.sign(back) == np.sign(xd))
    assert np.all(np.abs(xd - back) <= np.abs(xd) * 2.0 ** -20)
    # values with at most 21 significant bits are exact
    y = (rng.integers(-2 ** 20, 2 ** 20, 1000) * 2.0 ** rng.integers(-40, 40, 1000)).astype(np.float32)
    assert np.array_equal(segy.float_from_ibm(segy.ibm_from_float(y)), y.astype(np.float64))


def test_golden_file_bytes():
    ref = open(os.path.join(GOLD, "reference.sgy"), "rb").read()
    date = ref[DATE_AT].decode("cp037")
    out = os.path.join(os.environ.get("TMPDIR", "/tmp"), f"cfem_segy_{os.getpid()}.sgy")
    try:
        segy.convert(out, os.path.join(GOLD, "receivers.txt"), segy.VELOCITY, _nodes(os.path.join(GOLD, "nodes.txt")),
                     1, 123, date=date)
        assert open(out, "rb").read() == ref
    finally:
        if os.path.exists(out):
            os.remove(out)


def test_read_back(tmp_path):
    ids, times, tr = segy.read_receiver_text(os.path.join(GOLD, "receivers.txt"))
    text, bh, traces = segy.read_segy(os.path.join(GOLD, "reference.sgy"))
    assert "Velocity Along Y" in text and "CudaFEMproject" in text
    assert bh["traces"] == len(ids) and bh["samples"] == len(times) and bh["format"] == 1
    assert bh["interval"] == 50                            # 50000 us > 32767: stored in ms
    nodes = _nodes(os.path.join(GOLD, "nodes.txt"))
    for (th, s), nid, col in zip(traces, ids, tr.T):
        assert th["inline"] == nid and th["source_type"] == 2 and th["crossline"] == 1
        assert th["source_x"] == int(nodes[nid, 0]) and th["recv_group_elev"] == int(nodes[nid, 1])
        assert np.all(np.abs(s - col) <= np.abs(col.astype(np.float64)) * 2.0 ** -20)


def test_traces_to_segy(tmp_path):
    rng = np.random.default_rng(3)
    nodes = rng.uniform(-5, 5, (20, 3))
    trace = rng.standard_normal((7, 3, 3)) * 1e-4     # [steps][receivers][dim]
    rec = [2, 9, 19]
    path = str(tmp_path / "t.sgy")
    segy.traces_to_segy(path, nodes, 55, rec, 1e-4, trace, dof=2, date="Thu Jan  1 00:00:00 1970")
    text, bh, traces = segy.read_segy(path)
    assert bh["interval"] == 100 and bh["samples"] == 7 and len(traces) == 3
    assert "Displacement Along Z" in text
    for k, (th, s) in enumerate(traces):
        col = trace[:, k, 2].astype(np.float32).astype(np.float64)
        assert th["inline"] == rec[k] and th["source_type"] == 3
        assert np.all(np.abs(s - col) <= np.abs(col) * 2.0 ** -20)
    # the receiver text file keeps six significant digits (%g, as the reference's stream output)
    txt = str(tmp_path / "t.txt")
    times = np.arange(1, 8, dtype=np.float32) * np.float32(1e-4)
    segy.write_receiver_text(txt, rec, times, trace[:, :, 2])
    ids, t2, tr2 = segy.read_receiver_text(txt)
    assert ids == rec
    assert np.allclose(t2, times, rtol=1e-5, atol=0)
    assert np.allclose(tr2, trace[:, :, 2], rtol=1e-5, atol=0)


@pytest.mark.skipif(not os.path.exists(DRIVER), reason="reference driver not built (oracle/ref.mk)")
@pytest.mark.parametrize("dt,quantity,dof", [(1e-4, segy.DISPLACEMENT, 0), (3.3e-5, segy.VELOCITY, 1),
                                             (0.05, segy.ACCELERATION, 1), (2.5e-3, segy.PRESSURE, 0)])
def test_matches_reference_converter(tmp_path, dt, quantity, dof):
    rng = np.random.default_rng(int(dt * 1e6) + quantity)
    nodes = (rng.standard_normal((40, 2)) * 25).astype(np.float32)
    nodes[5] = [-2.9999998, 7.0]
    npath = str(tmp_path / "nodes.txt")
    with open(npath, "w") as f:
        f.write(f"{len(nodes)}\n" + "".join(" ".join(repr(float(v)) for v in x) + "\n" for x in nodes))
    ids = [5, 39, 0, 11, 5]
    times = np.arange(1, 33, dtype=np.float32) * np.float32(dt)
    tr = (rng.standard_normal((32, 5)) * 10.0 ** rng.integers(-20, 8, (32, 5))).astype(np.float32)
    txt = str(tmp_path / "rec.txt")
    segy.write_receiver_text(txt, ids, times, tr)
    ref_path, ours = str(tmp_path / "ref.sgy"), str(tmp_path / "ours.sgy")
    subprocess.run([DRIVER, "segy", ref_path, txt, npath, "2", str(dof), str(quantity), "999"], check=True,
                   capture_output=True)
    ref = open(ref_path, "rb").read()
    segy.convert(ours, txt, quantity, nodes, dof, 999, date=ref[DATE_AT].decode("cp037"))
    assert open(ours, "rb").read() == ref
