"""Output layout of src/bin/output/worker.rs:130-248 and the readers of
tools/DataStreamer.py and src/bin/init.rs (CPU only)."""
import lzma
import os
import struct

import numpy as np
import pytest

from stochasticsampling_gb300 import output as io
from stochasticsampling_gb300.settings import parse_settings

from test_settings import FULL


def _settings():
    import tomllib
    return parse_settings(tomllib.loads(FULL))


def test_codec_roundtrip_against_msgpack():
    msgpack = pytest.importorskip("msgpack")
    rng = np.random.default_rng(0)
    p = rng.random((333, 5))
    e = io.output_entry(7, distribution=io.distribution_record(rng.random((4, 3, 1, 2, 1)), (4, 3, 1, 2, 1),
                                                               (1.0, 2.0, 3.0)),
                        flowfield=rng.random((3, 4, 3, 1)), particles=p)
    ref = msgpack.unpackb(io.packb(e), raw=False)
    assert ref["timestep"] == 7 and ref["magneticfield"] is None
    assert np.array_equal(np.array(ref["particles"]), p)
    ff = ref["flowfield"]
    assert ff["v"] == 1 and np.array_equal(np.array(ff["data"]).reshape(ff["dim"]), e["flowfield"].a)
    d = ref["distribution"]
    assert list(d) == ["dist", "grid_width", "box_size", "grid_size"]
    assert d["grid_size"] == {"x": 4, "y": 3, "z": 1, "phi": 2, "theta": 1}
    for v in [0, 127, 128, 65536, 2 ** 40, -1, -33, -2 ** 40, 0.5, "", "s" * 40, [], {}, None, True, [1, [2.5]]]:
        assert msgpack.unpackb(io.packb(v), raw=False) == v
        assert io.unpackb(msgpack.packb(v, use_bin_type=True)) == v


def test_settings_header_record():
    rec = io.settings_record(_settings())
    assert list(rec) == ["simulation", "parameters", "environment"]
    sim = rec["simulation"]
    assert list(sim)[:5] == ["number_of_particles", "number_of_timesteps", "timestep", "init_distribution", "seed"]
    back = io.unpackb(io.packb(rec))
    assert back["simulation"]["init_distribution"] == [1, []]  # Homogeneous, rmp-serde 0.13 unit variant
    assert back["environment"]["output_format"] == [1, []]  # Bincode
    assert back["parameters"]["diffusion"] == {"translational": 1.0, "rotational": 0.5}


def test_worker_layout_and_reader(tmp_path):
    s = _settings()
    w = io.Worker(str(tmp_path), "run-x", "MsgPack", io_queue_size=2)
    w.write_metadata(s)
    rng = np.random.default_rng(1)
    entries = []
    for t in range(3):
        e = io.output_entry(t, flowfield=rng.random((3, 2, 2, 1)), particles=rng.random((4, 5)))
        entries.append(e)
        w.append(e)
    w.write_snapshot(io.snapshot_record(rng.random((4, 5)), 3))
    w.quit()
    idx = np.fromfile(tmp_path / "run-x.index", dtype="<u8")
    raw = open(tmp_path / "run-x.msgpack-lzma", "rb").read()
    assert len(idx) == 3 and idx[0] > 0 and np.all(np.diff(idx) > 0)
    header = io.unpackb(raw[:idx[0]])  # uncompressed settings first (DataStreamer.get_metadata)
    assert header["parameters"]["stress"]["active"] == 1.0
    # DataStreamer.__getitem__: blob i spans [index[i], index[i+1]) and is an xz stream
    sizes = np.diff(np.append(idx, len(raw)))
    for i, (o, n) in enumerate(zip(idx, sizes)):
        rec = io.unpackb(lzma.decompress(raw[int(o):int(o + n)]))
        assert rec["timestep"] == i
        assert np.array_equal(io.ndarray_from(rec["flowfield"]), entries[i]["flowfield"].a)
        assert np.array_equal(np.asarray(rec["particles"]), entries[i]["particles"])
    h2, es = io.read_output(str(tmp_path / "run-x.msgpack-lzma"))
    assert h2 == header and [e["timestep"] for e in es] == [0, 1, 2]
    snap = tmp_path / "run-x.snapshot.1.msgpack-lzma"
    parts, ts = io.read_particles_file(str(snap))
    assert ts == 3 and parts.shape == (4, 5)
    assert lzma.decompress(open(snap, "rb").read())  # xz container


def test_initial_condition_file(tmp_path):
    p = np.random.default_rng(2).random((50, 5))
    f = str(tmp_path / "init.msgpack-lzma")
    io.write_particles_file(f, p)
    got, ts = io.read_particles_file(f)
    assert ts is None and np.array_equal(got, p)
    with pytest.raises(ValueError, match="Do not recognise"):
        io.read_particles_file(str(tmp_path / "init.cbor"))


def test_output_id():
    oid = io.create_output_id("prefix.with.dots")
    assert oid.startswith("prefix.with.dots-") and oid.endswith("_v2_1_1")
