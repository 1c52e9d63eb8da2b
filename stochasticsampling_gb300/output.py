"""Output and input files in the reference's layout.

The reference's IO worker (src/bin/output/worker.rs:130-248) writes, per run:
  <id>.msgpack-lzma   the Settings as an uncompressed msgpack map, then one
                      xz blob (preset 1) per OutputEntry (src/output.rs:10-17)
  <id>.index          the byte offset of every blob, u64 little endian
  <id>.snapshot.<k>.msgpack-lzma   one xz-compressed Snapshot per snapshot
and reads initial conditions from xz-compressed msgpack particle lists
(src/bin/init.rs:23-48).  Records are written like rmp-serde's
`encode::write_named`: structs as maps keyed by field name, Option::None as
nil, sequences as arrays; an ndarray (ndarray 0.12 serde) is the map
{"v": 1, "dim": [...], "data": [...]} with data in C order; a Particle is
[x, y, z, phi, theta] (src/particle.rs:363-395); a unit enum variant is
[index, []] (rmp-serde 0.13).

The msgpack codec is self-contained (the container images carry no msgpack
package); arrays of doubles are encoded and decoded with numpy in one pass.
"""
import dataclasses
import lzma
import os
import queue
import struct
import threading
import time

import numpy as np

COMPRESSION = 1  # xz preset, worker.rs:18
EXTENSIONS = {"CBOR": "cbor-lzma", "Bincode": "bincode-lzma", "MsgPack": "msgpack-lzma"}


class UnitVariant:
    """A unit enum variant (rmp-serde 0.13 encodes it as [index, []])."""

    def __init__(self, index, name):
        self.index, self.name = index, name


class NDArray:
    """An ndarray to serialise as {"v": 1, "dim": [...], "data": [...]}."""

    def __init__(self, a):
        self.a = np.ascontiguousarray(a)


# --------------------------------------------------------------- encoding
def _f64_array_body(a):
    """msgpack float64 elements of a float array, vectorised."""
    flat = np.ascontiguousarray(a, dtype=np.float64).ravel()
    rec = np.empty(flat.size, dtype=[("tag", "u1"), ("val", ">f8")])
    rec["tag"] = 0xCB
    rec["val"] = flat
    return rec.tobytes()


def _u64_array_body(a):
    flat = np.ascontiguousarray(a, dtype=np.uint64).ravel()
    out = bytearray()
    for v in flat.tolist():
        _pack_int(out, v)
    return bytes(out)


def _array_header(out, n):
    if n < 16:
        out.append(0x90 | n)
    elif n < 1 << 16:
        out += b"\xdc" + struct.pack(">H", n)
    else:
        out += b"\xdd" + struct.pack(">I", n)


def _map_header(out, n):
    if n < 16:
        out.append(0x80 | n)
    elif n < 1 << 16:
        out += b"\xde" + struct.pack(">H", n)
    else:
        out += b"\xdf" + struct.pack(">I", n)


def _pack_int(out, v):
    if 0 <= v < 128:
        out.append(v)
    elif -32 <= v < 0:
        out.append(v & 0xFF)
    elif 0 <= v < 1 << 8:
        out += b"\xcc" + struct.pack(">B", v)
    elif 0 <= v < 1 << 16:
        out += b"\xcd" + struct.pack(">H", v)
    elif 0 <= v < 1 << 32:
        out += b"\xce" + struct.pack(">I", v)
    elif 0 <= v < 1 << 64:
        out += b"\xcf" + struct.pack(">Q", v)
    elif -(1 << 7) <= v:
        out += b"\xd0" + struct.pack(">b", v)
    elif -(1 << 15) <= v:
        out += b"\xd1" + struct.pack(">h", v)
    elif -(1 << 31) <= v:
        out += b"\xd2" + struct.pack(">i", v)
    else:
        out += b"\xd3" + struct.pack(">q", v)


def _pack(out, v):
    if v is None:
        out.append(0xC0)
    elif v is True:
        out.append(0xC3)
    elif v is False:
        out.append(0xC2)
    elif isinstance(v, (int, np.integer)):
        _pack_int(out, int(v))
    elif isinstance(v, (float, np.floating)):
        out += b"\xcb" + struct.pack(">d", float(v))
    elif isinstance(v, str):
        b = v.encode("utf-8")
        n = len(b)
        if n < 32:
            out.append(0xA0 | n)
        elif n < 1 << 8:
            out += b"\xd9" + struct.pack(">B", n)
        elif n < 1 << 16:
            out += b"\xda" + struct.pack(">H", n)
        else:
            out += b"\xdb" + struct.pack(">I", n)
        out += b
    elif isinstance(v, UnitVariant):
        _array_header(out, 2)
        _pack_int(out, v.index)
        _array_header(out, 0)
    elif isinstance(v, NDArray):
        a = v.a
        _map_header(out, 3)
        _pack(out, "v")
        _pack_int(out, 1)
        _pack(out, "dim")
        _pack(out, list(a.shape))
        _pack(out, "data")
        _array_header(out, a.size)
        if a.dtype.kind == "f":
            out += _f64_array_body(a)
        else:
            out += _u64_array_body(a)
    elif isinstance(v, np.ndarray):
        if v.ndim == 2 and v.dtype.kind == "f":  # list of fixed-size float rows (particles)
            rows, cols = v.shape
            _array_header(out, rows)
            head = bytearray()
            _array_header(head, cols)
            rec = np.empty((rows,), dtype=[("h", "u1", (len(head),)), ("vals", [("tag", "u1"), ("val", ">f8")],
                                                                           (cols,))])
            rec["h"] = np.frombuffer(bytes(head), dtype="u1")
            rec["vals"]["tag"] = 0xCB
            rec["vals"]["val"] = v
            out += rec.tobytes()
        else:
            _pack(out, v.tolist())
    elif isinstance(v, (list, tuple)):
        _array_header(out, len(v))
        for x in v:
            _pack(out, x)
    elif isinstance(v, dict):
        _map_header(out, len(v))
        for k, x in v.items():
            _pack(out, k)
            _pack(out, x)
    elif dataclasses.is_dataclass(v):
        fields = dataclasses.fields(v)
        _map_header(out, len(fields))
        for f in fields:
            _pack(out, f.name)
            _pack(out, getattr(v, f.name))
    else:
        raise TypeError(f"cannot encode {type(v)!r}")


def packb(v):
    out = bytearray()
    _pack(out, v)
    return bytes(out)


# --------------------------------------------------------------- decoding
class _Reader:
    def __init__(self, buf):
        self.b = memoryview(buf)
        self.i = 0

    def take(self, n):
        s = self.b[self.i:self.i + n]
        self.i += n
        return s

    def u(self, fmt, n):
        (v,) = struct.unpack(fmt, self.take(n))
        return v

    def float_run(self, n):
        """n consecutive msgpack float64 elements, or None if they are not."""
        end = self.i + 9 * n
        if end > len(self.b):
            return None
        rec = np.frombuffer(self.b[self.i:end], dtype=[("tag", "u1"), ("val", ">f8")])
        if not np.all(rec["tag"] == 0xCB):
            return None
        self.i = end
        return rec["val"].astype(np.float64)

    def value(self):
        t = self.b[self.i]
        self.i += 1
        if t <= 0x7F:
            return t
        if t >= 0xE0:
            return t - 256
        if 0x80 <= t <= 0x8F:
            return self.map(t & 0x0F)
        if 0x90 <= t <= 0x9F:
            return self.array(t & 0x0F)
        if 0xA0 <= t <= 0xBF:
            return bytes(self.take(t & 0x1F)).decode("utf-8")
        if t == 0xC0:
            return None
        if t == 0xC2:
            return False
        if t == 0xC3:
            return True
        if t in (0xC4, 0xC5, 0xC6):
            n = self.u({0xC4: ">B", 0xC5: ">H", 0xC6: ">I"}[t], {0xC4: 1, 0xC5: 2, 0xC6: 4}[t])
            return bytes(self.take(n))
        if t == 0xCA:
            return self.u(">f", 4)
        if t == 0xCB:
            return self.u(">d", 8)
        fmts = {0xCC: (">B", 1), 0xCD: (">H", 2), 0xCE: (">I", 4), 0xCF: (">Q", 8), 0xD0: (">b", 1),
                0xD1: (">h", 2), 0xD2: (">i", 4), 0xD3: (">q", 8)}
        if t in fmts:
            return self.u(*fmts[t])
        if t in (0xD9, 0xDA, 0xDB):
            n = self.u({0xD9: ">B", 0xDA: ">H", 0xDB: ">I"}[t], {0xD9: 1, 0xDA: 2, 0xDB: 4}[t])
            return bytes(self.take(n)).decode("utf-8")
        if t == 0xDC:
            return self.array(self.u(">H", 2))
        if t == 0xDD:
            return self.array(self.u(">I", 4))
        if t == 0xDE:
            return self.map(self.u(">H", 2))
        if t == 0xDF:
            return self.map(self.u(">I", 4))
        raise ValueError(f"unsupported msgpack type 0x{t:02x}")

    def array(self, n):
        if n > 8:
            run = self.float_run(n)
            if run is not None:
                return run
        return [self.value() for _ in range(n)]

    def map(self, n):
        return {self.value(): self.value() for _ in range(n)}


def unpackb(buf):
    return _Reader(buf).value()


def unpack_all(buf):
    """All msgpack values concatenated in buf."""
    r = _Reader(buf)
    out = []
    while r.i < len(r.b):
        out.append(r.value())
    return out


def ndarray_from(v):
    """An ndarray record {"v", "dim", "data"} as a numpy array."""
    return np.asarray(v["data"], dtype=np.float64).reshape(v["dim"])


# ---------------------------------------------------------------- records
def settings_record(settings):
    """Settings as rmp-serde write_named encodes it: unit enum variants as
    [index, []] (InitDistribution, OutputFormat)."""
    from .settings import INIT_DISTRIBUTIONS, OUTPUT_FORMATS
    d = dataclasses.asdict(settings)
    sim = d["simulation"]
    order = ["number_of_particles", "number_of_timesteps", "timestep", "init_distribution", "seed",
             "output_at_timestep", "box_size", "grid_size"]
    sim = {k: sim[k] for k in order}
    sim["init_distribution"] = UnitVariant(INIT_DISTRIBUTIONS.index(sim["init_distribution"]),
                                           sim["init_distribution"])
    out = sim["output_at_timestep"]
    sim["output_at_timestep"] = {k: out[k] for k in ["initial_condition", "final_snapshot", "distribution",
                                                      "flowfield", "magneticfield", "particles_head",
                                                      "particles", "snapshot"]}
    par = d["parameters"]
    par = {k: par[k] for k in ["magnetic_drag", "shape", "hydro_screening", "volume_exclusion",
                               "magnetic_reorientation", "diffusion", "stress", "magnetic_dipole"]}
    env = d["environment"]
    env = {"prefix": env["prefix"], "version": env["version"], "init_file": env["init_file"],
           "io_queue_size": env["io_queue_size"],
           "output_format": UnitVariant(OUTPUT_FORMATS.index(env["output_format"]), env["output_format"])}
    return {"simulation": sim, "parameters": par, "environment": env}


def distribution_record(dist, grid, box):
    """Distribution (src/distribution/mod.rs:27-36): dist, grid_width,
    box_size, grid_size."""
    gx, gy, gz, gp, gt = grid
    gw = {"x": box[0] / gx, "y": box[1] / gy, "z": box[2] / gz, "phi": 2 * np.pi / gp, "theta": np.pi / gt}
    return {"dist": NDArray(dist), "grid_width": gw, "box_size": {"x": box[0], "y": box[1], "z": box[2]},
            "grid_size": {"x": gx, "y": gy, "z": gz, "phi": gp, "theta": gt}}


def output_entry(timestep, distribution=None, flowfield=None, magneticfield=None, particles=None):
    """OutputEntry (src/output.rs:10-17) in field order."""
    return {"distribution": distribution,
            "flowfield": None if flowfield is None else NDArray(flowfield),
            "magneticfield": None if magneticfield is None else NDArray(magneticfield),
            "particles": None if particles is None else np.ascontiguousarray(particles, dtype=np.float64),
            "timestep": int(timestep)}


def snapshot_record(particles, timestep):
    """Snapshot (src/bin/simulation/mod.rs:80-86).  The noise here is Philox
    keyed by the settings' seed with the timestep as counter, so rng_state is
    empty: (seed, timestep) restores it."""
    return {"particles": np.ascontiguousarray(particles, dtype=np.float64), "rng_state": [],
            "timestep": int(timestep)}


# --------------------------------------------------------------- files
def create_output_id(prefix, version="2.1.1"):
    """create_output_id, src/bin/output/path.rs:44-54."""
    return "{}-{}_v{}".format(prefix, time.strftime("%Y-%m-%d_%H%M%S"), version.replace(".", "_"))


class Worker:
    """The IO worker of src/bin/output/worker.rs: a thread fed by a bounded
    queue (io_queue_size) that appends compressed blobs and their offsets."""

    def __init__(self, directory, output_id, output_format="MsgPack", io_queue_size=1):
        if output_format != "MsgPack":
            raise ValueError("only the MsgPack output format is written")
        self.dir = directory
        self.id = output_id
        os.makedirs(directory, exist_ok=True)
        self.path = os.path.join(directory, f"{output_id}.{EXTENSIONS[output_format]}")
        self.index_path = os.path.join(directory, f"{output_id}.index")
        self._f = open(self.path, "wb")
        self._idx = open(self.index_path, "wb")
        self._snap = 0
        self._q = queue.Queue(maxsize=max(1, int(io_queue_size)))
        self._err = None
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()

    def _run(self):
        while True:
            kind, payload = self._q.get()
            try:
                if kind == "quit":
                    break
                if kind == "settings":
                    self._f.write(packb(payload))
                elif kind == "output":
                    self._idx.write(struct.pack("<Q", self._f.tell()))
                    self._f.write(lzma.compress(packb(payload), preset=COMPRESSION))
                elif kind == "snapshot":
                    self._snap += 1
                    p = os.path.join(self.dir, f"{self.id}.snapshot.{self._snap}.msgpack-lzma")
                    with open(p, "wb") as f:
                        f.write(lzma.compress(packb(payload), preset=COMPRESSION))
            except Exception as exc:  # surfaced by the next call
                self._err = exc
            finally:
                self._q.task_done()

    def _put(self, kind, payload):
        if self._err is not None:
            raise RuntimeError(f"IO worker failed: {self._err}")
        self._q.put((kind, payload))

    def write_metadata(self, settings):
        self._put("settings", settings_record(settings))

    def append(self, entry):
        self._put("output", entry)

    def write_snapshot(self, snapshot):
        self._put("snapshot", snapshot)

    def quit(self):
        self._q.put(("quit", None))
        self._t.join()
        self._f.close()
        self._idx.close()
        if self._err is not None:
            raise RuntimeError(f"IO worker failed: {self._err}")


def read_index(path):
    return np.fromfile(path, dtype="<u8")


def read_output(path, index_path=None):
    """(settings record, [entries]) of an output file (DataStreamer.Streamer)."""
    index_path = index_path or os.path.splitext(path)[0] + ".index"
    idx = read_index(index_path)
    data = open(path, "rb").read()
    header = unpackb(data[:idx[0]]) if len(idx) else unpackb(data)
    ends = list(idx[1:]) + [len(data)]
    entries = [unpackb(lzma.decompress(data[int(a):int(b)])) for a, b in zip(idx, ends)]
    return header, entries


def read_particles_file(path):
    """An initial-condition or snapshot file (init.rs:23-48): xz-compressed
    msgpack; a particle list or a Snapshot map.  Returns (particles, timestep)
    with timestep None for a plain particle list."""
    ext = path.rsplit(".", 1)[-1] if "." in path else ""
    if not path.endswith("msgpack-lzma"):
        raise ValueError(f"Do not recognise file extension {ext}.")
    v = unpackb(lzma.decompress(open(path, "rb").read()))
    if isinstance(v, dict):
        return np.asarray(v["particles"], dtype=np.float64).reshape(-1, 5), int(v["timestep"])
    if isinstance(v, np.ndarray):
        return v.reshape(-1, 5), None
    return np.asarray(v, dtype=np.float64).reshape(-1, 5), None


def write_particles_file(path, particles):
    """An initial-condition file: the particle list, msgpack, xz preset 1."""
    with open(path, "wb") as f:
        f.write(lzma.compress(packb(np.ascontiguousarray(particles, dtype=np.float64)), preset=COMPRESSION))
