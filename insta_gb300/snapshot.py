"""instant-ngp / INSTA snapshots (`Testbed::save_snapshot` / `load_snapshot`,
instant-ngp/src/testbed.cu:2913-3016): a msgpack document holding the network configuration
(`encoding`, `network`, `rgb_network`, `dir_encoding`, ...) and a `snapshot` object with
`version`, `params_type`, `params_binary` (the trainer's flat parameters, density MLP, rgb MLP,
hash table in NerfNetwork::set_params order, NGP/nerf_network.h:492-525), `density_grid_size`
(128), `density_grid_binary` (FP16, n_cascades x 128^3, Morton order), `aabb`, `render_aabb`
(`{"min": [...], "max": [...]}`), `nerf.aabb_scale`, `training_step`, `loss`.

The msgpack codec here is a small self-contained implementation of the format's types that
nlohmann::json::to_msgpack writes (nil, bool, integers, float32/64, str, bin, array, map), so the
loader needs no third-party package.  Layout of the trainer's `params_binary` is tiny-cuda-nn's
(absent from the reference tree): it is taken as the concatenation above, unpinned until a real
snapshot is checked against it.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

SNAPSHOT_FORMAT_VERSION = 1
GRID = 128


# ------------------------------------------------------------------ msgpack
def _pack(obj, out: bytearray):
    if obj is None:
        out.append(0xC0)
    elif obj is True:
        out.append(0xC3)
    elif obj is False:
        out.append(0xC2)
    elif isinstance(obj, (int, np.integer)) and not isinstance(obj, bool):
        v = int(obj)
        if 0 <= v < 0x80:
            out.append(v)
        elif -32 <= v < 0:
            out.append(v & 0xFF)
        elif v >= 0:
            for tag, fmt, lim in ((0xCC, ">B", 1 << 8), (0xCD, ">H", 1 << 16), (0xCE, ">I", 1 << 32), (0xCF, ">Q", 1 << 64)):
                if v < lim:
                    out.append(tag)
                    out += struct.pack(fmt, v)
                    break
            else:
                raise ValueError("integer too large for msgpack")
        else:
            for tag, fmt, lim in ((0xD0, ">b", 1 << 7), (0xD1, ">h", 1 << 15), (0xD2, ">i", 1 << 31), (0xD3, ">q", 1 << 63)):
                if -lim <= v:
                    out.append(tag)
                    out += struct.pack(fmt, v)
                    break
            else:
                raise ValueError("integer too small for msgpack")
    elif isinstance(obj, (float, np.floating)):
        if isinstance(obj, np.float32):
            out.append(0xCA)
            out += struct.pack(">f", float(obj))
        else:
            out.append(0xCB)
            out += struct.pack(">d", float(obj))
    elif isinstance(obj, str):
        b = obj.encode("utf-8")
        n = len(b)
        if n < 32:
            out.append(0xA0 | n)
        elif n < 1 << 8:
            out += bytes([0xD9, n])
        elif n < 1 << 16:
            out.append(0xDA)
            out += struct.pack(">H", n)
        else:
            out.append(0xDB)
            out += struct.pack(">I", n)
        out += b
    elif isinstance(obj, (bytes, bytearray, memoryview)):
        b = bytes(obj)
        n = len(b)
        if n < 1 << 8:
            out += bytes([0xC4, n])
        elif n < 1 << 16:
            out.append(0xC5)
            out += struct.pack(">H", n)
        else:
            out.append(0xC6)
            out += struct.pack(">I", n)
        out += b
    elif isinstance(obj, (list, tuple)):
        n = len(obj)
        if n < 16:
            out.append(0x90 | n)
        elif n < 1 << 16:
            out.append(0xDC)
            out += struct.pack(">H", n)
        else:
            out.append(0xDD)
            out += struct.pack(">I", n)
        for x in obj:
            _pack(x, out)
    elif isinstance(obj, dict):
        n = len(obj)
        if n < 16:
            out.append(0x80 | n)
        elif n < 1 << 16:
            out.append(0xDE)
            out += struct.pack(">H", n)
        else:
            out.append(0xDF)
            out += struct.pack(">I", n)
        for k, v in obj.items():
            _pack(k, out)
            _pack(v, out)
    else:
        raise TypeError(f"cannot pack {type(obj).__name__}")


def packb(obj) -> bytes:
    out = bytearray()
    _pack(obj, out)
    return bytes(out)


def unpackb(data: bytes):
    buf = memoryview(data)
    pos = 0

    def take(n):
        nonlocal pos
        if pos + n > len(buf):
            raise ValueError("truncated msgpack document")
        b = buf[pos:pos + n]
        pos += n
        return b

    def read():
        t = take(1)[0]
        if t < 0x80:
            return t
        if t >= 0xE0:
            return t - 0x100
        if 0x80 <= t <= 0x8F:
            return {read(): read() for _ in range(t & 0x0F)}
        if 0x90 <= t <= 0x9F:
            return [read() for _ in range(t & 0x0F)]
        if 0xA0 <= t <= 0xBF:
            return bytes(take(t & 0x1F)).decode("utf-8")
        if t == 0xC0:
            return None
        if t == 0xC2:
            return False
        if t == 0xC3:
            return True
        if t in (0xC4, 0xC5, 0xC6):
            n = struct.unpack({0xC4: ">B", 0xC5: ">H", 0xC6: ">I"}[t], take({0xC4: 1, 0xC5: 2, 0xC6: 4}[t]))[0]
            return bytes(take(n))
        if t in (0xC7, 0xC8, 0xC9):   # ext: (type, data)
            n = struct.unpack({0xC7: ">B", 0xC8: ">H", 0xC9: ">I"}[t], take({0xC7: 1, 0xC8: 2, 0xC9: 4}[t]))[0]
            kind = struct.unpack(">b", take(1))[0]
            return (kind, bytes(take(n)))
        if t == 0xCA:
            return struct.unpack(">f", take(4))[0]
        if t == 0xCB:
            return struct.unpack(">d", take(8))[0]
        if 0xCC <= t <= 0xCF:
            fmt, n = {0xCC: (">B", 1), 0xCD: (">H", 2), 0xCE: (">I", 4), 0xCF: (">Q", 8)}[t]
            return struct.unpack(fmt, take(n))[0]
        if 0xD0 <= t <= 0xD3:
            fmt, n = {0xD0: (">b", 1), 0xD1: (">h", 2), 0xD2: (">i", 4), 0xD3: (">q", 8)}[t]
            return struct.unpack(fmt, take(n))[0]
        if 0xD4 <= t <= 0xD8:   # fixext 1..16
            n = {0xD4: 1, 0xD5: 2, 0xD6: 4, 0xD7: 8, 0xD8: 16}[t]
            kind = struct.unpack(">b", take(1))[0]
            return (kind, bytes(take(n)))
        if t in (0xD9, 0xDA, 0xDB):
            n = struct.unpack({0xD9: ">B", 0xDA: ">H", 0xDB: ">I"}[t], take({0xD9: 1, 0xDA: 2, 0xDB: 4}[t]))[0]
            return bytes(take(n)).decode("utf-8")
        if t in (0xDC, 0xDD):
            n = struct.unpack(">H" if t == 0xDC else ">I", take(2 if t == 0xDC else 4))[0]
            return [read() for _ in range(n)]
        if t in (0xDE, 0xDF):
            n = struct.unpack(">H" if t == 0xDE else ">I", take(2 if t == 0xDE else 4))[0]
            return {read(): read() for _ in range(n)}
        raise ValueError(f"msgpack type byte 0x{t:02x} is not supported")

    obj = read()
    if pos != len(buf):
        raise ValueError("trailing bytes after the msgpack document")
    return obj


def _binary(v) -> bytes:
    """nlohmann binaries come back as bytes (bin) or (subtype, bytes) (ext)."""
    if isinstance(v, tuple):
        return v[1]
    if isinstance(v, (bytes, bytearray)):
        return bytes(v)
    raise ValueError("expected a binary field")


# ------------------------------------------------------------------ snapshots
@dataclass
class Snapshot:
    params: np.ndarray                         # float16, NerfNetwork::set_params order
    density_grid: np.ndarray | None            # float16, n_cascades * 128^3 (Morton order per cascade)
    aabb: tuple                                # (min[3], max[3]), Testbed::m_aabb
    render_aabb: tuple                         # (min[3], max[3])
    aabb_scale: int = 1
    training_step: int = 0
    loss: float = 0.0
    config: dict = field(default_factory=dict)  # the network configuration (without "snapshot")
    bounding_radius: float = 1.0               # Testbed::m_bounding_radius (testbed.h:488)
    # the trainer's batch counters (Testbed::Nerf::Training::Counters, testbed.h:581-584), which
    # load_snapshot reads without a default (testbed.cu:2975-2977)
    rays_per_batch: int = 1 << 12
    measured_batch_size: int = 0
    measured_batch_size_before_compaction: int = 0

    @property
    def n_cascades(self) -> int:
        return 0 if self.density_grid is None else self.density_grid.size // GRID ** 3

    def field_config(self):
        """FieldConfig from the configuration's encoding / network / rgb_network blocks."""
        from .synthetic import FieldConfig
        enc, net, rgb = self.config.get("encoding", {}), self.config.get("network", {}), self.config.get("rgb_network", {})
        fc = FieldConfig()
        fc.n_levels = int(enc.get("n_levels", fc.n_levels))
        fc.n_features = int(enc.get("n_features_per_level", fc.n_features))
        fc.log2_table = int(enc.get("log2_hashmap_size", fc.log2_table))
        fc.base_res = int(enc.get("base_resolution", fc.base_res))
        fc.aabb_scale = int(self.aabb_scale)
        fc.n_extra = int(self.config.get("exp_params", 0))
        fc.density_hidden = int(net.get("n_neurons", fc.density_hidden))
        fc.density_layers = int(net.get("n_hidden_layers", fc.density_layers))
        fc.density_out = int(net.get("n_output_dims", fc.density_out))
        fc.rgb_hidden = int(rgb.get("n_neurons", fc.rgb_hidden))
        fc.rgb_layers = int(rgb.get("n_hidden_layers", fc.rgb_layers))
        return fc


def _box(j) -> tuple:
    return (np.asarray(j["min"], np.float32), np.asarray(j["max"], np.float32))


def read_snapshot(src) -> Snapshot:
    """Testbed::load_snapshot's reading side from a path or the document's bytes."""
    data = Path(src).read_bytes() if isinstance(src, (str, Path)) else bytes(src)
    doc = unpackb(data)
    if not isinstance(doc, dict) or "snapshot" not in doc:
        raise ValueError("the document does not contain a snapshot")
    snap = doc["snapshot"]
    if int(snap.get("version", 0)) < SNAPSHOT_FORMAT_VERSION:
        raise ValueError("snapshot uses an old format")
    kind = str(snap.get("params_type", "__half"))
    raw = _binary(snap["params_binary"])
    if kind in ("__half", "half"):
        params = np.frombuffer(raw, dtype=np.float16).copy()
    elif kind == "float":
        params = np.frombuffer(raw, dtype=np.float32).astype(np.float16)
    else:
        raise ValueError(f"unsupported params_type {kind!r}")
    grid = None
    if "density_grid_binary" in snap:
        if int(snap.get("density_grid_size", GRID)) != GRID:
            raise ValueError("incompatible grid size")
        g = np.frombuffer(_binary(snap["density_grid_binary"]), dtype=np.float16).copy()
        if g.size % GRID ** 3:
            raise ValueError("incompatible number of grid cascades")
        grid = g if g.size else None
    nerf = snap.get("nerf", {})
    rgb = nerf.get("rgb", {})
    cfg = {k: v for k, v in doc.items() if k != "snapshot"}
    unit = {"min": [0.0, 0.0, 0.0], "max": [1.0, 1.0, 1.0]}
    return Snapshot(params=params, density_grid=grid, aabb=_box(snap.get("aabb", unit)), render_aabb=_box(snap.get("render_aabb", unit)),
                    aabb_scale=int(nerf.get("aabb_scale", 1)), training_step=int(snap.get("training_step", 0)),
                    loss=float(snap.get("loss", 0.0)), config=cfg, bounding_radius=float(snap.get("bounding_radius", 1.0)),
                    rays_per_batch=int(rgb.get("rays_per_batch", 1 << 12)),
                    measured_batch_size=int(rgb.get("measured_batch_size", 0)),
                    measured_batch_size_before_compaction=int(rgb.get("measured_batch_size_before_compaction", 0)))


def write_snapshot(dst, s: Snapshot) -> bytes:
    """Testbed::save_snapshot's layout (FP16 parameters; testbed.cu:2916-2950): every key that
    Testbed::load_snapshot reads (testbed.cu:2952-3016) is written, an empty density_grid_binary
    standing for a grid that was never populated, as the reference allows.  Returns the bytes and
    writes them to dst when it is a path."""
    snap = {
        "version": SNAPSHOT_FORMAT_VERSION,
        "params_type": "__half",
        "n_params": int(s.params.size),
        "params_binary": np.ascontiguousarray(s.params, np.float16).tobytes(),
        "density_grid_size": GRID,
        "density_grid_binary": b"" if s.density_grid is None else np.ascontiguousarray(s.density_grid, np.float16).tobytes(),
        "nerf": {"aabb_scale": int(s.aabb_scale),
                 "rgb": {"rays_per_batch": int(s.rays_per_batch), "measured_batch_size": int(s.measured_batch_size),
                         "measured_batch_size_before_compaction": int(s.measured_batch_size_before_compaction)}},
        "training_step": int(s.training_step),
        "loss": float(s.loss),
        "aabb": {"min": [float(x) for x in s.aabb[0]], "max": [float(x) for x in s.aabb[1]]},
        "render_aabb": {"min": [float(x) for x in s.render_aabb[0]], "max": [float(x) for x in s.render_aabb[1]]},
        "bounding_radius": float(s.bounding_radius),
    }
    doc = dict(s.config)
    doc["snapshot"] = snap
    data = packb(doc)
    if isinstance(dst, (str, Path)):
        Path(dst).write_bytes(data)
    return data


def apply_snapshot(ctx, avatar: int, s: Snapshot, frame: int | None = None, precision: int = 0):
    """Load a snapshot into an avatar: parameters (insta_params_load), the train and render boxes
    and, for `frame`, the bitfield of the snapshot's density grid (insta_density_grid_load,
    update_density_grid_mean_and_bitfield)."""
    ctx.params_load(avatar, s.field_config(), s.params, precision)
    ctx.set_boxes(avatar, train=s.aabb, render=s.render_aabb)
    if frame is not None and s.density_grid is not None:
        ctx.density_grid_load(avatar, frame, s.density_grid, s.n_cascades)
