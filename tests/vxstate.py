"""Reader/writer for VXST0001 state files (parity fixtures and checkpoints).

Layout (all little-endian int64 / float64): magic, step, time, dt, Ex0, n, pre, post,
then arrays (int64 length + float64 data) By, Bz, Ey, Ez, Ay, Az (8 RK slots each),
a_squared, phi, charge, J, neutralizationCharge; then species -> levels -> patches with
x_pos, p_pos, n_x, n_p, depth, up, down, left, right and the 3-slot f block in the
reference's interleaved Index3 order.
"""
from __future__ import annotations

import io
import struct
from pathlib import Path

import numpy as np

FIELDS = ["By", "Bz", "Ey", "Ez", "Ay", "Az", "a_squared", "phi", "charge", "J", "neut"]


def read_state(path_or_bytes) -> dict:
    data = path_or_bytes if isinstance(path_or_bytes, (bytes, bytearray)) else Path(path_or_bytes).read_bytes()
    f = io.BytesIO(data)

    def i64():
        return struct.unpack("<q", f.read(8))[0]

    def f64():
        return struct.unpack("<d", f.read(8))[0]

    def arr():
        n = i64()
        return np.frombuffer(f.read(8 * n), dtype="<f8").copy()

    magic = f.read(8)
    assert magic == b"VXST0001", magic
    st = {"step": i64(), "time": f64(), "dt": f64(), "Ex0": f64(), "n": i64(), "pre": i64(), "post": i64()}
    for k in FIELDS:
        st[k] = arr()
    species = []
    for _ in range(i64()):
        levels = []
        for _ in range(i64()):
            rects = []
            for _ in range(i64()):
                hdr = [i64() for _ in range(9)]
                fv = arr()
                nx, np_ = hdr[2], hdr[3]
                f3 = fv.reshape(nx + 4, np_ + 4, 3)
                rects.append({"x_pos": hdr[0], "p_pos": hdr[1], "n_x": nx, "n_p": np_, "depth": hdr[4],
                              "up": hdr[5], "down": hdr[6], "left": hdr[7], "right": hdr[8], "f": f3})
            levels.append(rects)
        species.append(levels)
    st["species"] = species
    return st


def write_state(st: dict, path) -> None:
    out = io.BytesIO()
    out.write(b"VXST0001")
    out.write(struct.pack("<q", int(st["step"])))
    for k in ("time", "dt", "Ex0"):
        out.write(struct.pack("<d", float(st[k])))
    for k in ("n", "pre", "post"):
        out.write(struct.pack("<q", int(st[k])))
    for k in FIELDS:
        a = np.ascontiguousarray(st[k], dtype="<f8")
        out.write(struct.pack("<q", a.size))
        out.write(a.tobytes())
    out.write(struct.pack("<q", len(st["species"])))
    for levels in st["species"]:
        out.write(struct.pack("<q", len(levels)))
        for rects in levels:
            out.write(struct.pack("<q", len(rects)))
            for r in rects:
                for k in ("x_pos", "p_pos", "n_x", "n_p", "depth", "up", "down", "left", "right"):
                    out.write(struct.pack("<q", int(r[k])))
                a = np.ascontiguousarray(r["f"], dtype="<f8").reshape(-1)
                out.write(struct.pack("<q", a.size))
                out.write(a.tobytes())
    Path(path).write_bytes(out.getvalue())


def to_npz(st: dict, path) -> None:
    flat = {k: st[k] for k in FIELDS}
    meta = np.array([st["step"], st["n"], st["pre"], st["post"]], dtype=np.int64)
    flat["meta_i"] = meta
    flat["meta_f"] = np.array([st["time"], st["dt"], st["Ex0"]])
    layout = []
    for s, levels in enumerate(st["species"]):
        for l, rects in enumerate(levels):
            for k, r in enumerate(rects):
                layout.append([s, l, k] + [int(r[x]) for x in ("x_pos", "p_pos", "n_x", "n_p", "depth", "up", "down",
                                                               "left", "right")])
                flat[f"f_{s}_{l}_{k}"] = r["f"]
    flat["layout"] = np.array(layout, dtype=np.int64).reshape(-1, 12)
    flat["nlevels"] = np.array([len(levels) for levels in st["species"]], dtype=np.int64)
    np.savez_compressed(path, **flat)


def from_npz(path) -> dict:
    z = np.load(path)
    st = {k: z[k] for k in FIELDS}
    st["step"], st["n"], st["pre"], st["post"] = (int(v) for v in z["meta_i"])
    st["time"], st["dt"], st["Ex0"] = (float(v) for v in z["meta_f"])
    species = [[[] for _ in range(int(nl))] for nl in z["nlevels"]]
    for row in z["layout"]:
        s, l, k = int(row[0]), int(row[1]), int(row[2])
        keys = ("x_pos", "p_pos", "n_x", "n_p", "depth", "up", "down", "left", "right")
        r = {kk: int(v) for kk, v in zip(keys, row[3:])}
        r["f"] = z[f"f_{s}_{l}_{k}"]
        species[s][l].append(r)
    st["species"] = species
    return st


def rel_linf(a: np.ndarray, b: np.ndarray) -> float:
    """max|a-b| / max|b| (0 when both are zero)."""
    den = float(np.max(np.abs(b))) if b.size else 0.0
    num = float(np.max(np.abs(a - b))) if a.size else 0.0
    if den == 0.0:
        return num
    return num / den
