""".EAR scene files: the tagged binary format the Blender exporter writes
(blender/render_EAR/__init__.py:154-196) and the reference reads
(src/Datatype.cpp, src/EAR.cpp:92-119).

``write_ear(path, ...)`` encodes a scene the way the exporter's ``pack`` /
``writeblock`` do: ints as ``int4``, floats as ``flt4``, strings as ``str ``
padded with 1-4 NULs to a multiple of 4, float lists of length 2..9 as
``vecN`` (N = length), triangles as ``tri `` + 3 ``vec3``, blocks as a tag,
an int32 byte length and the packed items.  ``read_ear(path)`` parses one
back into plain Python structures.  The C++ command-line host has its own
reader (ear_gb300/csrc/cli/earfile.cpp); the tests check both agree.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence

import numpy as np


def _pack(d) -> bytes:
    if isinstance(d, bool):
        d = int(d)
    if isinstance(d, int):
        return b"int4" + struct.pack("<i", d)
    if isinstance(d, float):
        return b"flt4" + struct.pack("<f", d)
    if isinstance(d, str):
        e = d.encode("utf8")
        return b"str " + e + b"\x00" * (4 - len(e) % 4)
    if isinstance(d, bytes):
        return d
    if isinstance(d, (list, tuple)) and d and isinstance(d[0], (list, tuple)):
        return b"tri " + b"".join(_pack(list(map(float, v))) for v in d)
    if isinstance(d, (list, tuple)) and 1 < len(d) < 10:
        return ("vec%d" % len(d)).encode("ascii") + b"".join(_pack(float(x)) for x in d)
    raise ValueError(type(d))


def _block(tag: str, items) -> bytes:
    body = b"".join(_pack(x) for x in items)
    return tag.encode("ascii") + struct.pack("<i", len(body)) + body


def _loc(v):
    a = np.asarray(v, np.float32)
    if a.ndim == 1:
        return [float(x) for x in a]
    return _block("anim", [[float(x) for x in row] for row in a])


def encode(*, materials, meshes, sources, recorders, settings: Optional[dict] = None,
           keys: Optional[Sequence[float]] = None, freq=(0.3, 2.0, 6.0)) -> bytes:
    """materials: [(name, refl3, refr3|None, spec3|None)];
    meshes: [(material name, (n, 9) triangles)];
    sources: [dict(file=... | files=[low, mid, high], location=(3,)|(K,3), gain=...,
    offset=...)] (three files: a 3SRC block);
    recorders: [dict(file=..., location=..., channels=1|2, right_ear=...,
    head_size=..., head_absorption=(3,))]."""
    out = [b".EAR", _block("VRSN", [0])]
    for name, refl, refr, spec in materials:
        items = [name] + [float(x) for x in refl]
        if refr is not None:
            items += [float(x) for x in refr]
            if spec is not None:
                items += [float(x) for x in spec]
        out.append(_block("MAT ", items))
    st = settings if settings is not None else {
        "debug": 0, "absorption": [0.01, 0.02, 0.05], "drylevel": 1.0, "samples": 10 ** 5,
        "maxthreads": 8}
    items = []
    for k, v in st.items():
        items += [k, list(map(float, v)) if isinstance(v, (list, tuple)) else v]
    out.append(_block("SET ", items))
    if keys:
        out.append(_block("KEYS", [float(k) for k in keys]))
    out.append(_block("FREQ", [float(f) for f in freq]))
    for mat, tris in meshes:
        t = np.asarray(tris, np.float32).reshape(-1, 3, 3)
        out.append(_block("MESH", [mat] + [[list(map(float, v)) for v in tri] for tri in t]))
    for s in sources:
        files = s.get("files")
        triple = files is not None and len(files) == 3  # 3SRC: one WAV per band
        names = list(files) if triple else [s.get("file", files[0] if files else "dry.wav")]
        items = names + [_loc(s["location"]), float(s.get("gain", 1.0))]
        if "offset" in s:
            items.append(float(s["offset"]))
        out.append(_block("3SRC" if triple else "SSRC", items))
    for r in recorders:
        ch = int(r.get("channels", 1))
        items = [r.get("file", "out.wav"), 35.0, _loc(r["location"])]
        if ch == 2:
            items += [_loc(r["right_ear"]), float(r.get("head_size", 0.2)),
                      [float(x) for x in r.get("head_absorption", (0.1, 0.3, 0.9))]]
        out.append(_block("OUT%d" % ch, items))
    return b"".join(out)


def write_ear(path, **kw) -> None:
    with open(path, "wb") as f:
        f.write(encode(**kw))


def workload_to_ear(w, samples: int, keys=None, source_file: str = "dry.wav") -> bytes:
    """Encode a ``scenes.Workload`` (one MESH block per material, in
    material order, so triangle order follows material_ids grouping).
    ``source_file`` names the source's WAV; the reference's source printout
    wants a path with a directory (src/HelperFunctions.cpp:49-54), as the
    Blender exporter writes them."""
    mats = []
    for m in w.materials:
        mats.append((m.name, m.reflection, m.refraction if m.refraction is not None else
                     ([0.0, 0.0, 0.0] if m.specularity is not None else None), m.specularity))
    meshes = []
    for i, m in enumerate(w.materials):
        sel = w.vertices[w.material_ids == i]
        if len(sel):
            meshes.append((m.name, sel))
    air = list(w.render.get("air_absorption", (0.0, 0.0, 0.0)))
    settings = {"debug": 0, "absorption": air, "drylevel": float(w.render.get("dry", 1.0)),
                "samples": int(samples), "maxthreads": 8}
    src = {"file": source_file, "location": w.source.location, "gain": float(w.source.gain)}
    recs = []
    for r in w.recorders:
        recs.append({"file": "out.wav", "location": r.location, "channels": r.channels,
                     "right_ear": r.right_ear, "head_size": r.head_size,
                     "head_absorption": r.head_absorption})
    return encode(materials=mats, meshes=meshes, sources=[src], recorders=recs,
                  settings=settings, keys=keys)


# ------------------------------------------------------------------ reader
class _R:
    def __init__(self, b: bytes, pos: int = 0, end: Optional[int] = None):
        self.b, self.p, self.end = b, pos, len(b) if end is None else end

    def peek(self):
        return self.b[self.p:self.p + 4].decode("latin1") if self.p + 4 <= self.end else None

    def tag(self, want):
        t = self.peek()
        if t != want:
            raise ValueError(f"Found '{t}' while expecting '{want}'")
        self.p += 4

    def i32(self):
        v = struct.unpack_from("<i", self.b, self.p)[0]
        self.p += 4
        return v

    def flt(self):
        self.tag("flt4")
        v = struct.unpack_from("<f", self.b, self.p)[0]
        self.p += 4
        return v

    def integer(self):
        self.tag("int4")
        return self.i32()

    def string(self):
        self.tag("str ")
        q = self.b.index(b"\x00", self.p)
        s = self.b[self.p:q].decode("utf8")
        n = q - self.p
        self.p += n + 4 - n % 4
        return s

    def vec(self):
        t = self.peek()
        if t not in ("vec3", "vecf"):
            raise ValueError(f"Found '{t}' while expecting 'vec3'")
        self.p += 4
        return [self.flt(), self.flt(), self.flt()]

    def block(self, want):
        self.tag(want)
        n = self.i32()
        return self.p + n

    def location(self, end):
        if self.peek() == "anim":
            e = self.block("anim")
            frames = []
            while self.p < e:
                frames.append(self.vec())
            return np.array(frames, np.float32)
        return np.array(self.vec(), np.float32)


@dataclass
class EarScene:
    settings: Dict[str, object] = field(default_factory=dict)
    keys: List[float] = field(default_factory=list)
    freq: Optional[List[float]] = None
    materials: list = field(default_factory=list)   # (name, refl, refr|None, spec|None)
    meshes: list = field(default_factory=list)      # (material, (n, 9) float32)
    sources: list = field(default_factory=list)     # dict
    recorders: list = field(default_factory=list)   # dict
    unknown: List[str] = field(default_factory=list)


def decode(b: bytes) -> EarScene:
    if b[:4] != b".EAR":
        raise ValueError("Failed to read file")
    r = _R(b, 4)
    sc = EarScene()
    while r.peek():
        t = r.peek()
        if t == "MAT ":
            e = r.block("MAT ")
            name = r.string()
            refl = [r.flt() for _ in range(3)]
            refr = [r.flt() for _ in range(3)] if r.p < e and r.peek() == "flt4" else None
            spec = [r.flt() for _ in range(3)] if r.p < e and r.peek() == "flt4" else None
            sc.materials.append((name, refl, refr, spec))
            r.p = e
        elif t == "SET ":
            e = r.block("SET ")
            while r.p < e and r.peek() == "str ":
                k = r.string()
                vt = r.peek()
                if vt == "int4":
                    sc.settings[k] = r.integer()
                elif vt == "flt4":
                    sc.settings[k] = r.flt()
                elif vt in ("vec3", "vecf"):
                    sc.settings[k] = r.vec()
                else:
                    sc.settings[k] = r.string()
            r.p = e
        elif t == "KEYS":
            e = r.block("KEYS")
            while r.p < e:
                sc.keys.append(r.flt())
        elif t == "FREQ":
            e = r.block("FREQ")
            sc.freq = [r.flt() for _ in range(3)]
            r.p = e
        elif t == "MESH":
            e = r.block("MESH")
            mat = r.string()
            tris = []
            while r.p < e and r.peek() == "tri ":
                r.tag("tri ")
                tris.append(r.vec() + r.vec() + r.vec())
            sc.meshes.append((mat, np.array(tris, np.float32).reshape(-1, 9)))
            r.p = e
        elif t in ("OUT1", "OUT2"):
            e = r.block(t)
            d = {"file": r.string(), "unused": r.flt(), "channels": 2 if t == "OUT2" else 1}
            d["location"] = r.location(e)
            if t == "OUT2":
                d["right_ear"] = r.location(e)
                d["head_size"] = r.flt()
                d["head_absorption"] = r.vec()
            sc.recorders.append(d)
            r.p = e
        elif t in ("SSRC", "3SRC"):
            e = r.block(t)
            d = {"files": [r.string() for _ in range(3 if t == "3SRC" else 1)]}
            if r.peek() == "mesh":
                me = r.block("mesh")
                tris = []
                while r.p < me and r.peek() == "tri ":
                    r.tag("tri ")
                    tris.append(r.vec() + r.vec() + r.vec())
                d["emitter"] = np.array(tris, np.float32).reshape(-1, 9)
                r.p = me
            else:
                d["location"] = r.location(e)
            if r.p < e and r.peek() == "flt4":
                d["gain"] = r.flt()
            if r.p < e and r.peek() == "flt4":
                d["offset"] = r.flt()
            sc.sources.append(d)
            r.p = e
        else:
            if t != "VRSN":
                sc.unknown.append(t)
            if t in ("int4", "flt4"):
                r.p += 8
            else:
                r.p = r.block(t)
    return sc


def read_ear(path) -> EarScene:
    with open(path, "rb") as f:
        return decode(f.read())
