"""ctypes binding of the CPU restatement (oracle/ear_oracle.cpp).

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and
the CPU-baseline legs of bench.py, as the checker or the timed baseline.
The product (ear_gb300) never imports this package.  Pinned to the
reference itself: the ray-tracing restatement equals, bit for bit, the
reference's own Scene::Render compiled from its sources into oracle/_ref
(tests/test_ref_pin.py; a committed fixture of its output,
tests/golden/reference_render.json, pins it where the reference tree is
absent), and the band split equals the reference's own equalizer.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from ear_gb300 import _native as N
from ear_gb300.scene import make_params, recorders_at

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libear_oracle.so"


class OracleOutput(C.Structure):
    _fields_ = [("hist64", C.c_void_p), ("hist32", C.c_void_p), ("first_sample", C.c_void_p),
                ("last_sample", C.c_void_p), ("counters", C.c_void_p), ("debug_band", C.c_int32),
                ("debug_max_record", C.c_int32), ("debug_rays", C.c_int64), ("hit_tri", C.c_void_p),
                ("bounce_type", C.c_void_p), ("visible", C.c_void_p)]


_L = None


def lib():
    global _L
    if _L is None:
        if not LIB_PATH.exists():
            from ear_gb300.build import build_oracle
            build_oracle()
        L = C.CDLL(str(LIB_PATH))
        L.oracle_render.restype = C.c_int
        L.oracle_render.argtypes = [C.POINTER(N.EarSceneDesc), C.POINTER(N.EarSource),
                                    C.POINTER(N.EarRecorder), C.c_int32,
                                    C.POINTER(N.EarRenderParams), C.c_int32, C.c_int32,
                                    C.POINTER(OracleOutput)]
        L.oracle_render_adjoint.restype = C.c_int
        L.oracle_render_adjoint.argtypes = [C.POINTER(N.EarSceneDesc), C.POINTER(N.EarSource),
                                            C.POINTER(N.EarRecorder), C.c_int32,
                                            C.POINTER(N.EarRenderParams), C.c_int32, C.c_int32,
                                            C.c_void_p, C.c_void_p]
        L.oracle_last_error.restype = C.c_char_p
        L.oracle_powf.restype = C.c_float
        L.oracle_powf.argtypes = [C.c_float, C.c_float]
        L.oracle_philox.argtypes = [C.c_uint32] * 6 + [C.c_void_p]
        L.oracle_material.argtypes = [C.POINTER(N.EarMaterial), C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.c_void_p]
        L.oracle_closest_hit.argtypes = [C.POINTER(N.EarSceneDesc), C.c_int64, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_segment_blocked.argtypes = [C.POINTER(N.EarSceneDesc), C.c_int64, C.c_void_p,
                                             C.c_void_p, C.c_void_p]
        L.oracle_track_power.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_float]
        L.oracle_track_maximum.restype = C.c_float
        L.oracle_track_maximum.argtypes = [C.c_void_p, C.c_int32, C.c_int32]
        L.oracle_track_length.restype = C.c_int32
        L.oracle_track_length.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_float]
        L.oracle_track_t60.restype = C.c_float
        L.oracle_track_t60.argtypes = [C.c_void_p, C.c_int32, C.c_int32]
        L.oracle_band_split.argtypes = [C.c_void_p, C.c_int64, C.c_float, C.c_float, C.c_float,
                                        C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_process_direct.restype = C.c_int64
        L.oracle_process_direct.argtypes = ([C.c_void_p] + [C.c_int64] * 3 + [C.c_void_p]
                                            + [C.c_int64] * 3 + [C.c_void_p, C.c_int64, C.c_int64,
                                                                 C.c_void_p, C.c_int64])
        L.oracle_process_fft64.restype = C.c_int64
        L.oracle_process_fft64.argtypes = ([C.c_void_p, C.c_int64, C.c_int64, C.c_void_p,
                                            C.c_int64, C.c_int64, C.c_void_p, C.c_int64,
                                            C.c_int64, C.c_void_p, C.c_int64])
        _L = L
    return _L


def scene_desc(vertices, material_ids, materials):
    v = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 9)
    m = np.ascontiguousarray(material_ids, dtype=np.int32).reshape(-1)
    mats = (N.EarMaterial * max(1, len(materials)))()
    for i, mm in enumerate(materials):
        mats[i] = mm.to_c()
    d = N.EarSceneDesc()
    d.num_triangles = v.shape[0]
    d.vertices = v.ctypes.data_as(C.POINTER(C.c_float))
    d.material_ids = m.ctypes.data_as(C.POINTER(C.c_int32))
    d.num_materials = len(materials)
    d.materials = mats
    return d, (v, m, mats)


def render(vertices, material_ids, materials, source, recorders, *, keyframe=-1, threads=1,
           pow_mode=0, debug_band=-1, debug_rays=0, debug_max_record=0, **kw):
    """Scene::Render restated on the CPU for every band in kw['bands'].
    Returns a dict with hist64 (FP64 re-accumulation), hist32 (float
    accumulation in ray order per thread chunk), first/last sample, the
    counters and, when requested, the per-bounce debug record."""
    d, keep = scene_desc(vertices, material_ids, materials)
    src, _k2 = source.at(keyframe)
    recs = recorders_at(recorders, keyframe)
    p = make_params(**kw)
    tracks = sum(r.tracks for r in recorders)
    nb = p.num_bins
    h64 = np.zeros((max(tracks, 1), 3, nb), np.float64)
    h32 = np.zeros((max(tracks, 1), 3, nb), np.float32)
    first = np.zeros((max(tracks, 1), 3), np.int32)
    last = np.zeros((max(tracks, 1), 3), np.int32)
    cnt = np.zeros(5, np.uint64)
    o = OracleOutput()
    o.hist64, o.hist32 = h64.ctypes.data, h32.ctypes.data
    o.first_sample, o.last_sample, o.counters = first.ctypes.data, last.ctypes.data, cnt.ctypes.data
    dbg = None
    if debug_max_record > 0:
        hit = np.empty((debug_rays, debug_max_record), np.int32)
        bt = np.empty((debug_rays, debug_max_record), np.uint8)
        vis = np.empty((debug_rays, debug_max_record), np.uint32)
        o.debug_band, o.debug_max_record, o.debug_rays = debug_band, debug_max_record, debug_rays
        o.hit_tri, o.bounce_type, o.visible = hit.ctypes.data, bt.ctypes.data, vis.ctypes.data
        dbg = (hit, bt, vis)
    rc = lib().oracle_render(C.byref(d), C.byref(src), recs, len(recorders), C.byref(p),
                             int(threads), int(pow_mode), C.byref(o))
    if rc != 0:
        raise RuntimeError("oracle: " + lib().oracle_last_error().decode())
    out = {"hist64": h64[:tracks], "hist32": h32[:tracks], "first_sample": first[:tracks],
           "last_sample": last[:tracks],
           "counters": dict(zip(["rays", "segments", "shadow_queries", "contributions",
                                 "sampler_overflows"], [int(x) for x in cnt]))}
    if dbg is not None:
        out["debug"] = dbg
    return out


def adjoint(vertices, material_ids, materials, source, recorders, d_hist, *, keyframe=-1,
            threads=1, pow_mode=0, **kw):
    """FP64 path-replay gradient of sum(d_hist * h) with respect to every
    material's per-band (absorption, refraction), h being ``render``'s
    finalized histogram with the same arguments: (materials, 3, 2)."""
    d, keep = scene_desc(vertices, material_ids, materials)
    src, _k2 = source.at(keyframe)
    recs = recorders_at(recorders, keyframe)
    p = make_params(**kw)
    g = np.ascontiguousarray(d_hist, np.float64)
    tracks = sum(r.tracks for r in recorders)
    if g.shape != (tracks, 3, p.num_bins):
        raise ValueError("d_hist must be (tracks, 3, num_bins)")
    grad = np.zeros((max(1, len(materials)), 3, 2), np.float64)
    rc = lib().oracle_render_adjoint(C.byref(d), C.byref(src), recs, len(recorders), C.byref(p),
                                     int(threads), int(pow_mode), g.ctypes.data, grad.ctypes.data)
    if rc != 0:
        raise RuntimeError("oracle: " + lib().oracle_last_error().decode())
    return grad[:len(materials)]


def powf(x: float, y: float) -> float:
    return lib().oracle_powf(x, y)


def philox(counter, key):
    out = (C.c_uint32 * 4)()
    lib().oracle_philox(*[int(c) for c in counter], *[int(k) for k in key], out)
    return list(out)


def closest_hit(vertices, origins, dirs):
    d, keep = scene_desc(vertices, np.zeros(len(vertices), np.int32), [])
    o = np.ascontiguousarray(origins, np.float32)
    r = np.ascontiguousarray(dirs, np.float32)
    hit = np.empty(len(o), np.int32)
    t = np.empty(len(o), np.float32)
    lib().oracle_closest_hit(C.byref(d), len(o), o.ctypes.data, r.ctypes.data, hit.ctypes.data,
                             t.ctypes.data)
    return hit, t


def segment_blocked(vertices, origins, dirs):
    d, keep = scene_desc(vertices, np.zeros(len(vertices), np.int32), [])
    o = np.ascontiguousarray(origins, np.float32)
    r = np.ascontiguousarray(dirs, np.float32)
    out = np.empty(len(o), np.uint8)
    lib().oracle_segment_blocked(C.byref(d), len(o), o.ctypes.data, r.ctypes.data, out.ctypes.data)
    return out.astype(bool)


# ------------------------------------------------------------ auralisation
# Restatements of Equalizer::Split and RecorderTrack::Process; contexts are
# ear_gb300.aural.Context objects with numpy buffers.

def band_split(dry, freq_khz=(0.2, 1.0, 2.0)):
    x = np.ascontiguousarray(dry, np.float32)
    outs = [np.empty_like(x) for _ in range(3)]
    lib().oracle_band_split(x.ctypes.data, x.size, *[float(f) for f in freq_khz],
                            *[o.ctypes.data for o in outs])
    return tuple(outs)


def _track(t):
    a = np.ascontiguousarray(t.data, np.float32)
    return a, (a.ctypes.data if a.size else None), a.size


def process_direct(ctx, out_length):
    """RecorderTrack::Process without FFTW for one context: (track of
    out_length samples, FloatBuffer capacity)."""
    a, pa, ca = _track(ctx.ir)
    d = np.ascontiguousarray(ctx.dry, np.float32)
    out = np.zeros(int(out_length), np.float32)
    if ctx.ir_next is not None:
        b, pb, cb = _track(ctx.ir_next)
        nf, nl = ctx.ir_next.first, ctx.ir_next.length
    else:
        b, pb, cb, nf, nl = None, None, 0, 0, 0
    cap = lib().oracle_process_direct(pa, ca, ctx.ir.first, ctx.ir.length, pb, cb, nf, nl,
                                      d.ctypes.data if d.size else None, d.size, ctx.offset,
                                      out.ctypes.data, out.size)
    return out, int(cap)


def process_fft64(ctx, out_length):
    """The FFTW-build RecorderTrack::Process for one context in float64:
    (values of out_length samples, FloatBuffer capacity)."""
    a, pa, ca = _track(ctx.ir)
    d = np.ascontiguousarray(ctx.dry, np.float32)
    out = np.zeros(int(out_length), np.float64)
    if ctx.ir_next is not None:
        b, pb, cb = _track(ctx.ir_next)
        nl = ctx.ir_next.length
    else:
        b, pb, cb, nl = None, None, 0, 0
    cap = lib().oracle_process_fft64(pa, ca, ctx.ir.length, pb, cb, nl,
                                     d.ctypes.data if d.size else None, d.size, ctx.offset,
                                     out.ctypes.data, out.size)
    return out, int(cap)


def convolve_direct(contexts, out_length):
    """Recorder::Add of the processed tracks, in float32 and in order."""
    total = np.zeros(int(out_length), np.float32)
    caps = []
    for c in contexts:
        t, cap = process_direct(c, out_length)
        total = total + t
        caps.append(cap)
    return total, caps


def convolve_fft64(contexts, out_length):
    total = np.zeros(int(out_length), np.float64)
    caps = []
    for c in contexts:
        t, cap = process_fft64(c, out_length)
        total += t
        caps.append(cap)
    return total, caps


# ------------------------------------------------ the reference's own render
# oracle/_ref/libear_ref_render.so (built by oracle/build_ref.py where the
# reference tree exists): the reference's Scene::Render and parsers,
# compiled against a GMTL / Boost interface shim whose random generator
# replays a tape of uniforms recorded by the oracle.

REF_RENDER_PATH = Path(__file__).resolve().parent / "_ref" / "libear_ref_render.so"
_R = None


def ref_render_lib():
    """The reference-built render library, or None where it was not built."""
    global _R
    if _R is None:
        if not REF_RENDER_PATH.exists():
            return None
        lib()  # the oracle library it links (portable power function)
        R = C.CDLL(str(REF_RENDER_PATH))
        R.ref_render_band.restype = C.c_int
        R.ref_render_band.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_void_p, C.c_int64,
                                      C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                      C.c_void_p]
        R.ref_calc_t60.restype = C.c_int
        R.ref_calc_t60.argtypes = [C.c_char_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                                   C.c_void_p]
        R.ref_last_error.restype = C.c_char_p
        lib().oracle_random_tape.restype = C.c_int
        lib().oracle_random_tape.argtypes = [C.POINTER(N.EarSceneDesc), C.POINTER(N.EarSource),
                                             C.POINTER(N.EarRecorder), C.c_int32,
                                             C.POINTER(N.EarRenderParams), C.c_void_p, C.c_int64,
                                             C.c_void_p]
        _R = R
    return _R


def random_tape(vertices, material_ids, materials, source, recorders, *, band, keyframe=-1,
                **kw):
    """The uniforms a single-threaded oracle render of one band consumes, in
    the order the reference's global generator is called for the same
    paths (float32 array)."""
    ref_render_lib()
    d, keep = scene_desc(vertices, material_ids, materials)
    src, _k2 = source.at(keyframe)
    recs = recorders_at(recorders, keyframe)
    p = make_params(**dict(kw, bands=(band,)))
    used = C.c_int64(0)
    rc = lib().oracle_random_tape(C.byref(d), C.byref(src), recs, len(recorders), C.byref(p),
                                  None, 0, C.byref(used))
    if rc != 0:
        raise RuntimeError("oracle: " + lib().oracle_last_error().decode())
    tape = np.empty(max(1, used.value), np.float32)
    rc = lib().oracle_random_tape(C.byref(d), C.byref(src), recs, len(recorders), C.byref(p),
                                  tape.ctypes.data, tape.size, C.byref(used))
    if rc != 0:
        raise RuntimeError("oracle: " + lib().oracle_last_error().decode())
    return tape[:used.value]


def reference_render_band(ear_path, band, num_rays, tape, window, max_tracks=64):
    """Runs the reference's Scene::Render for one band on a .EAR file with
    `tape` as its random numbers.  Returns (tracks[:, :window], first_sample,
    real_length, uniforms consumed)."""
    R = ref_render_lib()
    if R is None:
        raise RuntimeError("oracle/_ref/libear_ref_render.so is not built")
    t = np.ascontiguousarray(tape, np.float32)
    out = np.zeros((max_tracks, window), np.float32)
    first = np.zeros(max_tracks, np.int32)
    real = np.zeros(max_tracks, np.int32)
    used = C.c_int64(0)
    n = R.ref_render_band(str(ear_path).encode(), int(band), int(num_rays), t.ctypes.data, t.size,
                          C.byref(used), int(window), int(max_tracks), out.ctypes.data,
                          first.ctypes.data, real.ctypes.data)
    if n < 0:
        raise RuntimeError("reference render: " + R.ref_last_error().decode())
    return out[:n], first[:n], real[:n], used.value


def grouped_by_material(w):
    """(vertices, material_ids) of a workload in the order a .EAR file
    lists them (one MESH block per material, in material order) -- the
    triangle order of the reference's combined mesh (src/Scene.cpp:103-106)."""
    order = np.argsort(w.material_ids, kind="stable")
    return w.vertices[order], w.material_ids[order]


def write_reference_scene(w, directory, samples=1000) -> Path:
    """Writes `w` as scene.ear (with a short silent dry.wav beside it, named
    by its full path as the Blender exporter writes it, and `samples` in its
    settings) into `directory`."""
    import wave

    from ear_gb300 import earfile

    d = Path(directory)
    d.mkdir(parents=True, exist_ok=True)
    wav = d / "dry.wav"
    with wave.open(str(wav), "wb") as f:
        f.setnchannels(1)
        f.setsampwidth(2)
        f.setframerate(44100)
        f.writeframes(np.zeros(64, np.int16).tobytes())
    ear = d / "scene.ear"
    ear.write_bytes(earfile.workload_to_ear(w, samples=int(samples), source_file=str(wav.resolve())))
    return ear


def reference_pin_params(w, num_rays, window):
    """Render arguments under which the oracle follows the reference's own
    loop: at most 1000 path vertices and the fixed 1e-8 cut-off
    (src/Scene.cpp:142,275)."""
    kw = dict(w.render)
    kw.update(num_rays=int(num_rays), max_bounces=N.EAR_REFERENCE_MAX_BOUNCES,
              cutoff=N.EAR_REFERENCE_CUTOFF, num_bins=int(window))
    return kw


def reference_render(w, directory, num_rays, window, bands=(0, 1, 2)):
    """The reference's own Scene::Render of workload `w` (point source,
    static) per band, on the oracle's random tape for the same rays.
    Returns dict(tracks (tracks, 3, window) float32, first_sample /
    real_length (tracks, 3), tape and used (per band))."""
    V, M = grouped_by_material(w)
    ear = write_reference_scene(w, directory)
    kw = reference_pin_params(w, num_rays, window)
    ntr = sum(r.tracks for r in w.recorders)
    out = {"tracks": np.zeros((ntr, 3, window), np.float32),
           "first_sample": np.zeros((ntr, 3), np.int64), "real_length": np.zeros((ntr, 3), np.int64),
           "tape": [0, 0, 0], "used": [0, 0, 0]}
    for b in bands:
        tape = random_tape(V, M, w.materials, w.source, w.recorders, band=b, **kw)
        tr, first, real, used = reference_render_band(ear, b, num_rays, tape, window)
        out["tracks"][:, b] = tr
        out["first_sample"][:, b] = first
        out["real_length"][:, b] = real
        out["tape"][b] = len(tape)
        out["used"][b] = used
    return out


def reference_calc_t60(w, directory, samples, window):
    """The reference's `EAR calc T60` (src/EAR.cpp:55-284: the mid band of
    the first source at samples / 10 rays, post-processed, T60 of recorder 0
    track 0, Sabine and Norris-Eyring on the first mesh) on workload `w`,
    with the oracle's random tape for those rays.  Returns dict(t60 =
    (ear, sabine, eyring) float32, num_rays, tape, used)."""
    R = ref_render_lib()
    if R is None:
        raise RuntimeError("oracle/_ref/libear_ref_render.so is not built")
    V, M = grouped_by_material(w)
    ear = write_reference_scene(w, directory, samples=samples)
    rays = int(samples) // 10
    kw = reference_pin_params(w, rays, window)
    tape = np.ascontiguousarray(
        random_tape(V, M, w.materials, w.source, w.recorders, band=1, **kw), np.float32)
    used = C.c_int64(0)
    nr = C.c_int32(0)
    out = np.zeros(3, np.float32)
    if R.ref_calc_t60(str(ear).encode(), tape.ctypes.data, tape.size, C.byref(used), C.byref(nr),
                      out.ctypes.data) != 0:
        raise RuntimeError("reference calc T60: " + R.ref_last_error().decode())
    return {"t60": out, "num_rays": nr.value, "tape": tape.size, "used": used.value}
