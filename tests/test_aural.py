"""Auralisation on the CPU: the oracle's band split is pinned bit for bit
to the reference's own Equalizer::Split (compiled from its sources into
oracle/_ref where the reference tree exists), the library's FloatBuffer
capacity rule agrees with the oracle's write-by-write simulation, and the
argument checks of the C ABI fire before any device work."""
import ctypes as C
import importlib.util
from pathlib import Path

import numpy as np
import pytest

import oracle
from ear_gb300 import _native as N
from ear_gb300.aural import Context, Track, processed_capacity, section

ROOT = Path(__file__).resolve().parent.parent
REF_LIB = ROOT / "oracle" / "_ref" / "libear_ref.so"


def ref_lib():
    spec = importlib.util.spec_from_file_location("build_ref", ROOT / "oracle" / "build_ref.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    path = mod.build()
    if path is None:
        pytest.skip("the reference tree is not present (oracle/_ref cannot be built)")
    L = C.CDLL(str(path))
    L.ref_equalizer_split.argtypes = [C.c_void_p] * 4 + [C.c_uint, C.c_float, C.c_float, C.c_float]
    L.ref_wave_to_float.restype = C.c_long
    L.ref_wave_to_float.argtypes = [C.c_char_p, C.c_void_p, C.c_uint]
    L.ref_wave_save_mono.argtypes = [C.c_char_p, C.c_void_p, C.c_int, C.c_int, C.c_float]
    L.ref_wave_save_stereo.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                       C.c_int]
    return L


@pytest.mark.parametrize("freq", [(0.2, 1.0, 2.0), (0.2, 1.0, 5.0), (0.1, 0.4, 8.0)])
def test_oracle_band_split_equals_reference_equalizer(freq):
    L = ref_lib()
    rng = np.random.default_rng(7)
    n = 60000
    x = (rng.standard_normal(n) * 0.25).astype(np.float32)
    x[1000:1010] = 0.0
    x[2000] = 1.0
    got = oracle.band_split(x, freq)
    ref = [np.empty(n, np.float32) for _ in range(3)]
    f = [np.float32(v) * np.float32(1000.0) for v in freq]
    L.ref_equalizer_split(x.ctypes.data, *[r.ctypes.data for r in ref], n, *[float(v) for v in f])
    for g, r in zip(got, ref):
        np.testing.assert_array_equal(g.view(np.uint32), r.view(np.uint32))
    # the three bands recombine (Linkwitz-Riley: low + mid + high is all-pass)
    assert np.abs(np.fft.rfft(sum(g.astype(np.float64) for g in got))).max() > 0


def random_context(rng, pair: bool, n=None, empty_ir=False):
    cap = int(rng.integers(50, 400))
    first = int(rng.integers(0, 40))
    length = first if empty_ir else int(rng.integers(first + 1, cap + 60))
    ir = Track(rng.random(cap).astype(np.float32), first, length)
    nxt = None
    if pair:
        cap2 = int(rng.integers(50, 400))
        f2 = int(rng.integers(0, 40))
        nxt = Track(rng.random(cap2).astype(np.float32), f2, int(rng.integers(f2 + 1, cap2 + 60)))
    n = int(rng.integers(0, 300)) if n is None else n
    off = int(rng.choice([0, int(rng.integers(0, 140000)), 132300 - 5, 176400 + 3]))
    return Context(ir, rng.standard_normal(n).astype(np.float32), off, nxt)


@pytest.mark.parametrize("mode", ["direct", "fft"])
def test_processed_capacity_matches_oracle_simulation(mode):
    """ear_conv_processed_capacity (closed form) == the oracle's FloatBuffer
    simulation of every write of RecorderTrack::Process."""
    rng = np.random.default_rng(11 if mode == "direct" else 12)
    fn = oracle.process_direct if mode == "direct" else oracle.process_fft64
    cases = [random_context(rng, pair=bool(i % 2), n=(0 if i % 7 == 0 else None),
                            empty_ir=(i % 11 == 5)) for i in range(40)]
    for c in cases:
        _, cap = fn(c, 1)
        assert processed_capacity(c, mode) == cap, (mode, c.offset, c.ir, len(c.dry))


def test_section_follows_soundfile_section():
    x = np.arange(10 * 44100, dtype=np.float32)
    s, off = section(x, 0.5, 0.25)
    assert off == 22050 and len(s) == 11025 and s[0] == 22050
    s, off = section(x, 9.9)  # to the end
    assert off == int(np.float32(9.9) * np.float32(44100)) and len(s) == len(x) - off
    s, off = section(x, 11.0)  # past the end: an empty section at offset 0
    assert off == 0 and len(s) == 0


def test_aural_arguments_are_checked_before_device_work():
    L = N.lib()
    f = (C.c_float * 3)(0.2, 1.0, 2.0)
    assert L.ear_band_split(None, 10, f, None, None, None, 0, None, 0) == N.EAR_ERR_INVALID_ARG
    bad = (C.c_float * 3)(0.2, 1.0, 30.0)
    x = np.zeros(4, np.float32)
    assert L.ear_band_split(x.ctypes.data, 4, bad, x.ctypes.data, x.ctypes.data, x.ctypes.data, 0,
                            None, 0) == N.EAR_ERR_INVALID_ARG
    assert L.ear_band_split(None, 0, f, None, None, None, 0, None, 0) == N.EAR_OK
    st = N.EarConvStats()
    out = np.zeros(8, np.float32)
    assert L.ear_convolve(None, 1, 0, out.ctypes.data, 8, 0, None, 0, C.byref(st)) == \
        N.EAR_ERR_INVALID_ARG
    ctx = (N.EarConvContext * 1)()
    ctx[0].dry_length = -1
    assert L.ear_convolve(ctx, 1, 0, out.ctypes.data, 8, 0, None, 0, C.byref(st)) == \
        N.EAR_ERR_INVALID_ARG
    ctx[0].dry_length = 0
    assert L.ear_convolve(ctx, 1, 7, out.ctypes.data, 8, 0, None, 0, C.byref(st)) == \
        N.EAR_ERR_INVALID_ARG
    assert b"mode" in L.ear_last_error()


CLI = ROOT / "ear_gb300" / "bin" / "EAR"


def write_pcm(path, frames, bits):
    """A canonical 44-byte-header PCM WAV; frames: (n, channels) ints."""
    frames = np.asarray(frames)
    ch = frames.shape[1]
    if bits == 8:
        data = (frames + 128).astype(np.uint8).tobytes()
    elif bits == 16:
        data = frames.astype("<i2").tobytes()
    else:
        v = frames.astype("<i4").reshape(-1)
        data = np.stack([v & 255, (v >> 8) & 255, (v >> 16) & 255], 1).astype(np.uint8).tobytes()
    hdr = b"RIFF" + (36 + len(data)).to_bytes(4, "little") + b"WAVEfmt " + (16).to_bytes(4, "little")
    hdr += (1).to_bytes(2, "little") + ch.to_bytes(2, "little") + (44100).to_bytes(4, "little")
    hdr += (44100 * ch * bits // 8).to_bytes(4, "little") + (ch * bits // 8).to_bytes(2, "little")
    hdr += bits.to_bytes(2, "little") + b"data" + len(data).to_bytes(4, "little")
    Path(path).write_bytes(hdr + data)


def run_cli(*args):
    import subprocess

    r = subprocess.run([str(CLI), *map(str, args)], capture_output=True, text=True, timeout=60)
    return r.returncode, r.stdout


@pytest.mark.parametrize("bits,channels", [(16, 1), (16, 2), (8, 1), (24, 2)])
def test_cli_wav_reader_equals_reference_wavefile(tmp_path, bits, channels):
    """The CLI reads a source WAV exactly as WaveFile::ToFloat does."""
    L = ref_lib()
    rng = np.random.default_rng(bits + channels)
    hi = 2 ** (bits - 1)
    frames = rng.integers(-hi, hi, size=(5001, channels))
    frames[0] = -hi
    frames[1] = hi - 1
    wav = tmp_path / "in.wav"
    write_pcm(wav, frames, bits)
    rc, out = run_cli("wav2raw", wav, tmp_path / "x.f32")
    assert rc == 0, out
    got = np.fromfile(tmp_path / "x.f32", np.float32)
    ref = np.empty(len(frames) + 8, np.float32)
    n = L.ref_wave_to_float(str(wav).encode(), ref.ctypes.data, ref.size)
    assert n == len(frames) == got.size
    np.testing.assert_array_equal(got.view(np.uint32), ref[:n].view(np.uint32))


@pytest.mark.parametrize("norm,mx,stereo", [(0, 1.0, False), (1, -1.0, False), (1, 0.37, False),
                                            (0, 1.0, True), (1, 1.0, True)])
def test_cli_wav_writer_equals_reference_wavefile(tmp_path, norm, mx, stereo):
    """The CLI writes WAVs byte for byte as WaveFile::FromFloat + Save."""
    L = ref_lib()
    rng = np.random.default_rng(3)
    a = (rng.standard_normal(3000) * 0.2).astype(np.float32)
    b = (rng.standard_normal(2500) * 0.2).astype(np.float32)
    a.tofile(tmp_path / "a.f32")
    b.tofile(tmp_path / "b.f32")
    args = ["raw2wav", tmp_path / "got.wav", norm, mx, tmp_path / "a.f32"]
    if stereo:
        args.append(tmp_path / "b.f32")
        L.ref_wave_save_stereo(str(tmp_path / "ref.wav").encode(), a.ctypes.data, b.ctypes.data,
                               a.size, b.size, norm)
    else:
        L.ref_wave_save_mono(str(tmp_path / "ref.wav").encode(), a.ctypes.data, a.size, norm, mx)
    rc, out = run_cli(*args)
    assert rc == 0, out
    assert (tmp_path / "got.wav").read_bytes() == (tmp_path / "ref.wav").read_bytes()


def test_convolve_tracks_arguments_are_checked_before_device_work():
    L = N.lib()
    ctx = (N.EarConvContext * 2)()
    track = np.array([0, 2], np.int32)  # track 2 of 2: out of range
    a = np.zeros(8, np.float32)
    b = np.zeros(8, np.float32)
    outs = (C.c_void_p * 2)(a.ctypes.data, b.ctypes.data)
    lens = (C.c_int64 * 2)(8, 8)
    st = N.EarConvStats()
    assert L.ear_convolve_tracks(ctx, track.ctypes.data, 2, 0, outs, lens, 2, 0, None, 0,
                                 C.byref(st)) == N.EAR_ERR_INVALID_ARG
    assert b"names track 2" in L.ear_last_error()
    # several tracks need a track index per context
    assert L.ear_convolve_tracks(ctx, None, 2, 0, outs, lens, 2, 0, None, 0,
                                 C.byref(st)) == N.EAR_ERR_INVALID_ARG
    # an output with samples but no buffer
    bad = (C.c_void_p * 2)(a.ctypes.data, None)
    track[1] = 1
    assert L.ear_convolve_tracks(ctx, track.ctypes.data, 2, 0, bad, lens, 2, 0, None, 0,
                                 C.byref(st)) == N.EAR_ERR_INVALID_ARG
    assert b"output track 1" in L.ear_last_error()
