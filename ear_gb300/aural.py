"""Auralisation: the band split of a dry sound and the convolution of
recorder tracks with it, on the GPU.

These are the steps of the reference's ``Render()`` after the impulse
responses (src/EAR.cpp:295-386): ``SoundFile::Band`` splits each dry sound
into three bands with ``Equalizer::Split`` (lib/equalizer/Equalizer.cpp),
``SoundFile::Section`` cuts the part that belongs to a keyframe
(src/SoundFile.cpp:164-173), ``RecorderTrack::Process`` convolves it with a
recorder track (src/Recorder.cpp:136-292) and ``Recorder::Add`` sums the
processed tracks of all (source x keyframe x band) contexts
(src/Recorder.cpp:432-441).

Inputs may be numpy arrays (host memory; the library copies them) or CUDA
torch tensors (device memory; no copies, work on the current stream).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from . import _native as N

SAMPLE_RATE = N.SAMPLE_RATE
DEFAULT_EQ_BANDS_KHZ = (0.2, 1.0, 2.0)  # src/SoundFile.cpp:238-240
MODES = {"fft": N.EAR_CONV_FFT, "direct": N.EAR_CONV_DIRECT}


def _is_cuda_tensor(x) -> bool:
    return hasattr(x, "is_cuda") and bool(x.is_cuda)


def _host(x) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    return a


def _ptr(a) -> int:
    if _is_cuda_tensor(a):
        return int(a.data_ptr())
    return int(a.ctypes.data) if a.size else 0


def _stream_of(t) -> int:
    import torch

    return int(torch.cuda.current_stream(t.device).cuda_stream)


def band_split(dry, freq_khz: Sequence[float] = DEFAULT_EQ_BANDS_KHZ, device: int = 0,
               chunked: bool = False):
    """``SoundFile::Band`` for all three bands: returns (low, mid, high),
    bit-identical to ``Equalizer::Split``.  ``freq_khz`` is the FREQ block
    (kHz, as the .EAR file stores it).  ``chunked`` evaluates the filters in
    parallel over 512-sample chunks: far faster for long sounds, as close
    to exact arithmetic as the sequential FP32 filters but not bit for bit
    (both drift up to ~1e-3 of the peak in the low band)."""
    f = (C.c_float * 3)(*[float(v) for v in freq_khz])
    L = N.lib()
    extra = N.EAR_SPLIT_CHUNKED if chunked else 0
    if _is_cuda_tensor(dry):
        import torch

        x = dry.contiguous().to(torch.float32)
        outs = [torch.empty_like(x) for _ in range(3)]
        N.check(L.ear_band_split(_ptr(x), x.numel(), f, _ptr(outs[0]), _ptr(outs[1]), _ptr(outs[2]),
                                 N.EAR_AURAL_DEVICE_MEMORY | extra, _stream_of(x),
                                 x.device.index or 0))
        return tuple(outs)
    x = _host(dry)
    outs = [np.empty_like(x) for _ in range(3)]
    N.check(L.ear_band_split(_ptr(x), x.size, f, _ptr(outs[0]), _ptr(outs[1]), _ptr(outs[2]),
                             extra, None, device))
    return tuple(outs)


@dataclass
class Track:
    """One recorder track as FloatBuffer keeps it: ``data`` (its buffer),
    ``first`` (first_sample) and ``length`` (real_length)."""
    data: object
    first: int
    length: int


@dataclass
class Context:
    """One RecorderContext applied to one track: ``ir`` convolved with the
    dry section ``dry`` landing at ``offset``; ``ir_next`` is the next
    keyframe's track for a keyframe pair."""
    ir: Track
    dry: object
    offset: int = 0
    ir_next: Optional[Track] = None


def section(signal, start_seconds: float, length_seconds: float = -1.0):
    """``SoundFile::Section(float, float)`` of a band with offset 0: returns
    (samples, offset)."""
    n = len(signal)
    start = int(np.float32(start_seconds) * np.float32(44100.0))
    if length_seconds < 0:
        length = n - start
    else:
        length = int(np.float32(length_seconds) * np.float32(44100.0))
    if start >= n:
        return signal[:0], 0
    return signal[start:start + min(length, n - start)], start


def _c_context(c: Context, keep: list) -> N.EarConvContext:
    def arr(x):
        if _is_cuda_tensor(x):
            keep.append(x)
            return x
        a = _host(x)
        keep.append(a)
        return a

    ir = arr(c.ir.data)
    e = N.EarConvContext()
    e.ir = _ptr(ir) or None
    e.ir_capacity = len(ir)
    e.ir_first = int(c.ir.first)
    e.ir_length = int(c.ir.length)
    if c.ir_next is not None:
        nx = arr(c.ir_next.data)
        e.ir_next = _ptr(nx) or None
        e.ir_next_capacity = len(nx)
        e.ir_next_first = int(c.ir_next.first)
        e.ir_next_length = int(c.ir_next.length)
        if e.ir_next is None:
            raise ValueError("a keyframe pair needs a next-keyframe track buffer")
    d = arr(c.dry)
    e.dry = _ptr(d) or None
    e.dry_length = len(d)
    e.offset = int(c.offset)
    return e


def processed_capacity(c: Context, mode: str = "fft") -> int:
    """Capacity of the FloatBuffer RecorderTrack::Process returns for `c`."""
    keep: list = []
    e = _c_context(c, keep)
    return int(N.lib().ear_conv_processed_capacity(C.byref(e), MODES[mode]))


def convolve(contexts: Sequence[Context], mode: str = "fft", out=None, out_length=None,
             device: int = 0):
    """Sum of RecorderTrack::Process over `contexts` (in order), as
    Recorder::Add forms one processed recorder track.  Returns (out, stats).

    ``out`` (optional) is added to; by default a zero track of ``out_length``
    samples, which defaults to the largest processed capacity (the reference's
    processed track then ends one sample earlier: its real_length).  mode
    "direct" is bit-identical to the reference built without FFTW; "fft"
    follows the FFTW build to FP32 transform accuracy."""
    if mode not in MODES:
        raise ValueError(f"mode must be one of {sorted(MODES)}")
    keep: list = []
    arr = (N.EarConvContext * max(len(contexts), 1))()
    for i, c in enumerate(contexts):
        arr[i] = _c_context(c, keep)
    L = N.lib()
    if out_length is None:
        out_length = max((int(L.ear_conv_processed_capacity(C.byref(arr[i]), MODES[mode]))
                          for i in range(len(contexts))), default=0)
    on_dev = any(_is_cuda_tensor(x) for x in keep) or _is_cuda_tensor(out)
    st = N.EarConvStats()
    if on_dev:
        import torch

        if not all(_is_cuda_tensor(x) for x in keep):
            raise TypeError("mix of host and device buffers: pass all numpy or all CUDA tensors")
        dev = next(x.device for x in keep)
        if out is None:
            out = torch.zeros(int(out_length), dtype=torch.float32, device=dev)
        N.check(L.ear_convolve(arr, len(contexts), MODES[mode], _ptr(out), out.numel(),
                               N.EAR_AURAL_DEVICE_MEMORY, _stream_of(out), dev.index or 0,
                               C.byref(st)))
    else:
        if out is None:
            out = np.zeros(int(out_length), np.float32)
        elif out.dtype != np.float32 or not out.flags.c_contiguous:
            raise TypeError("out must be a contiguous float32 array")
        N.check(L.ear_convolve(arr, len(contexts), MODES[mode], _ptr(out), out.size, 0, None,
                               device, C.byref(st)))
    stats = {"kernel_ms": st.kernel_ms, "launches": st.launches, "fft_points": st.fft_points,
             "multiply_adds": st.multiply_adds}
    return out, stats


def convolve_tracks(contexts: Sequence[Context], tracks: Sequence[int], mode: str = "fft",
                    outs=None, out_lengths=None, device: int = 0):
    """``convolve`` for several output tracks in one call: context i is added
    to output track ``tracks[i]`` (each track's contexts in their order).
    ``outs`` (optional) are added to; by default zero tracks whose lengths
    (``out_lengths``, default: each track's largest processed capacity) are
    as ``convolve`` picks them.  Returns (list of outputs, stats)."""
    if mode not in MODES:
        raise ValueError(f"mode must be one of {sorted(MODES)}")
    if len(tracks) != len(contexts):
        raise ValueError("one track index per context")
    num_tracks = (max(tracks) + 1 if len(tracks) else 0) if outs is None else len(outs)
    keep: list = []
    arr = (N.EarConvContext * max(len(contexts), 1))()
    for i, c in enumerate(contexts):
        arr[i] = _c_context(c, keep)
    L = N.lib()
    if out_lengths is None:
        out_lengths = [0] * num_tracks
        for i, t in enumerate(tracks):
            out_lengths[t] = max(out_lengths[t],
                                 int(L.ear_conv_processed_capacity(C.byref(arr[i]), MODES[mode])))
    on_dev = any(_is_cuda_tensor(x) for x in keep)
    if outs is None:
        if on_dev:
            import torch

            dev = next(x.device for x in keep if _is_cuda_tensor(x))
            outs = [torch.zeros(int(n), dtype=torch.float32, device=dev) for n in out_lengths]
        else:
            outs = [np.zeros(int(n), np.float32) for n in out_lengths]
    if on_dev and not all(_is_cuda_tensor(x) for x in list(keep) + list(outs)):
        raise TypeError("mix of host and device buffers: pass all numpy or all CUDA tensors")
    tr = np.ascontiguousarray(np.asarray(tracks, np.int32))
    ptrs = (C.c_void_p * max(num_tracks, 1))(*[_ptr(o) or None for o in outs])
    lens = (C.c_int64 * max(num_tracks, 1))(*[int(len(o)) for o in outs])
    st = N.EarConvStats()
    if on_dev:
        dev_index = next(x.device for x in keep if _is_cuda_tensor(x)).index or 0
        N.check(L.ear_convolve_tracks(arr, tr.ctypes.data, len(contexts), MODES[mode], ptrs, lens,
                                      num_tracks, N.EAR_AURAL_DEVICE_MEMORY, _stream_of(outs[0]),
                                      dev_index, C.byref(st)))
    else:
        N.check(L.ear_convolve_tracks(arr, tr.ctypes.data, len(contexts), MODES[mode], ptrs, lens,
                                      num_tracks, 0, None, device, C.byref(st)))
    stats = {"kernel_ms": st.kernel_ms, "launches": st.launches, "fft_points": st.fft_points,
             "multiply_adds": st.multiply_adds}
    return list(outs), stats
